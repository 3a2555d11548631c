/*
 * cl_runner.c -- CPU executor for a kernel rendered from myokit's
 * openclsim.cl, driven by a C restatement of the reference host loop.
 *
 * TEST INFRASTRUCTURE (the oracle): used only by tests/, smoke() and the
 * CPU baseline of bench.py, never by the product.
 *
 * Compiled once per kernel source:
 *   gcc -O2 -std=gnu99 -fPIC -shared -fopenmp -ffp-contract=off
 *       -DORC_KERNEL='"<kernel>.cl"' -DORC_DIFF=<0..3> cl_runner.c -lm
 * where ORC_DIFF selects the diffusion kernel the rendered source contains:
 * 0 none, 1 diff_step, 2 diff_hetero, 3 diff_arb_reset/diff_arb_step.
 *
 * Restated from the reference:
 *   - event pacing:           myokit/_sim/pacing.h:69-80, 168-212, 340-600
 *   - sim_init buffers:       myokit/_sim/openclsim.c:488-560
 *   - sim_step loop:          myokit/_sim/openclsim.c:1036-1211
 * Each NDRange launch becomes a loop over work items (OpenMP over cells for
 * the cell and grid-diffusion kernels; the connection kernel, whose float
 * atomics make the sum order arbitrary, runs serially in connection order
 * so that the oracle is deterministic).
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_shim.h"
#include ORC_KERNEL

#ifndef ORC_DIFF
#error "ORC_DIFF must be defined"
#endif

__thread unsigned long orc_gid[2];

/* ------------------------------------------------------------------------ */
/* Event pacing (pacing.h)                                                  */
/* ------------------------------------------------------------------------ */

typedef struct {
    double level, duration, start, period, multiplier;
    int next;
} OrcEvent;

static OrcEvent *ev = NULL;
static int n_ev = 0;
static int ev_head = -1, ev_fire = -1;
static double ev_time, ev_tnext, ev_tdown, ev_level;

#define ORC_PACE_SIMULTANEOUS -50
#define ORC_PACE_NEGATIVE_INCREMENT -40

static int orc_eq(double a, double b)
{
    double s;
    if (a == b) return 1;
    s = fabs(a) > fabs(b) ? fabs(a) : fabs(b);
    return fabs(a - b) / s < DBL_EPSILON;
}

static int orc_geq(double a, double b) { return a >= b || orc_eq(a, b); }

/* Queue insertion after all events starting no later (pacing.h:192-212) */
static int orc_schedule(int head, int i, int *err)
{
    int e;
    ev[i].next = -1;
    if (head < 0) return i;
    if (ev[i].start < ev[head].start) {
        ev[i].next = head;
        return i;
    }
    e = head;
    while (ev[e].next >= 0 && ev[i].start >= ev[ev[e].next].start)
        e = ev[e].next;
    if (ev[i].start == ev[e].start) *err = ORC_PACE_SIMULTANEOUS;
    ev[i].next = ev[e].next;
    ev[e].next = i;
    return head;
}

static int orc_pace_advance(double t)
{
    int err = 0;
    if (t < ev_time) return ORC_PACE_NEGATIVE_INCREMENT;
    ev_time = t;
    while (orc_geq(ev_time, ev_tnext)) {
        if (ev_fire >= 0 && orc_geq(ev_tnext, ev_tdown)) {
            ev_fire = -1;
            ev_level = 0;
        }
        if (ev_head >= 0 && orc_geq(ev_tnext, ev[ev_head].start)) {
            OrcEvent *f;
            ev_fire = ev_head;
            f = &ev[ev_fire];
            ev_head = f->next;
            ev_tdown = f->start + f->duration;
            ev_level = f->level;
            if (f->period > 0) {
                if (f->multiplier != 1) {
                    if (f->multiplier > 1) f->multiplier -= 1;
                    f->start += f->period;
                    ev_head = orc_schedule(ev_head, ev_fire, &err);
                    if (err) return err;
                } else {
                    f->period = 0;
                }
            }
            if (ev_head >= 0 && orc_eq(ev[ev_head].start, ev_tdown))
                ev_tdown = ev[ev_head].start;
        }
        ev_tnext = HUGE_VAL;
        if (ev_fire >= 0 && ev_tnext > ev_tdown) ev_tnext = ev_tdown;
        if (ev_head >= 0 && ev_tnext > ev[ev_head].start)
            ev_tnext = ev[ev_head].start;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Simulation state (openclsim.c globals)                                   */
/* ------------------------------------------------------------------------ */

static unsigned long nx, ny, ncell;
static Real *state = NULL, *idiff = NULL, *inter = NULL, *field = NULL;
static Real *gxv = NULL, *gyv = NULL;
static unsigned long *conn1 = NULL, *conn2 = NULL;
static Real *conng = NULL;
static unsigned long nconn = 0;
static Real arg_gx, arg_gy;
static double tmin_, tmax_, default_dt, log_interval_;
static double engine_time, engine_pace, tnext_pace, tnext_log;
static unsigned long istep, inext_log;
static int halt;
static int nthreads = 1;

/* Log columns: kind 0 time, 1 pace, 2 idiff[index], 3 state[index],
 * 4 inter[index] (openclsim.c:935-1001) */
static int *log_kind = NULL;
static long *log_index = NULL;
static long nlog = 0;
static int logging_states = 0;
static double *rows = NULL;
static long nrows = 0, cap_rows = 0;
static double *state_snap = NULL;

static void orc_free_all(void)
{
    free(ev); ev = NULL; n_ev = 0;
    free(state); state = NULL;
    free(idiff); idiff = NULL;
    free(inter); inter = NULL;
    free(field); field = NULL;
    free(gxv); gxv = NULL;
    free(gyv); gyv = NULL;
    free(conn1); conn1 = NULL;
    free(conn2); conn2 = NULL;
    free(conng); conng = NULL;
    free(log_kind); log_kind = NULL;
    free(log_index); log_index = NULL;
    free(rows); rows = NULL;
    free(state_snap); state_snap = NULL;
    nrows = cap_rows = 0;
}

void orc_clean(void) { orc_free_all(); }

int orc_n_state(void) { return n_state; }
int orc_n_inter(void) { return n_inter; }
int orc_n_field(void) { return n_field; }
int orc_real_bytes(void) { return (int)sizeof(Real); }

/*
 * Mirrors sim_init (openclsim.c:309-1031) for already-parsed arguments.
 * events: n_events rows of (level, start, duration, period, multiplier).
 */
int orc_init(long nx_in, long ny_in, double gx, double gy,
             const double *gxf, long ngx, const double *gyf, long ngy,
             const long *c1, const long *c2, const double *cg, long nc,
             double tmin, double tmax, double dt, double log_interval,
             const double *state_in, const double *field_data, long nfield,
             const double *events, long n_events, const int *kinds,
             const long *indices, long n_log, int threads)
{
    long i;
    int err = 0;
    orc_free_all();
    nx = (unsigned long)nx_in;
    ny = (unsigned long)ny_in;
    ncell = nx * ny;
    nthreads = threads > 0 ? threads : 1;
    arg_gx = (Real)gx;
    arg_gy = (Real)gy;
    tmin_ = tmin;
    tmax_ = tmax;
    default_dt = dt;
    log_interval_ = log_interval;

    /* Pacing (ESys_Create/Populate/AdvanceTime, openclsim.c:488-496) */
    n_ev = (int)n_events;
    ev = (OrcEvent *)calloc(n_ev > 0 ? n_ev : 1, sizeof(OrcEvent));
    for (i = 0; i < n_events; i++) {
        ev[i].level = events[5 * i + 0];
        ev[i].start = events[5 * i + 1];
        ev[i].duration = events[5 * i + 2];
        ev[i].period = events[5 * i + 3];
        ev[i].multiplier = events[5 * i + 4];
        ev[i].next = -1;
    }
    ev_head = -1;
    ev_fire = -1;
    for (i = 0; i < n_events; i++) {
        ev_head = orc_schedule(ev_head, (int)i, &err);
        if (err) return err;
    }
    ev_time = ev_tnext = ev_tdown = tmin;
    ev_level = 0;
    err = orc_pace_advance(tmin);
    if (err) return err;
    tnext_pace = ev_tnext;
    engine_pace = ev_level;
    engine_time = tmin;

    /* Vectors (openclsim.c:510-560) */
    state = (Real *)malloc(ncell * n_state * sizeof(Real));
    for (i = 0; i < (long)(ncell * n_state); i++) state[i] = (Real)state_in[i];
    idiff = (Real *)calloc(ncell, sizeof(Real));
    inter = (Real *)calloc(ncell * (n_inter > 0 ? n_inter : 1), sizeof(Real));
    field = (Real *)calloc(nfield > 0 ? nfield : 1, sizeof(Real));
    for (i = 0; i < nfield; i++) field[i] = (Real)field_data[i];
    gxv = (Real *)calloc(ngx > 0 ? ngx : 1, sizeof(Real));
    gyv = (Real *)calloc(ngy > 0 ? ngy : 1, sizeof(Real));
    for (i = 0; i < ngx; i++) gxv[i] = (Real)gxf[i];
    for (i = 0; i < ngy; i++) gyv[i] = (Real)gyf[i];
    nconn = (unsigned long)nc;
    conn1 = (unsigned long *)calloc(nc > 0 ? nc : 1, sizeof(unsigned long));
    conn2 = (unsigned long *)calloc(nc > 0 ? nc : 1, sizeof(unsigned long));
    conng = (Real *)calloc(nc > 0 ? nc : 1, sizeof(Real));
    for (i = 0; i < nc; i++) {
        conn1[i] = (unsigned long)c1[i];
        conn2[i] = (unsigned long)c2[i];
        conng[i] = (Real)cg[i];
    }

    /* Logging */
    nlog = n_log;
    log_kind = (int *)malloc((n_log > 0 ? n_log : 1) * sizeof(int));
    log_index = (long *)malloc((n_log > 0 ? n_log : 1) * sizeof(long));
    state_snap = (double *)malloc((n_log > 0 ? n_log : 1) * sizeof(double));
    logging_states = 0;
    for (i = 0; i < n_log; i++) {
        log_kind[i] = kinds[i];
        log_index[i] = indices[i];
        if (kinds[i] == 3) logging_states = 1;
    }
    istep = 1;
    inext_log = 0;
    tnext_log = tmin;
    halt = 0;
    return 0;
}

static void orc_add_row(void)
{
    long j;
    double *r;
    if (nrows == cap_rows) {
        cap_rows = cap_rows ? 2 * cap_rows : 64;
        rows = (double *)realloc(rows, cap_rows * (nlog > 0 ? nlog : 1) *
                                           sizeof(double));
    }
    r = rows + nrows * nlog;
    for (j = 0; j < nlog; j++) {
        switch (log_kind[j]) {
        case 0: r[j] = (double)(Real)engine_time; break;
        case 1: r[j] = (double)(Real)engine_pace; break;
        case 2: r[j] = (double)idiff[log_index[j]]; break;
        case 3: r[j] = state_snap[j]; break;
        default: r[j] = (double)inter[log_index[j]]; break;
        }
    }
    nrows++;
}

/*
 * Runs at most max_steps steps (sim_step, openclsim.c:1036-1177).
 * Returns 0 to continue, 1 when tmax is reached, 2 on the NaN halt, or a
 * negative pacing error. *t_out receives the engine time.
 */
int orc_step(long max_steps, double *t_out)
{
    long left = max_steps;
    while (1) {
        const int logging = engine_time >= tnext_log;
        int intermediary = 0;
        double dt = tmin_ + (double)istep * default_dt - engine_time;
        double d = tmax_ - engine_time;
        const Real arg_time = (Real)engine_time;
        Real arg_dt, arg_pace;
        long c, j;
        int err;
        if (d > 0 && d < dt) { dt = d; intermediary = 1; }
        d = tnext_pace - engine_time;
        if (d > 0 && d < dt) { dt = d; intermediary = 1; }
        d = tnext_log - engine_time;
        if (d > 0 && d < dt) { dt = d; intermediary = 1; }
        if (!intermediary) istep++;
        arg_dt = (Real)dt;
        arg_pace = (Real)engine_pace;

        /* Diffusion current at t */
#if ORC_DIFF == 1
        #pragma omp parallel for num_threads(nthreads) schedule(static)
        for (c = 0; c < (long)ncell; c++) {
            orc_gid[0] = (unsigned long)c % nx;
            orc_gid[1] = (unsigned long)c / nx;
            diff_step(nx, ny, arg_gx, arg_gy, state, idiff);
        }
#elif ORC_DIFF == 2
        #pragma omp parallel for num_threads(nthreads) schedule(static)
        for (c = 0; c < (long)ncell; c++) {
            orc_gid[0] = (unsigned long)c % nx;
            orc_gid[1] = (unsigned long)c / nx;
            diff_hetero(nx, ny, gxv, gyv, state, idiff);
        }
#elif ORC_DIFF == 3
        for (c = 0; c < (long)ncell; c++) {
            orc_gid[0] = (unsigned long)c;
            orc_gid[1] = 0;
            diff_arb_reset(ncell, idiff);
        }
        for (c = 0; c < (long)nconn; c++) {
            orc_gid[0] = (unsigned long)c;
            orc_gid[1] = 0;
            diff_arb_step(nconn, conn1, conn2, conng, state, idiff);
        }
#endif

        /* States at t for the log, and the NaN check on the first entry
         * (openclsim.c:1080-1089) */
        if (logging) {
            for (j = 0; j < nlog; j++)
                if (log_kind[j] == 3)
                    state_snap[j] = (double)state[log_index[j]];
            if (logging_states && isnan(state[0])) halt = 1;
        }

        /* Cell kernel: intermediaries at t, states to t + dt */
        #pragma omp parallel for num_threads(nthreads) schedule(static)
        for (c = 0; c < (long)ncell; c++) {
            orc_gid[0] = (unsigned long)c % nx;
            orc_gid[1] = (unsigned long)c / nx;
            cell_step(nx, ny, arg_time, arg_dt, arg_pace, state, idiff,
                      inter, field);
        }

        if (logging) {
            orc_add_row();
            inext_log++;
            tnext_log = tmin_ + (double)inext_log * log_interval_;
        }

        engine_time += dt;
        err = orc_pace_advance(engine_time);
        if (err) return err;
        tnext_pace = ev_tnext;
        engine_pace = ev_level;

        if (engine_time >= tmax_ || halt) break;
        if (--left == 0) {
            *t_out = engine_time;
            return 0;
        }
    }
    *t_out = engine_time;
    return halt ? 2 : 1;
}

long orc_rows(void) { return nrows; }

/* Copies the buffered log rows (rows x nlog) and empties the buffer. */
void orc_take_rows(double *out)
{
    if (nrows > 0 && nlog > 0)
        memcpy(out, rows, nrows * nlog * sizeof(double));
    nrows = 0;
}

void orc_get_state(double *out)
{
    unsigned long i;
    for (i = 0; i < ncell * n_state; i++) out[i] = (double)state[i];
}

/*
 * mkg_tissue.h -- C ABI of the GB300 tissue-simulation host library.
 *
 * This library replaces the per-simulation CPython module that myokit
 * generates from myokit/_sim/openclsim.c (module methods sim_init, sim_step
 * and sim_clean, openclsim.c:1216-1221) and the OpenCL runtime calls made
 * inside it. The arguments of sim_init (openclsim.c:385-407) are split over
 * one call per input so that every buffer crosses the boundary once, as a
 * plain pointer plus a size, instead of as a Python list of floats.
 *
 * Conventions
 *  - Every function returns an int status: MKG_OK (0), a positive run status
 *    (mkg_run_chunk only) or a negative error code. No function aborts.
 *  - After an error, mkg_last_error() returns a message for the handle (or
 *    for the thread, when no handle was created).
 *  - Host arrays are read or written only during the call; the library keeps
 *    no pointer to caller memory.
 *  - State vectors are "array of structures" doubles with the x index
 *    running fastest, the layout used by SimulationOpenCL.state()
 *    (openclsim.py:1727-1757). The device stores them as structure of arrays.
 *  - One handle owns one CUDA stream and its device buffers. A handle is not
 *    thread safe; different handles may be used from different threads.
 */
#ifndef MKG_TISSUE_H
#define MKG_TISSUE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes */
#define MKG_OK              0
#define MKG_DONE            1   /* run reached tmax (sim_step's final return) */
#define MKG_HALT_NAN        2   /* NaN halt: openclsim.c:1086-1089, 1199-1204 */
#define MKG_ERR_ARG        -1   /* invalid argument or size */
#define MKG_ERR_CUDA       -2   /* CUDA runtime error */
#define MKG_ERR_COMPILE    -3   /* NVRTC compilation failed (log in mkg_last_error) */
#define MKG_ERR_PACING     -4   /* invalid protocol (pacing.h ESys_POPULATE_*) */
#define MKG_ERR_TIMEOUT    -5   /* a bounded device-side wait ran out */
#define MKG_ERR_ORDER      -6   /* call made in the wrong order */
#define MKG_ERR_SIMULTANEOUS -7 /* two events at the same time (pacing.h:204-206) */
#define MKG_ERR_NOMEM      -8   /* host or device allocation failed */

/* Diffusion modes, one per reference kernel (openclsim.cl:384-573) */
#define MKG_DIFF_NONE       0   /* diffusion=False */
#define MKG_DIFF_GRID       1   /* diff_step: homogeneous 1D/2D grid */
#define MKG_DIFF_HETERO     2   /* diff_hetero: per-edge conductances */
#define MKG_DIFF_CONN       3   /* diff_arb_step: arbitrary connections */

/* Pacing modes (calculate_pacing, openclsim.cl:249-280, 325-330) */
#define MKG_PACE_ALL        0   /* diffusion disabled: every cell gets pace */
#define MKG_PACE_RECT       1   /* rectangle from set_paced_cells */
#define MKG_PACE_LIST       2   /* explicit cell list from set_paced_cell_list */
#define MKG_PACE_NONE       3   /* diffusion enabled, empty list: pace 0 */

/* Log items: what one log column records (openclsim.c:916-1022) */
#define MKG_ITEM_IDIFF(n_state)       (n_state)
#define MKG_ITEM_INTER(n_state, k)    ((n_state) + 1 + (k))

typedef struct mkg_sim mkg_sim;

/* Configuration fixed when the simulation program is built. */
typedef struct mkg_config {
    int64_t nx;             /* cells in x (sim_init nx, openclsim.c:389) */
    int64_t ny;             /* cells in y; 1 for 1D (openclsim.c:390) */
    int32_t real_bytes;     /* 4 = single, 8 = double precision */
    int32_t n_state;        /* states per cell (openclsim.cl "n_state") */
    int32_t n_inter;        /* logged intermediaries the kernel writes */
    int32_t n_field;        /* scalar fields (openclsim.cl "n_field") */
    int32_t i_vm;           /* index of V in the state; -1 without diffusion */
    int32_t diffusion;      /* MKG_DIFF_* */
    int32_t block_x;        /* CTA shape the kernel was generated for */
    int32_t block_y;
    int32_t device;         /* CUDA device ordinal */
    int32_t two_d;          /* 1: kernel tiles an (nx, ny) grid with
                               (block_x, block_y) CTAs; 0: cells are a
                               flat array covered by (block_x, 1) CTAs */
    int32_t hi_mode;        /* single precision only: 0 none, 1 selected
                               states stored and updated in FP64, 2 selected
                               states carry an FP32 Kahan compensation term */
    int32_t n_hi;           /* number of selected states (mkg_set_hi_states) */
    int32_t stage;          /* 1: the kernel copies each warp tile's inputs
                               into shared memory with TMA tensor copies and
                               takes the tensor maps as a second parameter;
                               2: the same with two buffers per warp (the
                               copies of the tile after the next run while
                               a tile computes); the dynamic shared memory
                               per CTA is warps x stage x bytes + 128 */
    int32_t v_double;       /* 1: V is stored and updated in FP64 (hi_mode 1
                               with V among the selected states) */
    int32_t split;          /* warps per warp tile (1, 2, 4, 8 or 16): the
                               kernel divides each tile's state updates
                               among that many warps, of one CTA or, when
                               more than the CTA holds, of a cluster of
                               whole CTAs (at most 8; 0 is taken as 1) */
} mkg_config;

/*
 * Shared-memory layout of a staged warp tile for this configuration, as the
 * library lays out its tensor copies: out[0] tile width (cells), out[1]
 * first staged state plane, out[2] staged state planes, out[3] staged V
 * rows, out[4] 1 if 1D conductances are staged, out[5] bytes of shared
 * memory per warp, out[6] bytes the copies of one tile deliver. All zero
 * when cfg->stage is 0. Needs no GPU. No counterpart in the reference.
 */
int mkg_stage_layout(const mkg_config *cfg, int64_t *out);

/*
 * Bounds every device-side wait of the step kernel (the grid barrier or the
 * waits on neighbouring warps between steps, and the tile-copy waits) to
 * timeout_ns (1 ms .. 60 s; default 2 s). A wait that runs out records
 * MKG_DEV_TIMEOUT, every block leaves the kernel, and mkg_run_chunk returns
 * MKG_ERR_TIMEOUT with the context still usable. skew (0 .. 65536) > 0
 * raises the target of every step wait so that it cannot be reached: a way
 * to exercise that path from the host (0 restores normal runs). No
 * counterpart in the reference.
 */
int mkg_set_wait(mkg_sim *sim, int64_t timeout_ns, int32_t skew);

/*
 * Couples a fiber simulation (sim, whose kernel is a fused fiber-tissue
 * kernel) to a tissue simulation (partner): from then on mkg_run_chunk on
 * sim advances both in one launch per chunk, with the junction current
 * gft (Vf - Vt) between fiber cell (nx - 1, y) and tissue cell (0, cty + y)
 * for every fiber row y. The partner's log rows of a chunk are read with
 * mkg_read_log(partner, ...). Replaces the two diff_step launches, the
 * diff_step_fiber_tissue launch and the two cell_step launches of each step
 * of the reference's fiber-tissue loop (fiber_tissue.c:1003-1130,
 * openclsim.cl:601-628). A NULL partner uncouples.
 */
int mkg_set_partner(mkg_sim *sim, mkg_sim *partner, double gft,
                    int64_t cty);

/*
 * Compiles generated CUDA C++ source to an sm_103a cubin with NVRTC.
 * Replaces clCreateProgramWithSource + clBuildProgram (openclsim.c:812-839).
 * On success *cubin (size *cubin_size) and *log are malloc'd; free them with
 * mkg_free. On a compile failure the return is MKG_ERR_COMPILE and *log
 * holds the compiler output.
 */
int mkg_compile(const char *source, const char *name,
                const char *const *options, int n_options,
                void **cubin, size_t *cubin_size, char **log);
void mkg_free(void *ptr);

/*
 * Creates a simulation from a cubin produced by mkg_compile. Allocates the
 * device buffers (openclsim.c:741-809). The kernel entry point must be named
 * "mkg_tissue_step".
 */
int mkg_create(const mkg_config *cfg, const void *cubin, size_t cubin_size,
               mkg_sim **sim);

/* Frees everything; safe on NULL and on a handle after any error.
 * Replaces sim_clean (openclsim.c:216-292). */
void mkg_destroy(mkg_sim *sim);

/* Last error message for this handle, or for the calling thread when sim is
 * NULL. Never returns NULL. */
const char *mkg_last_error(const mkg_sim *sim);

/* The states kept in the accumulation planes when cfg.hi_mode != 0, in
 * plane order (n == cfg.n_hi). Must be called before mkg_set_state. No
 * counterpart in the reference, which stores every state in one precision
 * (openclsim.cl:158-169). */
int mkg_set_hi_states(mkg_sim *sim, const int32_t *states, int32_t n);

/* Cell state, AoS doubles, n = nx*ny*n_state (state_in, openclsim.c:512-521;
 * state_out, openclsim.c:1185-1190). */
int mkg_set_state(mkg_sim *sim, const double *state, int64_t n);
int mkg_get_state(mkg_sim *sim, double *state, int64_t n);

/*
 * mkg_set_state, without any allocation. No counterpart in the reference:
 * its CPython module always allocates (openclsim.c uses malloc and
 * clCreateBuffer per run).
 *
 * mkg_set_state stages the doubles in a device buffer that the handle
 * allocates with cudaMalloc the first time. Some callers must not call
 * cudaMalloc where they upload a state: a host loop that paces a tissue in
 * real time (cudaMalloc can synchronise the whole device and stall every
 * stream), or a host that keeps device memory in its own pool or under a
 * fixed budget (a cudaMalloc outside that pool can fail). They use this
 * call: it stages through a fixed 16 MiB array in the library's device
 * image (held on every GPU that loads the library until the process exits)
 * and calls no cudaMalloc, cudaFree or other allocating routine.
 *
 * - n must equal nx*ny*n_state and be at most 2,097,152 (16 MiB of
 *   doubles); larger states are rejected with MKG_ERR_ARG.
 * - The first call on a device looks up the array's device address
 *   (cudaGetSymbolAddress, with that device made current and then restored);
 *   make that first call before any stream capture.
 * - All handles share the array, which keeps the last call's contents;
 *   each call overwrites the part it uses before reading it. Calls whose
 *   GPU work overlaps (different streams, no ordering) race on it.
 */
int mkg_set_state_static(mkg_sim *sim, const double *state, int64_t n);

/* Scalar fields, cell-major interleaved: field_data[cell*n_field + k]
 * (openclsim.py:1082-1089, openclsim.cl:201). n = nx*ny*n_field. */
int mkg_set_fields(mkg_sim *sim, const double *field_data, int64_t n);

/* Homogeneous conductances gx, gy (sim_init gx/gy, openclsim.c:395-396). */
int mkg_set_conductance(mkg_sim *sim, double gx, double gy);

/* Per-edge conductances in the reference layout: gx has ny*(nx-1) entries,
 * gy has (ny-1)*nx (openclsim.py:1380-1384, openclsim.cl:452-487). */
int mkg_set_conductance_field(mkg_sim *sim, const double *gx, int64_t ngx,
                              const double *gy, int64_t ngy);

/* Connections (cell1[i], cell2[i], g[i]) as validated by
 * SimulationOpenCL.set_connections (openclsim.py:1387-1449). Stored as a
 * per-cell neighbour list so each cell sums its currents in a fixed order. */
int mkg_set_connections(mkg_sim *sim, const int64_t *cell1,
                        const int64_t *cell2, const double *g, int64_t n);

/* Paced cells (calculate_pacing, openclsim.cl:249-280). */
int mkg_set_pacing_mode(mkg_sim *sim, int32_t mode);
int mkg_set_paced_rect(mkg_sim *sim, int64_t nx, int64_t ny, int64_t x,
                       int64_t y);
int mkg_set_paced_list(mkg_sim *sim, const int64_t *cells, int64_t n);

/* Protocol events, n rows of (level, start, duration, period, multiplier),
 * the attributes ESys_Populate reads (pacing.h:340-470). */
int mkg_set_protocol(mkg_sim *sim, const double *events, int64_t n);

/* Logged per-cell columns: column j records item[j] of cell[j]. item is a
 * state index, MKG_ITEM_IDIFF or MKG_ITEM_INTER (openclsim.c:941-1001).
 * nan_check = 1 applies the reference's NaN halt, which looks at the first
 * state entry at every log point when states are logged (openclsim.c:1080-
 * 1089). */
int mkg_set_log(mkg_sim *sim, const int32_t *item, const int64_t *cell,
                int64_t ncol, int32_t nan_check);

/* Starts a run over [tmin, tmax) with the given default step and log
 * interval (the scalar arguments of sim_init, openclsim.c:397-403, and its
 * pacing set-up, openclsim.c:488-496). */
int mkg_run_begin(mkg_sim *sim, double tmin, double tmax, double default_dt,
                  double log_interval);

/*
 * Advances the run by at most max_steps steps (sim_step, openclsim.c:1036-
 * 1211, with the reference's step-size schedule, pacing and logging). Sets
 * *t_out to the engine time reached and *rows_out to the log rows produced.
 * Returns MKG_OK while the run continues, MKG_DONE at tmax, MKG_HALT_NAN
 * after the reference's NaN halt, or a negative error.
 */
int mkg_run_chunk(mkg_sim *sim, int64_t max_steps, double *t_out,
                  int64_t *rows_out);

/* Copies the rows of the last chunk: time[r], pace[r] (the engine values
 * cast to the simulation precision, openclsim.c:1063, 1148-1155) and
 * values[r*ncol + j]. Any pointer may be NULL. */
int mkg_read_log(mkg_sim *sim, double *time, double *pace, double *values,
                 int64_t rows);

/* Launch tuning: steps fused into one launch (0 = the whole chunk in one
 * cooperative launch; 1 = one plain launch per step, no grid barrier),
 * blocks per SM for the cooperative grid (0 = occupancy maximum), and
 * whether a chunk's launches are captured once as a CUDA graph and
 * replayed (use_graphs != 0). */
int mkg_set_tuning(mkg_sim *sim, int32_t steps_per_launch,
                   int32_t blocks_per_sm, int32_t use_graphs);

/* Timing and counters of the last chunk: device milliseconds spent in
 * step kernels, number of kernel launches and cell-steps computed. */
int mkg_last_stats(const mkg_sim *sim, double *kernel_ms, int64_t *launches,
                   int64_t *cell_steps);

/*
 * Discrete adjoint (no counterpart in the reference, which has no
 * derivatives of its simulations). For a loss on logged V values it gives
 * the exact gradients of the discrete forward map with respect to the
 * scalar fields and to gx, gy.
 *
 * mkg_adj_attach loads the module generated by myokit_gb300.adjoint (the
 * forward kernel with trajectory output and the reverse kernel) and sets
 * the checkpoint segment length. mkg_adj_forward runs [tmin, tmax) like
 * mkg_run_begin + mkg_run_chunk, keeping a checkpoint every seg_steps steps
 * and all log rows (mkg_adj_read_log, rows x ncol). mkg_adj_backward takes
 * dL/d(log value) (rows x ncol; every column must log V) and writes the
 * field gradients (AoS, ncell x n_field) and dL/dgx, dL/dgy. Every
 * diffusion mode: with per-edge conductances or connections, dL/dgx is the
 * sum of the x-edge (or connection) gradients and dL/dgy of the y-edge
 * ones, and mkg_adj_conductance_gradient then gives each edge's gradient.
 * With an accumulation mode the forward and its recomputation run as the
 * simulation's own kernel; the reverse sweep runs in the kernel precision.
 */
int mkg_adj_attach(mkg_sim *sim, const void *cubin, size_t size,
                   int32_t seg_steps);
int mkg_adj_forward(mkg_sim *sim, double tmin, double tmax, double dt,
                    double log_interval, int64_t *rows);
int mkg_adj_read_log(mkg_sim *sim, double *values, int64_t rows);
int mkg_adj_backward(mkg_sim *sim, const double *lgrad, int64_t rows,
                     double *grad_fields, double *grad_g);

/*
 * After mkg_adj_backward: dL/dg of every edge. Per-edge conductances
 * (diff_hetero, openclsim.cl:452-487; layout of sim_init's gx_field and
 * gy_field, openclsim.py:1380-1384): n = ny*(nx-1) x-edges, then
 * (ny-1)*nx y-edges in 2D. Connections (diff_arb_step,
 * openclsim.cl:537-556; the list of mkg_set_connections): n = number of
 * connections, in their order. Other diffusion modes: MKG_ERR_ARG.
 */
int mkg_adj_conductance_gradient(mkg_sim *sim, double *out, int64_t n);

/*
 * Device frame buffer: when set (rows > 0), log rows are written by the
 * kernel into dev_ptr (Real[rows][ncol], a device allocation owned by the
 * caller, filled from row 0 on) and never copied to the host; mkg_read_log
 * then returns times and pace only. For full-frame recordings (every cell's
 * V every few ms) that would not fit a host round trip. No counterpart in
 * the reference, which appends every logged value to a Python list
 * (openclsim.c:1122-1131). dev_ptr NULL / rows 0 switches it off.
 */
int mkg_set_frame_buffer(mkg_sim *sim, void *dev_ptr, int64_t rows);

/* The cudaStream_t (as void*) all work of this handle is queued on, so a
 * caller can time it with events recorded on the same stream. */
int mkg_stream(const mkg_sim *sim, void **stream);

/* Kernels this handle has launched since it was created (tissue steps,
 * layout and precision conversions). */
int mkg_launch_count(const mkg_sim *sim, int64_t *count);

/*
 * Host-only view of the step schedule that mkg_run_chunk follows: the first
 * at most max_steps steps of a run over [tmin, tmax) with the given protocol
 * (events as in mkg_set_protocol). Writes t, dt, pace and log (0/1) per step
 * and returns the number of steps (or a negative error). Needs no GPU; it
 * exists so the schedule can be checked against the reference's
 * (openclsim.c:1051-1162) on any machine.
 */
int64_t mkg_schedule_preview(const double *events, int64_t n_events,
                             double tmin, double tmax, double default_dt,
                             double log_interval, int64_t max_steps,
                             double *t, double *dt, double *pace,
                             int32_t *log);

#ifdef __cplusplus
}
#endif

#endif /* MKG_TISSUE_H */

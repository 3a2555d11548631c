/*
 * mkg_kernel_abi.h -- argument block shared by the host library and the
 * generated tissue kernels. Included by mkg_host.cu and prepended (as text)
 * to every generated kernel compiled with NVRTC, so both sides agree on the
 * layout. Plain C types only (and C++11 alignas): NVRTC compiles it
 * without system headers.
 */
#ifndef MKG_KERNEL_ABI_H
#define MKG_KERNEL_ABI_H

/* Device error codes written to mkg_status.error */
#define MKG_DEV_OK        0
#define MKG_DEV_TIMEOUT   1   /* grid barrier wait exceeded timeout_ns */
#define MKG_DEV_STAGE     2   /* tile staging: the host's layout differs from
                                 the kernel's, or a copy wait timed out */
#define MKG_DEV_LAUNCH    3   /* the launch's cluster shape differs from the
                                 kernel's */

#define MKG_NO_HALT 0x7fffffff

/* One time step of the schedule, computed on the host exactly as the
 * reference's sim_step loop does (openclsim.c:1051-1063). The kernel casts
 * t, dt and pace to its Real type, as the reference casts its kernel
 * arguments (openclsim.c:1063, 1148, 1155). */
typedef struct mkg_step {
    double t;          /* engine time at the start of the step */
    double dt;         /* step size */
    double pace;       /* global pacing level during the step */
    float tf, dtf, pacef;  /* the same, rounded to single precision on the
                              host (what a single precision kernel uses) */
    int log_row;       /* row of the chunk log written at this step, or -1 */
} mkg_step;

/* Device-side status word, one per simulation. */
typedef struct mkg_status {
    unsigned int barrier;   /* grid barrier arrival counter (reset per chunk) */
    int error;              /* MKG_DEV_* */
    int halt_step;          /* first step of the chunk that saw the NaN halt */
    int timeout_block;      /* block that gave up waiting, for diagnostics */
} mkg_status;

/* Everything a tissue step launch needs. Passed by value. */
typedef struct mkg_launch {
    long long nx, ny;        /* grid shape */
    long long ncell;         /* nx * ny */
    long long pitch;         /* cells per plane in the SoA buffers */
    void *state;             /* Real[n_state][pitch] */
    void *vbuf;              /* Real[2][pitch]: V(t) and V(t+dt) ping-pong */
    const void *field;       /* Real[n_field][pitch] */
    const void *gx;          /* heterogeneous x conductances, ny*(nx-1) */
    const void *gy;          /* heterogeneous y conductances, (ny-1)*nx */
    const int *nbr_ptr;      /* CSR row pointers, ncell + 1 */
    const int *nbr_idx;      /* CSR neighbour cell ids */
    const void *nbr_g;       /* CSR conductances (Real) */
    double gxs, gys;         /* homogeneous conductances */
    float gxf, gyf;          /* the same, rounded to single precision */
    long long pace_x0, pace_x1, pace_y0, pace_y1;  /* paced rectangle */
    const unsigned int *pace_bits;                 /* paced list bitmap */
    const mkg_step *steps;   /* nsteps schedule entries */
    void *log;               /* Real[rows][log_ncol] */
    const int *log_items;    /* item id of each logged item slot */
    const int *log_cols;     /* int[n_log_items][pitch]: column or -1 */
    mkg_status *status;
    long long timeout_ns;    /* bound on each grid barrier wait */
    int pace_mode;           /* MKG_PACE_* */
    int nsteps;              /* steps in this launch */
    int v_sel;               /* plane of vbuf holding V(t) at step 0 */
    int log_ncol;
    int n_log_items;
    int nan_check;           /* apply the NaN halt at log rows */
    int ntiles_x, ntiles_y;  /* warp tiles (32 cells) per row, and rows */
    int stage_tx;            /* bytes the tensor copies of one staged tile
                                deliver, as the host laid them out; 0 when
                                the kernel does not stage tiles */
    int step0;               /* index of this launch's first step within
                                the chunk (for the NaN halt) */
    int epoch_base;          /* grid barriers completed by earlier launches
                                of this chunk (the barrier counter is reset
                                once per chunk) */
    int wait_skew;           /* added to every step-wait target: 0, or > 0
                                to make the waits unreachable (a test of
                                the bounded-wait path) */
    void *hi;                /* accumulation planes [n_hi][pitch], 8 bytes
                                per entry: FP64 states, or FP32 Kahan
                                compensation terms */
    void *traj;              /* adjoint forward pass only: the states at t
                                of every step, Real[nsteps][n_state][pitch] */
    unsigned int *warp_epoch; /* neighbour synchronisation: steps completed
                                by each warp of the grid (reset per chunk) */
} mkg_launch;

/* An opaque TMA tensor map (CUtensorMap: 128 bytes, 64-byte aligned) */
typedef struct mkg_tmap {
    alignas(64) unsigned long long m[16];
} mkg_tmap;

/* Tensor maps of the arrays a staging kernel copies per warp tile; passed
 * as a second, __grid_constant__ kernel parameter. */
typedef struct mkg_tmaps {
    mkg_tmap state;          /* Real[n_state][pitch] */
    mkg_tmap hi;             /* accumulation planes [n_hi][pitch] */
    mkg_tmap field;          /* Real[n_field][pitch] */
    mkg_tmap v;              /* VReal[2][pitch] */
    mkg_tmap gx;             /* Real[nx - 1]: 1D heterogeneous conductances */
} mkg_tmaps;

/* The fiber-tissue junction: fiber cell (nfx - 1, y) and tissue cell
 * (0, cty + y), y < nfy, are coupled by the conductance gft. */
typedef struct mkg_junction {
    double gft;
    float gftf;              /* gft rounded to single precision */
    int nfy;
    long long cty;
} mkg_junction;

/* Arguments of the adjoint kernel: one checkpoint segment in reverse. */
typedef struct mkg_adj_launch {
    mkg_launch f;            /* geometry, fields, pacing, schedule, status */
    const void *traj;        /* Real[nsteps][n_state][pitch] */
    void *lam;               /* Real[n_state][pitch]: own part of lambda */
    void *mu;                /* Real[2][pitch]: dL/d idiff, double buffered */
    void *gfield;            /* Real[n_field][pitch]: field gradients */
    void *gg;                /* Real[2][pitch]: dL/dgx and dL/dgy per cell */
    const int *probe_col;    /* int[pitch]: loss column of a cell or -1 */
    const void *lgrad;       /* Real[rows][nprobe]: dL/dV at logged points */
    int nprobe;
    int mu_sel;              /* plane of mu holding mu_{k+1} at entry */
    double *ge;              /* per-edge conductance gradient parts, each
                                cell's own: heterogeneous grids
                                double[4][pitch] (the edge to the left,
                                right, down and up neighbour), connections
                                double[n_nbr] (one per CSR entry) */
} mkg_adj_launch;

/* Accumulation modes for selected states of a single precision kernel */
#define MKG_HI_NONE   0
#define MKG_HI_DOUBLE 1   /* state stored and updated in FP64 */
#define MKG_HI_KAHAN  2   /* FP32 state plus FP32 compensation term */

#endif /* MKG_KERNEL_ABI_H */

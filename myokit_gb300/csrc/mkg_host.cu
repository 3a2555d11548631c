/*
 * mkg_host.cu -- host library behind include/mkg_tissue.h.
 *
 * Replaces the generated CPython module of myokit's SimulationOpenCL
 * (myokit/_sim/openclsim.c) and its OpenCL runtime calls (myokit/_sim/mcl.h):
 *
 *   openclsim.c sim_init  -> mkg_create + mkg_set_* + mkg_run_begin
 *   openclsim.c sim_step  -> mkg_run_chunk (+ mkg_read_log)
 *   openclsim.c sim_clean -> mkg_destroy
 *   clBuildProgram        -> mkg_compile (NVRTC, sm_103a cubin)
 *
 * Where the reference enqueues two kernels per step and copies the whole
 * state to the host at every log point, this library uploads a schedule of
 * many steps, runs them in one cooperative launch of the generated fused
 * kernel, and copies back only the logged columns of the logged steps.
 *
 * Also holds the fixed (not generated) kernels: AoS <-> SoA state
 * conversion and precision conversion of per-edge conductances.
 */
#include <cuda.h>            /* CUtensorMap types; the driver entry point is
                                looked up at run time */
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <algorithm>
#include <climits>
#include <map>
#include <mutex>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mkg_tissue.h"
#include "mkg_kernel_abi.h"
#include "mkg_pacing.h"

namespace {

thread_local std::string g_thread_error;

/* ------------------------------------------------------------------------ */
/* Fixed device kernels                                                     */
/* ------------------------------------------------------------------------ */

/* Where a state lives on the device */
struct Slots {
    int skip_var;        /* state held in the V plane (alt), or -1 */
    int v_double;        /* the V plane holds doubles */
    int hi_mode;         /* MKG_HI_* */
    const int *hi_slot;  /* per state: accumulation plane, or -1 (or null) */
    void *hi;            /* accumulation planes [n_hi][pitch] */
};

/* AoS doubles [ncell][nvar] -> SoA Real [nvar][pitch]. The V state goes to
 * the V plane (alt); states with an accumulation plane go there as FP64, or
 * (Kahan) as an FP32 value x plus a term c with x - c equal to the double. */
template <typename Real>
__global__ void k_aos_to_soa(const double *__restrict__ in, Real *out,
                             long long ncell, int nvar, long long pitch,
                             Slots sl, void *alt)
{
    const long long n = ncell * nvar;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
         i < n; i += (long long)gridDim.x * blockDim.x) {
        const int s = (int)(i / ncell);
        const long long c = i - (long long)s * ncell;
        const double v = in[c * nvar + s];
        const int j = sl.hi_slot ? sl.hi_slot[s] : -1;
        if (j >= 0 && sl.hi_mode == MKG_HI_DOUBLE) {
            if (s == sl.skip_var) ((double *)alt)[c] = v;
            else ((double *)sl.hi)[(long long)j * pitch + c] = v;
            continue;
        }
        const Real x = (Real)v;
        if (s == sl.skip_var) {
            if (sl.v_double) ((double *)alt)[c] = v;
            else ((Real *)alt)[c] = x;
        } else {
            out[(long long)s * pitch + c] = x;
        }
        if (j >= 0 && sl.hi_mode == MKG_HI_KAHAN)
            ((Real *)sl.hi)[(long long)j * pitch + c] = (Real)((double)x - v);
    }
}

/* SoA Real -> AoS doubles, the inverse of k_aos_to_soa. */
template <typename Real>
__global__ void k_soa_to_aos(const Real *__restrict__ in, double *out,
                             long long ncell, int nvar, long long pitch,
                             Slots sl, const void *alt)
{
    const long long n = ncell * nvar;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
         i < n; i += (long long)gridDim.x * blockDim.x) {
        const int s = (int)(i / ncell);
        const long long c = i - (long long)s * ncell;
        const int j = sl.hi_slot ? sl.hi_slot[s] : -1;
        double v;
        if (s == sl.skip_var)
            v = sl.v_double ? ((const double *)alt)[c]
                            : (double)((const Real *)alt)[c];
        else if (j >= 0 && sl.hi_mode == MKG_HI_DOUBLE)
            v = ((const double *)sl.hi)[(long long)j * pitch + c];
        else
            v = (double)in[(long long)s * pitch + c];
        if (j >= 0 && sl.hi_mode == MKG_HI_KAHAN)
            v -= (double)((const Real *)sl.hi)[(long long)j * pitch + c];
        out[c * nvar + s] = v;
    }
}

/* Tiled forms of the two conversions above, for nvar up to MKG_TILE_NVAR:
 * a block moves tiles of MKG_TILE_CELLS cells, whose AoS rows are one
 * contiguous run of nvar * MKG_TILE_CELLS doubles, through shared memory,
 * so that the AoS side is read or written in full contiguous runs and the
 * SoA side as MKG_TILE_CELLS consecutive cells per state. Same conversions,
 * bit for bit. A cell's row sits in shared memory at an odd stride
 * (nvar | 1 doubles): the 32 cells of one state, read or written by one
 * warp, then fall in distinct banks (at a stride of nvar doubles, an even
 * nvar put a half-warp's 16 accesses in one bank). */
#define MKG_TILE_CELLS 32
#define MKG_TILE_NVAR 96
#define MKG_TILE_STRIDE(nvar) ((nvar) | 1)

template <typename Real>
__global__ void __launch_bounds__(256)
k_aos_to_soa_tiled(const double *__restrict__ in, Real *out, long long ncell,
                   int nvar, long long pitch, Slots sl, void *alt)
{
    __shared__ double tile[MKG_TILE_CELLS * MKG_TILE_STRIDE(MKG_TILE_NVAR)];
    const int stride = MKG_TILE_STRIDE(nvar);
    const long long ntile = (ncell + MKG_TILE_CELLS - 1) / MKG_TILE_CELLS;
    for (long long t = blockIdx.x; t < ntile; t += gridDim.x) {
        const long long c0 = t * MKG_TILE_CELLS;
        const int nc = (int)min((long long)MKG_TILE_CELLS, ncell - c0);
        const int nv = nc * nvar;
        const double *src = in + c0 * nvar;
        for (int k = threadIdx.x; k < nv; k += blockDim.x) {
            const int cc = k / nvar;
            tile[cc * stride + (k - cc * nvar)] = src[k];
        }
        __syncthreads();
        for (int k = threadIdx.x; k < nvar * MKG_TILE_CELLS;
             k += blockDim.x) {
            const int s = k / MKG_TILE_CELLS;
            const int cc = k - s * MKG_TILE_CELLS;
            if (cc >= nc) continue;
            const long long c = c0 + cc;
            const double v = tile[cc * stride + s];
            const int j = sl.hi_slot ? sl.hi_slot[s] : -1;
            if (j >= 0 && sl.hi_mode == MKG_HI_DOUBLE) {
                if (s == sl.skip_var) ((double *)alt)[c] = v;
                else ((double *)sl.hi)[(long long)j * pitch + c] = v;
                continue;
            }
            const Real x = (Real)v;
            if (s == sl.skip_var) {
                if (sl.v_double) ((double *)alt)[c] = v;
                else ((Real *)alt)[c] = x;
            } else {
                out[(long long)s * pitch + c] = x;
            }
            if (j >= 0 && sl.hi_mode == MKG_HI_KAHAN)
                ((Real *)sl.hi)[(long long)j * pitch + c] =
                    (Real)((double)x - v);
        }
        __syncthreads();
    }
}

template <typename Real>
__global__ void __launch_bounds__(256)
k_soa_to_aos_tiled(const Real *__restrict__ in, double *out, long long ncell,
                   int nvar, long long pitch, Slots sl, const void *alt)
{
    __shared__ double tile[MKG_TILE_CELLS * MKG_TILE_STRIDE(MKG_TILE_NVAR)];
    const int stride = MKG_TILE_STRIDE(nvar);
    const long long ntile = (ncell + MKG_TILE_CELLS - 1) / MKG_TILE_CELLS;
    for (long long t = blockIdx.x; t < ntile; t += gridDim.x) {
        const long long c0 = t * MKG_TILE_CELLS;
        const int nc = (int)min((long long)MKG_TILE_CELLS, ncell - c0);
        for (int k = threadIdx.x; k < nvar * MKG_TILE_CELLS;
             k += blockDim.x) {
            const int s = k / MKG_TILE_CELLS;
            const int cc = k - s * MKG_TILE_CELLS;
            if (cc >= nc) continue;
            const long long c = c0 + cc;
            const int j = sl.hi_slot ? sl.hi_slot[s] : -1;
            double v;
            if (s == sl.skip_var)
                v = sl.v_double ? ((const double *)alt)[c]
                                : (double)((const Real *)alt)[c];
            else if (j >= 0 && sl.hi_mode == MKG_HI_DOUBLE)
                v = ((const double *)sl.hi)[(long long)j * pitch + c];
            else
                v = (double)in[(long long)s * pitch + c];
            if (j >= 0 && sl.hi_mode == MKG_HI_KAHAN)
                v -= (double)((const Real *)sl.hi)[(long long)j * pitch + c];
            tile[cc * stride + s] = v;
        }
        __syncthreads();
        const int nv = nc * nvar;
        double *dst = out + c0 * nvar;
        for (int k = threadIdx.x; k < nv; k += blockDim.x) {
            const int cc = k / nvar;
            dst[k] = tile[cc * stride + (k - cc * nvar)];
        }
        __syncthreads();
    }
}

template <typename Real>
__global__ void k_convert(const double *__restrict__ in, Real *out,
                          long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
         i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (Real)in[i];
}

template <typename Real>
__global__ void k_log_to_double(const Real *__restrict__ in, double *out,
                                long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
         i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

int grid_for(long long n)
{
    long long b = (n + 255) / 256;
    if (b < 1) b = 1;
    if (b > 152 * 32) b = 152 * 32;
    return (int)b;
}

}  // namespace

/* ------------------------------------------------------------------------ */
/* Warp-tile staging layout                                                 */
/* ------------------------------------------------------------------------ */

namespace {

/* Shared-memory layout of one staged warp tile (per warp). The same rule is
 * stated by stage_layout() in exporter.py, which writes it into the kernel;
 * the kernel compares its tile byte count with mkg_launch.stage_tx and
 * refuses to run on a mismatch. Tile inputs are copied from the tile's
 * first cell (rounded down to 4 cells when 2D rows are not 4-cell aligned,
 * width 36, else 32); V rows and 1D conductances start one cell earlier,
 * rounded down alike, 40 wide. Every copy destination is 128-byte aligned:
 * regions, and V rows within theirs, are padded to multiples of 128. */
const int kStageVW = 40;

struct StageLayout {
    int sw = 0, lo = 0, np = 0, v_rows = 0, gx = 0;
    int hsize = 0, vsize = 0;
    int64_t v_row = 0;                  /* bytes between staged V rows */
    int64_t off[5] = {0, 0, 0, 0, 0};   /* state, hi, field, v, gx */
    int64_t bytes = 0, tx = 0;
};

void compute_stage_layout(const mkg_config *c, StageLayout *L)
{
    *L = StageLayout();
    if (!c->stage) return;
    const int real = c->real_bytes;
    const bool grid = c->diffusion == MKG_DIFF_GRID ||
                      c->diffusion == MKG_DIFF_HETERO;
    const bool two_d = c->two_d && grid;
    L->sw = (two_d && c->nx % 4 != 0) ? 36 : 32;
    int lo = 0, hi = c->n_state;
    if (c->diffusion != MKG_DIFF_NONE && c->i_vm >= 0) {
        if (c->i_vm == 0) lo = 1;
        if (c->i_vm == c->n_state - 1) hi = c->n_state - 1;
    }
    L->lo = lo;
    L->np = std::max(0, hi - lo);
    L->v_rows = grid ? (two_d ? 3 : 1) : 0;
    L->gx = (c->diffusion == MKG_DIFF_HETERO && !two_d) ? 1 : 0;
    L->hsize = c->hi_mode == MKG_HI_DOUBLE ? 8 : real;
    L->vsize = c->v_double ? 8 : real;
    const int64_t size[5] = {
        (int64_t)L->np * L->sw * real,
        (int64_t)c->n_hi * L->sw * L->hsize,
        (int64_t)c->n_field * L->sw * real,
        (int64_t)L->v_rows * kStageVW * L->vsize,
        L->gx ? (int64_t)kStageVW * real : 0,
    };
    L->v_row = ((int64_t)kStageVW * L->vsize + 127) / 128 * 128;
    int64_t off = 0, tx = 0;
    for (int i = 0; i < 5; ++i) {
        L->off[i] = off;
        const int64_t room = i == 3 ? L->v_rows * L->v_row : size[i];
        off += (room + 127) / 128 * 128;
        tx += size[i];
    }
    L->bytes = off;
    L->tx = tx;
}

}  // namespace

/* ------------------------------------------------------------------------ */
/* Simulation handle                                                        */
/* ------------------------------------------------------------------------ */

struct mkg_sim {
    mkg_config cfg;
    std::string error;
    int real;                 /* bytes per Real */
    long long ncell, pitch;

    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaLibrary_t lib = nullptr;
    cudaKernel_t kernel = nullptr;
    int occ_blocks = 1;       /* co-resident blocks per SM */
    int num_sms = 1;

    /* device buffers */
    void *d_state = nullptr;  /* Real[n_state][pitch] */
    void *d_vbuf = nullptr;   /* Real[2][pitch] */
    void *d_field = nullptr;  /* Real[n_field][pitch] */
    void *d_gx = nullptr, *d_gy = nullptr;
    int *d_nbr_ptr = nullptr, *d_nbr_idx = nullptr;
    void *d_nbr_g = nullptr;
    unsigned int *d_pace_bits = nullptr;
    int *d_log_items = nullptr, *d_log_cols = nullptr;
    void *d_log = nullptr;
    double *d_log_dbl = nullptr;
    mkg_step *d_steps = nullptr;
    mkg_status *d_status = nullptr;
    unsigned int *d_warp_epoch = nullptr;  /* per-warp step counters */
    size_t n_warp_epoch = 0;
    double *d_stage = nullptr;   /* staging for double uploads */
    void *d_hi = nullptr;        /* accumulation planes [n_hi][pitch] x 8 B */
    int *d_hi_slot = nullptr;    /* per state: accumulation plane or -1 */
    int v_double = 0;            /* V plane holds doubles */
    int vbytes = 4;              /* bytes per V plane entry */
    size_t stage_bytes = 0;

    /* Warp-tile staging (cfg.stage): layout, dynamic shared memory per CTA
     * and the tensor maps passed to the kernel */
    StageLayout lay;
    size_t tile_smem = 0;
    mkg_tmaps tmaps;

    /* pinned host buffers */
    mkg_step *h_steps = nullptr;
    mkg_status *h_status = nullptr;
    double *h_log = nullptr;
    std::vector<double> h_time, h_pace, h_tend;

    int v_sel = 0;
    double gx = 0, gy = 0;
    int pace_mode = MKG_PACE_NONE;
    long long px0 = 0, px1 = 0, py0 = 0, py1 = 0;
    int n_log_items = 0;
    int log_ncol = 0;
    int nan_check = 0;
    int64_t cap_steps = 0;    /* schedule capacity */
    int64_t cap_rows = 0;     /* log row capacity */
    int64_t last_rows = 0;
    int steps_per_launch = 0;
    int blocks_per_sm = 0;
    long long timeout_ns = 2000000000LL;
    int wait_skew = 0;        /* mkg_set_wait: unreachable step waits */

    mkg::Pacer pacer;
    mkg::Schedule sched;
    bool running = false;
    bool halted = false;

    double last_ms = 0;
    int64_t last_launches = 0, last_cell_steps = 0;
    int64_t n_launches = 0;   /* every kernel launched by this handle */
    bool use_graphs = false;  /* replay multi-launch chunks as CUDA graphs */
    std::map<std::string, cudaGraphExec_t> graphs;

    /* Fiber-tissue: a second simulation (the tissue) advanced by this
     * one's fused kernel, and the junction between them (not owned) */
    mkg_sim *partner = nullptr;
    mkg_junction junction;

    /* Device frame buffer for log rows (not owned) */
    void *frame_buf = nullptr;
    int64_t frame_rows = 0, frame_next = 0;

    /* Logged columns (host copy) */
    std::vector<int> h_log_item;
    std::vector<long long> h_log_cell;

    /* Adjoint */
    cudaLibrary_t adj_lib = nullptr;
    cudaKernel_t adj_fwd = nullptr, adj_bwd = nullptr;
    int adj_occ_fwd = 1, adj_occ_bwd = 1;
    int adj_bwd_threads = 0;              /* reverse kernel CTA size */
    size_t ckpt_bytes = 0;                /* bytes per checkpoint */
    int adj_seg = 0;                      /* steps per checkpoint segment */
    void *d_traj = nullptr, *d_lam = nullptr, *d_mu = nullptr;
    void *d_gfield = nullptr, *d_gg = nullptr, *d_lgrad = nullptr;
    double *d_ge = nullptr;               /* per-edge gradient parts */
    size_t n_ge = 0;                      /* doubles in d_ge */
    std::vector<double> h_edge_grad;      /* per-edge / per-connection */
    long long n_nbr = 0;                  /* CSR entries (2 per connection) */
    std::vector<int> conn_pos;            /* CSR entries of connection c:
                                             conn_pos[2c], conn_pos[2c+1] */
    int *d_probe_col = nullptr;
    mkg_step *d_fsteps = nullptr, *d_bsteps = nullptr;
    std::vector<mkg_step> adj_sched;      /* full run, global log rows */
    std::vector<long long> adj_seg_start, adj_seg_len;
    std::vector<int> adj_seg_vsel;
    std::vector<void *> adj_ckpt;         /* state + V plane per segment */
    std::vector<double> adj_log;          /* rows x log_ncol */
    int64_t adj_rows = 0;
};

namespace {

int set_err(mkg_sim *s, int code, const char *fmt, ...)
{
    char buf[2048];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (s) s->error = buf;
    else g_thread_error = buf;
    return code;
}

#define CK(sim, call)                                                       \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess)                                              \
            return set_err(sim, MKG_ERR_CUDA, "%s failed: %s (%s:%d)",      \
                           #call, cudaGetErrorString(e_), __FILE__,        \
                           __LINE__);                                       \
    } while (0)

template <typename T>
void dfree(T *&p)
{
    if (p) cudaFree((void *)p);
    p = nullptr;
}

int ensure_stage(mkg_sim *s, size_t bytes)
{
    if (bytes <= s->stage_bytes) return MKG_OK;
    dfree(s->d_stage);
    s->stage_bytes = 0;
    CK(s, cudaMalloc((void **)&s->d_stage, bytes));
    s->stage_bytes = bytes;
    return MKG_OK;
}

/* Cached graphs bake in buffer pointers and launch parameters */
void clear_graphs(mkg_sim *s)
{
    for (auto &kv : s->graphs) cudaGraphExecDestroy(kv.second);
    s->graphs.clear();
}

int ensure_schedule(mkg_sim *s, int64_t steps, int64_t rows)
{
    if (steps > s->cap_steps || rows > s->cap_rows) clear_graphs(s);
    if (steps > s->cap_steps) {
        dfree(s->d_steps);
        if (s->h_steps) cudaFreeHost(s->h_steps);
        s->h_steps = nullptr;
        s->cap_steps = 0;
        CK(s, cudaMalloc((void **)&s->d_steps, steps * sizeof(mkg_step)));
        CK(s, cudaMallocHost((void **)&s->h_steps, steps * sizeof(mkg_step)));
        s->h_tend.resize(steps);
        s->cap_steps = steps;
    }
    if ((int64_t)s->h_time.size() < rows) {
        s->h_time.resize(rows);
        s->h_pace.resize(rows);
    }
    /* Log values are staged on the device and copied back, unless a
     * device frame buffer receives them. */
    if (!s->frame_buf && rows > s->cap_rows) {
        dfree(s->d_log);
        dfree(s->d_log_dbl);
        if (s->h_log) cudaFreeHost(s->h_log);
        s->h_log = nullptr;
        s->cap_rows = 0;
        const size_t n = (size_t)rows * (size_t)std::max(s->log_ncol, 1);
        CK(s, cudaMalloc(&s->d_log, n * s->real));
        CK(s, cudaMalloc((void **)&s->d_log_dbl, n * sizeof(double)));
        CK(s, cudaMallocHost((void **)&s->h_log, n * sizeof(double)));
        s->cap_rows = rows;
    }
    return MKG_OK;
}

Slots state_slots(const mkg_sim *s)
{
    Slots sl;
    sl.skip_var = s->cfg.diffusion != MKG_DIFF_NONE ? s->cfg.i_vm : -1;
    sl.v_double = s->v_double;
    sl.hi_mode = s->cfg.hi_mode;
    sl.hi_slot = s->d_hi_slot;
    sl.hi = s->d_hi;
    return sl;
}

Slots plain_slots()
{
    Slots sl;
    sl.skip_var = -1;
    sl.v_double = 0;
    sl.hi_mode = MKG_HI_NONE;
    sl.hi_slot = nullptr;
    sl.hi = nullptr;
    return sl;
}

/* Blocks for the tiled conversions: one tile of MKG_TILE_CELLS cells per
 * block and pass, at most 8 resident 256-thread blocks per SM */
int tile_grid(const mkg_sim *s)
{
    const long long tiles = (s->ncell + MKG_TILE_CELLS - 1) / MKG_TILE_CELLS;
    const long long cap = 8LL * std::max(s->num_sms, 1);
    return (int)std::max<long long>(1, std::min(tiles, cap));
}

template <typename Real>
int upload_soa(mkg_sim *s, const double *aos, int nvar, void *dst, Slots sl,
               void *alt)
{
    const size_t bytes = (size_t)s->ncell * nvar * sizeof(double);
    int r = ensure_stage(s, bytes);
    if (r) return r;
    CK(s, cudaMemcpyAsync(s->d_stage, aos, bytes, cudaMemcpyHostToDevice,
                          s->stream));
    s->n_launches++;
    if (nvar <= MKG_TILE_NVAR)
        k_aos_to_soa_tiled<Real><<<tile_grid(s), 256, 0, s->stream>>>(
            s->d_stage, (Real *)dst, s->ncell, nvar, s->pitch, sl, alt);
    else
        k_aos_to_soa<Real><<<grid_for(s->ncell * nvar), 256, 0,
                             s->stream>>>(
            s->d_stage, (Real *)dst, s->ncell, nvar, s->pitch, sl, alt);
    CK(s, cudaGetLastError());
    CK(s, cudaStreamSynchronize(s->stream));
    return MKG_OK;
}

template <typename Real>
int download_soa(mkg_sim *s, double *aos, int nvar, const void *src,
                 Slots sl, const void *alt)
{
    const size_t bytes = (size_t)s->ncell * nvar * sizeof(double);
    int r = ensure_stage(s, bytes);
    if (r) return r;
    s->n_launches++;
    if (nvar <= MKG_TILE_NVAR)
        k_soa_to_aos_tiled<Real><<<tile_grid(s), 256, 0, s->stream>>>(
            (const Real *)src, s->d_stage, s->ncell, nvar, s->pitch, sl,
            alt);
    else
        k_soa_to_aos<Real><<<grid_for(s->ncell * nvar), 256, 0,
                             s->stream>>>(
            (const Real *)src, s->d_stage, s->ncell, nvar, s->pitch, sl,
            alt);
    CK(s, cudaGetLastError());
    CK(s, cudaMemcpyAsync(aos, s->d_stage, bytes, cudaMemcpyDeviceToHost,
                          s->stream));
    CK(s, cudaStreamSynchronize(s->stream));
    return MKG_OK;
}

template <typename Real>
int upload_real(mkg_sim *s, const double *src, long long n, void *dst)
{
    if (n <= 0) return MKG_OK;
    int r = ensure_stage(s, (size_t)n * sizeof(double));
    if (r) return r;
    CK(s, cudaMemcpyAsync(s->d_stage, src, n * sizeof(double),
                          cudaMemcpyHostToDevice, s->stream));
    s->n_launches++;
    k_convert<Real><<<grid_for(n), 256, 0, s->stream>>>(s->d_stage,
                                                       (Real *)dst, n);
    CK(s, cudaGetLastError());
    CK(s, cudaStreamSynchronize(s->stream));
    return MKG_OK;
}

bool diffusion_on(const mkg_sim *s) { return s->cfg.diffusion != MKG_DIFF_NONE; }

int pacer_err(mkg_sim *s, int st)
{
    if (st == mkg::PACER_SIMULTANEOUS_EVENT)
        return set_err(s, MKG_ERR_SIMULTANEOUS,
                       "E-Pacing error: Event scheduled or re-occuring at the"
                       " same time as another event.");
    if (st == mkg::PACER_NEGATIVE_TIME_INCREMENT)
        return set_err(s, MKG_ERR_PACING,
                       "E-Pacing error: New time is before current time.");
    if (st == mkg::PACER_NON_ZERO_MULTIPLIER)
        return set_err(s, MKG_ERR_PACING,
                       "E-Pacing error: Non-zero multiplier found for"
                       " non-periodic stimulus.");
    if (st == mkg::PACER_NEGATIVE_PERIOD)
        return set_err(s, MKG_ERR_PACING,
                       "E-Pacing error: Pacing event period cannot be"
                       " negative.");
    if (st == mkg::PACER_NEGATIVE_MULTIPLIER)
        return set_err(s, MKG_ERR_PACING,
                       "E-Pacing error: Pacing event multiplier cannot be"
                       " negative.");
    return set_err(s, MKG_ERR_PACING, "E-Pacing error: Unlisted error %d",
                   st);
}

/* The launch block common to every tissue-step launch of a handle:
 * buffers, geometry (warp tiles), conductances, pacing, logging. */
void fill_launch(mkg_sim *s, mkg_launch *a)
{
    memset(a, 0, sizeof(*a));
    a->nx = s->cfg.nx;
    a->ny = s->cfg.ny;
    a->ncell = s->ncell;
    a->pitch = s->pitch;
    a->state = s->d_state;
    a->vbuf = s->d_vbuf;
    a->field = s->d_field;
    a->gx = s->d_gx;
    a->gy = s->d_gy;
    a->nbr_ptr = s->d_nbr_ptr;
    a->nbr_idx = s->d_nbr_idx;
    a->nbr_g = s->d_nbr_g;
    a->gxs = s->gx;
    a->gys = s->gy;
    a->gxf = (float)s->gx;
    a->gyf = (float)s->gy;
    a->pace_x0 = s->px0;
    a->pace_x1 = s->px1;
    a->pace_y0 = s->py0;
    a->pace_y1 = s->py1;
    a->pace_bits = s->d_pace_bits;
    a->pace_mode = s->pace_mode;
    a->log = s->d_log;
    a->log_items = s->d_log_items;
    a->log_cols = s->d_log_cols;
    a->log_ncol = s->log_ncol;
    a->n_log_items = s->n_log_items;
    a->nan_check = s->nan_check;
    a->status = s->d_status;
    a->timeout_ns = s->timeout_ns;
    a->wait_skew = s->wait_skew;
    a->hi = s->d_hi;
    a->warp_epoch = s->d_warp_epoch;
    /* Warp tiles: 32 consecutive cells of a row (2D) or of the flat cell
     * array (1D cables, connection graphs, diffusion-free simulations). */
    if (s->cfg.two_d) {
        a->ntiles_x = (int)((s->cfg.nx + 31) / 32);
        a->ntiles_y = (int)s->cfg.ny;
    } else {
        a->nx = s->ncell;
        a->ny = 1;
        a->ntiles_x = (int)((s->ncell + 31) / 32);
        a->ntiles_y = 1;
    }
}

/* cuTensorMapEncodeTiled, looked up once through the runtime (the library
 * does not link the driver API) */
typedef CUresult (*EncodeTiledFn)(
    CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
    const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
    CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
    CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled_fn()
{
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p,
                                             12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    });
    return fn;
}

/* A rank-1 (d1 == 0) or rank-2 tensor map of FP32 / FP64 elements over
 * d0 x d1 elements, rows d0 elements apart, copied in boxes b0 x b1 */
int encode_map(mkg_sim *s, mkg_tmap *out, const void *base, int elem,
               uint64_t d0, uint64_t d1, uint32_t b0, uint32_t b1)
{
    static_assert(sizeof(CUtensorMap) == sizeof(mkg_tmap),
                  "tensor map size");
    EncodeTiledFn fn = encode_tiled_fn();
    if (!fn)
        return set_err(s, MKG_ERR_CUDA,
                       "cuTensorMapEncodeTiled is not available");
    if (!base) return set_err(s, MKG_ERR_ARG, "a staged array is missing");
    CUtensorMap m;
    const cuuint32_t rank = d1 ? 2 : 1;
    const cuuint64_t dims[2] = {d0, d1 ? d1 : 1};
    const cuuint64_t strides[1] = {d0 * (cuuint64_t)elem};
    const cuuint32_t box[2] = {b0, b1 ? b1 : 1};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(
        &m, elem == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                      : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
        rank, const_cast<void *>(base), dims, strides, box, estr,
        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return set_err(s, MKG_ERR_CUDA, "tensor map encoding failed (%d)",
                       (int)r);
    memcpy(out, &m, sizeof(m));
    return MKG_OK;
}

/* Tensor maps of every staged array, for the current buffers */
int encode_stage_maps(mkg_sim *s)
{
    const StageLayout &L = s->lay;
    const mkg_config &c = s->cfg;
    memset(&s->tmaps, 0, sizeof(s->tmaps));
    int r;
    if (L.np > 0 &&
        (r = encode_map(s, &s->tmaps.state, s->d_state, s->real, s->pitch,
                        c.n_state, L.sw, L.np)))
        return r;
    if (c.n_hi > 0 &&
        (r = encode_map(s, &s->tmaps.hi, s->d_hi, L.hsize, s->pitch, c.n_hi,
                        L.sw, c.n_hi)))
        return r;
    if (c.n_field > 0 &&
        (r = encode_map(s, &s->tmaps.field, s->d_field, s->real, s->pitch,
                        c.n_field, L.sw, c.n_field)))
        return r;
    if (L.v_rows > 0 &&
        (r = encode_map(s, &s->tmaps.v, s->d_vbuf, L.vsize, s->pitch, 2,
                        kStageVW, 1)))
        return r;
    if (L.gx &&
        (r = encode_map(s, &s->tmaps.gx, s->d_gx, s->real,
                        std::max<int64_t>(s->ncell - 1, 1), 0, kStageVW, 0)))
        return r;
    return MKG_OK;
}

/* CTAs per cluster: a split team larger than the CTA is a cluster */
int cluster_ctas(const mkg_sim *s)
{
    const int nwarp = s->cfg.block_x / 32;
    return s->cfg.split > nwarp ? s->cfg.split / nwarp : 1;
}

/* CTAs needed to give every warp tile a warp (a team of cfg.split warps
 * when the kernel divides each tile's work) */
long long blocks_needed(const mkg_sim *s, const mkg_launch *a)
{
    const long long nwt = (long long)a->ntiles_x * a->ntiles_y;
    const int threads = s->cfg.block_x * s->cfg.block_y;
    const long long split = s->cfg.split > 1 ? s->cfg.split : 1;
    return (nwt * 32 * split + threads - 1) / threads;
}

}  // namespace

/* ------------------------------------------------------------------------ */
/* C ABI                                                                    */
/* ------------------------------------------------------------------------ */

extern "C" {

const char *mkg_last_error(const mkg_sim *sim)
{
    if (sim) return sim->error.c_str();
    return g_thread_error.c_str();
}

void mkg_free(void *ptr) { free(ptr); }

int mkg_compile(const char *source, const char *name,
                const char *const *options, int n_options, void **cubin,
                size_t *cubin_size, char **log)
{
    if (!source || !cubin || !cubin_size)
        return set_err(nullptr, MKG_ERR_ARG, "mkg_compile: null argument");
    *cubin = nullptr;
    *cubin_size = 0;
    if (log) *log = nullptr;
    nvrtcProgram prog;
    nvrtcResult r = nvrtcCreateProgram(&prog, source,
                                       name ? name : "mkg_tissue.cu", 0,
                                       nullptr, nullptr);
    if (r != NVRTC_SUCCESS)
        return set_err(nullptr, MKG_ERR_COMPILE, "nvrtcCreateProgram: %s",
                       nvrtcGetErrorString(r));
    r = nvrtcCompileProgram(prog, n_options, options);
    size_t log_size = 0;
    nvrtcGetProgramLogSize(prog, &log_size);
    std::string text(log_size > 0 ? log_size : 1, '\0');
    if (log_size > 1) nvrtcGetProgramLog(prog, &text[0]);
    if (log) {
        *log = (char *)malloc(text.size() + 1);
        if (*log) memcpy(*log, text.c_str(), text.size() + 1);
    }
    if (r != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        return set_err(nullptr, MKG_ERR_COMPILE,
                       "Kernel failed to compile (%s):\n%s",
                       nvrtcGetErrorString(r), text.c_str());
    }
    size_t n = 0;
    r = nvrtcGetCUBINSize(prog, &n);
    if (r != NVRTC_SUCCESS || n == 0) {
        nvrtcDestroyProgram(&prog);
        return set_err(nullptr, MKG_ERR_COMPILE, "no cubin produced");
    }
    void *out = malloc(n);
    if (!out) {
        nvrtcDestroyProgram(&prog);
        return set_err(nullptr, MKG_ERR_NOMEM, "out of host memory");
    }
    nvrtcGetCUBIN(prog, (char *)out);
    nvrtcDestroyProgram(&prog);
    *cubin = out;
    *cubin_size = n;
    return MKG_OK;
}

void mkg_destroy(mkg_sim *s)
{
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    clear_graphs(s);
    for (void *p : s->adj_ckpt) cudaFree(p);
    s->adj_ckpt.clear();
    dfree(s->d_traj);
    dfree(s->d_lam);
    dfree(s->d_mu);
    dfree(s->d_gfield);
    dfree(s->d_gg);
    dfree(s->d_ge);
    dfree(s->d_lgrad);
    dfree(s->d_probe_col);
    dfree(s->d_fsteps);
    dfree(s->d_bsteps);
    if (s->adj_lib) cudaLibraryUnload(s->adj_lib);
    dfree(s->d_state);
    dfree(s->d_vbuf);
    dfree(s->d_field);
    dfree(s->d_gx);
    dfree(s->d_gy);
    dfree(s->d_nbr_ptr);
    dfree(s->d_nbr_idx);
    dfree(s->d_nbr_g);
    dfree(s->d_pace_bits);
    dfree(s->d_log_items);
    dfree(s->d_log_cols);
    dfree(s->d_log);
    dfree(s->d_log_dbl);
    dfree(s->d_steps);
    dfree(s->d_status);
    dfree(s->d_warp_epoch);
    dfree(s->d_stage);
    dfree(s->d_hi);
    dfree(s->d_hi_slot);
    if (s->h_steps) cudaFreeHost(s->h_steps);
    if (s->h_status) cudaFreeHost(s->h_status);
    if (s->h_log) cudaFreeHost(s->h_log);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->lib) cudaLibraryUnload(s->lib);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

int mkg_create(const mkg_config *cfg, const void *cubin, size_t cubin_size,
               mkg_sim **out)
{
    if (!cfg || !cubin || !cubin_size || !out)
        return set_err(nullptr, MKG_ERR_ARG, "mkg_create: null argument");
    *out = nullptr;
    if (cfg->nx < 1 || cfg->ny < 1)
        return set_err(nullptr, MKG_ERR_ARG,
                       "The number of cells in any direction must be at"
                       " least 1.");
    if (cfg->real_bytes != 4 && cfg->real_bytes != 8)
        return set_err(nullptr, MKG_ERR_ARG,
                       "Only single and double precision are supported.");
    if (cfg->n_state < 1 || cfg->n_field < 0 || cfg->n_inter < 0)
        return set_err(nullptr, MKG_ERR_ARG, "invalid variable counts");
    if (cfg->hi_mode < MKG_HI_NONE || cfg->hi_mode > MKG_HI_KAHAN ||
        cfg->n_hi < 0 || cfg->n_hi > cfg->n_state ||
        (cfg->hi_mode != MKG_HI_NONE && cfg->real_bytes != 4))
        return set_err(nullptr, MKG_ERR_ARG,
                       "invalid accumulation mode (single precision only)");
    if (cfg->diffusion < MKG_DIFF_NONE || cfg->diffusion > MKG_DIFF_CONN)
        return set_err(nullptr, MKG_ERR_ARG, "invalid diffusion mode");
    if (cfg->diffusion != MKG_DIFF_NONE &&
        (cfg->i_vm < 0 || cfg->i_vm >= cfg->n_state))
        return set_err(nullptr, MKG_ERR_ARG, "invalid membrane potential index");
    if (cfg->block_x < 1 || cfg->block_y < 1 ||
        cfg->block_x * cfg->block_y > 1024)
        return set_err(nullptr, MKG_ERR_ARG, "invalid block shape");
    if (cfg->block_y != 1 || cfg->block_x % 32 != 0)
        return set_err(nullptr, MKG_ERR_ARG,
                       "the CTA must be (32*k, 1) threads");
    if (!cfg->two_d && cfg->ny != 1 && cfg->diffusion != MKG_DIFF_NONE)
        return set_err(nullptr, MKG_ERR_ARG, "2D diffusion needs two_d");
    if (cfg->v_double && cfg->hi_mode != MKG_HI_DOUBLE)
        return set_err(nullptr, MKG_ERR_ARG, "v_double needs hi_mode 1");
    if (cfg->stage < 0 || cfg->stage > 2)
        return set_err(nullptr, MKG_ERR_ARG, "stage must be 0, 1 or 2");
    if (cfg->split < 0 || cfg->split > 16 ||
        (cfg->split > 1 && (cfg->split & (cfg->split - 1))))
        return set_err(nullptr, MKG_ERR_ARG,
                       "split must be 1, 2, 4, 8 or 16");
    if (cfg->split > 1) {
        const int nwarp = cfg->block_x / 32;
        const bool cta_team = cfg->split <= nwarp &&
                              nwarp % cfg->split == 0 &&
                              nwarp / cfg->split <= 15;
        const bool cluster_team = cfg->split > nwarp &&
                                  cfg->split % nwarp == 0 &&
                                  cfg->split / nwarp <= 8;
        if ((!cta_team && !cluster_team) || cfg->stage ||
            cfg->hi_mode != MKG_HI_NONE)
            return set_err(nullptr, MKG_ERR_ARG,
                           "a split kernel needs whole teams of at most 15"
                           " per CTA, or teams of 2 to 8 whole CTAs, no"
                           " staging and no accumulation planes");
    }
    if (cfg->stage) {
        /* Tensor copy limits: 256 planes per box, int32 coordinates */
        StageLayout L;
        compute_stage_layout(cfg, &L);
        if (L.np > 256 || cfg->n_hi > 256 || cfg->n_field > 256 ||
            cfg->nx * cfg->ny + 64 > (int64_t)INT_MAX)
            return set_err(nullptr, MKG_ERR_ARG,
                           "this configuration cannot stage tiles");
    }

    mkg_sim *s = new mkg_sim();
    s->cfg = *cfg;
    s->real = cfg->real_bytes;
    s->ncell = cfg->nx * cfg->ny;
    s->pitch = (s->ncell + 31) / 32 * 32;
    s->pace_mode = cfg->diffusion == MKG_DIFF_NONE ? MKG_PACE_ALL
                                                   : MKG_PACE_NONE;
#define CKC(call)                                                           \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) {                                            \
            set_err(nullptr, MKG_ERR_CUDA, "%s failed: %s", #call,          \
                    cudaGetErrorString(e_));                                \
            mkg_destroy(s);                                                 \
            return MKG_ERR_CUDA;                                            \
        }                                                                   \
    } while (0)
    CKC(cudaSetDevice(cfg->device));
    CKC(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    CKC(cudaEventCreate(&s->ev0));
    CKC(cudaEventCreate(&s->ev1));
    CKC(cudaLibraryLoadData(&s->lib, cubin, nullptr, nullptr, 0, nullptr,
                            nullptr, 0));
    CKC(cudaLibraryGetKernel(&s->kernel, s->lib, "mkg_tissue_step"));
    CKC(cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount,
                               cfg->device));
    if (cfg->stage) {
        compute_stage_layout(cfg, &s->lay);
        /* One or two buffers per warp (cfg.stage); + 128: the kernel
         * rounds the base up to a 128-byte boundary */
        s->tile_smem = (size_t)(cfg->block_x / 32) * s->lay.bytes *
                           (size_t)cfg->stage + 128;
        CKC(cudaKernelSetAttributeForDevice(
            s->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
            (int)s->tile_smem, cfg->device));
    }
    CKC(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &s->occ_blocks, (const void *)s->kernel,
        cfg->block_x * cfg->block_y, s->tile_smem));
    if (s->occ_blocks < 1) {
        set_err(nullptr, MKG_ERR_CUDA,
                "the generated kernel cannot be resident on an SM");
        mkg_destroy(s);
        return MKG_ERR_CUDA;
    }

    const size_t plane = (size_t)s->pitch * s->real;
    CKC(cudaMalloc(&s->d_state, plane * cfg->n_state));
    CKC(cudaMemsetAsync(s->d_state, 0, plane * cfg->n_state, s->stream));
    /* V planes hold doubles when V is accumulated in FP64: 8 B entries */
    CKC(cudaMalloc(&s->d_vbuf, (size_t)s->pitch * 8 * 2));
    CKC(cudaMemsetAsync(s->d_vbuf, 0, (size_t)s->pitch * 8 * 2, s->stream));
    s->vbytes = s->real;
    if (cfg->hi_mode != MKG_HI_NONE && cfg->n_hi > 0) {
        CKC(cudaMalloc(&s->d_hi, (size_t)s->pitch * 8 * cfg->n_hi));
        CKC(cudaMemsetAsync(s->d_hi, 0, (size_t)s->pitch * 8 * cfg->n_hi,
                            s->stream));
        CKC(cudaMalloc((void **)&s->d_hi_slot, cfg->n_state * sizeof(int)));
        CKC(cudaMemsetAsync(s->d_hi_slot, 0xff, cfg->n_state * sizeof(int),
                            s->stream));
    }
    if (cfg->n_field > 0) {
        CKC(cudaMalloc(&s->d_field, plane * cfg->n_field));
        CKC(cudaMemsetAsync(s->d_field, 0, plane * cfg->n_field, s->stream));
    }
    CKC(cudaMalloc((void **)&s->d_status, sizeof(mkg_status)));
    CKC(cudaMallocHost((void **)&s->h_status, sizeof(mkg_status)));
    /* One step counter per warp of the largest co-resident grid */
    s->n_warp_epoch = (size_t)s->occ_blocks * s->num_sms *
                      (size_t)(cfg->block_x / 32);
    CKC(cudaMalloc((void **)&s->d_warp_epoch,
                   s->n_warp_epoch * sizeof(unsigned int)));
    CKC(cudaStreamSynchronize(s->stream));
#undef CKC
    *out = s;
    return MKG_OK;
}

int mkg_set_hi_states(mkg_sim *s, const int32_t *states, int32_t n)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (n != s->cfg.n_hi || (n > 0 && !states))
        return set_err(s, MKG_ERR_ARG, "expected %d accumulated states",
                       s->cfg.n_hi);
    std::vector<int> slot(s->cfg.n_state, -1);
    for (int j = 0; j < n; ++j) {
        if (states[j] < 0 || states[j] >= s->cfg.n_state ||
            slot[states[j]] >= 0)
            return set_err(s, MKG_ERR_ARG, "invalid accumulated state %d",
                           states[j]);
        slot[states[j]] = j;
    }
    CK(s, cudaMemcpyAsync(s->d_hi_slot, slot.data(),
                          slot.size() * sizeof(int), cudaMemcpyHostToDevice,
                          s->stream));
    CK(s, cudaStreamSynchronize(s->stream));
    s->v_double = (s->cfg.hi_mode == MKG_HI_DOUBLE && diffusion_on(s) &&
                   slot[s->cfg.i_vm] >= 0) ? 1 : 0;
    s->vbytes = s->v_double ? 8 : s->real;
    if (s->cfg.stage && s->v_double != s->cfg.v_double)
        return set_err(s, MKG_ERR_ARG,
                       "the accumulated states disagree with v_double");
    return MKG_OK;
}

int mkg_set_state(mkg_sim *s, const double *state, int64_t n)
{
    if (!s || !state) return set_err(s, MKG_ERR_ARG, "null argument");
    if (n != s->ncell * s->cfg.n_state)
        return set_err(s, MKG_ERR_ARG,
                       "'state_in' must have size nx * ny * n_states.");
    void *alt = (char *)s->d_vbuf + (size_t)s->v_sel * s->pitch * s->vbytes;
    if (s->real == 4)
        return upload_soa<float>(s, state, s->cfg.n_state, s->d_state,
                                 state_slots(s), alt);
    return upload_soa<double>(s, state, s->cfg.n_state, s->d_state,
                              state_slots(s), alt);
}

int mkg_get_state(mkg_sim *s, double *state, int64_t n)
{
    if (!s || !state) return set_err(s, MKG_ERR_ARG, "null argument");
    if (n != s->ncell * s->cfg.n_state)
        return set_err(s, MKG_ERR_ARG,
                       "'state_out' must have size nx * ny * n_states.");
    const void *alt =
        (const char *)s->d_vbuf + (size_t)s->v_sel * s->pitch * s->vbytes;
    if (s->real == 4)
        return download_soa<float>(s, state, s->cfg.n_state, s->d_state,
                                   state_slots(s), alt);
    return download_soa<double>(s, state, s->cfg.n_state, s->d_state,
                                state_slots(s), alt);
}

int mkg_set_fields(mkg_sim *s, const double *field_data, int64_t n)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (n != s->ncell * s->cfg.n_field)
        return set_err(s, MKG_ERR_ARG,
                       "field data must have nx * ny * n_field entries");
    if (n == 0) return MKG_OK;
    if (!field_data) return set_err(s, MKG_ERR_ARG, "null argument");
    if (s->real == 4)
        return upload_soa<float>(s, field_data, s->cfg.n_field, s->d_field,
                                 plain_slots(), nullptr);
    return upload_soa<double>(s, field_data, s->cfg.n_field, s->d_field,
                              plain_slots(), nullptr);
}

int mkg_set_conductance(mkg_sim *s, double gx, double gy)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (gx < 0) return set_err(s, MKG_ERR_ARG, "Invalid conductance gx=%g", gx);
    if (gy < 0) return set_err(s, MKG_ERR_ARG, "Invalid conductance gy=%g", gy);
    s->gx = gx;
    s->gy = gy;
    return MKG_OK;
}

int mkg_set_conductance_field(mkg_sim *s, const double *gx, int64_t ngx,
                              const double *gy, int64_t ngy)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    const long long nx = s->cfg.nx, ny = s->cfg.ny;
    if (ngx != ny * (nx - 1))
        return set_err(s, MKG_ERR_ARG, "gx must have ny * (nx - 1) entries");
    if (ngy != (ny - 1) * nx)
        return set_err(s, MKG_ERR_ARG, "gy must have (ny - 1) * nx entries");
    for (int64_t i = 0; i < ngx; ++i)
        if (!(gx[i] >= 0))
            return set_err(s, MKG_ERR_ARG,
                           "The argument `gx` can not contain negative"
                           " values.");
    for (int64_t i = 0; i < ngy; ++i)
        if (!(gy[i] >= 0))
            return set_err(s, MKG_ERR_ARG,
                           "The argument `gy` can not contain negative"
                           " values.");
    dfree(s->d_gx);
    dfree(s->d_gy);
    CK(s, cudaMalloc(&s->d_gx, std::max<int64_t>(ngx, 1) * s->real));
    CK(s, cudaMalloc(&s->d_gy, std::max<int64_t>(ngy, 1) * s->real));
    int r;
    if (s->real == 4) {
        if ((r = upload_real<float>(s, gx, ngx, s->d_gx))) return r;
        if ((r = upload_real<float>(s, gy, ngy, s->d_gy))) return r;
    } else {
        if ((r = upload_real<double>(s, gx, ngx, s->d_gx))) return r;
        if ((r = upload_real<double>(s, gy, ngy, s->d_gy))) return r;
    }
    return MKG_OK;
}

int mkg_set_connections(mkg_sim *s, const int64_t *c1, const int64_t *c2,
                        const double *g, int64_t n)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (n < 0 || (n > 0 && (!c1 || !c2 || !g)))
        return set_err(s, MKG_ERR_ARG, "invalid connection arrays");
    const long long nc = s->ncell;
    std::vector<int> deg(nc + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
        if (c1[i] < 0 || c2[i] < 0 || c1[i] >= nc || c2[i] >= nc ||
            c1[i] == c2[i])
            return set_err(s, MKG_ERR_ARG,
                           "Invalid connection: (%lld, %lld, %g)",
                           (long long)c1[i], (long long)c2[i], g[i]);
        if (!(g[i] >= 0))
            return set_err(s, MKG_ERR_ARG, "Invalid conductance: %g", g[i]);
        deg[c1[i]]++;
        deg[c2[i]]++;
    }
    std::vector<int> ptr(nc + 1, 0);
    for (long long i = 0; i < nc; ++i) ptr[i + 1] = ptr[i] + deg[i];
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    std::vector<int> idx(std::max<int64_t>(2 * n, 1));
    std::vector<double> gg(std::max<int64_t>(2 * n, 1));
    /* Each cell's list keeps the order of the connection list. */
    s->conn_pos.assign(2 * n, 0);
    for (int64_t i = 0; i < n; ++i) {
        const int a = (int)c1[i], b = (int)c2[i];
        s->conn_pos[2 * i] = fill[a];
        idx[fill[a]] = b;
        gg[fill[a]++] = g[i];
        s->conn_pos[2 * i + 1] = fill[b];
        idx[fill[b]] = a;
        gg[fill[b]++] = g[i];
    }
    s->n_nbr = 2 * n;
    dfree(s->d_nbr_ptr);
    dfree(s->d_nbr_idx);
    dfree(s->d_nbr_g);
    CK(s, cudaMalloc((void **)&s->d_nbr_ptr, (nc + 1) * sizeof(int)));
    CK(s, cudaMalloc((void **)&s->d_nbr_idx, idx.size() * sizeof(int)));
    CK(s, cudaMalloc(&s->d_nbr_g, gg.size() * s->real));
    CK(s, cudaMemcpyAsync(s->d_nbr_ptr, ptr.data(), (nc + 1) * sizeof(int),
                          cudaMemcpyHostToDevice, s->stream));
    CK(s, cudaMemcpyAsync(s->d_nbr_idx, idx.data(), idx.size() * sizeof(int),
                          cudaMemcpyHostToDevice, s->stream));
    CK(s, cudaStreamSynchronize(s->stream));
    if (s->real == 4)
        return upload_real<float>(s, gg.data(), (long long)gg.size(), s->d_nbr_g);
    return upload_real<double>(s, gg.data(), (long long)gg.size(), s->d_nbr_g);
}

int mkg_set_pacing_mode(mkg_sim *s, int32_t mode)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (mode < MKG_PACE_ALL || mode > MKG_PACE_NONE)
        return set_err(s, MKG_ERR_ARG, "invalid pacing mode");
    s->pace_mode = mode;
    return MKG_OK;
}

int mkg_set_paced_rect(mkg_sim *s, int64_t nx, int64_t ny, int64_t x,
                       int64_t y)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    s->px0 = x;
    s->px1 = x + nx;
    s->py0 = y;
    s->py1 = y + ny;
    s->pace_mode = MKG_PACE_RECT;
    return MKG_OK;
}

int mkg_set_paced_list(mkg_sim *s, const int64_t *cells, int64_t n)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    const long long words = (s->ncell + 31) / 32;
    std::vector<unsigned int> bits(words, 0u);
    for (int64_t i = 0; i < n; ++i) {
        if (cells[i] < 0 || cells[i] >= s->ncell)
            return set_err(s, MKG_ERR_ARG, "Cell index out of range: %lld.",
                           (long long)cells[i]);
        bits[cells[i] >> 5] |= 1u << (cells[i] & 31);
    }
    dfree(s->d_pace_bits);
    CK(s, cudaMalloc((void **)&s->d_pace_bits, words * sizeof(unsigned int)));
    CK(s, cudaMemcpyAsync(s->d_pace_bits, bits.data(),
                          words * sizeof(unsigned int),
                          cudaMemcpyHostToDevice, s->stream));
    CK(s, cudaStreamSynchronize(s->stream));
    s->pace_mode = n > 0 ? MKG_PACE_LIST : MKG_PACE_NONE;
    return MKG_OK;
}

int mkg_set_protocol(mkg_sim *s, const double *events, int64_t n)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (n < 0 || (n > 0 && !events))
        return set_err(s, MKG_ERR_ARG, "invalid event array");
    const int st = s->pacer.populate(events, n);
    if (st != mkg::PACER_OK) return pacer_err(s, st);
    return MKG_OK;
}

int mkg_set_log(mkg_sim *s, const int32_t *item, const int64_t *cell,
                int64_t ncol, int32_t nan_check)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (ncol < 0 || (ncol > 0 && (!item || !cell)) || ncol > INT_MAX)
        return set_err(s, MKG_ERR_ARG, "invalid log columns");
    const int n_items_total = s->cfg.n_state + 1 + s->cfg.n_inter;
    std::vector<int> slot_of(n_items_total, -1);
    std::vector<int> items;
    for (int64_t j = 0; j < ncol; ++j) {
        if (item[j] < 0 || item[j] >= n_items_total)
            return set_err(s, MKG_ERR_ARG, "invalid log item %d", item[j]);
        if (item[j] == s->cfg.n_state && !diffusion_on(s))
            return set_err(s, MKG_ERR_ARG,
                           "diffusion current logged without diffusion");
        if (cell[j] < 0 || cell[j] >= s->ncell)
            return set_err(s, MKG_ERR_ARG, "invalid log cell %lld",
                           (long long)cell[j]);
        if (slot_of[item[j]] < 0) {
            slot_of[item[j]] = (int)items.size();
            items.push_back(item[j]);
        }
    }
    std::vector<int> cols((size_t)std::max<size_t>(items.size(), 1) *
                          s->pitch, -1);
    for (int64_t j = 0; j < ncol; ++j)
        cols[(size_t)slot_of[item[j]] * s->pitch + cell[j]] = (int)j;
    dfree(s->d_log_items);
    dfree(s->d_log_cols);
    CK(s, cudaMalloc((void **)&s->d_log_items,
                     std::max<size_t>(items.size(), 1) * sizeof(int)));
    CK(s, cudaMalloc((void **)&s->d_log_cols, cols.size() * sizeof(int)));
    if (!items.empty())
        CK(s, cudaMemcpyAsync(s->d_log_items, items.data(),
                              items.size() * sizeof(int),
                              cudaMemcpyHostToDevice, s->stream));
    CK(s, cudaMemcpyAsync(s->d_log_cols, cols.data(),
                          cols.size() * sizeof(int), cudaMemcpyHostToDevice,
                          s->stream));
    CK(s, cudaStreamSynchronize(s->stream));
    s->n_log_items = (int)items.size();
    s->h_log_item.assign(item, item + ncol);
    s->h_log_cell.assign(cell, cell + ncol);
    /* A new column count invalidates the log buffers. */
    if ((int)ncol != s->log_ncol) {
        dfree(s->d_log);
        dfree(s->d_log_dbl);
        if (s->h_log) cudaFreeHost(s->h_log);
        s->h_log = nullptr;
        s->cap_rows = 0;
    }
    s->log_ncol = (int)ncol;
    s->nan_check = nan_check ? 1 : 0;
    return MKG_OK;
}

int mkg_set_tuning(mkg_sim *s, int32_t steps_per_launch,
                   int32_t blocks_per_sm, int32_t use_graphs)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (steps_per_launch < 0 || blocks_per_sm < 0)
        return set_err(s, MKG_ERR_ARG, "invalid tuning");
    clear_graphs(s);
    s->steps_per_launch = steps_per_launch;
    s->blocks_per_sm = blocks_per_sm;
    s->use_graphs = use_graphs != 0;
    return MKG_OK;
}

int mkg_run_begin(mkg_sim *s, double tmin, double tmax, double default_dt,
                  double log_interval)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (!(default_dt > 0))
        return set_err(s, MKG_ERR_ARG, "Step size must be greater than zero.");
    if (!(log_interval > 0))
        return set_err(s, MKG_ERR_ARG, "log interval must be positive");
    if (diffusion_on(s) && s->cfg.diffusion == MKG_DIFF_HETERO &&
        (!s->d_gx || !s->d_gy))
        return set_err(s, MKG_ERR_ORDER, "conductance field not set");
    if (s->cfg.diffusion == MKG_DIFF_CONN && !s->d_nbr_ptr)
        return set_err(s, MKG_ERR_ORDER, "connections not set");
    if (s->pace_mode == MKG_PACE_LIST && !s->d_pace_bits)
        return set_err(s, MKG_ERR_ORDER, "paced cell list not set");
    if (!s->d_log_cols) {
        int r = mkg_set_log(s, nullptr, nullptr, 0, 0);
        if (r) return r;
    }
    if (s->partner && !s->partner->d_log_cols) {
        int r = mkg_set_log(s->partner, nullptr, nullptr, 0, 0);
        if (r) return set_err(s, r, "%s", mkg_last_error(s->partner));
    }
    clear_graphs(s);
    const int st = s->sched.begin(s->pacer, tmin, tmax, default_dt,
                                  log_interval);
    if (st != mkg::PACER_OK) return pacer_err(s, st);
    s->running = true;
    s->halted = false;
    s->last_rows = 0;
    return MKG_OK;
}

int mkg_run_chunk(mkg_sim *s, int64_t max_steps, double *t_out,
                  int64_t *rows_out)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (rows_out) *rows_out = 0;
    if (!s->running)
        return set_err(s, MKG_ERR_ORDER, "mkg_run_chunk before mkg_run_begin");
    if (max_steps < 1) return set_err(s, MKG_ERR_ARG, "max_steps < 1");
    {
        /* The grid barrier counts (steps + skew) x CTAs arrivals per chunk
         * in the low 31 bits of its counter (the top bit carries a NaN
         * halt): a chunk is kept short enough not to overflow it */
        const int64_t ctas = std::max<int64_t>(
            1, (int64_t)s->occ_blocks * (int64_t)s->num_sms);
        const int64_t cap = (int64_t)0x7fffffff / ctas - 2 - s->wait_skew;
        max_steps = std::min<int64_t>(max_steps, std::max<int64_t>(cap, 1));
    }
    s->last_ms = 0;
    s->last_launches = 0;
    s->last_cell_steps = 0;
    s->last_rows = 0;
    if (s->sched.done()) {
        if (t_out) *t_out = s->sched.time();
        s->running = false;
        return MKG_DONE;
    }

    /* Log rows that fit a 256 MiB buffer, at least 16; with a device frame
     * buffer, the rows it has left. */
    const int64_t ncol = std::max(s->log_ncol, 1);
    int64_t row_cap = (int64_t)(256ll << 20) / (ncol * 8);
    row_cap = std::max<int64_t>(16, std::min<int64_t>(row_cap, max_steps));
    if (s->frame_buf) {
        row_cap = s->frame_rows - s->frame_next;
        if (row_cap <= 0 && s->sched.next_logs())
            return set_err(s, MKG_ERR_ARG, "the frame buffer is full");
        row_cap = std::max<int64_t>(row_cap, 0);
    }
    mkg_sim *p = s->partner;
    if (p) {
        const int64_t pcol = std::max(p->log_ncol, 1);
        row_cap = std::min<int64_t>(
            row_cap, std::max<int64_t>(16, (int64_t)(256ll << 20) /
                                               (pcol * 8)));
    }
    int r = ensure_schedule(s, max_steps, row_cap);
    if (r) return r;
    if (p && (r = ensure_schedule(p, 1, row_cap)))
        return set_err(s, r, "%s", mkg_last_error(p));

    /* Host schedule for this chunk (openclsim.c:1051-1162). */
    int64_t n = 0, rows = 0;
    while (n < max_steps && !s->sched.done()) {
        if (s->sched.next_logs() && rows == row_cap) break;
        mkg::StepRecord rec;
        const int st = s->sched.next(&rec);
        if (st != mkg::PACER_OK) {
            s->running = false;
            return pacer_err(s, st);
        }
        mkg_step &h = s->h_steps[n];
        h.t = rec.t;
        h.dt = rec.dt;
        h.pace = rec.pace;
        h.tf = (float)rec.t;
        h.dtf = (float)rec.dt;
        h.pacef = (float)rec.pace;
        if (rec.log) {
            h.log_row = (int)rows;
            if (s->real == 4) {
                s->h_time[rows] = (double)(float)rec.t;
                s->h_pace[rows] = (double)(float)rec.pace;
            } else {
                s->h_time[rows] = rec.t;
                s->h_pace[rows] = rec.pace;
            }
            rows++;
        } else {
            h.log_row = -1;
        }
        s->h_tend[n] = rec.t_end;
        n++;
    }
    CK(s, cudaMemcpyAsync(s->d_steps, s->h_steps, n * sizeof(mkg_step),
                          cudaMemcpyHostToDevice, s->stream));

    /* Launch geometry */
    const int bx = s->cfg.block_x, by = s->cfg.block_y;
    mkg_launch a;
    fill_launch(s, &a);
    if (s->frame_buf)
        a.log = (char *)s->frame_buf +
                (size_t)s->frame_next * s->log_ncol * s->real;
    if (s->cfg.stage) {
        r = encode_stage_maps(s);
        if (r) return r;
        a.stage_tx = (int)s->lay.tx;
    }
    const int threads = bx * by;
    /* The partner's launch block: its buffers, log and pacing; steps,
     * status and barrier are this simulation's */
    mkg_launch b;
    if (p) {
        fill_launch(p, &b);
        b.status = s->d_status;
        b.steps = nullptr;
    }
    const long long nblocks =
        p ? ((long long)(a.ntiles_x * (long long)a.ntiles_y +
                         b.ntiles_x * (long long)b.ntiles_y) * 32 +
             threads - 1) / threads
          : blocks_needed(s, &a);
    int bpsm = s->blocks_per_sm > 0 ? std::min(s->blocks_per_sm, s->occ_blocks)
                                    : s->occ_blocks;
    long long coop_blocks = std::min<long long>(nblocks,
                                                (long long)bpsm * s->num_sms);
    /* Split teams larger than the CTA are clusters of whole CTAs */
    const int ncl = cluster_ctas(s);
    coop_blocks -= coop_blocks % ncl;
    int spl = s->steps_per_launch > 0 ? s->steps_per_launch : 1 << 20;

    /* All launches of the chunk are queued without host synchronisation;
     * the status word is reset once. Launch i covers steps
     * [off_i, off_i + m_i); a NaN halt or device error makes every later
     * launch return at once. */
    mkg_status init;
    init.barrier = 0;
    init.error = MKG_DEV_OK;
    init.halt_step = MKG_NO_HALT;
    init.timeout_block = -1;
    *s->h_status = init;
    CK(s, cudaMemcpyAsync(s->d_status, s->h_status, sizeof(mkg_status),
                          cudaMemcpyHostToDevice, s->stream));
    CK(s, cudaMemsetAsync(s->d_warp_epoch, 0,
                          s->n_warp_epoch * sizeof(unsigned int), s->stream));
    CK(s, cudaEventRecord(s->ev0, s->stream));

    const int64_t nlaunch = (n + spl - 1) / spl;
    /* (graphs are not used with a partner, whose log buffers may grow
     * between chunks) */
    const bool graph = s->use_graphs && nlaunch > 1 && !p;
    const int v_sel0 = s->v_sel;
    cudaGraphExec_t exec = nullptr;
    if (graph) {
        const std::string key = std::to_string(n) + ":" +
                                std::to_string(spl) + ":" +
                                std::to_string(v_sel0);
        auto it = s->graphs.find(key);
        if (it != s->graphs.end()) exec = it->second;
        else {
            CK(s, cudaStreamBeginCapture(s->stream,
                                         cudaStreamCaptureModeThreadLocal));
        }
    }
    if (!exec) {
        int epoch = 0;
        for (int64_t off = 0; off < n; off += spl) {
            const int64_t m = std::min<int64_t>(n - off, spl);
            a.steps = s->d_steps + off;
            a.nsteps = (int)m;
            a.step0 = (int)off;
            a.epoch_base = epoch;
            a.v_sel = diffusion_on(s) ? (v_sel0 ^ (int)(off & 1)) : 0;
            void *args[] = {&a, &s->tmaps};
            void *args_p[] = {&a, &b, &s->junction};
            cudaLaunchConfig_t lc;
            memset(&lc, 0, sizeof(lc));
            cudaLaunchAttribute attr[1];
            lc.blockDim = dim3(threads, 1, 1);
            lc.stream = s->stream;
            lc.attrs = attr;
            long long grid;
            /* (a kernel with split teams larger than the CTA has its
             * cluster shape compiled in; grids are whole clusters) */
            if (m > 1) {
                grid = coop_blocks;
                attr[lc.numAttrs].id = cudaLaunchAttributeCooperative;
                attr[lc.numAttrs++].val.cooperative = 1;
                epoch += (int)(m - 1);
            } else {
                grid = std::min<long long>(nblocks, 1 << 30);
                grid -= grid % ncl;
            }
            lc.gridDim = dim3((unsigned)grid, 1, 1);
            lc.dynamicSmemBytes = s->tile_smem;
            const cudaError_t e = cudaLaunchKernelExC(
                &lc, (const void *)s->kernel, p ? args_p : args);
            if (e != cudaSuccess) {
                if (graph) {
                    cudaGraph_t g = nullptr;
                    cudaStreamEndCapture(s->stream, &g);
                    if (g) cudaGraphDestroy(g);
                }
                s->running = false;
                return set_err(s, MKG_ERR_CUDA,
                               "kernel launch failed: %s",
                               cudaGetErrorString(e));
            }
        }
        if (graph) {
            cudaGraph_t g = nullptr;
            CK(s, cudaStreamEndCapture(s->stream, &g));
            const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess)
                return set_err(s, MKG_ERR_CUDA, "graph instantiation: %s",
                               cudaGetErrorString(e));
            s->graphs[std::to_string(n) + ":" + std::to_string(spl) + ":" +
                      std::to_string(v_sel0)] = exec;
        }
    }
    if (graph) CK(s, cudaGraphLaunch(exec, s->stream));
    s->last_launches += nlaunch;
    s->n_launches += nlaunch;
    CK(s, cudaEventRecord(s->ev1, s->stream));
    CK(s, cudaMemcpyAsync(s->h_status, s->d_status, sizeof(mkg_status),
                          cudaMemcpyDeviceToHost, s->stream));
    CK(s, cudaStreamSynchronize(s->stream));
    if (s->h_status->error == MKG_DEV_LAUNCH) {
        s->running = false;
        return set_err(s, MKG_ERR_CUDA,
                       "the kernel was launched with clusters of another"
                       " size than it was generated for");
    }
    if (s->h_status->error != MKG_DEV_OK) {
        s->running = false;
        return set_err(s, MKG_ERR_TIMEOUT,
                       "device barrier wait timed out (block %d)",
                       s->h_status->timeout_block);
    }
    int64_t done = n;
    bool halted = false;
    if (s->h_status->halt_step != MKG_NO_HALT) {
        done = (int64_t)s->h_status->halt_step + 1;
        halted = true;
    }
    if (diffusion_on(s)) s->v_sel = v_sel0 ^ (int)(done & 1);
    if (p) p->v_sel = s->v_sel;
    s->last_cell_steps = done * s->ncell;

    /* Rows written by the executed steps */
    int64_t rows_done = 0;
    for (int64_t i = 0; i < done; ++i)
        if (s->h_steps[i].log_row >= 0) rows_done = s->h_steps[i].log_row + 1;
    if (s->frame_buf) {
        /* Frames stay on the device */
        s->frame_next += rows_done;
    } else if (rows_done > 0 && s->log_ncol > 0) {
        const long long cnt = rows_done * (long long)s->log_ncol;
        s->n_launches++;
        if (s->real == 4)
            k_log_to_double<float><<<grid_for(cnt), 256, 0, s->stream>>>(
                (const float *)s->d_log, s->d_log_dbl, cnt);
        else
            k_log_to_double<double><<<grid_for(cnt), 256, 0, s->stream>>>(
                (const double *)s->d_log, s->d_log_dbl, cnt);
        CK(s, cudaGetLastError());
        CK(s, cudaMemcpyAsync(s->h_log, s->d_log_dbl, cnt * sizeof(double),
                              cudaMemcpyDeviceToHost, s->stream));
    }
    if (p && rows_done > 0 && p->log_ncol > 0) {
        /* The partner's rows, through the same stream */
        const long long cnt = rows_done * (long long)p->log_ncol;
        s->n_launches++;
        if (p->real == 4)
            k_log_to_double<float><<<grid_for(cnt), 256, 0, s->stream>>>(
                (const float *)p->d_log, p->d_log_dbl, cnt);
        else
            k_log_to_double<double><<<grid_for(cnt), 256, 0, s->stream>>>(
                (const double *)p->d_log, p->d_log_dbl, cnt);
        CK(s, cudaGetLastError());
        CK(s, cudaMemcpyAsync(p->h_log, p->d_log_dbl, cnt * sizeof(double),
                              cudaMemcpyDeviceToHost, s->stream));
    }
    if (p) p->last_rows = rows_done;
    CK(s, cudaStreamSynchronize(s->stream));
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    s->last_ms = ms;
    s->last_rows = rows_done;
    if (rows_out) *rows_out = rows_done;
    const double t = done > 0 ? s->h_tend[done - 1] : s->sched.time();
    if (t_out) *t_out = t;
    if (halted) {
        s->running = false;
        s->halted = true;
        return MKG_HALT_NAN;
    }
    if (s->sched.done()) {
        s->running = false;
        return MKG_DONE;
    }
    return MKG_OK;
}

int mkg_read_log(mkg_sim *s, double *time, double *pace, double *values,
                 int64_t rows)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (rows < 0 || rows > s->last_rows)
        return set_err(s, MKG_ERR_ARG, "rows exceeds the rows of the last"
                       " chunk");
    if (time) memcpy(time, s->h_time.data(), rows * sizeof(double));
    if (pace) memcpy(pace, s->h_pace.data(), rows * sizeof(double));
    if (values && s->log_ncol > 0)
        memcpy(values, s->h_log, rows * s->log_ncol * sizeof(double));
    return MKG_OK;
}

int mkg_last_stats(const mkg_sim *s, double *kernel_ms, int64_t *launches,
                   int64_t *cell_steps)
{
    if (!s) return set_err(nullptr, MKG_ERR_ARG, "null argument");
    if (kernel_ms) *kernel_ms = s->last_ms;
    if (launches) *launches = s->last_launches;
    if (cell_steps) *cell_steps = s->last_cell_steps;
    return MKG_OK;
}

int mkg_set_wait(mkg_sim *s, int64_t timeout_ns, int32_t skew)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (timeout_ns < 1000000 || timeout_ns > 60000000000LL || skew < 0 ||
        skew > 65536)
        return set_err(s, MKG_ERR_ARG,
                       "the wait bound must be 1 ms to 60 s, the skew 0 to"
                       " 65536");
    clear_graphs(s);
    s->timeout_ns = timeout_ns;
    s->wait_skew = skew;
    return MKG_OK;
}

int mkg_set_partner(mkg_sim *s, mkg_sim *partner, double gft, int64_t cty)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (!partner) {
        s->partner = nullptr;
        clear_graphs(s);
        return MKG_OK;
    }
    const mkg_config &c = s->cfg, &d = partner->cfg;
    if (partner == s || c.device != d.device || c.real_bytes != d.real_bytes)
        return set_err(s, MKG_ERR_ARG,
                       "the partner must be another simulation of the same"
                       " precision on the same device");
    if (c.diffusion != MKG_DIFF_GRID || d.diffusion != MKG_DIFF_GRID ||
        !c.two_d || !d.two_d || c.stage || d.stage ||
        c.hi_mode != MKG_HI_NONE || d.hi_mode != MKG_HI_NONE ||
        c.split > 1 || d.split > 1)
        return set_err(s, MKG_ERR_ARG,
                       "fiber-tissue simulations use 2D grid diffusion"
                       " without staging, accumulation modes or split"
                       " tiles");
    if (c.ny > d.ny || cty < 0 || cty + c.ny > d.ny)
        return set_err(s, MKG_ERR_ARG,
                       "the junction rows must lie inside the tissue");
    clear_graphs(s);
    s->partner = partner;
    s->junction.gft = gft;
    s->junction.gftf = (float)gft;
    s->junction.nfy = (int)c.ny;
    s->junction.cty = cty;
    partner->v_sel = s->v_sel;
    return MKG_OK;
}

int mkg_stage_layout(const mkg_config *cfg, int64_t *out)
{
    if (!cfg || !out) return set_err(nullptr, MKG_ERR_ARG, "null argument");
    StageLayout L;
    compute_stage_layout(cfg, &L);
    const int64_t v[7] = {L.sw, L.lo, L.np, L.v_rows, L.gx, L.bytes, L.tx};
    memcpy(out, v, sizeof(v));
    return MKG_OK;
}

int mkg_set_frame_buffer(mkg_sim *s, void *dev_ptr, int64_t rows)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (rows < 0 || (rows > 0 && !dev_ptr))
        return set_err(s, MKG_ERR_ARG, "invalid frame buffer");
    clear_graphs(s);
    s->frame_buf = rows > 0 ? dev_ptr : nullptr;
    s->frame_rows = rows;
    s->frame_next = 0;
    return MKG_OK;
}

int mkg_launch_count(const mkg_sim *s, int64_t *count)
{
    if (!s || !count) return set_err(nullptr, MKG_ERR_ARG, "null argument");
    *count = s->n_launches;
    return MKG_OK;
}

int mkg_stream(const mkg_sim *s, void **stream)
{
    if (!s || !stream) return set_err(nullptr, MKG_ERR_ARG, "null argument");
    *stream = (void *)s->stream;
    return MKG_OK;
}

int64_t mkg_schedule_preview(const double *events, int64_t n_events,
                             double tmin, double tmax, double default_dt,
                             double log_interval, int64_t max_steps,
                             double *t, double *dt, double *pace,
                             int32_t *log)
{
    mkg::Pacer p;
    int st = p.populate(events, n_events);
    if (st != mkg::PACER_OK) return st;
    mkg::Schedule sc;
    st = sc.begin(p, tmin, tmax, default_dt, log_interval);
    if (st != mkg::PACER_OK) return st;
    int64_t n = 0;
    while (n < max_steps && !sc.done()) {
        mkg::StepRecord r;
        st = sc.next(&r);
        if (st != mkg::PACER_OK) return st;
        if (t) t[n] = r.t;
        if (dt) dt[n] = r.dt;
        if (pace) pace[n] = r.pace;
        if (log) log[n] = r.log ? 1 : 0;
        n++;
    }
    return n;
}

}  /* extern "C" */

/* ------------------------------------------------------------------------ */
/* State upload without allocation                                          */
/* ------------------------------------------------------------------------ */
/*
 * mkg_set_state stages the caller's doubles in a device buffer that the
 * handle allocates with cudaMalloc on first use. Some callers must not make
 * that call when they upload a state: a host loop driving pacing in real
 * time, where cudaMalloc's implicit device-wide synchronisation stalls
 * every stream, or a host that keeps device memory in its own pool or under
 * a fixed budget, where a cudaMalloc outside that pool can fail.
 * mkg_set_state_static stages through the fixed array below instead.
 *
 * The array lives in the library's device image: every GPU on which the
 * library's module is loaded holds these MKG_STATIC_STAGE_BYTES until the
 * process exits. Every call, from every handle, shares it and it keeps the
 * last call's contents; the whole used range is overwritten by each call's
 * copy before the conversion kernel reads it, so nothing needs clearing.
 * Calls whose work overlaps on the GPU (different streams, no ordering
 * between them) race on the array.
 */
#define MKG_STATIC_STAGE_DOUBLES (2ll * 1024 * 1024)   /* 16 MiB */

static __device__ __align__(256) double
    mkg_static_stage[MKG_STATIC_STAGE_DOUBLES];

namespace {

/* Same conversion as k_aos_to_soa, reading the fixed staging array. */
template <typename Real>
__global__ void k_aos_to_soa_static(Real *out, long long ncell, int nvar,
                                    long long pitch, int skip_var, Real *alt)
{
    const long long n = ncell * nvar;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
         i < n; i += (long long)gridDim.x * blockDim.x) {
        const int s = (int)(i / ncell);
        const long long c = i - (long long)s * ncell;
        const Real v = (Real)mkg_static_stage[c * nvar + s];
        if (s == skip_var) alt[c] = v;
        else out[(long long)s * pitch + c] = v;
    }
}

#define MKG_MAX_DEVICES 64
std::mutex g_static_mutex;
double *g_static_addr[MKG_MAX_DEVICES] = {nullptr};

/* Device address of the staging array on the given device, looked up once
 * per device with that device current. In host code the array's name is
 * only a host-side stand-in, not a device address. */
int static_stage_address(mkg_sim *s, double **addr)
{
    const int dev = s->cfg.device;
    if (dev < 0 || dev >= MKG_MAX_DEVICES)
        return set_err(s, MKG_ERR_ARG, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (!g_static_addr[dev]) {
        int prev = 0;
        CK(s, cudaGetDevice(&prev));
        CK(s, cudaSetDevice(dev));
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, mkg_static_stage);
        cudaSetDevice(prev);
        if (e != cudaSuccess)
            return set_err(s, MKG_ERR_CUDA,
                           "cudaGetSymbolAddress(mkg_static_stage) failed:"
                           " %s", cudaGetErrorString(e));
        g_static_addr[dev] = (double *)p;
    }
    *addr = g_static_addr[dev];
    return MKG_OK;
}

template <typename Real>
int upload_state_static(mkg_sim *s, const double *aos, double *stage)
{
    const int nvar = s->cfg.n_state;
    const size_t bytes = (size_t)s->ncell * nvar * sizeof(double);
    const int skip = diffusion_on(s) ? s->cfg.i_vm : -1;
    Real *alt = (Real *)((char *)s->d_vbuf +
                         (size_t)s->v_sel * s->pitch * s->real);
    CK(s, cudaMemcpyAsync(stage, aos, bytes, cudaMemcpyHostToDevice,
                          s->stream));
    s->n_launches++;
    k_aos_to_soa_static<Real><<<grid_for(s->ncell * nvar), 256, 0,
                                 s->stream>>>(
        (Real *)s->d_state, s->ncell, nvar, s->pitch, skip, alt);
    CK(s, cudaGetLastError());
    CK(s, cudaStreamSynchronize(s->stream));
    return MKG_OK;
}

}  // namespace

extern "C" int mkg_set_state_static(mkg_sim *s, const double *state,
                                    int64_t n)
{
    if (!s || !state) return set_err(s, MKG_ERR_ARG, "null argument");
    if (n != s->ncell * s->cfg.n_state)
        return set_err(s, MKG_ERR_ARG,
                       "'state_in' must have size nx * ny * n_states.");
    if (s->cfg.hi_mode != MKG_HI_NONE)
        return set_err(s, MKG_ERR_ARG,
                       "mkg_set_state_static: not available for simulations"
                       " with accumulated states; use mkg_set_state");
    if (n > MKG_STATIC_STAGE_DOUBLES)
        return set_err(s, MKG_ERR_ARG,
                       "mkg_set_state_static: a state of %lld values exceeds"
                       " the static staging area of %lld values (16 MiB);"
                       " use mkg_set_state for this simulation",
                       (long long)n, (long long)MKG_STATIC_STAGE_DOUBLES);
    double *stage = nullptr;
    const int r = static_stage_address(s, &stage);
    if (r) return r;
    if (s->real == 4) return upload_state_static<float>(s, state, stage);
    return upload_state_static<double>(s, state, stage);
}


/* ------------------------------------------------------------------------ */
/* Discrete adjoint                                                         */
/* ------------------------------------------------------------------------ */

extern "C" int mkg_adj_attach(mkg_sim *s, const void *cubin, size_t size,
                              int32_t seg_steps)
{
    if (!s || !cubin || !size) return set_err(s, MKG_ERR_ARG, "null argument");
    if (seg_steps < 1) return set_err(s, MKG_ERR_ARG, "seg_steps < 1");
    if (s->adj_lib) {
        cudaLibraryUnload(s->adj_lib);
        s->adj_lib = nullptr;
    }
    CK(s, cudaLibraryLoadData(&s->adj_lib, cubin, nullptr, nullptr, 0,
                              nullptr, nullptr, 0));
    CK(s, cudaLibraryGetKernel(&s->adj_fwd, s->adj_lib, "mkg_tissue_step"));
    CK(s, cudaLibraryGetKernel(&s->adj_bwd, s->adj_lib,
                               "mkg_tissue_adjoint"));
    const int threads = s->cfg.block_x * s->cfg.block_y;
    /* The trajectory kernel stages tiles like the simulation's kernel */
    if (s->cfg.stage)
        CK(s, cudaKernelSetAttributeForDevice(
                  s->adj_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                  (int)s->tile_smem, s->cfg.device));
    CK(s, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &s->adj_occ_fwd, (const void *)s->adj_fwd, threads, s->tile_smem));
    /* The reverse kernel's CTA size is its launch bound */
    cudaFuncAttributes fa;
    CK(s, cudaFuncGetAttributes(&fa, (const void *)s->adj_bwd));
    s->adj_bwd_threads = fa.maxThreadsPerBlock;
    if (s->adj_bwd_threads < 32 || s->adj_bwd_threads % 32)
        return set_err(s, MKG_ERR_ARG, "invalid reverse kernel CTA size");
    CK(s, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &s->adj_occ_bwd, (const void *)s->adj_bwd, s->adj_bwd_threads, 0));
    if (s->adj_occ_fwd < 1 || s->adj_occ_bwd < 1)
        return set_err(s, MKG_ERR_CUDA, "adjoint kernels cannot be resident");
    {
        /* The trajectory kernel's grid may be larger than the forward's */
        const size_t nw = (size_t)s->adj_occ_fwd * s->num_sms *
                          (size_t)(s->cfg.block_x / 32);
        if (nw > s->n_warp_epoch) {
            dfree(s->d_warp_epoch);
            CK(s, cudaMalloc((void **)&s->d_warp_epoch,
                             nw * sizeof(unsigned int)));
            s->n_warp_epoch = nw;
        }
    }
    const size_t plane = (size_t)s->pitch * s->real;
    dfree(s->d_traj);
    dfree(s->d_lam);
    dfree(s->d_mu);
    dfree(s->d_gfield);
    dfree(s->d_gg);
    dfree(s->d_probe_col);
    dfree(s->d_fsteps);
    dfree(s->d_bsteps);
    CK(s, cudaMalloc(&s->d_traj, plane * s->cfg.n_state * seg_steps));
    CK(s, cudaMalloc(&s->d_lam, plane * s->cfg.n_state));
    CK(s, cudaMalloc(&s->d_mu, plane * 2));
    CK(s, cudaMalloc(&s->d_gfield, plane * std::max(s->cfg.n_field, 1)));
    CK(s, cudaMalloc(&s->d_gg, plane * 2));
    CK(s, cudaMalloc((void **)&s->d_probe_col, s->pitch * sizeof(int)));
    CK(s, cudaMalloc((void **)&s->d_fsteps, seg_steps * sizeof(mkg_step)));
    CK(s, cudaMalloc((void **)&s->d_bsteps, seg_steps * sizeof(mkg_step)));
    s->adj_seg = seg_steps;
    return MKG_OK;
}

extern "C" int mkg_adj_forward(mkg_sim *s, double tmin, double tmax,
                               double dt, double log_interval,
                               int64_t *rows_out)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (!s->adj_lib) return set_err(s, MKG_ERR_ORDER, "mkg_adj_attach first");
    int r = mkg_run_begin(s, tmin, tmax, dt, log_interval);
    if (r) return r;
    s->adj_sched.clear();
    s->adj_seg_start.clear();
    s->adj_seg_len.clear();
    s->adj_seg_vsel.clear();
    s->adj_log.clear();
    s->adj_rows = 0;
    const size_t plane = (size_t)s->pitch * s->real;
    const size_t vplane = (size_t)s->pitch * s->vbytes;
    const size_t hi_bytes = s->d_hi ? (size_t)s->pitch * 8 * s->cfg.n_hi : 0;
    const size_t ckpt_bytes = plane * s->cfg.n_state + vplane + hi_bytes;
    if (s->ckpt_bytes != ckpt_bytes) {
        for (void *p : s->adj_ckpt) cudaFree(p);
        s->adj_ckpt.clear();
        s->ckpt_bytes = ckpt_bytes;
    }
    size_t nseg = 0;
    int status = MKG_OK;
    while (status == MKG_OK) {
        /* Checkpoint: state planes, the current V plane and the
         * accumulation planes (FP64 states or compensation terms) */
        if (nseg >= s->adj_ckpt.size()) {
            void *p = nullptr;
            CK(s, cudaMalloc(&p, ckpt_bytes));
            s->adj_ckpt.push_back(p);
        }
        char *ck = (char *)s->adj_ckpt[nseg];
        CK(s, cudaMemcpyAsync(ck, s->d_state, plane * s->cfg.n_state,
                              cudaMemcpyDeviceToDevice, s->stream));
        CK(s, cudaMemcpyAsync(ck + plane * s->cfg.n_state,
                              (char *)s->d_vbuf + (size_t)s->v_sel * vplane,
                              vplane, cudaMemcpyDeviceToDevice, s->stream));
        if (hi_bytes)
            CK(s, cudaMemcpyAsync(ck + plane * s->cfg.n_state + vplane,
                                  s->d_hi, hi_bytes,
                                  cudaMemcpyDeviceToDevice, s->stream));
        s->adj_seg_vsel.push_back(s->v_sel);
        double t = 0;
        int64_t rows = 0;
        status = mkg_run_chunk(s, s->adj_seg, &t, &rows);
        if (status < 0) return status;
        if (status == MKG_HALT_NAN)
            return set_err(s, MKG_ERR_ARG,
                           "NaN in the forward pass of the adjoint");
        const long long done = s->last_cell_steps / s->ncell;
        s->adj_seg_start.push_back((long long)s->adj_sched.size());
        s->adj_seg_len.push_back(done);
        for (long long i = 0; i < done; ++i) {
            mkg_step st = s->h_steps[i];
            if (st.log_row >= 0) st.log_row += (int)s->adj_rows;
            s->adj_sched.push_back(st);
        }
        s->adj_log.insert(s->adj_log.end(), s->h_log,
                          s->h_log + rows * s->log_ncol);
        s->adj_rows += rows;
        nseg++;
    }
    if (rows_out) *rows_out = s->adj_rows;
    return MKG_OK;
}

extern "C" int mkg_adj_read_log(mkg_sim *s, double *values, int64_t rows)
{
    if (!s || !values) return set_err(s, MKG_ERR_ARG, "null argument");
    if (rows != s->adj_rows)
        return set_err(s, MKG_ERR_ARG, "expected %lld rows",
                       (long long)s->adj_rows);
    memcpy(values, s->adj_log.data(), rows * s->log_ncol * sizeof(double));
    return MKG_OK;
}

namespace {

template <typename Real>
__global__ void k_sum_planes(const Real *__restrict__ in, long long n,
                             long long pitch, double *out)
{
    /* out[p] = sum over the first n entries of plane p (one block per
     * plane, fixed order: deterministic) */
    __shared__ double part[256];
    const Real *x = in + (long long)blockIdx.x * pitch;
    double acc = 0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) acc += (double)x[i];
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = part[0];
}

int launch_coop(mkg_sim *s, cudaKernel_t k, void *arg, int occ,
                long long need, size_t smem = 0, int threads = 0)
{
    cudaLaunchConfig_t lc;
    memset(&lc, 0, sizeof(lc));
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    lc.blockDim = dim3(threads ? threads : s->cfg.block_x * s->cfg.block_y,
                       1, 1);
    lc.gridDim = dim3((unsigned)std::min<long long>(
        need, (long long)occ * s->num_sms), 1, 1);
    lc.stream = s->stream;
    lc.dynamicSmemBytes = smem;
    /* A staging kernel takes the tensor maps as a second parameter */
    void *args[] = {arg, &s->tmaps};
    CK(s, cudaLaunchKernelExC(&lc, (const void *)k, args));
    s->n_launches++;
    return MKG_OK;
}

template <typename Real>
int adj_backward(mkg_sim *s, const double *lgrad, int64_t rows,
                 double *grad_fields, double *grad_g)
{
    const size_t plane = (size_t)s->pitch * s->real;
    const int ncol = s->log_ncol;
    /* Loss gradient (as Real) and the probe column of each cell */
    dfree(s->d_lgrad);
    const long long nl = std::max<long long>(rows * ncol, 1);
    CK(s, cudaMalloc(&s->d_lgrad, nl * s->real));
    if (rows * ncol > 0) {
        int r = upload_real<Real>(s, lgrad, rows * ncol, s->d_lgrad);
        if (r) return r;
    }
    std::vector<int> pc(s->pitch, -1);
    for (int j = 0; j < ncol; ++j) {
        if (s->h_log_item[j] != s->cfg.i_vm)
            return set_err(s, MKG_ERR_ARG,
                           "the adjoint loss needs V columns only");
        if (pc[s->h_log_cell[j]] >= 0)
            return set_err(s, MKG_ERR_ARG, "cell logged twice");
        pc[s->h_log_cell[j]] = j;
    }
    CK(s, cudaMemcpyAsync(s->d_probe_col, pc.data(), pc.size() * sizeof(int),
                          cudaMemcpyHostToDevice, s->stream));
    CK(s, cudaMemsetAsync(s->d_lam, 0, plane * s->cfg.n_state, s->stream));
    CK(s, cudaMemsetAsync(s->d_mu, 0, plane * 2, s->stream));
    CK(s, cudaMemsetAsync(s->d_gfield, 0,
                          plane * std::max(s->cfg.n_field, 1), s->stream));
    CK(s, cudaMemsetAsync(s->d_gg, 0, plane * 2, s->stream));
    /* Per-edge gradient parts: four per cell on heterogeneous grids, one
     * per CSR entry with connections */
    size_t n_ge = 0;
    if (s->cfg.diffusion == MKG_DIFF_HETERO) n_ge = 4 * (size_t)s->pitch;
    if (s->cfg.diffusion == MKG_DIFF_CONN) n_ge = (size_t)s->n_nbr;
    if (n_ge != s->n_ge) {
        dfree(s->d_ge);
        s->n_ge = 0;
        if (n_ge) {
            CK(s, cudaMalloc((void **)&s->d_ge, n_ge * sizeof(double)));
            s->n_ge = n_ge;
        }
    }
    if (s->n_ge)
        CK(s, cudaMemsetAsync(s->d_ge, 0, s->n_ge * sizeof(double),
                              s->stream));
    s->h_edge_grad.clear();
    int mu_sel = 0;
    /* The whole schedule on the device, once: the reverse kernel reads the
     * logged rows, the trajectory kernel logs nothing */
    const size_t total = s->adj_sched.size();
    std::vector<mkg_step> fsteps(s->adj_sched);
    for (mkg_step &st : fsteps) st.log_row = -1;
    dfree(s->d_fsteps);
    dfree(s->d_bsteps);
    CK(s, cudaMalloc((void **)&s->d_fsteps,
                     std::max<size_t>(total, 1) * sizeof(mkg_step)));
    CK(s, cudaMalloc((void **)&s->d_bsteps,
                     std::max<size_t>(total, 1) * sizeof(mkg_step)));
    if (total) {
        CK(s, cudaMemcpyAsync(s->d_fsteps, fsteps.data(),
                              total * sizeof(mkg_step),
                              cudaMemcpyHostToDevice, s->stream));
        CK(s, cudaMemcpyAsync(s->d_bsteps, s->adj_sched.data(),
                              total * sizeof(mkg_step),
                              cudaMemcpyHostToDevice, s->stream));
    }
    mkg_status init;
    init.barrier = 0;
    init.error = MKG_DEV_OK;
    init.halt_step = MKG_NO_HALT;
    init.timeout_block = -1;
    if (s->cfg.stage) {
        int r = encode_stage_maps(s);
        if (r) return r;
    }
    /* Segments are queued without host synchronisation. The status word
     * is set once; before each launch only its barrier counter restarts, so
     * a device error stays recorded (every launch checks it first and
     * returns) and is read once at the end. */
    *s->h_status = init;
    CK(s, cudaMemcpyAsync(s->d_status, s->h_status, sizeof(mkg_status),
                          cudaMemcpyHostToDevice, s->stream));
    for (long long g = (long long)s->adj_seg_len.size() - 1; g >= 0; --g) {
        const long long n = s->adj_seg_len[g];
        if (n == 0) continue;
        const long long st0 = s->adj_seg_start[g];
        /* Restore the segment's checkpoint */
        const char *ck = (const char *)s->adj_ckpt[g];
        const int vsel = s->adj_seg_vsel[g];
        const size_t vplane = (size_t)s->pitch * s->vbytes;
        CK(s, cudaMemcpyAsync(s->d_state, ck, plane * s->cfg.n_state,
                              cudaMemcpyDeviceToDevice, s->stream));
        CK(s, cudaMemcpyAsync((char *)s->d_vbuf + (size_t)vsel * vplane,
                              ck + plane * s->cfg.n_state, vplane,
                              cudaMemcpyDeviceToDevice, s->stream));
        if (s->d_hi && s->cfg.n_hi > 0)
            CK(s, cudaMemcpyAsync(s->d_hi,
                                  ck + plane * s->cfg.n_state + vplane,
                                  (size_t)s->pitch * 8 * s->cfg.n_hi,
                                  cudaMemcpyDeviceToDevice, s->stream));
        /* Forward over the segment, recording the trajectory */
        mkg_launch a;
        fill_launch(s, &a);
        a.n_log_items = 0;
        a.log_ncol = 0;
        a.nan_check = 0;
        a.steps = s->d_fsteps + st0;
        a.nsteps = (int)n;
        a.v_sel = vsel;
        a.traj = s->d_traj;
        if (s->cfg.stage) a.stage_tx = (int)s->lay.tx;
        CK(s, cudaMemsetAsync(&s->d_status->barrier, 0, sizeof(unsigned),
                              s->stream));
        CK(s, cudaMemsetAsync(s->d_warp_epoch, 0,
                              s->n_warp_epoch * sizeof(unsigned int),
                              s->stream));
        int r = launch_coop(s, s->adj_fwd, &a, s->adj_occ_fwd,
                            blocks_needed(s, &a), s->tile_smem);
        if (r) return r;
        /* The segment in reverse */
        mkg_adj_launch b;
        memset(&b, 0, sizeof(b));
        b.f = a;
        b.f.steps = s->d_bsteps + st0;
        b.f.traj = nullptr;
        b.traj = s->d_traj;
        b.lam = s->d_lam;
        b.mu = s->d_mu;
        b.gfield = s->d_gfield;
        b.gg = s->d_gg;
        b.ge = s->d_ge;
        b.probe_col = s->d_probe_col;
        b.lgrad = s->d_lgrad;
        b.nprobe = ncol;
        b.mu_sel = mu_sel;
        CK(s, cudaMemsetAsync(&s->d_status->barrier, 0, sizeof(unsigned),
                              s->stream));
        const long long bwd_blocks =
            ((long long)a.ntiles_x * a.ntiles_y * 32 + s->adj_bwd_threads -
             1) / s->adj_bwd_threads;
        r = launch_coop(s, s->adj_bwd, &b, s->adj_occ_bwd, bwd_blocks, 0,
                        s->adj_bwd_threads);
        if (r) return r;
        mu_sel ^= (int)(n & 1);
    }
    CK(s, cudaMemcpyAsync(s->h_status, s->d_status, sizeof(mkg_status),
                          cudaMemcpyDeviceToHost, s->stream));
    CK(s, cudaStreamSynchronize(s->stream));
    if (s->h_status->error != MKG_DEV_OK)
        return set_err(s, MKG_ERR_TIMEOUT,
                       s->h_status->error == MKG_DEV_STAGE
                           ? "tile staging failed in the adjoint"
                           : "device barrier wait timed out in the adjoint");
    /* Field gradients (AoS doubles) and the conductance gradients */
    if (grad_fields && s->cfg.n_field > 0) {
        int r = download_soa<Real>(s, grad_fields, s->cfg.n_field,
                                   s->d_gfield, plain_slots(), nullptr);
        if (r) return r;
    }
    if (grad_g) {
        double *d_out = nullptr;
        CK(s, cudaMalloc((void **)&d_out, 2 * sizeof(double)));
        s->n_launches++;
        k_sum_planes<Real><<<2, 256, 0, s->stream>>>(
            (const Real *)s->d_gg, s->ncell, s->pitch, d_out);
        cudaError_t e = cudaMemcpyAsync(grad_g, d_out, 2 * sizeof(double),
                                        cudaMemcpyDeviceToHost, s->stream);
        cudaStreamSynchronize(s->stream);
        cudaFree(d_out);
        if (e != cudaSuccess)
            return set_err(s, MKG_ERR_CUDA, "gradient copy failed");
    }
    /* Per-edge gradients: the two cells' parts of every edge */
    if (s->n_ge) {
        std::vector<double> part(s->n_ge);
        CK(s, cudaMemcpyAsync(part.data(), s->d_ge, s->n_ge * sizeof(double),
                              cudaMemcpyDeviceToHost, s->stream));
        CK(s, cudaStreamSynchronize(s->stream));
        if (s->cfg.diffusion == MKG_DIFF_CONN) {
            const size_t nc = s->conn_pos.size() / 2;
            s->h_edge_grad.resize(nc);
            for (size_t c = 0; c < nc; ++c)
                s->h_edge_grad[c] = part[s->conn_pos[2 * c]] +
                                    part[s->conn_pos[2 * c + 1]];
        } else {
            /* gx edges (ix, iy)-(ix+1, iy) at iy*(nx-1)+ix: the right part
             * of the left cell plus the left part of the right cell; gy
             * edges (ix, iy)-(ix, iy+1) at iy*nx+ix: up part plus down */
            const long long nx = s->cfg.nx, ny = s->cfg.ny;
            const long long p = s->pitch;
            const double *L = part.data(), *R = L + p, *D = R + p, *U = D + p;
            s->h_edge_grad.clear();
            for (long long iy = 0; iy < ny; ++iy)
                for (long long ix = 0; ix + 1 < nx; ++ix) {
                    const long long c = ix + iy * nx;
                    s->h_edge_grad.push_back(R[c] + L[c + 1]);
                }
            if (s->cfg.two_d)
                for (long long iy = 0; iy + 1 < ny; ++iy)
                    for (long long ix = 0; ix < nx; ++ix) {
                        const long long c = ix + iy * nx;
                        s->h_edge_grad.push_back(U[c] + D[c + nx]);
                    }
        }
    }
    return MKG_OK;
}

}  // namespace

extern "C" int mkg_adj_conductance_gradient(mkg_sim *s, double *out,
                                            int64_t n)
{
    if (!s || (n > 0 && !out)) return set_err(s, MKG_ERR_ARG,
                                              "null argument");
    if (s->cfg.diffusion != MKG_DIFF_HETERO &&
        s->cfg.diffusion != MKG_DIFF_CONN)
        return set_err(s, MKG_ERR_ARG,
                       "per-edge gradients need per-edge conductances or"
                       " connections");
    if (n != (int64_t)s->h_edge_grad.size())
        return set_err(s, MKG_ERR_ARG,
                       "expected %lld edge gradients (after"
                       " mkg_adj_backward)",
                       (long long)s->h_edge_grad.size());
    if (n > 0) memcpy(out, s->h_edge_grad.data(), n * sizeof(double));
    return MKG_OK;
}

extern "C" int mkg_adj_backward(mkg_sim *s, const double *lgrad,
                                int64_t rows, double *grad_fields,
                                double *grad_g)
{
    if (!s) return set_err(s, MKG_ERR_ARG, "null argument");
    if (!s->adj_lib) return set_err(s, MKG_ERR_ORDER, "mkg_adj_attach first");
    if (rows != s->adj_rows)
        return set_err(s, MKG_ERR_ARG, "expected %lld rows",
                       (long long)s->adj_rows);
    if (rows * s->log_ncol > 0 && !lgrad)
        return set_err(s, MKG_ERR_ARG, "null loss gradient");
    if (s->real == 4)
        return adj_backward<float>(s, lgrad, rows, grad_fields, grad_g);
    return adj_backward<double>(s, lgrad, rows, grad_fields, grad_g);
}

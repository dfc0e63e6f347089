// tl_internal.cuh -- shared definitions of the GB300 TeaLeaf runtime.
//
// Data layout in HBM.  Every 2-D field is stored row-major, x fastest, in the
// reference's padded coordinates (column c, row r in [0, n+2h)), but each row
// is padded to a pitch that is a multiple of 32 elements and shifted so that
// the first interior cell (c = h) of every row starts on a 256-byte boundary.
// A field pointer f addresses padded (c, r) as f[c + r * pitch]; the
// allocation starts `lead` elements before f.  All solver kernels touch the
// interior only, plus the x/y neighbours of interior cells.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/tealeaf_capi.h"

namespace tl {

constexpr int kStrip = 4;          // block-Jacobi strip height (cuda_kernel_header.hpp:11)
constexpr int kWarpCols = 32;      // columns per warp: one column per lane
constexpr int kBlockWarps = 8;     // warps per CTA; each warp owns one 4-row strip
constexpr int kBlockThreads = kWarpCols * kBlockWarps;
constexpr int kMaxRedBlocks = 152 * 8;  // grid cap for reducing kernels (SMs x 8)

// Scalars of the device-resident solve (the tea_solve.f90 locals).
struct DevScalars {
    double rro, pw, rrn, alpha, beta;
    double error, old_error, initial_residual, eps, epslim;
    double rr, bb;
    double sum[4];                 // generic reduction outputs
    double inner_rr;               // mixed-precision inner scalars
    double theta;                  // Chebyshev / PPCG centre of the spectrum
    // inner FP32 Krylov solve of the mixed form (its scalars stay FP64)
    double in_rro, in_pw, in_rrn, in_alpha, in_beta, in_target;
    // FP32 CG presteps of mixed PPCG: where the inner epilogues record the
    // Lanczos coefficients (the cg_alphas / cg_betas of the FP64 path)
    double *lanczos_a, *lanczos_b;
    int in_n, in_max;
    int prestep;                   // 1: the inner epilogues act as the CG phase's
    int n;                         // current iteration (1-based)
    int max_iters;
    int done;                      // 0 running, 1 converged, 2 max_iters, 3 switch, 4 breakdown
    int n_exit;
    int cheby_calc_steps;
    int est_itc;
    int solver;
    int first;
    int presteps;
    int ppcg_inner;
    int ppcg_iters;                // PPCG outer iterations taken in this solve
    int pad;
};

enum DoneCode { kRunning = 0, kConverged = 1, kMaxIters = 2, kSwitch = 3, kBreakdown = 4 };

// What the last CTA of a kernel does with the grid-wide sums.
enum Epilogue : int {
    kEpiNone = 0,
    kEpiStore,        // sum[0..nv) <- totals
    kEpiResid,        // old_error = rr; initial_residual = sqrt|rr|
    kEpiRro,          // rro = total
    kEpiCgW,          // pw; alpha = rro/pw; cg_alphas[n] = alpha
    kEpiCgUr,         // rrn; beta = rrn/rro; cg_betas[n]; error = rro = rrn
    kEpiFinish,       // end-of-iteration exit test (tea_solve.f90:400-417)
    kEpiPpcgZr,       // rro = r.z; alpha = rro/pw
    kEpiPpcgRrn,      // rrn; beta = rrn/rro; error = rro = rrn
    kEpiChebyNorm,    // rr (the residual norm of this Chebyshev step)
    kEpiChebyFinish,  // optional norm, cheby_calc_steps++, exit test
    kEpiJacobi,       // error = sum |du|, exit test
    kEpiPw,           // pw = p.w
    kEpiFinishNoSwitch,  // exit test once Chebyshev/PPCG has taken over
    kEpiPwZr,         // pw = sum 0, rro = sum 1, alpha = rro/pw (PPCG outer)
};

struct Geo {
    int nx, ny, h;
    int pitch;
    int nstrips;        // ceil(ny / 4)
    int tiles_x;        // ceil(nx / 32)
    int tiles_y;        // ceil(nstrips / 8)
    int tiles;
};

struct RedCtx {
    double *partials;            // kMaxRedBlocks * 4 doubles
    unsigned int *counter;
    DevScalars *sc;
    double *cg_alphas, *cg_betas;
    const int *done;             // early-exit flag (nullptr: always run)
    int epi;
};

struct Chunk {
    tl_config_t cfg;
    int device;
    cudaStream_t stream;
    Geo g;
    int nx, ny, h, pitch, rows, lead;
    size_t alloc_elems;          // per field
    // fields (padded reference coordinates)
    double *density, *energy0, *energy1, *u, *u0, *p, *r, *w, *z, *mi, *kx, *ky, *sd,
        *rtemp, *utemp, *r_store, *cp, *bfp, *volume, *un;
    double *diag;                // diag(A), refreshed with Kx/Ky by common_init
    double *stage;               // (rows x (nx + 2h)) contiguous copy buffer of
                                 // tl_get_field / tl_set_field (allocated on first use)
    std::vector<void *> allocations;
    // mesh
    double *vertexx, *vertexy, *cellx, *celly, *celldx, *celldy;
    std::vector<double> h_vertexx, h_vertexy, h_cellx, h_celly;
    double dx, dy, dt;
    // reductions and scalars
    double *partials;
    unsigned int *counter;
    DevScalars *sc;              // device
    DevScalars *sc_host;         // pinned mirror
    DevScalars *poll_host;       // two pinned slots polled by the solve loop
    cudaEvent_t poll_ev[2];
    double *cg_alphas, *cg_betas;          // device, max_iters + 2
    double *ch_alphas, *ch_betas;          // device coefficient arrays
    int n_coefs_cap;
    // state carried across timesteps (tea_solve.f90:55,58 SAVE variables)
    bool first;
    double eigmin, eigmax, theta, cn;
    // graphs of the device-resident loop
    cudaGraphExec_t graphs[6];   // CG, PPCG, Chebyshev, Jacobi, mixed inner
    long long graph_kernels[6];
    long long launches;
    int grid_red;                // CTAs of the grid-stride kernels
    // mixed precision state (allocated on first use)
    void *mixed;
    int inner_fuse;              // FP32 PPCG inner steps per HBM pass (1: one kernel per step)
    int inner_seg;               // 4-row strips per CTA share of the fused inner kernel (0: automatic)
    bool inner_fold_rrn;         // the last fused inner pass also sums PPCG's rrn
    int sms;                     // multiprocessors of the device
    // learned warm start model and buffers (tl_warm.cu)
    void *warm;
    int warm_history;            // previous increments the warm start combines (1..8)
    int warm_projection;         // TL_WARM_PROJ_*: energy (Galerkin) or minimal residual
    double rx, ry;
    // per-kernel profiling (CUDA events around eager launches)
    bool profiling;
    bool capturing;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
    std::vector<const char *> prof_names;
    std::vector<long long> prof_launches;
    std::vector<double> prof_ms;
};

// ---------------------------------------------------------------- helpers
void set_error(const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);
#define TL_CUDA(call)                                       \
    do {                                                    \
        cudaError_t _e = (call);                            \
        if (_e != cudaSuccess) return cuda_fail(_e, #call); \
    } while (0)

inline RedCtx red_ctx(Chunk *c, int epi, bool fast) {
    RedCtx r;
    r.partials = c->partials;
    r.counter = c->counter;
    r.sc = c->sc;
    r.cg_alphas = c->cg_alphas;
    r.cg_betas = c->cg_betas;
    r.done = fast ? &c->sc->done : nullptr;
    r.epi = epi;
    return r;
}

double *field_ptr(Chunk *c, int field);
// cudaMalloc, except when tl_test_fail_alloc has armed a simulated failure
cudaError_t device_malloc(void **p, size_t bytes);

// ------------------------------------------------ kernel launch wrappers
// (tl_kernels.cu).  `fast` selects the device-resident form: scalars are
// read from / written to DevScalars and the kernel is skipped once done.
int launch_common_init(Chunk *c, int coefficient, double rx, double ry, const int zero[4],
                       int reflective);
int launch_residual(Chunk *c, int epi);
int launch_norm(Chunk *c, const double *a, const double *b, int epi);
int launch_cg_init(Chunk *c, int epi);
int launch_cg_w(Chunk *c, int epi, bool fast);
int launch_cg_ur(Chunk *c, double alpha, int epi, bool fast);
int launch_cg_p(Chunk *c, double beta, int epi, bool fast);
int launch_cheby_init(Chunk *c, double theta);
int launch_cheby_calc_p(Chunk *c, int step, int epi, bool fast);
int launch_cheby_calc_u(Chunk *c, int epi, bool fast);
int launch_ppcg_init(Chunk *c, int step, int epi);
int launch_ppcg_init_sd(Chunk *c, double theta);
int launch_ppcg_init_sd_new(Chunk *c, double theta, bool fast);  // fast: theta from DevScalars
int launch_ppcg_update_r(Chunk *c, bool fast);
int launch_ppcg_calc_sd_new(Chunk *c, int step, bool fast);
int launch_copy(Chunk *c, double *dst, const double *src, bool fast);
int launch_ppcg_rrn(Chunk *c, int epi, bool fast);
int launch_ppcg_zr(Chunk *c, int epi, bool fast);
int launch_ppcg_w_store_zr(Chunk *c, bool fast, bool five);  // cg_w + ppcg_store_zr, one pass
int launch_ppcg_up(Chunk *c, int epi, bool fast);  // u += alpha p, p = z + beta p (mixed, fused passes)
int launch_ppcg_p(Chunk *c, double beta, int epi, bool fast);
int launch_jacobi(Chunk *c, int epi, bool fast);
int launch_finalise(Chunk *c);
int launch_field_summary(Chunk *c);
int launch_set_field(Chunk *c);
int launch_generate(Chunk *c, int nstates, const tl_state_t *states);
int launch_fill(Chunk *c, double *f, double v);
int launch_reflect(Chunk *c, double *f, int depth);

// ------------------------------------------------------ profiling
// bracket one launch with events when profiling (call before / after)
int prof_begin(Chunk *c, const char *name, int *slot);
void prof_end(Chunk *c, int slot);
int prof_flush(Chunk *c);   // after a stream sync: accumulate elapsed times

// ------------------------------------------------------ chunk operations
int chunk_sync_scalars(Chunk *c);        // device -> pinned host mirror
int chunk_push_scalars(Chunk *c);        // pinned host mirror -> device
int chunk_initialise_mesh(Chunk *c, double xmin, double ymin, double dx, double dy);
int chunk_update_halo(Chunk *c, const int *fields, int depth);
int chunk_upload_coefs(Chunk *c, const double *a, const double *b, int n);
int solve_timestep(Chunk *c, tl_solve_info_t *info);       // tl_solve.cu
// run `iters`-iteration graphs of `body` (graph slot `phase`) until the
// device sets DevScalars::done; *done_out receives it (tl_solve.cu)
int run_phase(Chunk *c, int (*body)(Chunk *), int iters, int phase, int *done_out);
constexpr int kPhaseMixedInner = 4;
constexpr int kPhaseMixedPre = 5;
int solve_timestep_mixed(Chunk *c, tl_solve_info_t *info); // tl_mixed.cu
void mixed_free(Chunk *c);
int mixed_ppcg_prepare(Chunk *c);  // FP32 operator + preconditioner copies
// the CG presteps of the first PPCG solve in FP32 (FP64 scalars and Lanczos
// coefficients): runs until the switch test, then u += d and r = u0 - A u in
// FP64; *done_out gets the device's exit code (kSwitch when it switched)
int mixed_ppcg_presteps(Chunk *c, int *done_out);
int mixed_ppcg_inner(Chunk *c);    // PPCG inner steps in FP32, z in FP64
// the outer u/r update fused with the inner start, then the steps; *did_rrn
// tells whether the last pass also summed (r - r_store).z (kEpiPpcgRrn)
int mixed_ppcg_ur_inner(Chunk *c, bool *did_rrn);
// whether mixed PPCG runs its inner steps as fused passes: its outer pass
// then updates r alone, and u += alpha p moves into the p pass (launch_ppcg_up)
bool mixed_fused(const Chunk *c);
void drop_graphs(Chunk *c);        // after a change that captured graphs depend on
constexpr int kFusedMax = 5;           // most FP32 PPCG inner steps fused into one pass
constexpr int kInnerFuseDefault = 5;
constexpr int kInnerSegDefault = 0;
// warm starts (tl_warm.cu)
void warm_free(Chunk *c);
void warm_reset(Chunk *c);                // forget u^(n-1) (tl_start)
long long warm_param_count();
int warm_set_options(Chunk *c, int history, int projection);
int warm_set_model(Chunk *c, const float *params, long long n);
bool warm_ready(Chunk *c);                // a network is loaded
int warm_features(Chunk *c, float *dst);  // [ny][nx][8] inputs + target
// Galerkin warm start after common_init: sets u and r, returns the plain
// start's residual norm in *r0 and the chosen start's r.r in *rr
int warm_start_or_fallback(Chunk *c, tl_solve_info_t *info, double *r0, double *rr);

}  // namespace tl

// tl_mixed.cu -- the mixed-precision form of the implicit solve: FP32 inner
// Krylov iterations inside an FP64 iterative-refinement loop.
//
// FP64 state: u, u0, density, Kx, Ky, energy (the chunk's fields).  Each
// timestep:
//   r = u0 - A u in FP64 (the operator of tea_leaf_common.cuknl:19-39);
//   stop once ||r|| < tl_eps * ||r_0||, the test of tea_solve.f90:407, with
//   ||r_0|| the initial residual of the plain solve from u = u0;
//   otherwise solve A d = r with preconditioned CG in FP32 to tl_inner_eps
//   relative, u += d in FP64, and repeat.  Refinement also stops when an
//   outer step no longer halves ||r|| (the FP64 residual floor).
// The inner CG keeps its vectors, the operator coefficients (Kx, Ky and the
// Jacobi diagonal, rounded to FP32) and the arithmetic in FP32; its dot
// products are Kahan-compensated FP32 sums per thread and per warp, combined
// across warps and CTAs in FP64, and alpha, beta and the exit test are FP64
// scalars on the device, as in the FP64 path.
//
// The FP32 operator uses the difference form
//     A x = x_c + Ky_n (x_c - x_n) + Ky_c (x_c - x_s) + Kx_e (x_c - x_e) + Kx_c (x_c - x_w)
// which is the same matrix as the reference's diag*x_c - sum K x_nb but avoids
// the cancellation of two large terms when Kx is ~1e4 and x is smooth.
#include <math.h>
#include <string.h>

#include <chrono>

#include "tl_internal.cuh"

namespace tl {

namespace {

struct Mixed {
    float *kx, *ky, *mi, *d, *r, *p, *w, *z;
    std::vector<void *> allocs;
};

constexpr int kItersInner = 16;
constexpr int kMaxOuter = 40;

enum InnerEpi { kInNone = 0, kInInit, kInW, kInUr };

// ------------------------------------------------ compensated FP32 sums
struct CSum {
    float s, e;  // value ~= s + e
};

__device__ __forceinline__ void csum_add(CSum &a, float x) {
    // Kahan-Babuska: e carries the low part lost by each addition
    const float y = x + a.e;
    const float t = a.s + y;
    a.e = y - (t - a.s);
    a.s = t;
}

__device__ __forceinline__ CSum csum_merge(CSum a, CSum b) {
    // TwoSum of the high parts, then the low parts
    const float s = a.s + b.s;
    const float bb = s - a.s;
    const float err = (a.s - (s - bb)) + (b.s - bb);
    CSum r;
    r.s = s;
    r.e = err + (a.e + b.e);
    return r;
}

__device__ void inner_epilogue(DevScalars *s, int epi, double tot) {
    switch (epi) {
    case kInInit:
        s->in_rro = tot;
        s->in_target = s->in_target * sqrt(fabs(tot));  // in_target holds inner_eps on entry
        s->in_n = 0;
        if (!(sqrt(fabs(tot)) > 0.0)) s->done = kConverged;
        break;
    case kInW:
        s->in_pw = tot;
        s->in_alpha = s->in_rro / s->in_pw;
        break;
    case kInUr: {
        s->in_rrn = tot;
        s->in_beta = s->in_rrn / s->in_rro;
        s->in_rro = s->in_rrn;
        s->in_n += 1;
        const double e = sqrt(fabs(tot));
        if (isnan(e)) s->done = kBreakdown;
        else if (e < s->in_target || s->in_n >= s->in_max) s->done = kConverged;
        break;
    }
    default:
        break;
    }
}

// grid-stride strip kernel over FP32 bodies with one compensated dot product
template <class Body>
__global__ void __launch_bounds__(kBlockThreads) k_mixed(Geo g, int pitch32, Body body,
                                                         double *partials, unsigned int *counter,
                                                         DevScalars *sc, int epi, int check_done) {
    if (check_done && *(volatile const int *)&sc->done) return;
    body.setup(sc);
    CSum acc = {0.f, 0.f};
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = blockIdx.x; t < g.tiles; t += gridDim.x) {
        const int tx = t % g.tiles_x, ty = t / g.tiles_x;
        const int i = tx * kWarpCols + lane;
        const int s = ty * kBlockWarps + warp;
        if (i < g.nx && s < g.nstrips) {
            const int j0 = s * kStrip;
            const int m = min(kStrip, g.ny - j0);
            const int64_t b32 = (int64_t)(i + g.h) + (int64_t)(j0 + g.h) * pitch32;
            const int64_t b64 = (int64_t)(i + g.h) + (int64_t)(j0 + g.h) * g.pitch;
            body(b32, b64, m, acc);
        }
    }
    if (epi == kInNone) return;
    // warp: compensated butterfly; CTA and grid: FP64
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        CSum o;
        o.s = __shfl_xor_sync(0xffffffffu, acc.s, off);
        o.e = __shfl_xor_sync(0xffffffffu, acc.e, off);
        acc = csum_merge(acc, o);
    }
    __shared__ double sh[kBlockWarps];
    __shared__ int is_last;
    if (lane == 0) sh[warp] = (double)acc.s + (double)acc.e;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kBlockWarps; ++w) t += sh[w];
        partials[blockIdx.x] = t;
        __threadfence();
        is_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double t = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) t += __ldcg(&partials[b]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    __syncthreads();
    if (lane == 0) sh[warp] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < kBlockWarps; ++w) tot += sh[w];
        inner_epilogue(sc, epi, tot);
        __threadfence();
        *counter = 0u;
    }
}

// A x in FP32, difference form, on the m rows of a strip
__device__ __forceinline__ void strip_apply32(const float *__restrict__ kx,
                                              const float *__restrict__ ky,
                                              const float *__restrict__ x, int pitch, int64_t base,
                                              int m, float (&xc)[4], float (&ax)[4]) {
    float xr[6], kyr[5];
#pragma unroll
    for (int k = -1; k <= 4; ++k)
        if (k <= m) xr[k + 1] = x[base + (int64_t)k * pitch];
#pragma unroll
    for (int k = 0; k <= 4; ++k)
        if (k <= m) kyr[k] = ky[base + (int64_t)k * pitch];
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (k < m) {
            const int64_t i = base + (int64_t)k * pitch;
            const float c = xr[k + 1];
            float v = fmaf(kyr[k + 1], c - xr[k + 2], c);
            v = fmaf(kyr[k], c - xr[k], v);
            v = fmaf(kx[i + 1], c - x[i + 1], v);
            v = fmaf(kx[i], c - x[i - 1], v);
            ax[k] = v;
            xc[k] = c;
        }
}

// Kx, Ky -> FP32; Mi = 1/diag(A) computed in FP64, stored in FP32
struct BodyConvert {
    const double *kx64, *ky64;
    float *kx, *ky, *mi;
    int pitch32, pitch64, nx, ny, h;
    __device__ void setup(DevScalars *) {}
    __device__ void operator()(int64_t b32, int64_t b64, int m, CSum &) const {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = b64 + (int64_t)k * pitch64, j = b32 + (int64_t)k * pitch32;
                const double diag = (1.0 + (ky64[i + pitch64] + ky64[i])) + (kx64[i + 1] + kx64[i]);
                kx[j] = (float)kx64[i];
                ky[j] = (float)ky64[i];
                mi[j] = (float)(1.0 / diag);
                // the east face of the last column and the north face of the top row
                kx[j + 1] = (float)kx64[i + 1];
                ky[j + pitch32] = (float)ky64[i + pitch64];
            }
    }
};

template <bool DIAG>
struct BodyInnerInit {  // r = (float) r64; z = M^-1 r; p = z; d = 0; sum r.z
    const double *r64;
    const float *mi;
    float *r, *z, *p, *d;
    int pitch32, pitch64;
    __device__ void setup(DevScalars *) {}
    __device__ void operator()(int64_t b32, int64_t b64, int m, CSum &acc) const {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t j = b32 + (int64_t)k * pitch32;
                const float rv = (float)r64[b64 + (int64_t)k * pitch64];
                const float zv = DIAG ? rv * mi[j] : rv;
                r[j] = rv;
                z[j] = zv;
                p[j] = zv;
                d[j] = 0.f;
                csum_add(acc, rv * zv);
            }
    }
};

struct BodyInnerW {  // w = A p; sum p.w
    const float *p, *kx, *ky;
    float *w;
    int pitch32;
    __device__ void setup(DevScalars *) {}
    __device__ void operator()(int64_t b32, int64_t, int m, CSum &acc) const {
        float xc[4], ax[4];
        strip_apply32(kx, ky, p, pitch32, b32, m, xc, ax);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                w[b32 + (int64_t)k * pitch32] = ax[k];
                csum_add(acc, xc[k] * ax[k]);
            }
    }
};

template <bool DIAG>
struct BodyInnerUr {  // d += alpha p; r -= alpha w; z = M^-1 r; sum r.z
    float *d, *r, *z;
    const float *p, *w, *mi;
    int pitch32;
    float alpha;
    __device__ void setup(DevScalars *s) { alpha = (float)s->in_alpha; }
    __device__ void operator()(int64_t b32, int64_t, int m, CSum &acc) const {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t j = b32 + (int64_t)k * pitch32;
                d[j] = fmaf(alpha, p[j], d[j]);
                const float rv = fmaf(-alpha, w[j], r[j]);
                r[j] = rv;
                const float zv = DIAG ? rv * mi[j] : rv;
                if (DIAG) z[j] = zv;
                csum_add(acc, rv * zv);
            }
    }
};

struct BodyInnerP {  // p = z + beta p
    float *p;
    const float *z;
    int pitch32;
    float beta;
    __device__ void setup(DevScalars *s) { beta = (float)s->in_beta; }
    __device__ void operator()(int64_t b32, int64_t, int m, CSum &) const {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t j = b32 + (int64_t)k * pitch32;
                p[j] = fmaf(beta, p[j], z[j]);
            }
    }
};

struct BodyUpdateU {  // u += d (FP64)
    double *u;
    const float *d;
    int pitch32, pitch64;
    __device__ void setup(DevScalars *) {}
    __device__ void operator()(int64_t b32, int64_t b64, int m, CSum &) const {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = b64 + (int64_t)k * pitch64;
                u[i] = u[i] + (double)d[b32 + (int64_t)k * pitch32];
            }
    }
};

Mixed *mixed_of(Chunk *c) { return (Mixed *)c->mixed; }

int mixed_alloc(Chunk *c) {
    if (c->mixed) return TL_OK;
    Mixed *mx = new Mixed();
    c->mixed = mx;
    const size_t n = (size_t)c->lead + (size_t)c->pitch * (size_t)c->rows + 32;
    float **arr[] = {&mx->kx, &mx->ky, &mx->mi, &mx->d, &mx->r, &mx->p, &mx->w, &mx->z};
    for (float **a : arr) {
        void *p = nullptr;
        cudaError_t e = cudaMalloc(&p, n * sizeof(float));
        if (e != cudaSuccess) return cuda_fail(e, "mixed cudaMalloc");
        mx->allocs.push_back(p);
        TL_CUDA(cudaMemsetAsync(p, 0, n * sizeof(float), c->stream));
        *a = (float *)p + c->lead;
    }
    return TL_OK;
}

template <class Body>
int run32(Chunk *c, const char *name, const Body &b, int epi, bool check_done) {
    const int grid = c->g.tiles < c->grid_red ? c->g.tiles : c->grid_red;
    int slot = -1;
    if (c->profiling && !c->capturing) prof_begin(c, name, &slot);
    k_mixed<Body><<<grid, kBlockThreads, 0, c->stream>>>(c->g, c->pitch, b, c->partials, c->counter,
                                                         c->sc, epi, check_done ? 1 : 0);
    if (slot >= 0) prof_end(c, slot);
    c->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "mixed kernel launch");
    return TL_OK;
}

int inner_body(Chunk *c) {
    Mixed *mx = mixed_of(c);
    const bool diag = c->cfg.precond != TL_PREC_NONE;
    int rc;
    BodyInnerW bw{mx->p, mx->kx, mx->ky, mx->w, c->pitch};
    if ((rc = run32(c, "mixed_w", bw, kInW, true))) return rc;
    if (diag) {
        BodyInnerUr<true> bu{mx->d, mx->r, mx->z, mx->p, mx->w, mx->mi, c->pitch, 0.f};
        if ((rc = run32(c, "mixed_ur", bu, kInUr, true))) return rc;
    } else {
        BodyInnerUr<false> bu{mx->d, mx->r, mx->z, mx->p, mx->w, mx->mi, c->pitch, 0.f};
        if ((rc = run32(c, "mixed_ur", bu, kInUr, true))) return rc;
    }
    BodyInnerP bp{mx->p, diag ? mx->z : mx->r, c->pitch, 0.f};
    return run32(c, "mixed_p", bp, kInNone, true);
}

}  // namespace

void mixed_free(Chunk *c) {
    Mixed *mx = mixed_of(c);
    if (!mx) return;
    for (void *p : mx->allocs) cudaFree(p);
    delete mx;
    c->mixed = nullptr;
}

int solve_timestep_mixed(Chunk *c, tl_solve_info_t *info) {
    const auto t0 = std::chrono::steady_clock::now();
    memset(info, 0, sizeof *info);
    const tl_config_t &cf = c->cfg;
    if (cf.solver != TL_SOLVER_CG || cf.precond == TL_PREC_JAC_BLOCK || cf.reflective_boundary) {
        set_error("tl_precision mixed supports tl_use_cg with none or jac_diag and non-reflective "
                  "boundaries");
        return TL_ERR_ARG;
    }
    int rc;
    if ((rc = mixed_alloc(c))) return rc;
    Mixed *mx = mixed_of(c);
    const bool diag = cf.precond == TL_PREC_JAC_DIAG;

    // tea_leaf_common_init (FP64), then the FP32 copies of the operator
    const double rx = c->dt / (c->dx * c->dx), ry = c->dt / (c->dy * c->dy);
    c->rx = rx;
    c->ry = ry;
    const int zero[4] = {1, 1, 1, 1};
    if ((rc = launch_common_init(c, cf.coefficient, rx, ry, zero, 0))) return rc;
    BodyConvert bc{c->kx, c->ky, mx->kx, mx->ky, mx->mi, c->pitch, c->pitch, c->nx, c->ny, c->h};
    if ((rc = run32(c, "mixed_convert", bc, kInNone, false))) return rc;

    DevScalars &h = *c->sc_host;
    memset(&h, 0, sizeof h);
    if ((rc = chunk_push_scalars(c))) return rc;
    // r = u0 - A u, ||r||^2 (FP64)
    if ((rc = launch_residual(c, kEpiResid))) return rc;
    if ((rc = chunk_sync_scalars(c))) return rc;
    const double r0 = h.initial_residual;
    const double target = cf.eps * r0;
    double rn = r0, rn_prev = 0.0;
    int outer = 0, inner_total = 0;
    int status = TL_OK;
    while (true) {
        if (rn < target) break;
        if (outer > 0 && rn > 0.5 * rn_prev) break;  // FP64 residual floor reached
        if (outer >= kMaxOuter || inner_total >= cf.max_iters) {
            status = TL_WARN_MAXITER;
            break;
        }
        // inner FP32 PCG on A d = r
        h.done = kRunning;
        h.in_target = cf.inner_eps;
        h.in_max = cf.max_iters - inner_total;
        if ((rc = chunk_push_scalars(c))) return rc;
        if (diag) {
            BodyInnerInit<true> bi{c->r, mx->mi, mx->r, mx->z, mx->p, mx->d, c->pitch, c->pitch};
            if ((rc = run32(c, "mixed_init", bi, kInInit, false))) return rc;
        } else {
            BodyInnerInit<false> bi{c->r, mx->mi, mx->r, mx->z, mx->p, mx->d, c->pitch, c->pitch};
            if ((rc = run32(c, "mixed_init", bi, kInInit, false))) return rc;
        }
        int done = kRunning;
        if ((rc = run_phase(c, inner_body, kItersInner, kPhaseMixedInner, &done))) return rc;
        if (done == kBreakdown) {
            set_error("mixed solve: breakdown in the FP32 inner iteration");
            status = TL_ERR_BREAKDOWN;
            break;
        }
        inner_total += h.in_n;
        // u += d (FP64), r = u0 - A u (FP64)
        BodyUpdateU bu{c->u, mx->d, c->pitch, c->pitch};
        if ((rc = run32(c, "mixed_update_u", bu, kInNone, false))) return rc;
        if ((rc = launch_residual(c, kEpiStore))) return rc;
        if ((rc = chunk_sync_scalars(c))) return rc;
        rn_prev = rn;
        rn = sqrt(fabs(h.sum[0]));
        outer++;
    }
    info->status = status;
    info->outer_iters = outer;
    info->inner_iters = inner_total;
    info->iterations = inner_total;
    info->initial_residual = r0;
    info->error = rn;
    info->error_ratio = rn / r0;
    if (cf.check_result) info->exact_error_ratio = rn / r0;
    if ((rc = launch_finalise(c))) return rc;
    TL_CUDA(cudaStreamSynchronize(c->stream));
    if ((rc = prof_flush(c))) return rc;
    info->rx = rx;
    info->ry = ry;
    info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return status < 0 ? status : TL_OK;
}

}  // namespace tl

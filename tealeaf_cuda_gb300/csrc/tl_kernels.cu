// tl_kernels.cu -- FP64 solver kernels of the GB300 TeaLeaf runtime.
//
// Thread mapping: a warp owns 32 adjacent interior columns of one 4-row strip
// (rows 4s..4s+3, the block-Jacobi strip of tea_block_jacobi.cuknl), one
// column per lane, so every global access of a warp is a contiguous 256-byte
// row segment.  A CTA is 8 warps (32 columns x 32 rows); CTAs walk the tiles
// with a grid-stride loop so a reduction has at most kMaxRedBlocks partials.
//
// Arithmetic follows the reference kernels (kernel_files/*.cuknl) with every
// a*b+c the reference writes evaluated as one explicit fma(); the file is
// built with -fmad=false so nvcc adds no other contraction.  The CPU oracle
// uses the same convention, so a single kernel agrees with it bit for bit.
//
// Reductions are deterministic: lanes combine with an xor butterfly, warps in
// index order, CTAs write one partial each, and the last CTA to finish (an
// atomic ticket) sums the partials in index order and runs the epilogue that
// the device-resident solve needs (alpha, beta, exit test).  No CTA ever
// waits for another.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>

#include "tl_internal.cuh"
#include "tl_device.cuh"

namespace tl {

// ------------------------------------------------------------ epilogues

__device__ void finish_iteration(DevScalars *s, bool allow_switch) {
    // tea_solve.f90:400-417: error = sqrt|error|; exit when below eps*||r0||
    double e = sqrt(fabs(s->error));
    s->error = e;
    if (fabs(e) < s->eps * s->initial_residual) {
        s->done = kConverged;
        s->n_exit = s->n;
        return;
    }
    if (isnan(e)) {  // breakdown: the reference would carry NaN to max_iters
        s->done = kBreakdown;
        s->n_exit = s->n;
        return;
    }
    s->old_error = e;
    s->n += 1;
    if (s->n > s->max_iters) {
        s->done = kMaxIters;
        s->n_exit = s->n;
        return;
    }
    if (allow_switch && (s->solver == TL_SOLVER_CHEBYSHEV || s->solver == TL_SOLVER_PPCG)) {
        // tea_solve.f90:157-171, evaluated at the top of the next iteration
        bool sw = (!s->first && s->solver == TL_SOLVER_PPCG && s->n > 1) ||
                  (fabs(s->old_error) <= s->epslim && s->n >= s->presteps);
        if (sw) s->done = kSwitch;
    }
}

__device__ void run_epilogue(const RedCtx &red, const double *tot, int nv) {
    DevScalars *s = red.sc;
    switch (red.epi) {
    case kEpiStore:
        for (int v = 0; v < nv; ++v) s->sum[v] = tot[v];
        break;
    case kEpiResid:
        s->sum[0] = tot[0];
        s->old_error = tot[0];
        s->initial_residual = sqrt(fabs(tot[0]));
        break;
    case kEpiRro:
        s->sum[0] = tot[0];
        s->rro = tot[0];
        break;
    case kEpiCgW:
        s->pw = tot[0];
        s->alpha = s->rro / s->pw;
        red.cg_alphas[s->n] = s->alpha;
        break;
    case kEpiCgUr:
        s->rrn = tot[0];
        s->beta = s->rrn / s->rro;
        red.cg_betas[s->n] = s->beta;
        s->error = s->rrn;
        s->rro = s->rrn;
        break;
    case kEpiFinish:
        finish_iteration(s, true);
        break;
    case kEpiFinishNoSwitch:
        finish_iteration(s, false);
        break;
    case kEpiPw:
        s->pw = tot[0];
        break;
    case kEpiPpcgZr:
        s->rro = tot[0];
        s->alpha = s->rro / s->pw;
        break;
    case kEpiPwZr:
        s->pw = tot[0];
        s->rro = tot[1];
        s->alpha = s->rro / s->pw;
        break;
    case kEpiPpcgRrn:
        s->rrn = tot[0];
        s->beta = s->rrn / s->rro;
        s->error = s->rrn;
        s->rro = s->rrn;
        s->ppcg_iters += 1;
        break;
    case kEpiChebyNorm:
        s->rr = tot[0];
        break;
    case kEpiChebyFinish:
        // tea_solve.f90:266-283: the residual is read every 10th iteration
        // after est_itc; cheby_calc_steps += 1 at :284
        if (s->n >= s->est_itc && s->n % 10 == 0) s->error = s->rr;
        s->cheby_calc_steps += 1;
        finish_iteration(s, false);
        break;
    case kEpiJacobi:
        s->error = tot[0];
        finish_iteration(s, false);
        break;
    default:
        break;
    }
}

template <int NV>
__device__ __forceinline__ void grid_reduce(double (&acc)[NV > 0 ? NV : 1], const RedCtx &red) {
    __shared__ double sh[kBlockWarps][NV > 0 ? NV : 1];
    __shared__ int is_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        double x = acc[v];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
        if (lane == 0) sh[warp][v] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            double t = 0.0;
            for (int w = 0; w < kBlockWarps; ++w) t += sh[w][v];
            red.partials[v * kMaxRedBlocks + blockIdx.x] = t;
        }
        __threadfence();
        unsigned int ticket = atomicAdd(red.counter, 1u);
        is_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double tot[NV > 0 ? NV : 1];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        double t = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
            t += __ldcg(&red.partials[v * kMaxRedBlocks + b]);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
        __syncthreads();
        if (lane == 0) sh[warp][v] = t;
        __syncthreads();
        double s = 0.0;
        for (int w = 0; w < kBlockWarps; ++w) s += sh[w][v];
        tot[v] = s;
    }
    if (threadIdx.x == 0) {
        run_epilogue(red, tot, NV);
        __threadfence();
        *red.counter = 0u;
    }
}

// The grid-stride strip kernel: Body processes one strip column.
template <int NV, class Body>
__global__ void __launch_bounds__(kBlockThreads) k_strips(Geo g, Body body, RedCtx red) {
    if (red.done && *(volatile const int *)red.done) return;
    double acc[NV > 0 ? NV : 1];
#pragma unroll
    for (int v = 0; v < (NV > 0 ? NV : 1); ++v) acc[v] = 0.0;
    body.setup();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = blockIdx.x; t < g.tiles; t += gridDim.x) {
        const int tx = t % g.tiles_x, ty = t / g.tiles_x;
        const int i = tx * kWarpCols + lane;
        const int s = ty * kBlockWarps + warp;
        if (i < g.nx && s < g.nstrips) {
            const int j0 = s * kStrip;
            const int m = min(kStrip, g.ny - j0);
            const int64_t base = (int64_t)(i + g.h) + (int64_t)(j0 + g.h) * g.pitch;
            body(base, m, acc);
        }
    }
    if (red.epi != kEpiNone) grid_reduce<NV>(acc, red);
}

// ------------------------------------------------------------- helpers

// diag(A) of tea_leaf_common.cuknl:137-139: (1 + (Ky_n + Ky_c)) + (Kx_e + Kx_c)
__device__ __forceinline__ double diag_at(const double *__restrict__ kx,
                                          const double *__restrict__ ky, int64_t i, int pitch) {
    return (1.0 + (ky[i + pitch] + ky[i])) + (kx[i + 1] + kx[i]);
}

// A x on the m rows of a strip (tea_leaf_common.cuknl:28-34).  xc receives
// the centre values.  Rows beyond m are neither read nor written.
// FIVE: the same operator as one product and four fused subtractions
// (5 FP64 instructions instead of 6; other rounding, so only for callers
// that do not need the reference's bits)
template <class X, bool FIVE = false>
__device__ __forceinline__ void strip_apply(const double *__restrict__ kx,
                                            const double *__restrict__ ky,
                                            const double *__restrict__ dg, int pitch,
                                            int64_t base, int m, X x, double (&xc)[4],
                                            double (&ax)[4]) {
    double xr[6];   // rows -1..4
    double kyr[5];  // faces of rows 0..4
#pragma unroll
    for (int k = -1; k <= 4; ++k)
        if (k <= m) xr[k + 1] = x(base + (int64_t)k * pitch);
#pragma unroll
    for (int k = 0; k <= 4; ++k)
        if (k <= m) kyr[k] = ky[base + (int64_t)k * pitch];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (k < m) {
            const int64_t i = base + (int64_t)k * pitch;
            const double kxc = kx[i], kxe = kx[i + 1];
            const double xw = x(i - 1), xe = x(i + 1);
            const double diag = dg[i];
            if (FIVE) {
                double v = diag * xr[k + 1];
                v = fma(-kyr[k + 1], xr[k + 2], v);
                v = fma(-kyr[k], xr[k], v);
                v = fma(-kxe, xe, v);
                ax[k] = fma(-kxc, xw, v);
            } else {
                const double a = fma(kyr[k + 1], xr[k + 2], kyr[k] * xr[k]);
                const double b = fma(kxe, xe, kxc * xw);
                ax[k] = fma(diag, xr[k + 1], -a) - b;
            }
            xc[k] = xr[k + 1];
        }
    }
}

struct LoadX {
    const double *__restrict__ f;
    __device__ __forceinline__ double operator()(int64_t i) const { return f[i]; }
};

__device__ __forceinline__ double coef(const double *p, double v) { return p ? *p : v; }

// ------------------------------------------------------------- bodies

struct BodyResidual {  // r = u0 - A u  (+ r.r)
    const double *dg;  // diag(A), stored by the diag kernel
    const double *u, *u0, *kx, *ky;
    double *r;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
        double xc[4], ax[4];
        strip_apply(kx, ky, dg, pitch, base, m, LoadX{u}, xc, ax);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                const double rv = u0[i] - ax[k];
                r[i] = rv;
                acc[0] = fma(rv, rv, acc[0]);
            }
    }
};

struct BodyNorm {  // sum a.b
    const double *a, *b;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                acc[0] = fma(a[i], b[i], acc[0]);
            }
    }
};

template <int PC>
struct BodyCgInit {  // tea_leaf_kernel_cuda.cu:164-186 fused per strip
    const double *dg;  // diag(A), stored by the diag kernel
    const double *r, *kx, *ky;
    double *p, *z, *mi, *cp, *bfp;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
        double rv[4], zv[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) rv[k] = r[base + (int64_t)k * pitch];
        if (PC == TL_PREC_JAC_BLOCK) {
            // block_init (tea_block_jacobi.cuknl:83-111)
            double cprev = (-ky[base + pitch]) / dg[base];
            cp[base] = cprev;
#pragma unroll
            for (int k = 1; k < 4; ++k)
                if (k < m) {
                    const int64_t i = base + (int64_t)k * pitch;
                    const double bf = 1.0 / fma(ky[i], cprev, dg[i]);
                    bfp[i] = bf;
                    cprev = (-ky[i + pitch]) * bf;
                    cp[i] = cprev;
                }
            strip_block_solve(dg, ky, cp, bfp, pitch, base, m, rv, zv);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                double pv;
                if (PC == TL_PREC_JAC_BLOCK) {
                    z[i] = zv[k];
                    pv = zv[k];
                } else if (PC == TL_PREC_JAC_DIAG) {
                    const double mv = 1.0 / dg[i];
                    mi[i] = mv;
                    const double zz = rv[k] * mv;
                    z[i] = zz;
                    pv = zz;
                } else {
                    pv = rv[k];
                }
                p[i] = pv;
                acc[0] = fma(rv[k], pv, acc[0]);
            }
    }
};

struct BodyCgW {  // w = A p; p.w  (tea_leaf_cg.cuknl:43-68)
    const double *dg;  // diag(A), stored by the diag kernel
    const double *p, *kx, *ky;
    double *w;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
        double xc[4], ax[4];
        strip_apply(kx, ky, dg, pitch, base, m, LoadX{p}, xc, ax);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                w[base + (int64_t)k * pitch] = ax[k];
                acc[0] = fma(xc[k], ax[k], acc[0]);
            }
    }
};

template <int PC>
struct BodyCgUr {  // tea_leaf_cg.cuknl:72-137
    const double *dg;  // diag(A), stored by the diag kernel
    double *u, *r, *z;
    const double *p, *w, *mi, *kx, *ky, *cp, *bfp;
    const double *alpha_p;
    double alpha_v;
    int pitch;
    double alpha;
    __device__ void setup() { alpha = coef(alpha_p, alpha_v); }
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
        // every load of the strip before the first store (the arrays may
        // alias as far as the compiler knows, so it would not hoist them)
        double uv[4], pv[4], wv[4], rv[4], mv[4], zv[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                uv[k] = u[i];
                pv[k] = p[i];
                wv[k] = w[i];
                rv[k] = r[i];
                if (PC == TL_PREC_JAC_DIAG) mv[k] = mi[i];
            }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                uv[k] = fma(alpha, pv[k], uv[k]);
                rv[k] = fma(-alpha, wv[k], rv[k]);
            }
        if (PC == TL_PREC_JAC_BLOCK) strip_block_solve(dg, ky, cp, bfp, pitch, base, m, rv, zv);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                u[i] = uv[k];
                r[i] = rv[k];
                if (PC == TL_PREC_JAC_BLOCK) {
                    z[i] = zv[k];
                    acc[0] = fma(rv[k], zv[k], acc[0]);
                } else if (PC == TL_PREC_JAC_DIAG) {
                    const double zz = rv[k] * mv[k];
                    z[i] = zz;
                    acc[0] = fma(rv[k], zz, acc[0]);
                } else {
                    acc[0] = fma(rv[k], rv[k], acc[0]);
                }
            }
    }
};

struct BodyAxpyP {  // p = src + beta p  (tea_leaf_cg.cuknl:141-161, tea_leaf_ppcg.cuknl:301-313)
    double *p;
    const double *src;
    const double *beta_p;
    double beta_v;
    int pitch;
    double beta;
    __device__ void setup() { beta = coef(beta_p, beta_v); }
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
        double pv[4], sv[4];  // loads first: see BodyCgUr
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                pv[k] = p[i];
                sv[k] = src[i];
            }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) p[base + (int64_t)k * pitch] = fma(beta, pv[k], sv[k]);
    }
};

// mixed PPCG with fused inner passes: u += alpha p (the u half of the outer
// update, tea_leaf_cg.cuknl:72-137), then p = z + beta p
// (tea_leaf_ppcg.cuknl:301-313), in one pass over the old p
struct BodyPpcgUP {
    double *p, *u;
    const double *z;
    const double *alpha_p, *beta_p;
    int pitch;
    double alpha, beta;
    __device__ void setup() {
        alpha = *alpha_p;
        beta = *beta_p;
    }
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
        double pv[4], uv[4], zv[4];  // loads first: see BodyCgUr
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                pv[k] = p[i];
                uv[k] = u[i];
                zv[k] = z[i];
            }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                u[i] = fma(alpha, pv[k], uv[k]);
                p[i] = fma(beta, pv[k], zv[k]);
            }
    }
};

template <int PC>
struct BodyChebyInitP {  // tea_leaf_cheby.cuknl:5-68
    const double *dg;  // diag(A), stored by the diag kernel
    const double *u, *u0, *kx, *ky, *mi, *cp, *bfp;
    double *p, *r, *w;
    double theta;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
        double xc[4], ax[4], rv[4], zv[4];
        strip_apply(kx, ky, dg, pitch, base, m, LoadX{u}, xc, ax);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                w[i] = ax[k];
                rv[k] = u0[i] - ax[k];
                r[i] = rv[k];
            }
        if (PC == TL_PREC_JAC_BLOCK) strip_block_solve(dg, ky, cp, bfp, pitch, base, m, rv, zv);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                if (PC == TL_PREC_JAC_BLOCK) p[i] = zv[k] / theta;
                else if (PC == TL_PREC_JAC_DIAG) p[i] = (mi[i] * rv[k]) / theta;
                else p[i] = rv[k] / theta;
            }
    }
};

template <int PC>
struct BodyChebyCalcP {  // tea_leaf_cheby.cuknl:84-152 (+ r.r for the exit test)
    const double *dg;  // diag(A), stored by the diag kernel
    const double *u, *u0, *kx, *ky, *mi, *cp, *bfp, *alphas, *betas;
    double *p, *r, *w;
    const int *step_p;   // device cheby_calc_steps, or nullptr
    int step_v;          // 1-based step
    int pitch;
    double al, be;
    __device__ void setup() {
        const int st = step_p ? *step_p : step_v;
        al = alphas[st - 1];
        be = betas[st - 1];
    }
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
        double xc[4], ax[4], rv[4], zv[4];
        strip_apply(kx, ky, dg, pitch, base, m, LoadX{u}, xc, ax);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                w[i] = ax[k];
                rv[k] = u0[i] - ax[k];
                r[i] = rv[k];
                acc[0] = fma(rv[k], rv[k], acc[0]);
            }
        if (PC == TL_PREC_JAC_BLOCK) strip_block_solve(dg, ky, cp, bfp, pitch, base, m, rv, zv);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                if (PC == TL_PREC_JAC_BLOCK) p[i] = fma(al, p[i], be * zv[k]);
                else if (PC == TL_PREC_JAC_DIAG) p[i] = fma(al, p[i], (be * mi[i]) * rv[k]);
                else p[i] = fma(al, p[i], be * rv[k]);
            }
    }
};

struct BodyAdd {  // u += p  (tea_leaf_cheby.cuknl:71-82)
    double *u;
    const double *p;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                u[i] += p[i];
            }
    }
};

template <int PC>
struct BodyPpcgInit {  // tea_leaf_ppcg.cuknl:319-420
    const double *dg;  // diag(A), stored by the diag kernel
    const double *r, *mi, *kx, *ky, *cp, *bfp;
    double *p, *z;
    int step, pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
        double zv[4], rv[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) rv[k] = r[base + (int64_t)k * pitch];
        const bool do_z = (PC != TL_PREC_NONE || step == 3) && (step == 1 || step == 2);
        if (do_z && PC == TL_PREC_JAC_BLOCK) strip_block_solve(dg, ky, cp, bfp, pitch, base, m, rv, zv);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                double pv = 0.0, zz = 0.0;
                if (step == 3) zz = z[i];
                if (PC != TL_PREC_NONE || step == 3) {
                    if (step == 1 || step == 2) {
                        if (PC == TL_PREC_JAC_BLOCK) zz = zv[k];
                        else if (PC == TL_PREC_JAC_DIAG) zz = mi[i] * rv[k];
                        z[i] = zz;
                    }
                    if (step == 1 || step == 3) pv = zz;
                } else if (step == 1) {
                    pv = rv[k];
                    z[i] = 0.0;
                }
                if (step == 1 || step == 3) {
                    p[i] = pv;
                    acc[0] = fma(rv[k], pv, acc[0]);
                }
            }
    }
};

template <int PC>
struct BodyPpcgInitSd {  // tea_leaf_ppcg.cuknl:5-55 (not used by the driver)
    const double *dg;  // diag(A), stored by the diag kernel
    const double *r, *mi, *kx, *ky, *cp, *bfp;
    double *sd;
    double theta;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
        double rv[4], zv[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) rv[k] = r[base + (int64_t)k * pitch];
        if (PC == TL_PREC_JAC_BLOCK) strip_block_solve(dg, ky, cp, bfp, pitch, base, m, rv, zv);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                if (PC == TL_PREC_JAC_BLOCK) sd[i] = zv[k] / theta;
                else if (PC == TL_PREC_JAC_DIAG) sd[i] = rv[k] * mi[i] / theta;
                else sd[i] = rv[k] / theta;
            }
    }
};

template <int PC>
struct BodyPpcgInitSdNew {  // tea_leaf_ppcg.cuknl:58-89
    const double *r, *z;
    double *sd, *rtemp, *utemp;
    const double *theta_p;
    double theta;
    int pitch;
    __device__ void setup() { theta = coef(theta_p, theta); }
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
        const double theta_r = 1.0 / theta;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                const double src = (PC != TL_PREC_NONE) ? z[i] : r[i];
                const double s = src * theta_r;
                sd[i] = s;
                rtemp[i] = r[i];
                utemp[i] = s;
            }
    }
};

struct BodyPpcgUpdateR {  // rtemp -= A sd  (tea_leaf_ppcg.cuknl:154-173)
    const double *dg;  // diag(A), stored by the diag kernel
    const double *sd, *kx, *ky;
    double *rtemp;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
        double xc[4], ax[4];
        strip_apply(kx, ky, dg, pitch, base, m, LoadX{sd}, xc, ax);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                rtemp[i] = rtemp[i] - ax[k];
            }
    }
};

template <int PC>
struct BodyPpcgCalcSdNew {  // tea_leaf_ppcg.cuknl:178-244
    const double *dg;  // diag(A), stored by the diag kernel
    const double *rtemp, *mi, *kx, *ky, *cp, *bfp, *alphas, *betas;
    double *sd, *utemp;
    int step;  // 1-based inner step
    int pitch;
    double al, be;
    __device__ void setup() {
        al = alphas[step - 1];
        be = betas[step - 1];
    }
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
        double rv[4], zv[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) rv[k] = rtemp[base + (int64_t)k * pitch];
        if (PC == TL_PREC_JAC_BLOCK) strip_block_solve(dg, ky, cp, bfp, pitch, base, m, rv, zv);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                double s;
                if (PC == TL_PREC_JAC_BLOCK) s = fma(al, sd[i], be * zv[k]);
                else if (PC == TL_PREC_JAC_DIAG) s = fma(al, sd[i], (be * rv[k]) * mi[i]);
                else s = fma(al, sd[i], be * rv[k]);
                sd[i] = s;
                utemp[i] = utemp[i] + s;
            }
    }
};

struct BodyCopy {
    double *dst;
    const double *src;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                dst[i] = src[i];
            }
    }
};

template <bool FIVE>
struct BodyCgWStoreZr {  // BodyCgW and BodyStoreZr in one pass: w = A p, r_store = r;
                         // sums p.w and r.z, each in its own kernel's order
                         // (FIVE: the 5-instruction operator, mixed precision only)
    const double *dg;
    const double *p, *kx, *ky, *r, *z;
    double *w, *r_store;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[2]) const {
        double xc[4], ax[4];
        strip_apply<LoadX, FIVE>(kx, ky, dg, pitch, base, m, LoadX{p}, xc, ax);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                w[i] = ax[k];
                acc[0] = fma(xc[k], ax[k], acc[0]);
                const double rv = r[i];
                r_store[i] = rv;
                acc[1] = fma(rv, z[i], acc[1]);
            }
    }
};

struct BodyPpcgRrn {  // sum (r - r_store).z  (tea_leaf_ppcg.cuknl:279-297)
    const double *r, *r_store, *z;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                acc[0] = fma(r[i] - r_store[i], z[i], acc[0]);
            }
    }
};

struct BodyJacobi {  // tea_leaf_jacobi.cuknl:19-46 (un holds the previous u)
    const double *un, *u0, *kx, *ky;
    double *u;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                double num = fma(kx[i + 1], un[i + 1], u0[i]);
                num = fma(kx[i], un[i - 1], num);
                num = fma(ky[i + pitch], un[i + pitch], num);
                num = fma(ky[i], un[i - pitch], num);
                const double den = (1.0 + (kx[i] + kx[i + 1])) + (ky[i] + ky[i + pitch]);
                const double v = num / den;
                u[i] = v;
                acc[0] += fabs(v - un[i]);
            }
    }
};

struct BodyFinalise {  // energy1 = u / density (tea_leaf_common.cuknl:5-17)
    const double *u, *density;
    double *energy1;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                energy1[i] = u[i] / density[i];
            }
    }
};

struct BodyFieldSummary {  // field_summary_kernel.cuknl:5-58
    const double *volume, *density, *energy1, *u;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[4]) const {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                const double cv = volume[i];
                const double cm = cv * density[i];
                acc[0] += cv;
                acc[1] += cm;
                acc[2] += cm * energy1[i];
                acc[3] += cm * u[i];
            }
    }
};

struct BodyDiag {  // diag(A) of tea_leaf_common.cuknl:137-139, once per solve
    const double *kx, *ky;
    double *dg;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = base + (int64_t)k * pitch;
                dg[i] = diag_at(kx, ky, i, pitch);
            }
    }
};

struct BodyFill {
    double *f;
    double v;
    int pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) f[base + (int64_t)k * pitch] = v;
    }
};

struct BodyGenerate {  // generate_chunk_kernel.cuknl:5-99, states in order
    double *density, *energy0, *u, *u0;
    const double *vertexx, *vertexy, *cellx, *celly;
    const tl_state_t *states;
    int nstates, h, pitch;
    __device__ void setup() {}
    __device__ void operator()(int64_t base, int m, double (&acc)[1]) const {
        const int c = (int)(base % pitch);
        const int r0 = (int)(base / pitch);
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int r = r0 + k;
                const int64_t i = base + (int64_t)k * pitch;
                double d = states[0].density, e = states[0].energy;
                for (int s = 1; s < nstates; ++s) {
                    const tl_state_t st = states[s];
                    bool hit = false;
                    if (st.geometry == TL_GEOM_RECTANGLE) {
                        hit = vertexx[c + 1] >= st.xmin && vertexx[c] < st.xmax &&
                              vertexy[r + 1] >= st.ymin && vertexy[r] < st.ymax;
                    } else if (st.geometry == TL_GEOM_CIRCLE) {
                        const double xp = cellx[c] - st.xmin, yp = celly[r] - st.ymin;
                        hit = sqrt(xp * xp + yp * yp) <= st.radius;
                    } else if (st.geometry == TL_GEOM_POINT) {
                        hit = vertexx[c] == st.xmin && vertexy[r] == st.ymin;
                    }
                    if (hit) {
                        d = st.density;
                        e = st.energy;
                    }
                }
                density[i] = d;
                energy0[i] = e;
                u[i] = e * d;
                u0[i] = e * d;
            }
    }
};

// face coefficients (tea_leaf_common.cuknl:60-129): one thread per padded
// cell of [h, nx+h] x [h, ny+h]; Kx on interior rows, Ky on interior columns;
// boundary faces zeroed unless reflective; u = u0 = energy1 * density
__global__ void k_common_init(Geo g, const double *__restrict__ density,
                              const double *__restrict__ energy1, double *__restrict__ kx,
                              double *__restrict__ ky, double *__restrict__ u,
                              double *__restrict__ u0, double rx, double ry, int recip, int zl,
                              int zr, int zb, int zt) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x + g.h;
    const int r = blockIdx.y * blockDim.y + threadIdx.y + g.h;
    if (c > g.nx + g.h || r > g.ny + g.h) return;
    const int64_t i = (int64_t)c + (int64_t)r * g.pitch;
    double dc = density[i], dl = density[i - 1], dd = density[i - g.pitch];
    if (recip) {
        dc = 1.0 / dc;
        dl = 1.0 / dl;
        dd = 1.0 / dd;
    }
    const bool row_in = r < g.ny + g.h, col_in = c < g.nx + g.h;
    if (row_in) {
        double v = (dl + dc) / (2.0 * dl * dc);
        v *= rx;
        if ((zl && c == g.h) || (zr && c == g.nx + g.h)) v = 0.0;
        kx[i] = v;
    }
    if (col_in) {
        double v = (dd + dc) / (2.0 * dd * dc);
        v *= ry;
        if ((zb && r == g.h) || (zt && r == g.ny + g.h)) v = 0.0;
        ky[i] = v;
    }
    if (row_in && col_in) {
        const double e = energy1[i] * density[i];
        u[i] = e;
        u0[i] = e;
    }
}

// reflective boundary for one field: TeaLeaf's mirror semantics.  Pass 0
// mirrors rows (bottom/top) over columns [h-depth, nx+h+depth), pass 1 then
// mirrors columns (left/right) over rows [h-depth, ny+h+depth).
__global__ void k_reflect(Geo g, double *__restrict__ f, int depth, int pass) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y;  // 0..depth-1
    if (pass == 0) {
        const int c = g.h - depth + t;
        if (c >= g.nx + g.h + depth) return;
        f[c + (int64_t)(g.h - 1 - k) * g.pitch] = f[c + (int64_t)(g.h + k) * g.pitch];
        f[c + (int64_t)(g.ny + g.h + k) * g.pitch] = f[c + (int64_t)(g.ny + g.h - 1 - k) * g.pitch];
    } else {
        const int r = g.h - depth + t;
        if (r >= g.ny + g.h + depth) return;
        const int64_t row = (int64_t)r * g.pitch;
        f[row + g.h - 1 - k] = f[row + g.h + k];
        f[row + g.nx + g.h + k] = f[row + g.nx + g.h - 1 - k];
    }
}

// ------------------------------------------------------------- launchers

template <int NV, class Body>
static int run(Chunk *c, const char *name, const Body &body, int epi, bool fast) {
    const int grid = c->g.tiles < c->grid_red ? c->g.tiles : c->grid_red;
    int slot = -1;
    if (c->profiling && !c->capturing) prof_begin(c, name, &slot);
    k_strips<NV, Body><<<grid, kBlockThreads, 0, c->stream>>>(c->g, body, red_ctx(c, epi, fast));
    if (slot >= 0) prof_end(c, slot);
    c->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    return TL_OK;
}

int launch_common_init(Chunk *c, int coefficient, double rx, double ry, const int zero[4],
                       int reflective) {
    dim3 block(32, 8);
    dim3 grid((c->nx + 1 + 31) / 32, (c->ny + 1 + 7) / 8);
    int zl = reflective ? 0 : zero[0], zr = reflective ? 0 : zero[1];
    int zb = reflective ? 0 : zero[2], zt = reflective ? 0 : zero[3];
    int slot = -1;
    if (c->profiling && !c->capturing) prof_begin(c, "common_init", &slot);
    k_common_init<<<grid, block, 0, c->stream>>>(c->g, c->density, c->energy1, c->kx, c->ky, c->u,
                                                 c->u0, rx, ry,
                                                 coefficient == TL_COEF_RECIP_CONDUCTIVITY, zl, zr,
                                                 zb, zt);
    if (slot >= 0) prof_end(c, slot);
    c->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "common_init launch");
    BodyDiag bd{c->kx, c->ky, c->diag, c->pitch};
    return run<1>(c, "diag", bd, kEpiNone, false);
}

int launch_residual(Chunk *c, int epi) {
    BodyResidual b{c->diag, c->u, c->u0, c->kx, c->ky, c->r, c->pitch};
    return run<1>(c, "residual", b, epi, false);
}

int launch_norm(Chunk *c, const double *a, const double *bb, int epi) {
    BodyNorm b{a, bb, c->pitch};
    return run<1>(c, "norm", b, epi, false);
}

int launch_cg_init(Chunk *c, int epi) {
    switch (c->cfg.precond) {
    case TL_PREC_JAC_BLOCK: {
        BodyCgInit<TL_PREC_JAC_BLOCK> b{c->diag, c->r, c->kx, c->ky, c->p, c->z, c->mi, c->cp, c->bfp, c->pitch};
        return run<1>(c, "cg_init", b, epi, false);
    }
    case TL_PREC_JAC_DIAG: {
        BodyCgInit<TL_PREC_JAC_DIAG> b{c->diag, c->r, c->kx, c->ky, c->p, c->z, c->mi, c->cp, c->bfp, c->pitch};
        return run<1>(c, "cg_init", b, epi, false);
    }
    default: {
        BodyCgInit<TL_PREC_NONE> b{c->diag, c->r, c->kx, c->ky, c->p, c->z, c->mi, c->cp, c->bfp, c->pitch};
        return run<1>(c, "cg_init", b, epi, false);
    }
    }
}

int launch_cg_w(Chunk *c, int epi, bool fast) {
    BodyCgW b{c->diag, c->p, c->kx, c->ky, c->w, c->pitch};
    return run<1>(c, "cg_w", b, epi, fast);
}

template <int PC>
static int cg_ur(Chunk *c, double alpha, int epi, bool fast) {
    BodyCgUr<PC> b{c->diag, c->u, c->r, c->z, c->p, c->w, c->mi, c->kx, c->ky, c->cp, c->bfp,
                   fast ? &c->sc->alpha : nullptr, alpha, c->pitch, 0.0};
    return run<1>(c, "cg_ur", b, epi, fast);
}

int launch_cg_ur(Chunk *c, double alpha, int epi, bool fast) {
    switch (c->cfg.precond) {
    case TL_PREC_JAC_BLOCK: return cg_ur<TL_PREC_JAC_BLOCK>(c, alpha, epi, fast);
    case TL_PREC_JAC_DIAG: return cg_ur<TL_PREC_JAC_DIAG>(c, alpha, epi, fast);
    default: return cg_ur<TL_PREC_NONE>(c, alpha, epi, fast);
    }
}

int launch_cg_p(Chunk *c, double beta, int epi, bool fast) {
    const double *src = c->cfg.precond != TL_PREC_NONE ? c->z : c->r;
    BodyAxpyP b{c->p, src, fast ? &c->sc->beta : nullptr, beta, c->pitch, 0.0};
    return run<1>(c, "cg_p", b, epi, fast);
}

int launch_cheby_init(Chunk *c, double theta) {
    switch (c->cfg.precond) {
    case TL_PREC_JAC_BLOCK: {
        BodyChebyInitP<TL_PREC_JAC_BLOCK> b{c->diag, c->u, c->u0, c->kx, c->ky, c->mi, c->cp, c->bfp,
                                            c->p, c->r, c->w, theta, c->pitch};
        return run<1>(c, "cheby_init", b, kEpiNone, false);
    }
    case TL_PREC_JAC_DIAG: {
        BodyChebyInitP<TL_PREC_JAC_DIAG> b{c->diag, c->u, c->u0, c->kx, c->ky, c->mi, c->cp, c->bfp,
                                           c->p, c->r, c->w, theta, c->pitch};
        return run<1>(c, "cheby_init", b, kEpiNone, false);
    }
    default: {
        BodyChebyInitP<TL_PREC_NONE> b{c->diag, c->u, c->u0, c->kx, c->ky, c->mi, c->cp, c->bfp,
                                       c->p, c->r, c->w, theta, c->pitch};
        return run<1>(c, "cheby_init", b, kEpiNone, false);
    }
    }
}

template <int PC>
static int cheby_p(Chunk *c, int step, int epi, bool fast) {
    BodyChebyCalcP<PC> b{c->diag, c->u, c->u0, c->kx, c->ky, c->mi, c->cp, c->bfp, c->ch_alphas,
                         c->ch_betas, c->p, c->r, c->w,
                         fast ? &c->sc->cheby_calc_steps : nullptr, step, c->pitch, 0.0, 0.0};
    return run<1>(c, "cheby_p", b, epi, fast);
}

int launch_cheby_calc_p(Chunk *c, int step, int epi, bool fast) {
    switch (c->cfg.precond) {
    case TL_PREC_JAC_BLOCK: return cheby_p<TL_PREC_JAC_BLOCK>(c, step, epi, fast);
    case TL_PREC_JAC_DIAG: return cheby_p<TL_PREC_JAC_DIAG>(c, step, epi, fast);
    default: return cheby_p<TL_PREC_NONE>(c, step, epi, fast);
    }
}

int launch_cheby_calc_u(Chunk *c, int epi, bool fast) {
    BodyAdd b{c->u, c->p, c->pitch};
    return run<1>(c, "cheby_calc_u", b, epi, fast);
}

template <int PC>
static int ppcg_init(Chunk *c, int step, int epi) {
    BodyPpcgInit<PC> b{c->diag, c->r, c->mi, c->kx, c->ky, c->cp, c->bfp, c->p, c->z, step, c->pitch};
    return run<1>(c, "ppcg_init", b, epi, false);
}

int launch_ppcg_init(Chunk *c, int step, int epi) {
    switch (c->cfg.precond) {
    case TL_PREC_JAC_BLOCK: return ppcg_init<TL_PREC_JAC_BLOCK>(c, step, epi);
    case TL_PREC_JAC_DIAG: return ppcg_init<TL_PREC_JAC_DIAG>(c, step, epi);
    default: return ppcg_init<TL_PREC_NONE>(c, step, epi);
    }
}

int launch_ppcg_init_sd(Chunk *c, double theta) {
    switch (c->cfg.precond) {
    case TL_PREC_JAC_BLOCK: {
        BodyPpcgInitSd<TL_PREC_JAC_BLOCK> b{c->diag, c->r, c->mi, c->kx, c->ky, c->cp, c->bfp, c->sd, theta, c->pitch};
        return run<1>(c, "ppcg_init_sd", b, kEpiNone, false);
    }
    case TL_PREC_JAC_DIAG: {
        BodyPpcgInitSd<TL_PREC_JAC_DIAG> b{c->diag, c->r, c->mi, c->kx, c->ky, c->cp, c->bfp, c->sd, theta, c->pitch};
        return run<1>(c, "ppcg_init_sd", b, kEpiNone, false);
    }
    default: {
        BodyPpcgInitSd<TL_PREC_NONE> b{c->diag, c->r, c->mi, c->kx, c->ky, c->cp, c->bfp, c->sd, theta, c->pitch};
        return run<1>(c, "ppcg_init_sd", b, kEpiNone, false);
    }
    }
}

int launch_ppcg_init_sd_new(Chunk *c, double theta, bool fast) {
    const double *tp = fast ? &c->sc->theta : nullptr;
    if (c->cfg.precond != TL_PREC_NONE) {
        BodyPpcgInitSdNew<TL_PREC_JAC_DIAG> b{c->r, c->z, c->sd, c->rtemp, c->utemp, tp, theta, c->pitch};
        return run<1>(c, "ppcg_init_sd_new", b, kEpiNone, fast);
    }
    BodyPpcgInitSdNew<TL_PREC_NONE> b{c->r, c->z, c->sd, c->rtemp, c->utemp, tp, theta, c->pitch};
    return run<1>(c, "ppcg_init_sd_new", b, kEpiNone, fast);
}

int launch_ppcg_update_r(Chunk *c, bool fast) {
    BodyPpcgUpdateR b{c->diag, c->sd, c->kx, c->ky, c->rtemp, c->pitch};
    return run<1>(c, "ppcg_update_r", b, kEpiNone, fast);
}

template <int PC>
static int ppcg_sd(Chunk *c, int step, bool fast) {
    BodyPpcgCalcSdNew<PC> b{c->diag, c->rtemp, c->mi, c->kx, c->ky, c->cp, c->bfp, c->ch_alphas,
                            c->ch_betas, c->sd, c->utemp, step, c->pitch, 0.0, 0.0};
    return run<1>(c, "ppcg_sd", b, kEpiNone, fast);
}

int launch_ppcg_calc_sd_new(Chunk *c, int step, bool fast) {
    switch (c->cfg.precond) {
    case TL_PREC_JAC_BLOCK: return ppcg_sd<TL_PREC_JAC_BLOCK>(c, step, fast);
    case TL_PREC_JAC_DIAG: return ppcg_sd<TL_PREC_JAC_DIAG>(c, step, fast);
    default: return ppcg_sd<TL_PREC_NONE>(c, step, fast);
    }
}

int launch_copy(Chunk *c, double *dst, const double *src, bool fast) {
    BodyCopy b{dst, src, c->pitch};
    return run<1>(c, "copy", b, kEpiNone, fast);
}

int launch_ppcg_rrn(Chunk *c, int epi, bool fast) {
    BodyPpcgRrn b{c->r, c->r_store, c->z, c->pitch};
    return run<1>(c, "ppcg_rrn", b, epi, fast);
}

int launch_ppcg_zr(Chunk *c, int epi, bool fast) {
    BodyNorm b{c->r, c->z, c->pitch};
    return run<1>(c, "ppcg_zr", b, epi, fast);
}

int launch_ppcg_w_store_zr(Chunk *c, bool fast, bool five) {
    if (five) {
        BodyCgWStoreZr<true> b{c->diag, c->p, c->kx, c->ky, c->r, c->z, c->w, c->r_store, c->pitch};
        return run<2>(c, "ppcg_w_zr", b, kEpiPwZr, fast);
    }
    BodyCgWStoreZr<false> b{c->diag, c->p, c->kx, c->ky, c->r, c->z, c->w, c->r_store, c->pitch};
    return run<2>(c, "ppcg_w_zr", b, kEpiPwZr, fast);
}

int launch_ppcg_up(Chunk *c, int epi, bool fast) {
    BodyPpcgUP b{c->p, c->u, c->z, &c->sc->alpha, &c->sc->beta, c->pitch, 0.0, 0.0};
    return run<1>(c, "ppcg_up", b, epi, fast);
}

int launch_ppcg_p(Chunk *c, double beta, int epi, bool fast) {
    BodyAxpyP b{c->p, c->z, fast ? &c->sc->beta : nullptr, beta, c->pitch, 0.0};
    return run<1>(c, "ppcg_p", b, epi, fast);
}

int launch_jacobi(Chunk *c, int epi, bool fast) {
    int rc = launch_copy(c, c->un, c->u, fast);
    if (rc) return rc;
    BodyJacobi b{c->un, c->u0, c->kx, c->ky, c->u, c->pitch};
    return run<1>(c, "jacobi", b, epi, fast);
}

int launch_finalise(Chunk *c) {
    BodyFinalise b{c->u, c->density, c->energy1, c->pitch};
    return run<1>(c, "finalise", b, kEpiNone, false);
}

int launch_field_summary(Chunk *c) {
    BodyFieldSummary b{c->volume, c->density, c->energy1, c->u, c->pitch};
    return run<4>(c, "field_summary", b, kEpiStore, false);
}

int launch_set_field(Chunk *c) { return launch_copy(c, c->energy1, c->energy0, false); }

int launch_fill(Chunk *c, double *f, double v) {
    BodyFill b{f, v, c->pitch};
    return run<1>(c, "fill", b, kEpiNone, false);
}

int launch_generate(Chunk *c, int nstates, const tl_state_t *states_dev) {
    BodyGenerate b{c->density, c->energy0, c->u, c->u0, c->vertexx, c->vertexy, c->cellx,
                   c->celly, states_dev, nstates, c->h, c->pitch};
    return run<1>(c, "generate", b, kEpiNone, false);
}

int launch_reflect(Chunk *c, double *f, int depth) {
    if (depth > c->h) depth = c->h;
    if (depth < 1) return TL_OK;
    const int n0 = c->nx + 2 * depth, n1 = c->ny + 2 * depth;
    dim3 g0((n0 + 127) / 128, depth), g1((n1 + 127) / 128, depth);
    k_reflect<<<g0, 128, 0, c->stream>>>(c->g, f, depth, 0);
    k_reflect<<<g1, 128, 0, c->stream>>>(c->g, f, depth, 1);
    c->launches += 2;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "reflect launch");
    return TL_OK;
}

}  // namespace tl

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
#include <type_traits>

#include "tl_internal.cuh"
#include "tl_device.cuh"

namespace tl {

namespace {

struct Mixed {
    float *kx, *ky, *mi, *d, *r, *p, *w, *z;
    float *sd[2], *rtemp, *utemp, *cp, *bfp;   // PPCG inner steps
    float *rtemp2;                             // second rtemp of the fused inner passes
    double *fpartials;                         // one per CTA of a fused inner pass
    double *partials;            // one per CTA of the vectorised kernels
    unsigned int *counter;
    int vtiles_x, vtiles;        // tiles of the vectorised kernels
    std::vector<void *> allocs;
};

// Vectorised FP32 kernels of the inner iteration: a lane owns four adjacent
// columns (one float4, 16-byte aligned: the interior starts on a 128-byte
// boundary) and walks kVRows rows keeping the rows above and below in
// registers; x-neighbours across lanes come from warp shuffles.  A CTA is
// 8 warps stacked in y: a 128-column x 64-row tile.
constexpr int kVRows = 8;
constexpr int kVCols = 128;
constexpr int kVTileRows = kVRows * kBlockWarps;

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
        if (isnan(tot)) {  // a NaN start is a breakdown, not "nothing to solve"
            s->done = kBreakdown;
            s->n_exit = s->n;
        } else if (!(sqrt(fabs(tot)) > 0.0)) {
            s->done = kConverged;
        }
        break;
    case kInW:
        s->in_pw = tot;
        s->in_alpha = s->in_rro / s->in_pw;
        if (s->prestep) s->lanczos_a[s->n] = s->in_alpha;  // cg_alphas (tea_leaf_cg.f90)
        break;
    case kInUr: {
        s->in_rrn = tot;
        s->in_beta = s->in_rrn / s->in_rro;
        s->in_rro = s->in_rrn;
        s->in_n += 1;
        const double e = sqrt(fabs(tot));
        if (s->prestep) {
            // the CG phase of tea_solve.f90:400-417 and its switch test
            // (:157-171), as the FP64 path's finish_iteration
            s->lanczos_b[s->n] = s->in_beta;
            s->error = e;
            if (fabs(e) < s->eps * s->initial_residual) {
                s->done = kConverged;
                s->n_exit = s->n;
            } else if (isnan(e)) {
                s->done = kBreakdown;
                s->n_exit = s->n;
            } else {
                s->old_error = e;
                s->n += 1;
                if (s->n > s->max_iters) {
                    s->done = kMaxIters;
                    s->n_exit = s->n;
                } else if ((!s->first && s->n > 1) || (fabs(s->old_error) <= s->epslim && s->n >= s->presteps)) {
                    s->done = kSwitch;
                }
            }
            break;
        }
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

// ------------------------------------------------ vectorised inner kernels

struct GeoV {
    int nx, ny, h, pitch;
    int tiles_x, tiles;
};

__device__ __forceinline__ float4 ld4(const float *__restrict__ f, int64_t i) {
    return *reinterpret_cast<const float4 *>(f + i);
}

// store the first `nv` of four values (all four when nv == 4)
__device__ __forceinline__ void st4(float *__restrict__ f, int64_t i, float4 v, int nv) {
    if (nv >= 4) {
        *reinterpret_cast<float4 *>(f + i) = v;
    } else {
        if (nv > 0) f[i] = v.x;
        if (nv > 1) f[i + 1] = v.y;
        if (nv > 2) f[i + 2] = v.z;
    }
}

__device__ __forceinline__ float cell_apply(float c, float n, float s, float w, float e, float kyn,
                                            float kyc, float kxe, float kxc) {
    float v = fmaf(kyn, c - n, c);
    v = fmaf(kyc, c - s, v);
    v = fmaf(kxe, c - e, v);
    return fmaf(kxc, c - w, v);
}

// block + grid reduction of a compensated sum; the last CTA runs the inner
// epilogue.  Every thread of the CTA must call it.
__device__ __forceinline__ void reduce_v(CSum acc, double *partials, unsigned int *counter,
                                         DevScalars *sc, int epi) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
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

// w = A p on a 128 x 64 tile; sum p.w
__global__ void __launch_bounds__(kBlockThreads) k_v_w(GeoV g, const float *__restrict__ p,
                                                       const float *__restrict__ kx,
                                                       const float *__restrict__ ky,
                                                       float *__restrict__ w, double *partials,
                                                       unsigned int *counter, DevScalars *sc) {
    if (*(volatile const int *)&sc->done) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = (blockIdx.x % g.tiles_x) * kVCols + lane * 4;
    const int j0 = (blockIdx.x / g.tiles_x) * kVTileRows + warp * kVRows;
    const int nv = min(4, g.nx - c);           // valid columns of this lane
    const bool live = c < g.nx + 4;            // lanes that load (the first one past nx reads the halo)
    CSum acc = {0.f, 0.f};
    if (j0 < g.ny) {
        const int64_t P = g.pitch;
        int64_t i = (int64_t)(c + g.h) + (int64_t)(j0 + g.h) * P;
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        // software pipeline, two rows deep: while row rr is computed, the p
        // and Ky rows rr+2 and the Kx row rr+1 (with the lanes' edge values)
        // are in flight.  A row is loaded only when it exists: padded rows
        // run to ny + h, so row ny (the halo) is the last one read.
        auto ldrow = [&](const float *f, int64_t at, int row) { return (live && row <= g.ny) ? ld4(f, at) : z4; };
        float4 xm = ldrow(p, i - P, j0 - 1);
        float4 x0 = ldrow(p, i, j0);
        float4 xp = ldrow(p, i + P, j0 + 1);
        float4 ky0 = ldrow(ky, i, j0);
        float4 ky1 = ldrow(ky, i + P, j0 + 1);
        float4 kxv = ldrow(kx, i, j0);
        float kxe_edge = 0.f, xe_edge = 0.f, xw_edge = 0.f;  // the last / first lane's neighbours
        if (lane == 31 && live) {
            kxe_edge = kx[i + 4];
            xe_edge = p[i + 4];
        }
        if (lane == 0 && live) xw_edge = p[i - 1];
#pragma unroll
        for (int rr = 0; rr < kVRows; ++rr) {
            if (j0 + rr >= g.ny) break;
            const int64_t in = i + P, inn = i + 2 * P;
            const int rn = j0 + rr + 1, rnn = j0 + rr + 2;
            const float4 xpp = ldrow(p, inn, rnn);
            const float4 ky2 = ldrow(ky, inn, rnn);
            const float4 kxn = ldrow(kx, in, rn);
            float kxe_n = 0.f, xe_n = 0.f, xw_n = 0.f;
            if (lane == 31 && live && rn <= g.ny) {
                kxe_n = kx[in + 4];
                xe_n = p[in + 4];
            }
            if (lane == 0 && live && rn <= g.ny) xw_n = p[in - 1];
            float kxe = __shfl_down_sync(0xffffffffu, kxv.x, 1);
            float xe = __shfl_down_sync(0xffffffffu, x0.x, 1);
            float xw = __shfl_up_sync(0xffffffffu, x0.w, 1);
            if (lane == 31 && live) {
                kxe = kxe_edge;
                xe = xe_edge;
            }
            if (lane == 0 && live) xw = xw_edge;
            float4 o;
            o.x = cell_apply(x0.x, xp.x, xm.x, xw, x0.y, ky1.x, ky0.x, kxv.y, kxv.x);
            o.y = cell_apply(x0.y, xp.y, xm.y, x0.x, x0.z, ky1.y, ky0.y, kxv.z, kxv.y);
            o.z = cell_apply(x0.z, xp.z, xm.z, x0.y, x0.w, ky1.z, ky0.z, kxv.w, kxv.z);
            o.w = cell_apply(x0.w, xp.w, xm.w, x0.z, xe, ky1.w, ky0.w, kxe, kxv.w);
            if (nv > 0) {
                st4(w, i, o, nv);
                csum_add(acc, x0.x * o.x);
                if (nv > 1) csum_add(acc, x0.y * o.y);
                if (nv > 2) csum_add(acc, x0.z * o.z);
                if (nv > 3) csum_add(acc, x0.w * o.w);
            }
            xm = x0;
            x0 = xp;
            xp = xpp;
            ky0 = ky1;
            ky1 = ky2;
            kxv = kxn;
            kxe_edge = kxe_n;
            xe_edge = xe_n;
            xw_edge = xw_n;
            i += P;
        }
    }
    reduce_v(acc, partials, counter, sc, kInW);
}

// d += alpha p; r -= alpha w; z = M^-1 r; sum r.z.  PC: TL_PREC_NONE (z = r,
// not stored), TL_PREC_JAC_DIAG (z = Mi r) or TL_PREC_JAC_BLOCK (the 4-row
// strip solve of k_pp_step on the warp's two strips; ky, cp and bfp with
// 1/diag in each strip's first row)
template <int PC>
__global__ void __launch_bounds__(kBlockThreads) k_v_ur(GeoV g, float *__restrict__ d,
                                                        float *__restrict__ r,
                                                        float *__restrict__ z,
                                                        const float *__restrict__ p,
                                                        const float *__restrict__ w,
                                                        const float *__restrict__ mi,
                                                        const float *__restrict__ ky,
                                                        const float *__restrict__ cp,
                                                        const float *__restrict__ bfp,
                                                        double *partials, unsigned int *counter,
                                                        DevScalars *sc) {
    constexpr bool DIAG = PC == TL_PREC_JAC_DIAG;
    if (*(volatile const int *)&sc->done) return;
    const float alpha = (float)sc->in_alpha;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = (blockIdx.x % g.tiles_x) * kVCols + lane * 4;
    const int j0 = (blockIdx.x / g.tiles_x) * kVTileRows + warp * kVRows;
    const int nv = min(4, g.nx - c);
    CSum acc = {0.f, 0.f};
    if (PC == TL_PREC_JAC_BLOCK && j0 < g.ny && nv > 0) {
        const int64_t P = g.pitch;
#pragma unroll
        for (int s0 = 0; s0 < kVRows; s0 += 4) {
            if (j0 + s0 >= g.ny) break;
            const int m = min(4, g.ny - (j0 + s0));
            const int64_t i0 = (int64_t)(c + g.h) + (int64_t)(j0 + s0 + g.h) * P;
            float4 rv[4], zv[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (k >= m) break;
                const int64_t i = i0 + (int64_t)k * P;
                const float4 pv = ld4(p, i), wv = ld4(w, i), rv0 = ld4(r, i), dv0 = ld4(d, i);
                float4 dv;
                dv.x = fmaf(alpha, pv.x, dv0.x);
                dv.y = fmaf(alpha, pv.y, dv0.y);
                dv.z = fmaf(alpha, pv.z, dv0.z);
                dv.w = fmaf(alpha, pv.w, dv0.w);
                rv[k].x = fmaf(-alpha, wv.x, rv0.x);
                rv[k].y = fmaf(-alpha, wv.y, rv0.y);
                rv[k].z = fmaf(-alpha, wv.z, rv0.z);
                rv[k].w = fmaf(-alpha, wv.w, rv0.w);
                st4(d, i, dv, nv);
                st4(r, i, rv[k], nv);
                // Thomas forward sweep: dp0 = x0 / b0, dp_k = (x_k + Ky_k dp_{k-1}) bfp_k
                const float4 bf = ld4(bfp, i);
                if (k == 0) {
                    zv[0] = make_float4(rv[0].x * bf.x, rv[0].y * bf.y, rv[0].z * bf.z, rv[0].w * bf.w);
                } else {
                    const float4 kyk = ld4(ky, i);
                    zv[k].x = fmaf(kyk.x, zv[k - 1].x, rv[k].x) * bf.x;
                    zv[k].y = fmaf(kyk.y, zv[k - 1].y, rv[k].y) * bf.y;
                    zv[k].z = fmaf(kyk.z, zv[k - 1].z, rv[k].z) * bf.z;
                    zv[k].w = fmaf(kyk.w, zv[k - 1].w, rv[k].w) * bf.w;
                }
            }
#pragma unroll
            for (int k = 2; k >= 0; --k) {
                if (k >= m - 1) continue;
                const float4 cv = ld4(cp, i0 + (int64_t)k * P);
                zv[k].x = fmaf(-cv.x, zv[k + 1].x, zv[k].x);
                zv[k].y = fmaf(-cv.y, zv[k + 1].y, zv[k].y);
                zv[k].z = fmaf(-cv.z, zv[k + 1].z, zv[k].z);
                zv[k].w = fmaf(-cv.w, zv[k + 1].w, zv[k].w);
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (k >= m) break;
                st4(z, i0 + (int64_t)k * P, zv[k], nv);
                csum_add(acc, rv[k].x * zv[k].x);
                if (nv > 1) csum_add(acc, rv[k].y * zv[k].y);
                if (nv > 2) csum_add(acc, rv[k].z * zv[k].z);
                if (nv > 3) csum_add(acc, rv[k].w * zv[k].w);
            }
        }
    } else if (j0 < g.ny && nv > 0) {
        const int64_t P = g.pitch;
        int64_t i = (int64_t)(c + g.h) + (int64_t)(j0 + g.h) * P;
#pragma unroll
        for (int rr = 0; rr < kVRows; ++rr) {
            if (j0 + rr >= g.ny) break;
            const float4 pv = ld4(p, i), wv = ld4(w, i), rv0 = ld4(r, i), dv0 = ld4(d, i);
            float4 dv, rv, zv;
            dv.x = fmaf(alpha, pv.x, dv0.x);
            dv.y = fmaf(alpha, pv.y, dv0.y);
            dv.z = fmaf(alpha, pv.z, dv0.z);
            dv.w = fmaf(alpha, pv.w, dv0.w);
            rv.x = fmaf(-alpha, wv.x, rv0.x);
            rv.y = fmaf(-alpha, wv.y, rv0.y);
            rv.z = fmaf(-alpha, wv.z, rv0.z);
            rv.w = fmaf(-alpha, wv.w, rv0.w);
            if (DIAG) {
                const float4 m = ld4(mi, i);
                zv = make_float4(rv.x * m.x, rv.y * m.y, rv.z * m.z, rv.w * m.w);
                st4(z, i, zv, nv);
            } else {
                zv = rv;
            }
            st4(d, i, dv, nv);
            st4(r, i, rv, nv);
            csum_add(acc, rv.x * zv.x);
            if (nv > 1) csum_add(acc, rv.y * zv.y);
            if (nv > 2) csum_add(acc, rv.z * zv.z);
            if (nv > 3) csum_add(acc, rv.w * zv.w);
            i += P;
        }
    }
    reduce_v(acc, partials, counter, sc, kInUr);
}

// p = z + beta p
__global__ void __launch_bounds__(kBlockThreads) k_v_p(GeoV g, float *__restrict__ p,
                                                       const float *__restrict__ z,
                                                       DevScalars *sc) {
    if (*(volatile const int *)&sc->done) return;
    const float beta = (float)sc->in_beta;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = (blockIdx.x % g.tiles_x) * kVCols + lane * 4;
    const int j0 = (blockIdx.x / g.tiles_x) * kVTileRows + warp * kVRows;
    const int nv = min(4, g.nx - c);
    if (j0 >= g.ny || nv <= 0) return;
    const int64_t P = g.pitch;
    int64_t i = (int64_t)(c + g.h) + (int64_t)(j0 + g.h) * P;
#pragma unroll
    for (int rr = 0; rr < kVRows; ++rr) {
        if (j0 + rr >= g.ny) break;
        const float4 pv = ld4(p, i), zv = ld4(z, i);
        float4 o;
        o.x = fmaf(beta, pv.x, zv.x);
        o.y = fmaf(beta, pv.y, zv.y);
        o.z = fmaf(beta, pv.z, zv.z);
        o.w = fmaf(beta, pv.w, zv.w);
        st4(p, i, o, nv);
        i += P;
    }
}

// ------------------------------------ PPCG inner steps in FP32 (mixed form)
//
// The polynomial preconditioner of PPCG (tea_leaf_ppcg.f90:174-230):
//   sd = z / theta, rtemp = r, utemp = sd;  for k = 1..inner:
//   rtemp -= A sd; sd = alpha_k sd + beta_k M^-1 rtemp; utemp += sd;  z = utemp
// runs here in FP32, one fused kernel per inner step (sd ping-pongs between
// two buffers so the stencil reads the previous step); the last step writes
// z back in FP64.  The outer flexible CG stays FP64, so the inexact FP32
// preconditioner only changes how fast it converges, not what it converges
// to.  Block-Jacobi strips (4 rows) are solved in registers, a float4 of
// columns per lane; the FP32 copy keeps 1/diag of each strip's first row in
// bfp (which the FP64 factorisation leaves unused there).

// sd = (z or r) / theta; rtemp = r; utemp = sd
template <bool USE_Z>
__global__ void __launch_bounds__(kBlockThreads) k_pp_init(GeoV g, int pitch64, const double *__restrict__ r64,
                                                           const double *__restrict__ z64, float *__restrict__ sd,
                                                           float *__restrict__ rtemp, float *__restrict__ utemp,
                                                           const DevScalars *__restrict__ sc) {
    if (*(volatile const int *)&sc->done) return;
    const double theta_r = 1.0 / sc->theta;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = (blockIdx.x % g.tiles_x) * kVCols + lane * 4;
    const int j0 = (blockIdx.x / g.tiles_x) * kVTileRows + warp * kVRows;
    const int nv = min(4, g.nx - c);
    if (j0 >= g.ny || nv <= 0) return;
#pragma unroll
    for (int rr = 0; rr < kVRows; ++rr) {
        const int j = j0 + rr;
        if (j >= g.ny) break;
        const int64_t i32 = (int64_t)(c + g.h) + (int64_t)(j + g.h) * g.pitch;
        const int64_t i64 = (int64_t)(c + g.h) + (int64_t)(j + g.h) * pitch64;
        float4 rv, sv;
        float *rp = &rv.x, *sp = &sv.x;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double rq = q < nv ? r64[i64 + q] : 0.0;
            const double zq = USE_Z ? (q < nv ? z64[i64 + q] : 0.0) : rq;
            rp[q] = (float)rq;
            sp[q] = (float)(zq * theta_r);
        }
        st4(rtemp, i32, rv, nv);
        st4(sd, i32, sv, nv);
        st4(utemp, i32, sv, nv);
    }
}

// one inner step; PC: preconditioner, LAST: write z (FP64) = utemp instead
// of rtemp / sd / utemp
template <int PC, bool LAST>
__global__ void __launch_bounds__(kBlockThreads) k_pp_step(
    GeoV g, int pitch64, const float *__restrict__ sd_in, float *__restrict__ sd_out,
    float *__restrict__ rtemp, float *__restrict__ utemp, const float *__restrict__ kx,
    const float *__restrict__ ky, const float *__restrict__ mi, const float *__restrict__ cp,
    const float *__restrict__ bfp, const double *__restrict__ alphas, const double *__restrict__ betas,
    int step, double *__restrict__ z64, const DevScalars *__restrict__ sc) {
    if (*(volatile const int *)&sc->done) return;
    const float al = (float)alphas[step - 1], be = (float)betas[step - 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = (blockIdx.x % g.tiles_x) * kVCols + lane * 4;
    const int j0 = (blockIdx.x / g.tiles_x) * kVTileRows + warp * kVRows;
    const int nv = min(4, g.nx - c);
    const bool live = c < g.nx + 4;
    if (j0 >= g.ny) return;
    const int64_t P = g.pitch;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    int64_t i = (int64_t)(c + g.h) + (int64_t)(j0 + g.h) * P;
    float4 xm = live ? ld4(sd_in, i - P) : z4;
    float4 x0 = live ? ld4(sd_in, i) : z4;
    float4 ky0 = live ? ld4(ky, i) : z4;
    // sd = alpha sd + beta z; utemp += sd; store (z64 on the last step)
    auto finish = [&](int64_t ik, int row, float4 sdo, float4 zv) {
        if (nv <= 0) return;
        float4 sn;
        sn.x = fmaf(al, sdo.x, be * zv.x);
        sn.y = fmaf(al, sdo.y, be * zv.y);
        sn.z = fmaf(al, sdo.z, be * zv.z);
        sn.w = fmaf(al, sdo.w, be * zv.w);
        const float4 ut = ld4(utemp, ik);
        const float4 un = make_float4(ut.x + sn.x, ut.y + sn.y, ut.z + sn.z, ut.w + sn.w);
        if (LAST) {
            const int64_t i64 = (int64_t)(c + g.h) + (int64_t)(row + g.h) * pitch64;
            const float *uq = &un.x;
            for (int q = 0; q < nv; ++q) z64[i64 + q] = (double)uq[q];
        } else {
            st4(sd_out, ik, sn, nv);
            st4(utemp, ik, un, nv);
        }
    };
    // rtemp - A sd for the row at ik (advances the row window)
    auto stencil_row = [&](int64_t ik) {
        const float4 xp = live ? ld4(sd_in, ik + P) : z4;
        const float4 ky1 = live ? ld4(ky, ik + P) : z4;
        const float4 kxv = live ? ld4(kx, ik) : z4;
        float kxe = __shfl_down_sync(0xffffffffu, kxv.x, 1);
        float xe = __shfl_down_sync(0xffffffffu, x0.x, 1);
        float xw = __shfl_up_sync(0xffffffffu, x0.w, 1);
        if (lane == 31 && live) {
            kxe = kx[ik + 4];
            xe = sd_in[ik + 4];
        }
        if (lane == 0 && live) xw = sd_in[ik - 1];
        const float4 r0 = live ? ld4(rtemp, ik) : z4;
        float4 o;
        o.x = r0.x - cell_apply(x0.x, xp.x, xm.x, xw, x0.y, ky1.x, ky0.x, kxv.y, kxv.x);
        o.y = r0.y - cell_apply(x0.y, xp.y, xm.y, x0.x, x0.z, ky1.y, ky0.y, kxv.z, kxv.y);
        o.z = r0.z - cell_apply(x0.z, xp.z, xm.z, x0.y, x0.w, ky1.z, ky0.z, kxv.w, kxv.z);
        o.w = r0.w - cell_apply(x0.w, xp.w, xm.w, x0.z, xe, ky1.w, ky0.w, kxe, kxv.w);
        xm = x0;
        x0 = xp;
        ky0 = ky1;
        if (!LAST) st4(rtemp, ik, o, nv);
        return o;
    };
    if constexpr (PC != TL_PREC_JAC_BLOCK) {
        // pointwise preconditioner: finish each row as soon as it is computed
#pragma unroll
        for (int rr = 0; rr < kVRows; ++rr) {
            if (j0 + rr >= g.ny) break;
            const int64_t ik = i + (int64_t)rr * P;
            const float4 sdo = x0;
            const float4 rt = stencil_row(ik);
            float4 zv = rt;
            if (PC == TL_PREC_JAC_DIAG) {
                const float4 mv = live ? ld4(mi, ik) : z4;
                zv = make_float4(rt.x * mv.x, rt.y * mv.y, rt.z * mv.z, rt.w * mv.w);
            }
            finish(ik, j0 + rr, sdo, zv);
        }
    } else {
#pragma unroll
    for (int s0 = 0; s0 < kVRows; s0 += 4) {
        if (j0 + s0 >= g.ny) break;
        const int m = min(4, g.ny - (j0 + s0));
        // rtemp of the strip's rows, then z = M^-1 rtemp in place (Thomas:
        // dp0 = x0 / b0, dp_k = (x_k + Ky_k dp_{k-1}) bfp_k, z_k = dp_k - cp_k z_{k+1})
        float4 v[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (k >= m) break;
            const int64_t ik = i + (int64_t)(s0 + k) * P;
            const float4 kyk = ky0;  // the face below row k, before the window moves
            const float4 rt = stencil_row(ik);
            const float4 bf = live ? ld4(bfp, ik) : z4;
            if (k == 0) {
                v[0] = make_float4(rt.x * bf.x, rt.y * bf.y, rt.z * bf.z, rt.w * bf.w);
            } else {
                v[k].x = fmaf(kyk.x, v[k - 1].x, rt.x) * bf.x;
                v[k].y = fmaf(kyk.y, v[k - 1].y, rt.y) * bf.y;
                v[k].z = fmaf(kyk.z, v[k - 1].z, rt.z) * bf.z;
                v[k].w = fmaf(kyk.w, v[k - 1].w, rt.w) * bf.w;
            }
        }
#pragma unroll
        for (int k = 2; k >= 0; --k) {
            if (k >= m - 1) continue;
            const float4 cv = live ? ld4(cp, i + (int64_t)(s0 + k) * P) : z4;
            v[k].x = fmaf(-cv.x, v[k + 1].x, v[k].x);
            v[k].y = fmaf(-cv.y, v[k + 1].y, v[k].y);
            v[k].z = fmaf(-cv.z, v[k + 1].z, v[k].z);
            v[k].w = fmaf(-cv.w, v[k + 1].w, v[k].w);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (k >= m) break;
            const int64_t ik = i + (int64_t)(s0 + k) * P;
            finish(ik, j0 + s0 + k, live ? ld4(sd_in, ik) : z4, v[k]);
        }
    }
    }
}

// ---------------------------- temporally blocked PPCG inner steps (FP32)
//
// T inner steps per pass over HBM (the matrix-powers idea of the
// reference's halo_depth > 1 PPCG, tea_leaf_ppcg.f90:199-221, done inside one
// chunk).  A CTA spans fused_threads<T>() columns (one column per thread:
// a band of owned columns and T columns of halo on each side, recomputed)
// and takes an equal share of the band-major sequence of (band, 4-row
// strip) pairs.  It streams down the strips of its share as a pipeline: at
// iteration s, level 0 takes strip s (sd, rtemp, utemp and the strip's
// coefficients, loaded from HBM during iteration s-1; the strip after that
// is prefetched into L2) and level t = 1..T
// applies inner step t to strip s - t, from level t-1's strips s-t-1 (last
// row), s-t and s-t+1 (first row).  Vertical neighbours stay in the
// thread's registers; horizontal ones go through shared memory (a buffer
// per level and iteration parity), and so do the coefficients (a ring of the
// T+1 strips in flight), so a coefficient is read from HBM once per pass and
// the levels never wait on global loads: one barrier per strip.  Shared
// memory keeps a column's strip as one float4 (its 4 rows) per array, so a
// level reads its coefficients, its west and east neighbours' sd and the
// east neighbour's Kx with one 16-byte load each.  Level T
// stores its strip when it lies in the CTA's band and share.  sd and rtemp
// are read in halos that other CTAs own, so they ping-pong between launches;
// utemp is read and written only at owned cells (its halo values are never
// stored) and is updated in place.  Every value is computed with the
// operations of k_pp_step in the same order, so T fused steps give the bits
// of T single steps.
constexpr int kFusedPrefetch = 1;  // strips beyond the next one that are prefetched into L2

// CTA width (threads = columns) of a T-step pass.  Two CTAs run on an SM;
// an SM sub-partition holds 16 K registers, so 7-warp CTAs get 128
// registers a thread and 6-warp CTAs 168 (T >= 2 needs more than 128).
template <int T>
__host__ __device__ constexpr int fused_threads() {
    return T >= 2 ? 192 : 224;
}
constexpr int kFusedThreadsMax = 224;
constexpr int kFusedBandMin = 192 - 2 * kFusedMax;  // the narrowest band of any pass

// the columns a T-step pass's CTA owns (the rest is halo)
inline int fused_band(int T) {
    const int nt = T >= 5   ? fused_threads<5>()
                   : T == 4 ? fused_threads<4>()
                   : T == 3 ? fused_threads<3>()
                   : T == 2 ? fused_threads<2>()
                            : fused_threads<1>();
    return nt - 2 * T;
}

struct PpFusedArgs {
    int nx, ny, h, pitch, pitch64;
    int band;    // columns a CTA owns (fused_band(T))
    int nbands;  // bands across the field
    int chunk;   // strips a CTA takes from the band-major (band, strip) sequence
    const float *sd_in, *rt_in;
    float *sd_out, *rt_out, *utemp;
    const float *kx, *ky, *mi, *cp, *bfp;
    const double *alphas, *betas;
    int step0;                      // inner step of level 1 (1-based)
    double *z64;                    // LAST: z = utemp in FP64
    // LAST with rrn: also sum (r - r_store).z, the PPCG outer rrn
    // (tea_leaf_ppcg.cuknl:279-297), and run its scalar update
    int rrn;
    const double *r64, *rs64;
    double *partials;
    unsigned int *counter;
};

// CTA + grid sum of the fused pass's rrn (deterministic: warps, then CTAs,
// in index order); the last CTA updates the PPCG scalars as the FP64
// path's ppcg_rrn epilogue does: rrn, beta = rrn / rro, error = rro = rrn,
// one more outer iteration.
// Every thread of the CTA calls it.
__device__ void fused_rrn_reduce(double acc, double *partials, unsigned int *counter, DevScalars *sc) {
    __shared__ double sh[kFusedThreadsMax / 32];
    const int NW = blockDim.x >> 5;
    __shared__ int is_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (lane == 0) sh[warp] = acc;
    __syncthreads();
    const unsigned nb = gridDim.x * gridDim.y, b = blockIdx.y * gridDim.x + blockIdx.x;
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < NW; ++w) t += sh[w];
        partials[b] = t;
        __threadfence();
        is_last = atomicAdd(counter, 1u) == nb - 1;
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double t = 0.0;
    for (unsigned i = threadIdx.x; i < nb; i += blockDim.x) t += __ldcg(&partials[i]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    __syncthreads();
    if (lane == 0) sh[warp] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < NW; ++w) tot += sh[w];
        sc->rrn = tot;
        sc->beta = tot / sc->rro;
        sc->error = tot;
        sc->rro = tot;
        sc->ppcg_iters += 1;
        __threadfence();
        *counter = 0u;
    }
}

// coefficient arrays staged per strip: Kx, Ky, then cp, bfp (block) or Mi (diag)
template <int PC>
__host__ __device__ constexpr int fused_narr() {
    return PC == TL_PREC_JAC_BLOCK ? 4 : (PC == TL_PREC_JAC_DIAG ? 3 : 2);
}

// shared memory holds, per strip and array, one float4 per column: the
// strip's 4 rows.  A row of columns has one entry per thread plus a zero
// at each end, so the west / east neighbours of the band's edge threads
// read zeros.
template <int T, int PC>
__host__ __device__ constexpr size_t fused_smem() {
    return sizeof(float4) * (fused_threads<T>() + 2) * (fused_narr<PC>() * (T + 1) + 2 * T);
}

// row k (0..3, known at compile time) of a column's strip
__device__ __forceinline__ float row_of(const float4 &v, int k) {
    return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

// Paired FP32 arithmetic (f32x2): two rows of a strip in one instruction,
// each lane rounded exactly as the scalar operation (round to nearest, no
// flush to zero), so a paired step gives the scalar step's bits.
using f2 = unsigned long long;
__device__ __forceinline__ f2 pk2(float lo, float hi) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void up2(f2 v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
// cell_apply on rows (k, k+1): the same four fused steps in the same order
__device__ __forceinline__ f2 cell_apply2(f2 c, f2 n, f2 s, f2 w, f2 e, f2 kyn, f2 kyc, f2 kxe, f2 kxc) {
    f2 v = fma2(kyn, sub2(c, n), c);
    v = fma2(kyc, sub2(c, s), v);
    v = fma2(kxe, sub2(c, e), v);
    return fma2(kxc, sub2(c, w), v);
}

// LAST: the last pass of a solve (writes z in FP64).  FIRST: the first pass
// of a solve, which starts the inner steps from r (FP64): rtemp = r, sd =
// utemp = M^-1 r / theta (the start BodyPpUr<PC, true> writes), instead of
// reading sd, rtemp and utemp.  RRN (with LAST only): the pass also sums
// the outer (r - r_store).z (a template flag, so that passes without the sum
// carry none of its registers)
template <int T, int PC, bool LAST, bool FIRST, bool RRN = false>
__global__ void __launch_bounds__(fused_threads<T>(), 2) k_pp_fused(PpFusedArgs a, DevScalars *sc) {
    static_assert(!RRN || LAST, "the rrn sum belongs to the last pass");
    if (*(volatile const int *)&sc->done) return;
    constexpr int NT = fused_threads<T>();
    constexpr int SR = NT + 2;  // shared-memory row stride
    constexpr int NA = fused_narr<PC>();
    constexpr int R = T + 1;  // ring slots
    extern __shared__ float4 smem4[];
    const int tid = threadIdx.x;
    float4 *const cfb = smem4 + 1;                // [R][NA][SR]: coefficients by strip slot
    float4 *const xsb = smem4 + R * NA * SR + 1;  // [T][2][SR]: sd by producer level and parity
    const int nstrips = (a.ny + 3) >> 2;
    float al[T], be[T];
#pragma unroll
    for (int t = 0; t < T; ++t) {
        al[t] = (float)a.alphas[a.step0 + t - 1];
        be[t] = (float)a.betas[a.step0 + t - 1];
    }
    for (int k = tid; k < (R * NA + 2 * T) * SR; k += NT) smem4[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    const float theta_r = FIRST ? (float)(1.0 / sc->theta) : 0.f;
    double racc = 0.0;  // LAST with rrn: this thread's (r - r_store).z
    // the CTA's share of the band-major sequence of (band, strip) pairs: a
    // share that reaches the end of a band goes on at the top of the next
    // one with a new pipeline (what a pipeline holds before its first strip
    // never reaches a stored value)
    // (32-bit: a field has fewer than 2^31 cells, so fewer (band, strip) pairs)
    const int w_end = min((int)(blockIdx.x + 1) * a.chunk, a.nbands * nstrips);
    for (int w = (int)blockIdx.x * a.chunk; w < w_end;) {
        const int band = w / nstrips;
        const int sb = w - band * nstrips;
        const int se = min(nstrips, sb + (w_end - w));
        w += se - sb;
        const int col = band * a.band - T + tid;
        const bool incol = col >= 0 && col < a.nx;
        const bool own = incol && tid >= T && tid < T + a.band;
        // the pipeline registers carried from one strip to the next: per
        // producer level l < T its output strip of the previous iteration
        // (sd, rtemp, utemp) and the last sd row of the one before.  For
        // T <= 3 the strip loop is unrolled by two with two sets that swap
        // roles, so nothing is copied from one set to the other.  Level 0's
        // loads of the next strip are one set (Ld): an iteration has used
        // them up before it loads the next strip into them.
        struct Pipe {
            float sdP[T][4], sdL[T], rtP[T][4], utP[T][4];
        };
        struct Ld {
            float ldS[4], ldR[4], ldU[4], ldC[NA][4];
            double ldR64[FIRST ? 4 : 1];  // FIRST: r (FP64) in place of sd, rtemp, utemp
        };
        Pipe pa, pb;
        Ld ld;
#pragma unroll
        for (int l = 0; l < T; ++l) {
            pa.sdL[l] = 0.f;
#pragma unroll
            for (int k = 0; k < 4; ++k) pa.sdP[l][k] = pa.rtP[l][k] = pa.utP[l][k] = 0.f;
        }
        // level 0 loads, one strip ahead (32-bit offsets, FP64 fields too: a
        // field has < 2^31 elements)
        const int cbase = col + a.h;
        auto load = [&](int s, Ld &o) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int row = 4 * s + k;
                const bool v = incol && s >= 0 && row < a.ny;
                const int i = cbase + (row + a.h) * a.pitch;
                if constexpr (FIRST) {
                    o.ldR64[k] = v ? a.r64[cbase + (row + a.h) * a.pitch64] : 0.0;
                } else {
                    o.ldS[k] = v ? a.sd_in[i] : 0.f;
                    o.ldR[k] = v ? a.rt_in[i] : 0.f;
                    o.ldU[k] = v ? a.utemp[i] : 0.f;
                }
                o.ldC[0][k] = v ? __ldg(&a.kx[i]) : 0.f;
                o.ldC[1][k] = v ? __ldg(&a.ky[i]) : 0.f;
                if (PC == TL_PREC_JAC_BLOCK) {
                    o.ldC[2][k] = v ? __ldg(&a.cp[i]) : 0.f;
                    o.ldC[3][k] = v ? __ldg(&a.bfp[i]) : 0.f;
                } else if (PC == TL_PREC_JAC_DIAG) {
                    o.ldC[NA - 1][k] = v ? __ldg(&a.mi[i]) : 0.f;
                }
            }
        };
        // L2 prefetch of the strip kFusedPrefetch after the next one, so that
        // level 0's loads find it in L2: lane l < 4 (NA + 3) of each warp takes
        // array l / 4 and row l % 4 and touches the lines of the warp's first
        // and last columns (clamped to the field)
        const int lane = tid & 31;
        const int wc0 = max(col - lane, 0), wc1 = min(col - lane + 31, a.nx - 1);
        const int pf_arr = lane >> 2, pf_k = lane & 3;
        const float *const pf_base = pf_arr == 0   ? a.sd_in
                                     : pf_arr == 1 ? a.rt_in
                                     : pf_arr == 2 ? a.utemp
                                     : pf_arr == 3 ? a.kx
                                     : pf_arr == 4 ? a.ky
                                     : pf_arr == 5 ? (PC == TL_PREC_JAC_BLOCK ? a.cp : a.mi)
                                                   : a.bfp;
        // (the first pass reads r (FP64) in place of sd, rtemp and utemp)
        const bool pf_on = pf_arr < NA + 3 && wc0 <= wc1 && !(FIRST && (pf_arr == 1 || pf_arr == 2));
        auto prefetch = [&](int s2) {
            const int row = 4 * s2 + pf_k;
            if (pf_on && s2 >= 0 && row < a.ny) {
                if (FIRST && pf_arr == 0) {
                    const double *p = a.r64 + (int64_t)(row + a.h) * a.pitch64 + a.h;
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(p + wc0));
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(p + wc1));
                } else {
                    const float *p = pf_base + (row + a.h) * a.pitch + a.h;
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(p + wc0));
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(p + wc1));
                }
            }
        };
        load(sb - T, ld);
#pragma unroll
        for (int d = 1; d <= kFusedPrefetch; ++d) prefetch(sb - T + d);
        int slot = (sb - T + 8 * R) % R;  // ring slot of strip s (sb - T >= -2T >= -8)
        const int s_end = se + T;
        __syncthreads();
        // one strip iteration: level 0 takes strip s from `in`, levels 1..T
        // advance, and what the next iteration needs goes to `out`
        auto iter = [&](const int s, const Pipe &in, Pipe &out) {
            // level 0's strip s: sd, rtemp, utemp
            float s0[4], r0[4], u0[4];
            if constexpr (FIRST) {
                // the start of the inner steps from r on the strip's mm rows:
                // rtemp = r, z = M^-1 rtemp, sd = utemp = z / theta (BodyPpUr's
                // operations, row for row)
                const int mm = (incol && s >= 0) ? max(0, min(4, a.ny - 4 * s)) : 0;
                float zf[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    r0[k] = (float)ld.ldR64[k];
                    zf[k] = 0.f;
                }
                if constexpr (PC == TL_PREC_JAC_BLOCK) {
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (k < mm)
                            zf[k] = k == 0 ? r0[0] * ld.ldC[3][0]
                                           : fmaf(ld.ldC[1][k], zf[k > 0 ? k - 1 : 0], r0[k]) * ld.ldC[3][k];
#pragma unroll
                    for (int k = 2; k >= 0; --k)
                        if (k < mm - 1) zf[k] = fmaf(-ld.ldC[2][k], zf[k + 1], zf[k]);
                } else {
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (k < mm) zf[k] = PC == TL_PREC_JAC_DIAG ? r0[k] * ld.ldC[NA - 1][k] : r0[k];
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) s0[k] = u0[k] = k < mm ? zf[k] * theta_r : 0.f;
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    s0[k] = ld.ldS[k];
                    r0[k] = ld.ldR[k];
                    u0[k] = ld.ldU[k];
                }
            }
            {
                float4 *cf = cfb + slot * NA * SR + tid;
                xsb[(s & 1) * SR + tid] = make_float4(s0[0], s0[1], s0[2], s0[3]);
#pragma unroll
                for (int q = 0; q < NA; ++q)
                    cf[q * SR] = make_float4(ld.ldC[q][0], ld.ldC[q][1], ld.ldC[q][2], ld.ldC[q][3]);
            }
            if (s + 1 < s_end) load(s + 1, ld);
            if (s + 1 + kFusedPrefetch < s_end) prefetch(s + 1 + kFusedPrefetch);
            // levels 1..T; FULL: every level's strip lies in the field and has 4
            // rows, so no level tests rows (columns outside the field compute on
            // the zeros they loaded and are never stored) and the levels form one
            // block of straight-line code
            auto levels = [&](auto full) {
                constexpr bool FULL = decltype(full)::value;
                float cS[4], cR[4], cU[4];  // level t-1's output of this iteration
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    cS[k] = s0[k];
                    cR[k] = r0[k];
                    cU[k] = u0[k];
                }
#pragma unroll
                for (int t = 1; t <= T; ++t) {
                    const int q = s - t;
                    const int m = FULL ? 4 : (q >= 0 && q < nstrips && incol) ? min(4, a.ny - 4 * q) : 0;
                    const int sq = slot - t < 0 ? slot - t + R : slot - t;  // ring slot of strip q
                    const int sn = sq + 1 == R ? 0 : sq + 1;                  // and of strip q + 1
                    const float4 *cf = cfb + sq * NA * SR + tid;
                    const float4 *xp = xsb + ((t - 1) * 2 + ((s - 1) & 1)) * SR + tid;
                    const float(&x0)[4] = in.sdP[t - 1];
                    float oS[4], oR[4], oU[4];
                    // the strip's coefficients, its west / east neighbours' sd and the
                    // east neighbour's Kx: one float4 (4 rows) each
                    const float4 kx4 = cf[0], ky4 = cf[SR], kxe4 = cf[1];
                    const float ky_top = cfb[sn * NA * SR + SR + tid].x;  // the face above row 3
                    const float4 xw4 = xp[-1], xe4 = xp[1];
                    // one inner step on the strip's first mm rows (mm == 4: no row tests)
                    auto step = [&](const int mm) {
                        float z[4];
                        if (mm == 4) {
                            // a full strip: the stencil of rows (0, 1) and (2, 3) as
                            // f32x2 pairs
                            const f2 c01 = pk2(x0[0], x0[1]), c23 = pk2(x0[2], x0[3]);
                            const f2 x12 = pk2(x0[1], x0[2]);  // north of rows 0, 1 and south of rows 2, 3
                            const f2 r01 = sub2(pk2(in.rtP[t - 1][0], in.rtP[t - 1][1]),
                                                cell_apply2(c01, x12, pk2(in.sdL[t - 1], x0[0]), pk2(xw4.x, xw4.y),
                                                            pk2(xe4.x, xe4.y), pk2(ky4.y, ky4.z), pk2(ky4.x, ky4.y),
                                                            pk2(kxe4.x, kxe4.y), pk2(kx4.x, kx4.y)));
                            const f2 r23 = sub2(pk2(in.rtP[t - 1][2], in.rtP[t - 1][3]),
                                                cell_apply2(c23, pk2(x0[3], cS[0]), x12, pk2(xw4.z, xw4.w),
                                                            pk2(xe4.z, xe4.w), pk2(ky4.w, ky_top), pk2(ky4.z, ky4.w),
                                                            pk2(kxe4.z, kxe4.w), pk2(kx4.z, kx4.w)));
                            up2(r01, oR[0], oR[1]);
                            up2(r23, oR[2], oR[3]);
                        } else {
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            oS[k] = oR[k] = oU[k] = z[k] = 0.f;
                            if (k < mm) {
                                const float c = x0[k];
                                const float n = k < 3 ? x0[k + 1] : cS[0];
                                const float sv = k > 0 ? x0[k - 1] : in.sdL[t - 1];
                                const float kyn = k < 3 ? row_of(ky4, k + 1) : ky_top;
                                oR[k] = in.rtP[t - 1][k] - cell_apply(c, n, sv, row_of(xw4, k), row_of(xe4, k), kyn,
                                                                      row_of(ky4, k), row_of(kxe4, k), row_of(kx4, k));
                            }
                        }
                        }
                        if constexpr (PC == TL_PREC_JAC_BLOCK) {
                            // Thomas: dp0 = x0 / b0, dp_k = (x_k + Ky_k dp_{k-1}) bfp_k,
                            // z_k = dp_k - cp_k z_{k+1}
                            const float4 bf4 = cf[3 * SR];
#pragma unroll
                            for (int k = 0; k < 4; ++k) {
                                if (k < mm)
                                    z[k] = k == 0 ? oR[0] * row_of(bf4, 0)
                                                  : fmaf(row_of(ky4, k), z[k > 0 ? k - 1 : 0], oR[k]) * row_of(bf4, k);
                            }
                            const float4 cp4 = cf[2 * SR];
#pragma unroll
                            for (int k = 2; k >= 0; --k)
                                if (k < mm - 1) z[k] = fmaf(-row_of(cp4, k), z[k + 1], z[k]);
                        } else if constexpr (PC == TL_PREC_JAC_DIAG) {
                            const float4 mi4 = cf[2 * SR];
#pragma unroll
                            for (int k = 0; k < 4; ++k)
                                if (k < mm) z[k] = oR[k] * row_of(mi4, k);
                        } else {
#pragma unroll
                            for (int k = 0; k < 4; ++k)
                                if (k < mm) z[k] = oR[k];
                        }
                        if (mm == 4 && !LAST) {
                            // paired updates too, except in the last pass (whose FP64
                            // stores leave no registers for them)
                            const f2 al2 = pk2(al[t - 1], al[t - 1]), be2 = pk2(be[t - 1], be[t - 1]);
                            const f2 s01 = fma2(al2, pk2(x0[0], x0[1]), mul2(be2, pk2(z[0], z[1])));
                            const f2 s23 = fma2(al2, pk2(x0[2], x0[3]), mul2(be2, pk2(z[2], z[3])));
                            up2(s01, oS[0], oS[1]);
                            up2(s23, oS[2], oS[3]);
                            up2(add2(pk2(in.utP[t - 1][0], in.utP[t - 1][1]), s01), oU[0], oU[1]);
                            up2(add2(pk2(in.utP[t - 1][2], in.utP[t - 1][3]), s23), oU[2], oU[3]);
                        } else {
#pragma unroll
                            for (int k = 0; k < 4; ++k) {
                                if (k < mm) {
                                    oS[k] = fmaf(al[t - 1], x0[k], be[t - 1] * z[k]);
                                    oU[k] = in.utP[t - 1][k] + oS[k];
                                }
                            }
                        }
                    };
                    if (FULL || m == 4) step(4);
                    else step(m);
                    // level t-1's output of this iteration is what level t reads next time
                    out.sdL[t - 1] = x0[3];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        out.sdP[t - 1][k] = cS[k];
                        out.rtP[t - 1][k] = cR[k];
                        out.utP[t - 1][k] = cU[k];
                        cS[k] = oS[k];
                        cR[k] = oR[k];
                        cU[k] = oU[k];
                    }
                    if (t < T) {
                        xsb[(t * 2 + (s & 1)) * SR + tid] = make_float4(oS[0], oS[1], oS[2], oS[3]);
                    } else if (own && q >= sb && q < se) {
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            if (k < m) {
                                const int row = 4 * q + k;
                                if (LAST) {
                                    const int i64 = cbase + (row + a.h) * a.pitch64;
                                    const double zv = (double)oU[k];
                                    a.z64[i64] = zv;
                                    if (RRN) racc = fma(a.r64[i64] - a.rs64[i64], zv, racc);
                                } else {
                                    const int i = cbase + (row + a.h) * a.pitch;
                                    a.sd_out[i] = oS[k];
                                    a.rt_out[i] = oR[k];
                                    a.utemp[i] = oU[k];
                                }
                            }
                        }
                    }
                }
            };
            if (s - T >= 0 && 4 * s <= a.ny) levels(std::true_type{});
            else levels(std::false_type{});
            slot = slot + 1 == R ? 0 : slot + 1;
            __syncthreads();
        };
        if constexpr (T <= 3) {
            int s = sb - T;
            for (; s + 1 < s_end; s += 2) {
                iter(s, pa, pb);
                iter(s + 1, pb, pa);
            }
            if (s < s_end) iter(s, pa, pb);
        } else {
            // T >= 4 has no registers for two sets
            for (int s = sb - T; s < s_end; ++s) {
                iter(s, pa, pb);
                pa = pb;
            }
        }
    }
    if (RRN) fused_rrn_reduce(racc, a.partials, a.counter, sc);
}

// FP32 copies of the preconditioner: Mi = 1/diag, block cp, and bfp with
// 1/diag at each strip's first row
__global__ void k_pp_convert(GeoV g, int pitch64, const double *__restrict__ dg, const double *__restrict__ cp64,
                             const double *__restrict__ bfp64, float *__restrict__ mi, float *__restrict__ cp,
                             float *__restrict__ bfp) {
    const long long n = (long long)g.nx * g.ny;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k % g.nx), j = (int)(k / g.nx);
        const int64_t a = (int64_t)(i + g.h) + (int64_t)(j + g.h) * g.pitch;
        const int64_t b = (int64_t)(i + g.h) + (int64_t)(j + g.h) * pitch64;
        mi[a] = (float)(1.0 / dg[b]);
        cp[a] = (float)cp64[b];
        bfp[a] = (j % 4 == 0) ? (float)(1.0 / dg[b]) : (float)bfp64[b];
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

template <int PC>
struct BodyInnerInit {  // r = (float) r64; z = M^-1 r; p = z; d = 0; sum r.z
    const double *r64;
    const float *mi, *ky, *cp, *bfp;
    float *r, *z, *p, *d;
    int pitch32, pitch64;
    __device__ void setup(DevScalars *) {}
    __device__ void operator()(int64_t b32, int64_t b64, int m, CSum &acc) const {
        float rv[4], zv[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t j = b32 + (int64_t)k * pitch32;
                rv[k] = (float)r64[b64 + (int64_t)k * pitch64];
                if (PC == TL_PREC_JAC_BLOCK)
                    zv[k] = k == 0 ? rv[0] * bfp[j] : fmaf(ky[j], zv[k - 1], rv[k]) * bfp[j];
                else
                    zv[k] = PC == TL_PREC_JAC_DIAG ? rv[k] * mi[j] : rv[k];
            }
        if (PC == TL_PREC_JAC_BLOCK) {
#pragma unroll
            for (int k = 2; k >= 0; --k)
                if (k < m - 1) zv[k] = fmaf(-cp[b32 + (int64_t)k * pitch32], zv[k + 1], zv[k]);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t j = b32 + (int64_t)k * pitch32;
                r[j] = rv[k];
                z[j] = zv[k];
                p[j] = zv[k];
                d[j] = 0.f;
                csum_add(acc, rv[k] * zv[k]);
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

// PPCG outer update fused with the start of the FP32 inner steps:
// u += alpha p, r -= alpha w (FP64, as BodyCgUr of tl_kernels.cu), then
// rtemp = r, z = M^-1 r and sd = utemp = z / theta in FP32 (as k_pp_init):
// z only seeds the FP32 polynomial preconditioner, so M^-1 uses the FP32
// operator copies (the block solve of k_pp_step, 1/diag in bfp's first row).
// START false: the r update alone (the first fused inner pass then starts
// the inner steps from r itself, and u += alpha p runs in the p pass,
// BodyPpcgUP)
template <int PC, bool START>
struct BodyPpUr {
    const double *p, *w;
    double *u, *r;
    const float *mi, *ky, *cp, *bfp;
    float *sd, *rtemp, *utemp;
    int pitch32, pitch64;
    double alpha;
    float theta_r;
    __device__ void setup(DevScalars *sc) {
        alpha = sc->alpha;
        theta_r = (float)(1.0 / sc->theta);
    }
    __device__ void operator()(int64_t b32, int64_t b64, int m, CSum &) const {
        // every load of the strip before the first store (the arrays may
        // alias as far as the compiler knows, so it would not hoist them)
        double uv[4], pv[4], wv[4], rv[4];
        float kyv[4], cpv[4], bfv[4], miv[4], rf[4], zf[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = b64 + (int64_t)k * pitch64;
                const int64_t j = b32 + (int64_t)k * pitch32;
                if (START) {
                    uv[k] = u[i];
                    pv[k] = p[i];
                }
                wv[k] = w[i];
                rv[k] = r[i];
                if (!START) {
                } else if (PC == TL_PREC_JAC_BLOCK) {
                    kyv[k] = ky[j];
                    cpv[k] = cp[j];
                    bfv[k] = bfp[j];
                } else if (PC == TL_PREC_JAC_DIAG) {
                    miv[k] = mi[j];
                }
            }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t i = b64 + (int64_t)k * pitch64;
                if (START) u[i] = fma(alpha, pv[k], uv[k]);
                rv[k] = fma(-alpha, wv[k], rv[k]);
                r[i] = rv[k];
                rf[k] = (float)rv[k];
            }
        if (!START) return;
        if (PC == TL_PREC_JAC_BLOCK) {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (k < m) zf[k] = k == 0 ? rf[0] * bfv[0] : fmaf(kyv[k], zf[k - 1], rf[k]) * bfv[k];
#pragma unroll
            for (int k = 2; k >= 0; --k)
                if (k < m - 1) zf[k] = fmaf(-cpv[k], zf[k + 1], zf[k]);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (k < m) zf[k] = PC == TL_PREC_JAC_DIAG ? rf[k] * miv[k] : rf[k];
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (k < m) {
                const int64_t j = b32 + (int64_t)k * pitch32;
                rtemp[j] = rf[k];
                const float sv = zf[k] * theta_r;
                sd[j] = sv;
                utemp[j] = sv;
            }
    }
};

Mixed *mixed_of(Chunk *c) { return (Mixed *)c->mixed; }

// the FP32 state; on failure nothing of it is kept (mixed_alloc frees it)
int mixed_alloc_fields(Chunk *c) {
    Mixed *mx = new Mixed();
    c->mixed = mx;
    const size_t n = (size_t)c->lead + (size_t)c->pitch * (size_t)c->rows + 32;
    float **arr[] = {&mx->kx, &mx->ky, &mx->mi,    &mx->d,     &mx->r,  &mx->p,  &mx->w,
                     &mx->z,  &mx->sd[0], &mx->sd[1], &mx->rtemp, &mx->utemp, &mx->cp, &mx->bfp,
                     &mx->rtemp2};
    for (float **a : arr) {
        void *p = nullptr;
        cudaError_t e = device_malloc(&p, n * sizeof(float));
        if (e != cudaSuccess) return cuda_fail(e, "mixed cudaMalloc");
        mx->allocs.push_back(p);
        TL_CUDA(cudaMemsetAsync(p, 0, n * sizeof(float), c->stream));
        *a = (float *)p + c->lead;
    }
    mx->vtiles_x = (c->nx + kVCols - 1) / kVCols;
    mx->vtiles = mx->vtiles_x * ((c->ny + kVTileRows - 1) / kVTileRows);
    void *p = nullptr;
    cudaError_t e = device_malloc(&p, sizeof(double) * (size_t)mx->vtiles + 256);
    if (e != cudaSuccess) return cuda_fail(e, "mixed cudaMalloc");
    mx->allocs.push_back(p);
    TL_CUDA(cudaMemsetAsync(p, 0, sizeof(double) * (size_t)mx->vtiles + 256, c->stream));
    mx->counter = (unsigned int *)p;
    mx->partials = (double *)((char *)p + 256);
    // the most CTAs a fused pass can have: the narrowest band, one strip per share
    const size_t fcta = (size_t)((c->nx + kFusedBandMin - 1) / kFusedBandMin) * (size_t)((c->ny + 3) / 4);
    e = device_malloc(&p, sizeof(double) * fcta);
    if (e != cudaSuccess) return cuda_fail(e, "mixed cudaMalloc");
    mx->allocs.push_back(p);
    mx->fpartials = (double *)p;
    return TL_OK;
}

int mixed_alloc(Chunk *c) {
    if (c->mixed) return TL_OK;
    const int rc = mixed_alloc_fields(c);
    if (rc) mixed_free(c);
    return rc;
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

// launch one vectorised kernel with the profiling bracket
template <class F>
int launch_v(Chunk *c, const char *name, F &&launch) {
    int slot = -1;
    if (c->profiling && !c->capturing) prof_begin(c, name, &slot);
    launch();
    if (slot >= 0) prof_end(c, slot);
    c->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, name);
    return TL_OK;
}

template <int PC>
int inner_body_pc(Chunk *c) {
    Mixed *mx = mixed_of(c);
    const bool diag = PC != TL_PREC_NONE;
    const GeoV g{c->nx, c->ny, c->h, c->pitch, mx->vtiles_x, mx->vtiles};
    const unsigned grid = (unsigned)mx->vtiles;
    cudaStream_t s = c->stream;
    int rc;
    if ((rc = launch_v(c, "mixed_w", [&] {
             k_v_w<<<grid, kBlockThreads, 0, s>>>(g, mx->p, mx->kx, mx->ky, mx->w, mx->partials,
                                                   mx->counter, c->sc);
         })))
        return rc;
    if ((rc = launch_v(c, "mixed_ur", [&] {
             k_v_ur<PC><<<grid, kBlockThreads, 0, s>>>(g, mx->d, mx->r, mx->z, mx->p, mx->w, mx->mi, mx->ky,
                                                       mx->cp, mx->bfp, mx->partials, mx->counter, c->sc);
         })))
        return rc;
    return launch_v(c, "mixed_p", [&] {
        k_v_p<<<grid, kBlockThreads, 0, s>>>(g, mx->p, diag ? mx->z : mx->r, c->sc);
    });
}

// the inner CG iteration of the mixed CG solve (none or jac_diag)
int inner_body(Chunk *c) {
    return c->cfg.precond == TL_PREC_JAC_DIAG ? inner_body_pc<TL_PREC_JAC_DIAG>(c)
                                              : inner_body_pc<TL_PREC_NONE>(c);
}

// the FP32 CG presteps of mixed PPCG (any preconditioner)
int prestep_body(Chunk *c) {
    switch (c->cfg.precond) {
    case TL_PREC_JAC_BLOCK: return inner_body_pc<TL_PREC_JAC_BLOCK>(c);
    case TL_PREC_JAC_DIAG: return inner_body_pc<TL_PREC_JAC_DIAG>(c);
    default: return inner_body_pc<TL_PREC_NONE>(c);
    }
}

}  // namespace

// FP32 copies of the operator and of the PPCG preconditioner, after cg_init
// has built the FP64 ones
int mixed_ppcg_prepare(Chunk *c) {
    int rc;
    if ((rc = mixed_alloc(c))) return rc;
    Mixed *mx = mixed_of(c);
    BodyConvert bc{c->kx, c->ky, mx->kx, mx->ky, mx->mi, c->pitch, c->pitch, c->nx, c->ny, c->h};
    if ((rc = run32(c, "mixed_convert", bc, kInNone, false))) return rc;
    const GeoV g{c->nx, c->ny, c->h, c->pitch, mx->vtiles_x, mx->vtiles};
    return launch_v(c, "mixed_pp_convert", [&] {
        k_pp_convert<<<1216, 256, 0, c->stream>>>(g, c->pitch, c->diag, c->cp, c->bfp, mx->mi, mx->cp, mx->bfp);
    });
}

template <int T, int PC, bool LAST, bool FIRST, bool RRN>
void launch_fused2(dim3 grid, cudaStream_t s, const PpFusedArgs &a, DevScalars *sc) {
    constexpr size_t bytes = fused_smem<T, PC>();
    static bool configured = false;  // the attribute belongs to the kernel: set once
    if (!configured) {
        cudaFuncSetAttribute(k_pp_fused<T, PC, LAST, FIRST, RRN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)bytes);
        cudaFuncSetAttribute(k_pp_fused<T, PC, LAST, FIRST, RRN>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             100);
        configured = true;
    }
    k_pp_fused<T, PC, LAST, FIRST, RRN><<<grid, fused_threads<T>(), bytes, s>>>(a, sc);
}

template <int T, int PC, bool LAST, bool FIRST>
void launch_fused1(dim3 grid, cudaStream_t s, const PpFusedArgs &a, DevScalars *sc) {
    if (LAST && a.rrn) launch_fused2<T, PC, LAST, FIRST, LAST>(grid, s, a, sc);
    else launch_fused2<T, PC, LAST, FIRST, false>(grid, s, a, sc);
}

template <int T, int PC>
void launch_fused(dim3 grid, cudaStream_t s, const PpFusedArgs &a, bool last, bool first, DevScalars *sc) {
    if (last && first) launch_fused1<T, PC, true, true>(grid, s, a, sc);
    else if (last) launch_fused1<T, PC, true, false>(grid, s, a, sc);
    else if (first) launch_fused1<T, PC, false, true>(grid, s, a, sc);
    else launch_fused1<T, PC, false, false>(grid, s, a, sc);
}

template <int T>
void launch_fused_pc(dim3 grid, cudaStream_t s, const PpFusedArgs &a, int pc, bool last, bool first,
                     DevScalars *sc) {
    if (pc == TL_PREC_JAC_BLOCK) launch_fused<T, TL_PREC_JAC_BLOCK>(grid, s, a, last, first, sc);
    else if (pc == TL_PREC_JAC_DIAG) launch_fused<T, TL_PREC_JAC_DIAG>(grid, s, a, last, first, sc);
    else launch_fused<T, TL_PREC_NONE>(grid, s, a, last, first, sc);
}

// the inner steps of tea_leaf_ppcg.f90:174-230 in FP32; z (FP64) at the end.
// With c->inner_fuse > 1 the steps run as ceil(inner / inner_fuse) passes of
// k_pp_fused (sizes as even as possible, larger first); otherwise one
// k_pp_step per step.
namespace {

// the inner steps proper, from sd[0], rtemp, utemp to z (FP64)
// rrn: the last fused pass also sums (r - r_store).z and updates the PPCG
// scalars (*did_rrn reports whether it did: only fused passes can)
// FP32 inner steps per fused pass (1: one kernel per step).  The fused
// kernel addresses FP32 fields with 32-bit offsets; fields of 2^31 elements
// or more take the one-kernel-per-step path (64-bit)
int fused_steps(const Chunk *c) {
    const bool fits32 = (size_t)c->lead + (size_t)c->pitch * (size_t)c->rows < ((size_t)1 << 31);
    return !fits32 ? 1 : c->inner_fuse < 1 ? 1 : (c->inner_fuse > kFusedMax ? kFusedMax : c->inner_fuse);
}

// first: the first fused pass starts the inner steps from r (FP64) itself
int inner_steps(Chunk *c, bool rrn, bool *did_rrn, bool first) {
    Mixed *mx = mixed_of(c);
    *did_rrn = false;
    const int inner = c->cfg.ppcg_inner_steps;
    const GeoV g{c->nx, c->ny, c->h, c->pitch, mx->vtiles_x, mx->vtiles};
    const unsigned grid = (unsigned)mx->vtiles;
    cudaStream_t s = c->stream;
    const int pc = c->cfg.precond;
    int rc;
    const int fuse = fused_steps(c);
    if (fuse > 1) {
        float *rt[2] = {mx->rtemp, mx->rtemp2};
        const int passes = (inner + fuse - 1) / fuse;
        const int nstrips = (c->ny + 3) / 4;
        int done = 0;
        for (int l = 0; l < passes; ++l) {
            const int T = (inner - done + (passes - l) - 1) / (passes - l);
            const bool last = l == passes - 1;
            PpFusedArgs a;
            a.nx = c->nx;
            a.ny = c->ny;
            a.h = c->h;
            a.pitch = c->pitch;
            a.pitch64 = c->pitch;
            a.band = fused_band(T);
            a.nbands = (c->nx + a.band - 1) / a.band;
            const long long work = (long long)a.nbands * nstrips;  // (band, strip) pairs
            long long chunk = c->inner_seg;
            if (chunk < 1) {
                // automatic: equal shares for one wave of 2 CTAs per SM (each
                // share recomputes 2T strips of pipeline warm-up, and 2T more
                // where it goes on into the next band)
                chunk = (work + 2 * c->sms - 1) / (2 * c->sms);
                if (chunk < 4 * T) chunk = 4 * T;
            }
            if (chunk > nstrips) chunk = nstrips;
            a.chunk = (int)chunk;
            a.sd_in = mx->sd[l & 1];
            a.sd_out = mx->sd[(l + 1) & 1];
            a.rt_in = rt[l & 1];
            a.rt_out = rt[(l + 1) & 1];
            a.utemp = mx->utemp;
            a.kx = mx->kx;
            a.ky = mx->ky;
            a.mi = mx->mi;
            a.cp = mx->cp;
            a.bfp = mx->bfp;
            a.alphas = c->ch_alphas;
            a.betas = c->ch_betas;
            a.step0 = done + 1;
            const bool fst = first && l == 0;
            a.z64 = c->z;
            a.rrn = (rrn && last) ? 1 : 0;
            a.r64 = c->r;
            a.rs64 = c->r_store;
            a.partials = mx->fpartials;
            a.counter = mx->counter;
            const dim3 fg((unsigned)((work + chunk - 1) / chunk));
            rc = launch_v(c, "mixed_pp_fused", [&] {
                switch (T) {
                case 1: launch_fused_pc<1>(fg, s, a, pc, last, fst, c->sc); break;
                case 2: launch_fused_pc<2>(fg, s, a, pc, last, fst, c->sc); break;
                case 3: launch_fused_pc<3>(fg, s, a, pc, last, fst, c->sc); break;
                case 4: launch_fused_pc<4>(fg, s, a, pc, last, fst, c->sc); break;
                default: launch_fused_pc<5>(fg, s, a, pc, last, fst, c->sc); break;
                }
            });
            if (rc) return rc;
            done += T;
        }
        *did_rrn = rrn;
        return TL_OK;
    }
    for (int st = 1; st <= inner; ++st) {
        const float *si = mx->sd[(st - 1) & 1];
        float *so = mx->sd[st & 1];
        const bool last = st == inner;
#define TL_PP_STEP(PC, L)                                                                              \
    k_pp_step<PC, L><<<grid, kBlockThreads, 0, s>>>(g, c->pitch, si, so, mx->rtemp, mx->utemp, mx->kx, \
                                                    mx->ky, mx->mi, mx->cp, mx->bfp, c->ch_alphas,     \
                                                    c->ch_betas, st, c->z, c->sc)
        rc = launch_v(c, "mixed_pp_step", [&] {
            if (pc == TL_PREC_JAC_BLOCK) {
                if (last) TL_PP_STEP(TL_PREC_JAC_BLOCK, true);
                else TL_PP_STEP(TL_PREC_JAC_BLOCK, false);
            } else if (pc == TL_PREC_JAC_DIAG) {
                if (last) TL_PP_STEP(TL_PREC_JAC_DIAG, true);
                else TL_PP_STEP(TL_PREC_JAC_DIAG, false);
            } else {
                if (last) TL_PP_STEP(TL_PREC_NONE, true);
                else TL_PP_STEP(TL_PREC_NONE, false);
            }
        });
#undef TL_PP_STEP
        if (rc) return rc;
    }
    return TL_OK;
}

bool inner_ready(Chunk *c) {
    if (!mixed_of(c) || c->cfg.ppcg_inner_steps < 1) {
        set_error("mixed PPCG needs tl_ppcg_inner_steps >= 1 and a prepared chunk");
        return false;
    }
    return true;
}

}  // namespace

int mixed_ppcg_inner(Chunk *c) {
    if (!inner_ready(c)) return TL_ERR_STATE;
    Mixed *mx = mixed_of(c);
    const GeoV g{c->nx, c->ny, c->h, c->pitch, mx->vtiles_x, mx->vtiles};
    const unsigned grid = (unsigned)mx->vtiles;
    cudaStream_t s = c->stream;
    int rc;
    if ((rc = launch_v(c, "mixed_pp_init", [&] {
             if (c->cfg.precond == TL_PREC_NONE)
                 k_pp_init<false><<<grid, kBlockThreads, 0, s>>>(g, c->pitch, c->r, c->z, mx->sd[0], mx->rtemp,
                                                                 mx->utemp, c->sc);
             else
                 k_pp_init<true><<<grid, kBlockThreads, 0, s>>>(g, c->pitch, c->r, c->z, mx->sd[0], mx->rtemp,
                                                                mx->utemp, c->sc);
         })))
        return rc;
    bool did_rrn;
    return inner_steps(c, false, &did_rrn, false);
}

bool mixed_fused(const Chunk *c) { return fused_steps(c) > 1; }

int mixed_ppcg_ur_inner(Chunk *c, bool *did_rrn) {
    if (!inner_ready(c)) return TL_ERR_STATE;
    Mixed *mx = mixed_of(c);
    int rc;
    // with fused passes the first pass starts the inner steps from r, and
    // this pass only updates r (u += alpha p runs in the p pass)
    const bool start = fused_steps(c) == 1;
#define TL_PP_UR(PC, S)                                                                                       \
    BodyPpUr<PC, S>{c->p, c->w, c->u, c->r, mx->mi, mx->ky, mx->cp, mx->bfp, mx->sd[0], mx->rtemp, mx->utemp, \
                    c->pitch, c->pitch, 0.0, 0.f}
    if (!start) rc = run32(c, "mixed_pp_ur", TL_PP_UR(TL_PREC_NONE, false), kInNone, true);
    else if (c->cfg.precond == TL_PREC_JAC_BLOCK)
        rc = run32(c, "mixed_pp_ur", TL_PP_UR(TL_PREC_JAC_BLOCK, true), kInNone, true);
    else if (c->cfg.precond == TL_PREC_JAC_DIAG)
        rc = run32(c, "mixed_pp_ur", TL_PP_UR(TL_PREC_JAC_DIAG, true), kInNone, true);
    else rc = run32(c, "mixed_pp_ur", TL_PP_UR(TL_PREC_NONE, true), kInNone, true);
#undef TL_PP_UR
    if (rc) return rc;
    return inner_steps(c, c->inner_fold_rrn, did_rrn, !start);
}

int mixed_ppcg_presteps(Chunk *c, int *done_out) {
    Mixed *mx = mixed_of(c);
    if (!mx) {
        set_error("mixed PPCG presteps need a prepared chunk");
        return TL_ERR_STATE;
    }
    int rc;
    DevScalars &h = *c->sc_host;
    if ((rc = chunk_sync_scalars(c))) return rc;
    h.prestep = 1;
    h.lanczos_a = c->cg_alphas;
    h.lanczos_b = c->cg_betas;
    h.in_target = 0.0;
    if ((rc = chunk_push_scalars(c))) return rc;
    // r = (float) r, z = M^-1 r, p = z, d = 0, in_rro = r.z
#define TL_PRE_INIT(PC)                                                                                        \
    run32(c, "mixed_init", BodyInnerInit<PC>{c->r, mx->mi, mx->ky, mx->cp, mx->bfp, mx->r, mx->z, mx->p, mx->d, \
                                              c->pitch, c->pitch},                                             \
          kInInit, false)
    if (c->cfg.precond == TL_PREC_JAC_BLOCK) rc = TL_PRE_INIT(TL_PREC_JAC_BLOCK);
    else if (c->cfg.precond == TL_PREC_JAC_DIAG) rc = TL_PRE_INIT(TL_PREC_JAC_DIAG);
    else rc = TL_PRE_INIT(TL_PREC_NONE);
#undef TL_PRE_INIT
    if (rc) return rc;
    int done = kRunning;
    if ((rc = run_phase(c, prestep_body, kItersInner, kPhaseMixedPre, &done))) return rc;
    // u += d, r = u0 - A u (FP64): the phase after the switch starts from the
    // true residual
    BodyUpdateU bu{c->u, mx->d, c->pitch, c->pitch};
    if ((rc = run32(c, "mixed_update_u", bu, kInNone, false))) return rc;
    if ((rc = launch_residual(c, kEpiNone))) return rc;
    if ((rc = chunk_sync_scalars(c))) return rc;
    h.prestep = 0;
    if ((rc = chunk_push_scalars(c))) return rc;
    *done_out = done;
    return TL_OK;
}

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
    double r0, rn;
    if (cf.warm_start) {
        // Galerkin warm start; the target stays tl_eps times the plain
        // start's residual
        double rr = 0.0;
        if ((rc = warm_start_or_fallback(c, info, &r0, &rr))) return rc;
        rn = sqrt(fabs(rr));
    } else {
        // r = u0 - A u, ||r||^2 (FP64)
        if ((rc = launch_residual(c, kEpiResid))) return rc;
        if ((rc = chunk_sync_scalars(c))) return rc;
        r0 = h.initial_residual;
        rn = r0;
    }
    const double target = cf.eps * r0;
    double rn_prev = 0.0;
    int outer = 0, inner_total = 0;
    int status = TL_OK;
    bool capped = false;  // an inner solve stopped at tl_max_iters before tl_inner_eps
    while (true) {
        if (isnan(rn)) {  // a NaN residual never meets the tests below
            set_error("mixed solve: breakdown (NaN in the FP64 residual) after %d refinement steps", outer);
            status = TL_ERR_BREAKDOWN;
            break;
        }
        if (rn < target) break;
        if (outer > 0 && rn > 0.5 * rn_prev) break;  // FP64 residual floor reached
        if (outer >= kMaxOuter) {
            status = TL_WARN_MAXITER;
            break;
        }
        // inner FP32 PCG on A d = r; tl_max_iters bounds each inner solve as
        // it bounds one CG solve of the FP64 path
        h.done = kRunning;
        h.in_target = cf.inner_eps;
        h.in_max = cf.max_iters;
        if ((rc = chunk_push_scalars(c))) return rc;
        if (diag) {
            BodyInnerInit<TL_PREC_JAC_DIAG> bi{c->r, mx->mi, mx->ky, mx->cp, mx->bfp, mx->r, mx->z, mx->p, mx->d,
                                               c->pitch, c->pitch};
            if ((rc = run32(c, "mixed_init", bi, kInInit, false))) return rc;
        } else {
            BodyInnerInit<TL_PREC_NONE> bi{c->r, mx->mi, mx->ky, mx->cp, mx->bfp, mx->r, mx->z, mx->p, mx->d,
                                           c->pitch, c->pitch};
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
        if (h.in_n >= cf.max_iters) capped = true;
        // u += d (FP64), r = u0 - A u (FP64)
        BodyUpdateU bu{c->u, mx->d, c->pitch, c->pitch};
        if ((rc = run32(c, "mixed_update_u", bu, kInNone, false))) return rc;
        if ((rc = launch_residual(c, kEpiStore))) return rc;
        if ((rc = chunk_sync_scalars(c))) return rc;
        rn_prev = rn;
        rn = sqrt(fabs(h.sum[0]));
        outer++;
    }
    if (capped && status == TL_OK) {
        status = TL_WARN_MAXITER;
        set_error("mixed solve: an inner FP32 solve reached tl_max_iters (%d) before tl_inner_eps", cf.max_iters);
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

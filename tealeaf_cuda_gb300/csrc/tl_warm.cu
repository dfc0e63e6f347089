// tl_warm.cu -- warm starts of the implicit solve (no reference counterpart).
//
// The system of a timestep is A u = u^n with A = I + the Kx/Ky stencil
// (tea_leaf_common.cuknl:28-34); the plain start is u = u^n, whose residual
// is r0 = u^n - A u^n, and the exact correction is du = A^-1 r0.  A warm
// start adds a combination of search directions to u^n:
//   d_net   = the residual network's prediction of du (tl_warm_start learned)
//   d_1..d_k = the last k increments u^(n-j+1) - u^(n-j) (both modes,
//              k <= the chunk's warm_history, 8 by default)
// with the coefficients that minimise the energy
//   phi(u) = 1/2 u.Au - u.u^n   over   u = u^n + sum_i c_i d_i,
// i.e. the Galerkin system [d_i.Ad_j] c = [d_i.r0] (projection onto previous
// solutions, as for sequences of right-hand sides: with A fixed, the
// increments are repeated applications of A^-1, so they span the smooth,
// slowly decaying part of the next correction).  The small system is solved
// on the host by A-orthonormalising the directions (Gram-Schmidt in the
// inner product G, twice, dropping directions that are numerically
// dependent).  Because A is SPD, phi - phi(u*) = 1/2 |u - u*|_A^2, so the
// chosen start never has a larger A-norm error than the plain one.  The
// solve's exit test stays tl_eps times the plain start's residual, so the
// answer meets the same tolerance.  (TL_WARM_PROJ_RESIDUAL minimises the
// residual's 2-norm instead: [Ad_i.Ad_j] c = [Ad_i.r0].  Measured on the
// 8192^2 standard deck it keeps the start's residual below the plain one's
// but takes slightly more iterations than the energy projection.)
//
// The network corrects what the history leaves: its input residual is that
// of the history start u_h = u^n + (the increments' projection alone),
// r_h = u^n - A u_h, and it predicts A^-1 r_h; the final start is the joint
// projection over the network's direction and the increments.  Input per
// cell (channels 0..6, BF16, NHWC, 1-pixel zero halo):
//   u^n / max|u^n|, log density, log1p(Kx west face), log1p(Ky south face),
//   100 dt, r_h / max|r_h|, d_1 / max|r_h| (the latest increment);
// output channel 0 is (u^{n+1} - u_h) / max|r_h| (the network is
// linear-equivariant in the residual's scale).
//
// Model parameters (FP32, flat, in this order per layer: W [9][coutp][cin]
// then b [coutp]):
//   layer 1: cin 16 (inputs 0..6 used), coutp 32, GELU
//   layers 2-5: cin 32, coutp 32, x + GELU(conv x)
//   layer 6: cin 32, coutp 16 (output channel 0 used), linear head
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <vector>

#include "tl_internal.cuh"

extern "C" int tl_nn_conv(int mode, int cin, int coutp, const void *in, const void *w, const float *bias,
                          const void *res, void *out, void *pre, float *outf, int B, int H, int W,
                          void *stream);
extern "C" int tl_nn_pack(const float *w, void *wf, void *wb, int cin, int coutp, void *stream);

namespace tl {

namespace {

using bf16 = __nv_bfloat16;

constexpr int kLayers = 6;
constexpr int kCin[kLayers] = {16, 32, 32, 32, 32, 32};
constexpr int kCout[kLayers] = {32, 32, 32, 32, 32, 16};
constexpr int kInputs = 7;          // network input channels in use
constexpr int kFeatures = kInputs + 1;  // + the training target
constexpr int kGramBlocks = 608;    // 152 SMs x 4
constexpr int kHist = 8;            // previous increments kept (the ring; a chunk uses up to warm_history)
constexpr int kMaxDirs = kHist + 1; // + the network's direction
constexpr int kGramPairs = kMaxDirs * (kMaxDirs + 1) / 2;
constexpr int kGramSums = kGramPairs + kMaxDirs + 1;  // d_i.Ad_j (i <= j), d_i.r0, r0.r0
constexpr float kClamp = 64.f;      // bound of the scaled inputs
// The network is consulted while it pays: when its direction adds less than
// kNetMinShare of the joint projection's energy decrease, the next
// kNetSkip solves start from the increment history alone (its inference
// and Gram sums cost a few per cent of a solve), then it is tried again.
constexpr double kNetMinShare = 0.01;
constexpr int kNetSkip = 8;

struct Warm {
    // previous-step tracking (both warm start modes)
    double *uprev;              // u^(n-1), field layout
    double *hist[kHist];        // ring of the last increments (zero halo)
    int nhist;                  // increments in the ring
    int head;                   // slot the next increment goes to
    int cur;                    // slot holding the current step's increment
    double *dnet;               // network direction (field layout, zero halo)
    double *r0;                 // u^n - A u^n (the plain start's residual)
    double *ustart;             // u_h, the history start of the current step
    double *rh;                 // u^n - A u_h
    double *partials;           // [kGramBlocks][kGramSums]
    float *scale;               // device [0] max|u^n|, [1] max|r0|
    bool have_prev;             // u^(n-1) is known
    int ring;                   // history slots in use (the chunk's warm_history)
    int net_skip;               // solves left before the network is consulted again
    std::vector<void *> allocs;
    // the network (learned mode)
    bool model;
    float *params;              // FP32 master copy on the device
    bf16 *wf[kLayers];          // BF16 [9][coutp][cin]
    float *bias[kLayers];
    bf16 *x, *h0, *h1, *pre;    // activations [1][ny+2][nxp+2][C]
    float *y;                   // [ny][nxp] predicted du / max|r0|
    int nxp;
    std::vector<void *> model_allocs;
};

long long layer_floats(int l) { return 9LL * kCin[l] * kCout[l] + kCout[l]; }

__device__ __forceinline__ int64_t cell_of(const Geo &g, long long k, int *i, int *j) {
    *i = (int)(k % g.nx);
    *j = (int)(k / g.nx);
    return (int64_t)(*i + g.h) + (int64_t)(*j + g.h) * g.pitch;
}

// (A v)[c]: the operator of tea_leaf_common.cuknl:28-34 with the stored diagonal
__device__ __forceinline__ double apply_a(const double *__restrict__ v, const double *__restrict__ dg,
                                          const double *__restrict__ kx, const double *__restrict__ ky,
                                          int64_t c, int pitch) {
    const double a = fma(ky[c + pitch], v[c + pitch], ky[c] * v[c - pitch]);
    const double b = fma(kx[c + 1], v[c + 1], kx[c] * v[c - 1]);
    return fma(dg[c], v[c], -a) - b;
}

// out[0] = max |a|, out[1] = max |b| over the interior (b may be null);
// non-negative floats compare as unsigned ints
__global__ void k_absmax2(Geo g, const double *__restrict__ a, const double *__restrict__ b,
                          float *__restrict__ out) {
    float ma = 0.f, mb = 0.f;
    const long long n = (long long)g.nx * g.ny;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        int i, j;
        const int64_t c = cell_of(g, k, &i, &j);
        ma = fmaxf(ma, (float)fabs(a[c]));
        if (b) mb = fmaxf(mb, (float)fabs(b[c]));
    }
    for (int off = 16; off > 0; off >>= 1) {
        ma = fmaxf(ma, __shfl_xor_sync(0xffffffffu, ma, off));
        mb = fmaxf(mb, __shfl_xor_sync(0xffffffffu, mb, off));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(reinterpret_cast<unsigned int *>(out), __float_as_uint(ma));
        atomicMax(reinterpret_cast<unsigned int *>(out + 1), __float_as_uint(mb));
    }
}

// r = u0 - A v on the interior
__global__ void k_resid_of(Geo g, const double *__restrict__ u0, const double *__restrict__ v,
                           const double *__restrict__ dg, const double *__restrict__ kx,
                           const double *__restrict__ ky, double *__restrict__ r) {
    const long long n = (long long)g.nx * g.ny;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        int i, j;
        const int64_t c = cell_of(g, k, &i, &j);
        r[c] = u0[c] - apply_a(v, dg, kx, ky, c, g.pitch);
    }
}

// dprev = u0 - uprev (zero without a previous step); uprev = u0
__global__ void k_prev(Geo g, const double *__restrict__ u0, double *__restrict__ uprev,
                       double *__restrict__ dprev, int have) {
    const long long n = (long long)g.nx * g.ny;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        int i, j;
        const int64_t c = cell_of(g, k, &i, &j);
        const double v = u0[c];
        dprev[c] = have ? v - uprev[c] : 0.0;
        uprev[c] = v;
    }
}

__device__ __forceinline__ float clampf(float v) { return fminf(fmaxf(v, -kClamp), kClamp); }

// network inputs of cell (i, j), as BF16 into the padded NHWC input
// (x != nullptr) and/or as FP32 [ny][nx][kFeatures] with the target
// (u - ubase) / max|rr| (f != nullptr); rr is the residual of ubase
__global__ void k_features(Geo g, const double *__restrict__ u0, const double *__restrict__ u,
                           const double *__restrict__ ubase, const double *__restrict__ rr,
                           const double *__restrict__ dprev,
                           const double *__restrict__ density, const double *__restrict__ kx,
                           const double *__restrict__ ky, const float *__restrict__ scale, double dt,
                           bf16 *__restrict__ x, int nxp, float *__restrict__ f) {
    const long long n = (long long)g.nx * g.ny;
    const double su = fmax((double)scale[0], 1e-300), sr = fmax((double)scale[1], 1e-300);
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        int i, j;
        const int64_t c = cell_of(g, k, &i, &j);
        float v[kInputs];
        v[0] = (float)(u0[c] / su);
        v[1] = logf((float)density[c]);
        v[2] = log1pf((float)kx[c]);
        v[3] = log1pf((float)ky[c]);
        v[4] = (float)(100.0 * dt);
        v[5] = clampf((float)(rr[c] / sr));
        v[6] = clampf((float)(dprev[c] / sr));
        if (x) {
            bf16 *d = x + (((int64_t)(j + 1)) * (nxp + 2) + i + 1) * 16;
            for (int q = 0; q < kInputs; ++q) d[q] = __float2bfloat16(v[q]);
        }
        if (f) {
            float *d = f + k * kFeatures;
            for (int q = 0; q < kInputs; ++q) d[q] = v[q];
            d[kInputs] = (float)((u[c] - ubase[c]) / sr);
        }
    }
}

// dnet = max|r0| * y on the interior (the halo stays zero)
__global__ void k_dnet(Geo g, const float *__restrict__ y, int nxp, const float *__restrict__ scale,
                       double *__restrict__ dnet) {
    const long long n = (long long)g.nx * g.ny;
    const double sr = (double)scale[1];
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        int i, j;
        const int64_t c = cell_of(g, k, &i, &j);
        dnet[c] = sr * (double)y[(int64_t)j * nxp + i];
    }
}

// the search directions of one warm start (null beyond n)
struct Dirs {
    const double *d[kMaxDirs];
    int n;
};

// index of d_i.Ad_j (i <= j) among the Gram sums
__host__ __device__ constexpr int pair_index(int i, int j) { return i * kMaxDirs - i * (i - 1) / 2 + (j - i); }

// Gram entries of the projection, per CTA in a fixed order.  Energy
// (Galerkin): d_i.Ad_j for i <= j, then d_i.r0, then r0.r0.  MR (minimal
// residual): Ad_i.Ad_j, then Ad_i.r0, then r0.r0.
template <bool MR>
__global__ void __launch_bounds__(256) k_gram(Geo g, Dirs D, const double *__restrict__ r0,
                                              const double *__restrict__ dg, const double *__restrict__ kx,
                                              const double *__restrict__ ky, double *__restrict__ partials) {
    double s[kGramSums];
#pragma unroll
    for (int q = 0; q < kGramSums; ++q) s[q] = 0.0;
    const long long n = (long long)g.nx * g.ny;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        int i, j;
        const int64_t c = cell_of(g, k, &i, &j);
        const double r = r0[c];
        double dv[kMaxDirs], av[kMaxDirs];
#pragma unroll
        for (int a = 0; a < kMaxDirs; ++a) {
            dv[a] = av[a] = 0.0;
            if (a < D.n) {
                dv[a] = D.d[a][c];
                av[a] = apply_a(D.d[a], dg, kx, ky, c, g.pitch);
            }
        }
#pragma unroll
        for (int a = 0; a < kMaxDirs; ++a) {
#pragma unroll
            const double la = MR ? av[a] : dv[a];
            for (int b = a; b < kMaxDirs; ++b) s[pair_index(a, b)] = fma(la, av[b], s[pair_index(a, b)]);
            s[kGramPairs + a] = fma(la, r, s[kGramPairs + a]);
        }
        s[kGramSums - 1] = fma(r, r, s[kGramSums - 1]);
    }
    __shared__ double red[8][kGramSums];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < kGramSums; ++q) {
        double v = s[q];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == 0) red[warp][q] = v;
    }
    __syncthreads();
    if (threadIdx.x < kGramSums) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += red[w][threadIdx.x];
        partials[(int64_t)blockIdx.x * kGramSums + threadIdx.x] = t;
    }
}

struct Coefs {
    double c[kMaxDirs];
};

// u = u0 + sum_i c_i d_i on the interior
__global__ void k_combine(Geo g, const double *__restrict__ u0, Dirs D, Coefs C, double *__restrict__ u) {
    const long long n = (long long)g.nx * g.ny;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        int i, j;
        const int64_t c = cell_of(g, k, &i, &j);
        double v = u0[c];
#pragma unroll
        for (int a = 0; a < kMaxDirs; ++a)
            if (a < D.n) v = fma(C.c[a], D.d[a][c], v);
        u[c] = v;
    }
}

Warm *warm_of(Chunk *c) { return (Warm *)c->warm; }

int dmalloc(std::vector<void *> &list, void **p, size_t bytes, cudaStream_t s) {
    cudaError_t e = device_malloc(p, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "warm start cudaMalloc");
    list.push_back(*p);
    e = cudaMemsetAsync(*p, 0, bytes, s);
    return e == cudaSuccess ? TL_OK : cuda_fail(e, "warm start memset");
}

int launched(Chunk *c, const char *what, int n = 1) {
    c->launches += n;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TL_OK : cuda_fail(e, what);
}

void free_model(Warm *w) {
    for (void *p : w->model_allocs) cudaFree(p);
    w->model_allocs.clear();
    w->model = false;
}

// the per-chunk warm start state, created on first use; on failure nothing
// of it is kept
int warm_state_fields(Chunk *c, Warm **out);
int warm_state(Chunk *c, Warm **out) {
    if (c->warm) {
        *out = warm_of(c);
        return TL_OK;
    }
    const int rc = warm_state_fields(c, out);
    if (rc) warm_free(c);
    return rc;
}

int warm_state_fields(Chunk *c, Warm **out) {
    Warm *w = new Warm();
    c->warm = w;
    const size_t bytes = sizeof(double) * c->alloc_elems;
    const int64_t off = c->lead;  // field pointers start `lead` elements into the allocation
    cudaStream_t s = c->stream;
    int rc;
    void *p;
    double **fields[5] = {&w->uprev, &w->dnet, &w->r0, &w->ustart, &w->rh};
    for (double **f : fields) {
        if ((rc = dmalloc(w->allocs, &p, bytes, s))) return rc;
        *f = (double *)p + off;
    }
    for (int k = 0; k < kHist; ++k) {
        if (k >= c->warm_history) {  // slots beyond the chunk's history length stay unallocated
            w->hist[k] = nullptr;
            continue;
        }
        if ((rc = dmalloc(w->allocs, &p, bytes, s))) return rc;
        w->hist[k] = (double *)p + off;
    }
    w->ring = c->warm_history;
    if ((rc = dmalloc(w->allocs, &p, sizeof(double) * kGramBlocks * kGramSums, s))) return rc;
    w->partials = (double *)p;
    if ((rc = dmalloc(w->allocs, &p, 256, s))) return rc;
    w->scale = (float *)p;
    *out = w;
    return TL_OK;
}

// max|u0| and max|r_h| into w->scale
int scales(Chunk *c, Warm *w) {
    TL_CUDA(cudaMemsetAsync(w->scale, 0, 2 * sizeof(float), c->stream));
    k_absmax2<<<kGramBlocks, 256, 0, c->stream>>>(c->g, c->u0, w->rh, w->scale);
    return launched(c, "absmax launch");
}

// dnet = network(features) (with u_h, r_h and the current increment in place)
int net_direction(Chunk *c, Warm *w) {
    cudaStream_t s = c->stream;
    int rc;
    k_features<<<1216, 256, 0, s>>>(c->g, c->u0, c->u, w->ustart, w->rh, w->hist[w->cur], c->density, c->kx,
                                    c->ky, w->scale, c->dt, w->x, w->nxp, nullptr);
    if ((rc = launched(c, "features launch"))) return rc;
    bf16 *h = w->h0, *hn = w->h1;
    if ((rc = tl_nn_conv(0, 16, 32, w->x, w->wf[0], w->bias[0], nullptr, h, w->pre, nullptr, 1, c->ny,
                         w->nxp, s)))
        return rc;
    for (int l = 1; l < 5; ++l) {
        if ((rc = tl_nn_conv(1, 32, 32, h, w->wf[l], w->bias[l], h, hn, w->pre, nullptr, 1, c->ny, w->nxp, s)))
            return rc;
        bf16 *t = h;
        h = hn;
        hn = t;
    }
    if ((rc = tl_nn_conv(2, 32, 16, h, w->wf[5], w->bias[5], nullptr, nullptr, nullptr, w->y, 1, c->ny,
                         w->nxp, s)))
        return rc;
    c->launches += 6;
    k_dnet<<<1216, 256, 0, s>>>(c->g, w->y, w->nxp, w->scale, w->dnet);
    return launched(c, "network direction");
}

// coefficients c minimising phi over u0 + sum_i c_i d_i (n directions)
// from the Gram sums S: Gram-Schmidt in the inner product G_ij = d_i.Ad_j,
// done twice, dropping a direction whose remaining G-norm^2 is below 1e-10
// of its own (numerically dependent on the earlier ones); returns twice the
// energy decrease, 0 when no direction helps
double project(const double *S, int n, double *coef) {
    double G[kMaxDirs][kMaxDirs], bv[kMaxDirs], Q[kMaxDirs][kMaxDirs];
    for (int i = 0; i < n; ++i) {
        coef[i] = 0.0;
        bv[i] = S[kGramPairs + i];
        for (int j = i; j < n; ++j) G[i][j] = G[j][i] = S[pair_index(i, j)];
    }
    auto ip = [&](const double *x, const double *y) {
        double t = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) t += x[i] * G[i][j] * y[j];
        return t;
    };
    int m = 0;
    for (int i = 0; i < n; ++i) {
        if (!(G[i][i] > 0.0) || !isfinite(G[i][i]) || !isfinite(bv[i])) continue;
        double v[kMaxDirs] = {};
        v[i] = 1.0;
        for (int pass = 0; pass < 2; ++pass)
            for (int q = 0; q < m; ++q) {
                const double h = ip(Q[q], v);
                for (int k = 0; k < n; ++k) v[k] -= h * Q[q][k];
            }
        const double nrm2 = ip(v, v);
        if (!(nrm2 > 1e-10 * G[i][i]) || !isfinite(nrm2)) continue;
        const double inv = 1.0 / sqrt(nrm2);
        for (int k = 0; k < n; ++k) Q[m][k] = v[k] * inv;
        ++m;
    }
    double gain = 0.0;
    for (int q = 0; q < m; ++q) {
        double t = 0.0;
        for (int k = 0; k < n; ++k) t += Q[q][k] * bv[k];
        gain += t * t;
        for (int k = 0; k < n; ++k) coef[k] += t * Q[q][k];
    }
    if (!isfinite(gain)) {
        for (int k = 0; k < n; ++k) coef[k] = 0.0;
        return 0.0;
    }
    return gain;
}

// Gram sums of the directions D (k_gram, partials summed on the host in CTA
// order) and their projection: coefficients into *C, twice the energy
// decrease into *gain (0 when D is empty or nothing helps)
int gram_project(Chunk *c, Warm *w, const Dirs &D, Coefs *C, double *gain) {
    for (int a = 0; a < kMaxDirs; ++a) C->c[a] = 0.0;
    *gain = 0.0;
    if (D.n == 0) return TL_OK;
    cudaStream_t s = c->stream;
    int rc;
    if (c->warm_projection == TL_WARM_PROJ_RESIDUAL)
        k_gram<true><<<kGramBlocks, 256, 0, s>>>(c->g, D, w->r0, c->diag, c->kx, c->ky, w->partials);
    else
        k_gram<false><<<kGramBlocks, 256, 0, s>>>(c->g, D, w->r0, c->diag, c->kx, c->ky, w->partials);
    if ((rc = launched(c, "gram launch"))) return rc;
    std::vector<double> part((size_t)kGramBlocks * kGramSums);
    TL_CUDA(cudaMemcpyAsync(part.data(), w->partials, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, s));
    TL_CUDA(cudaStreamSynchronize(s));
    double S[kGramSums];
    for (int q = 0; q < kGramSums; ++q) S[q] = 0.0;
    for (int b = 0; b < kGramBlocks; ++b)
        for (int q = 0; q < kGramSums; ++q) S[q] += part[(size_t)b * kGramSums + q];
    *gain = project(S, D.n, C->c);
    return TL_OK;
}

}  // namespace

void warm_free(Chunk *c) {
    Warm *w = warm_of(c);
    if (!w) return;
    free_model(w);
    for (void *p : w->allocs) cudaFree(p);
    delete w;
    c->warm = nullptr;
}

int warm_set_options(Chunk *c, int history, int projection) {
    if (history < 1 || history > kHist ||
        (projection != TL_WARM_PROJ_ENERGY && projection != TL_WARM_PROJ_RESIDUAL)) {
        set_error("tl_set_warm_start_options: history %d (1..%d), projection %d", history, kHist, projection);
        return TL_ERR_ARG;
    }
    c->warm_history = history;
    c->warm_projection = projection;
    Warm *w = warm_of(c);
    if (!w) return TL_OK;  // the state is made with these options on first use
    for (int k = 0; k < history; ++k)
        if (!w->hist[k]) {
            void *p;
            int rc = dmalloc(w->allocs, &p, sizeof(double) * c->alloc_elems, c->stream);
            if (rc) return rc;
            w->hist[k] = (double *)p + c->lead;
        }
    w->ring = history;
    w->nhist = w->head = w->cur = 0;  // restart the history (u^(n-1) stays known)
    return TL_OK;
}

void warm_reset(Chunk *c) {
    if (Warm *w = warm_of(c)) {
        w->have_prev = false;
        w->net_skip = 0;
        w->nhist = w->head = w->cur = 0;
    }
}

long long warm_param_count() {
    long long n = 0;
    for (int l = 0; l < kLayers; ++l) n += layer_floats(l);
    return n;
}

int warm_set_model(Chunk *c, const float *params, long long n) {
    if (n != warm_param_count()) {
        set_error("warm start model: %lld parameters, expected %lld", n, warm_param_count());
        return TL_ERR_ARG;
    }
    Warm *w;
    int rc;
    if ((rc = warm_state(c, &w))) return rc;
    free_model(w);
    cudaStream_t s = c->stream;
    void *p;
    auto &L = w->model_allocs;
    if ((rc = dmalloc(L, &p, sizeof(float) * n, s))) return rc;
    w->params = (float *)p;
    TL_CUDA(cudaMemcpyAsync(w->params, params, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    long long off = 0;
    for (int l = 0; l < kLayers; ++l) {
        if ((rc = dmalloc(L, &p, sizeof(bf16) * 9 * kCin[l] * kCout[l], s))) return rc;
        w->wf[l] = (bf16 *)p;
        if ((rc = tl_nn_pack(w->params + off, w->wf[l], nullptr, kCin[l], kCout[l], s))) return rc;
        w->bias[l] = w->params + off + 9LL * kCin[l] * kCout[l];
        off += layer_floats(l);
    }
    w->nxp = (c->nx + 15) / 16 * 16;
    const size_t px = (size_t)(c->ny + 2) * (w->nxp + 2);
    if ((rc = dmalloc(L, &p, sizeof(bf16) * px * 16, s))) return rc;
    w->x = (bf16 *)p;
    bf16 **acts[3] = {&w->h0, &w->h1, &w->pre};
    for (bf16 **a : acts) {
        if ((rc = dmalloc(L, &p, sizeof(bf16) * px * 32, s))) return rc;
        *a = (bf16 *)p;
    }
    if ((rc = dmalloc(L, &p, sizeof(float) * (size_t)c->ny * w->nxp, s))) return rc;
    w->y = (float *)p;
    TL_CUDA(cudaStreamSynchronize(s));
    w->model = true;
    return TL_OK;
}

bool warm_ready(Chunk *c) { return warm_of(c) != nullptr && warm_of(c)->model; }

int warm_start_or_fallback(Chunk *c, tl_solve_info_t *info, double *r0, double *rr) {
    const bool learned = c->cfg.warm_start == TL_WARM_LEARNED;
    Warm *w;
    int rc;
    if ((rc = warm_state(c, &w))) return rc;
    if (learned && !w->model) {
        set_error("warm start requested but no model is loaded (tl_set_warm_start_model)");
        return TL_ERR_STATE;
    }
    info->warm_used = 0;
    info->warm_ratio = 1.0;
    info->warm_net_share = 0.0;
    cudaStream_t s = c->stream;
    // the plain start u = u^n: r = u^n - A u^n, its norm defines the exit test
    if ((rc = launch_residual(c, kEpiStore))) return rc;
    if ((rc = launch_copy(c, w->r0, c->r, false))) return rc;
    const bool have_prev = w->have_prev;
    // the increment of this step, u^n - u^(n-1), into the history ring
    w->cur = w->head;
    k_prev<<<1216, 256, 0, s>>>(c->g, c->u0, w->uprev, w->hist[w->cur], have_prev ? 1 : 0);
    if ((rc = launched(c, "previous step launch"))) return rc;
    if (have_prev) {
        w->nhist = w->nhist < w->ring ? w->nhist + 1 : w->ring;
        w->head = (w->head + 1) % w->ring;
    }
    w->have_prev = true;
    // the history start u_h: the increments' projection alone
    Dirs H;
    H.n = 0;
    for (int a = 0; a < kMaxDirs; ++a) H.d[a] = nullptr;
    for (int j = 0; j < w->nhist; ++j) H.d[H.n++] = w->hist[(w->cur - j + w->ring) % w->ring];
    Coefs CH;
    double gh = 0.0;
    if ((rc = gram_project(c, w, H, &CH, &gh))) return rc;
    if (gh > 0.0) k_combine<<<1216, 256, 0, s>>>(c->g, c->u0, H, CH, w->ustart);
    else k_combine<<<1216, 256, 0, s>>>(c->g, c->u0, Dirs{{nullptr}, 0}, CH, w->ustart);
    if ((rc = launched(c, "history start"))) return rc;
    Dirs D = H;
    Coefs C = CH;
    double gain = gh;
    const bool consult = learned && w->net_skip == 0;
    if (learned && !consult) w->net_skip--;
    if (consult) {
        // the network corrects u_h: input r_h = u^n - A u_h; then the joint
        // projection over its direction and the increments
        k_resid_of<<<1216, 256, 0, s>>>(c->g, c->u0, w->ustart, c->diag, c->kx, c->ky, w->rh);
        if ((rc = launched(c, "history residual"))) return rc;
        if ((rc = scales(c, w))) return rc;
        if ((rc = net_direction(c, w))) return rc;
        D.n = 0;
        D.d[D.n++] = w->dnet;
        for (int j = 0; j < w->nhist; ++j) D.d[D.n++] = w->hist[(w->cur - j + w->ring) % w->ring];
        if ((rc = gram_project(c, w, D, &C, &gain))) return rc;
        info->warm_net_share = gain > 0.0 && gain >= gh ? (gain - gh) / gain : 0.0;
        if (!(info->warm_net_share > kNetMinShare)) w->net_skip = kNetSkip;
        if (!(gain >= gh)) {
            // the network's direction is unusable (not finite, e.g. a model
            // of NaNs) or adds nothing: fall back to the history start
            D = H;
            C = CH;
            gain = gh;
        }
    }
    if ((rc = chunk_sync_scalars(c))) return rc;
    const double rr0 = c->sc_host->sum[0];
    *r0 = sqrt(fabs(rr0));
    *rr = rr0;
    if (!(gain > 0.0)) return TL_OK;  // the plain start: u = u^n, r = r0
    k_combine<<<1216, 256, 0, s>>>(c->g, c->u0, D, C, c->u);
    if ((rc = launched(c, "warm start combine"))) return rc;
    if ((rc = launch_residual(c, kEpiStore))) return rc;
    if ((rc = chunk_sync_scalars(c))) return rc;
    const double rrw = c->sc_host->sum[0];
    info->warm_used = 1;
    info->warm_ratio = sqrt(fabs(rrw)) / (*r0 > 0.0 ? *r0 : 1.0);
    *rr = rrw;
    return TL_OK;
}

// FP32 [ny][nx][8] network inputs + target of the solved step into dst
// (device); needs the previous-step tracking of a warm-started solve
int warm_features(Chunk *c, float *dst) {
    Warm *w = warm_of(c);
    if (!w || !w->have_prev) {
        set_error("tl_warm_start_features: solve the step with tl_warm_start prev or learned first");
        return TL_ERR_STATE;
    }
    cudaStream_t s = c->stream;
    int rc;
    // the history start of this step and its residual: the network learns
    // the correction of u_h
    k_resid_of<<<1216, 256, 0, s>>>(c->g, c->u0, w->ustart, c->diag, c->kx, c->ky, w->rh);
    if ((rc = launched(c, "residual launch"))) return rc;
    if ((rc = scales(c, w))) return rc;
    k_features<<<1216, 256, 0, s>>>(c->g, c->u0, c->u, w->ustart, w->rh, w->hist[w->cur], c->density, c->kx,
                                    c->ky, w->scale, c->dt, nullptr, 0, dst);
    if ((rc = launched(c, "features launch"))) return rc;
    TL_CUDA(cudaStreamSynchronize(s));
    return TL_OK;
}

}  // namespace tl

extern "C" long long tl_warm_start_param_count(void) { return tl::warm_param_count(); }

// tl_warm.cu -- the learned warm start inside the solve (no reference
// counterpart): features of the current step, the residual network's
// forward pass on the tensor-core kernels of tl_conv.cu, and u = u^n + du.
// The solve compares the residual of this start with that of the plain
// start u = u^n and keeps the better one (the fallback); its exit test stays
// tl_eps times the plain start's residual.
//
// Model parameters (FP32, flat, in this order per layer: W [9][coutp][cin]
// then b [coutp]):
//   layer 1: cin 16 (inputs 0..4 used), coutp 32, GELU
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

struct Warm {
    float *params;              // FP32 master copy on the device
    bf16 *wf[kLayers];          // BF16 [9][coutp][cin]
    float *bias[kLayers];
    bf16 *x, *h0, *h1, *pre;    // activations [1][ny+2][nxp+2][C]
    float *y;                   // [ny][nxp] predicted du / s
    float *scale;               // device max |u0|
    int nxp;
    std::vector<void *> allocs;
};

long long layer_floats(int l) { return 9LL * kCin[l] * kCout[l] + kCout[l]; }

// max |u0| over the interior (non-negative floats compare as unsigned ints)
__global__ void k_absmax(Geo g, const double *__restrict__ u0, float *__restrict__ out) {
    float m = 0.f;
    const long long n = (long long)g.nx * g.ny;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k % g.nx), j = (int)(k / g.nx);
        m = fmaxf(m, (float)fabs(u0[(int64_t)(i + g.h) + (int64_t)(j + g.h) * g.pitch]));
    }
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned int *>(out), __float_as_uint(m));
}

// features of cell (i, j): u0 / s, log density, log1p(Kx west face),
// log1p(Ky south face), 100 dt; written as BF16 into the padded NHWC input
// (x != nullptr) and/or as FP32 [ny][nx][6] with the target (u - u0) / s
// (f != nullptr)
__global__ void k_features(Geo g, const double *__restrict__ u0, const double *__restrict__ u,
                           const double *__restrict__ density, const double *__restrict__ kx,
                           const double *__restrict__ ky, const float *__restrict__ scale, double dt,
                           bf16 *__restrict__ x, int nxp, float *__restrict__ f) {
    const long long n = (long long)g.nx * g.ny;
    const float s = fmaxf(*scale, 1e-30f);
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k % g.nx), j = (int)(k / g.nx);
        const int64_t c = (int64_t)(i + g.h) + (int64_t)(j + g.h) * g.pitch;
        float v[5];
        v[0] = (float)(u0[c] / s);
        v[1] = logf((float)density[c]);
        v[2] = log1pf((float)kx[c]);
        v[3] = log1pf((float)ky[c]);
        v[4] = (float)(100.0 * dt);
        if (x) {
            bf16 *d = x + (((int64_t)(j + 1)) * (nxp + 2) + i + 1) * 16;
            for (int q = 0; q < 5; ++q) d[q] = __float2bfloat16(v[q]);
        }
        if (f) {
            float *d = f + k * 6;
            for (int q = 0; q < 5; ++q) d[q] = v[q];
            d[5] = (float)((u[c] - u0[c]) / s);
        }
    }
}

// u = u0 + s * du on the interior
__global__ void k_apply(Geo g, const double *__restrict__ u0, double *__restrict__ u, const float *__restrict__ du,
                        int nxp, const float *__restrict__ scale) {
    const long long n = (long long)g.nx * g.ny;
    const double s = (double)fmaxf(*scale, 1e-30f);
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k % g.nx), j = (int)(k / g.nx);
        const int64_t c = (int64_t)(i + g.h) + (int64_t)(j + g.h) * g.pitch;
        u[c] = u0[c] + s * (double)du[(int64_t)j * nxp + i];
    }
}

Warm *warm_of(Chunk *c) { return (Warm *)c->warm; }

int dmalloc(Warm *w, void **p, size_t bytes, cudaStream_t s) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "warm start cudaMalloc");
    w->allocs.push_back(*p);
    e = cudaMemsetAsync(*p, 0, bytes, s);
    return e == cudaSuccess ? TL_OK : cuda_fail(e, "warm start memset");
}

}  // namespace

void warm_free(Chunk *c) {
    Warm *w = warm_of(c);
    if (!w) return;
    for (void *p : w->allocs) cudaFree(p);
    delete w;
    c->warm = nullptr;
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
    warm_free(c);
    Warm *w = new Warm();
    c->warm = w;
    cudaStream_t s = c->stream;
    int rc;
    void *p;
    if ((rc = dmalloc(w, &p, sizeof(float) * n, s))) return rc;
    w->params = (float *)p;
    TL_CUDA(cudaMemcpyAsync(w->params, params, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    long long off = 0;
    for (int l = 0; l < kLayers; ++l) {
        if ((rc = dmalloc(w, &p, sizeof(bf16) * 9 * kCin[l] * kCout[l], s))) return rc;
        w->wf[l] = (bf16 *)p;
        if ((rc = tl_nn_pack(w->params + off, w->wf[l], nullptr, kCin[l], kCout[l], s))) return rc;
        w->bias[l] = w->params + off + 9LL * kCin[l] * kCout[l];
        off += layer_floats(l);
    }
    w->nxp = (c->nx + 15) / 16 * 16;
    const size_t px = (size_t)(c->ny + 2) * (w->nxp + 2);
    if ((rc = dmalloc(w, &p, sizeof(bf16) * px * 16, s))) return rc;
    w->x = (bf16 *)p;
    if ((rc = dmalloc(w, &p, sizeof(bf16) * px * 32, s))) return rc;
    w->h0 = (bf16 *)p;
    if ((rc = dmalloc(w, &p, sizeof(bf16) * px * 32, s))) return rc;
    w->h1 = (bf16 *)p;
    if ((rc = dmalloc(w, &p, sizeof(bf16) * px * 32, s))) return rc;
    w->pre = (bf16 *)p;
    if ((rc = dmalloc(w, &p, sizeof(float) * (size_t)c->ny * w->nxp, s))) return rc;
    w->y = (float *)p;
    if ((rc = dmalloc(w, &p, 256, s))) return rc;
    w->scale = (float *)p;
    TL_CUDA(cudaStreamSynchronize(s));
    return TL_OK;
}

bool warm_ready(Chunk *c) { return warm_of(c) != nullptr; }

int warm_scale(Chunk *c, float *scale_dev) {
    TL_CUDA(cudaMemsetAsync(scale_dev, 0, sizeof(float), c->stream));
    k_absmax<<<608, 256, 0, c->stream>>>(c->g, c->u0, scale_dev);
    c->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TL_OK : cuda_fail(e, "absmax launch");
}

// u = u0 + network(features): call after common_init (u0, Kx, Ky current)
int warm_apply(Chunk *c) {
    Warm *w = warm_of(c);
    if (!w) {
        set_error("warm start requested but no model is loaded (tl_set_warm_start_model)");
        return TL_ERR_STATE;
    }
    cudaStream_t s = c->stream;
    int rc;
    if ((rc = warm_scale(c, w->scale))) return rc;
    k_features<<<1216, 256, 0, s>>>(c->g, c->u0, c->u, c->density, c->kx, c->ky, w->scale, c->dt, w->x,
                                    w->nxp, nullptr);
    c->launches++;
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
    k_apply<<<1216, 256, 0, s>>>(c->g, c->u0, c->u, w->y, w->nxp, w->scale);
    c->launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TL_OK : cuda_fail(e, "warm start apply");
}

int warm_start_or_fallback(Chunk *c, tl_solve_info_t *info, double *r0, double *rr) {
    int rc;
    // the plain start u = u^n: its residual defines the exit test
    if ((rc = launch_residual(c, kEpiStore))) return rc;
    if ((rc = chunk_sync_scalars(c))) return rc;
    const double rr0 = c->sc_host->sum[0];
    *r0 = sqrt(fabs(rr0));
    *rr = rr0;
    info->warm_used = 0;
    info->warm_ratio = 1.0;
    if ((rc = warm_apply(c))) return rc;
    if ((rc = launch_residual(c, kEpiStore))) return rc;
    if ((rc = chunk_sync_scalars(c))) return rc;
    const double rrw = c->sc_host->sum[0];
    info->warm_ratio = sqrt(fabs(rrw)) / (*r0 > 0.0 ? *r0 : 1.0);
    if (isfinite(rrw) && rrw < rr0) {
        info->warm_used = 1;
        *rr = rrw;
        return TL_OK;
    }
    // fallback to the plain start
    if ((rc = launch_copy(c, c->u, c->u0, false))) return rc;
    return launch_residual(c, kEpiNone);
}

// FP32 [ny][nx][6] features + target of the solved step into dst (device)
int warm_features(Chunk *c, float *dst) {
    float *scale = nullptr;
    TL_CUDA(cudaMallocAsync((void **)&scale, 256, c->stream));
    int rc = warm_scale(c, scale);
    if (rc == TL_OK) {
        k_features<<<1216, 256, 0, c->stream>>>(c->g, c->u0, c->u, c->density, c->kx, c->ky, scale, c->dt,
                                                nullptr, 0, dst);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda_fail(e, "features launch");
    }
    cudaFreeAsync(scale, c->stream);
    TL_CUDA(cudaStreamSynchronize(c->stream));
    return rc;
}

}  // namespace tl

extern "C" long long tl_warm_start_param_count(void) { return tl::warm_param_count(); }

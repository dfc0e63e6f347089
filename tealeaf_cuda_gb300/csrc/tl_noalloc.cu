// tl_noalloc.cu -- tl_dot_noalloc: the dot-product reduction of
// tea_leaf_calc_2norm (sum of a*b over an interior) for callers that cannot
// let this library allocate device memory.
//
// Who cannot allocate: a host that sets up its whole device-memory budget
// once (as the reference's TealeafCudaChunk does in initBuffers) and then
// runs under a fixed cap, so a cudaMalloc in the middle of a run could fail
// or fragment that budget; a host whose device memory belongs to another
// allocator (a framework's caching allocator) that must stay the only owner;
// and any host that cannot afford the device-wide synchronisation cudaMalloc
// and cudaFree imply.  Such a caller passes its own device arrays and a device
// output slot; the reduction's scratch (the per-CTA partial sums and the
// last-CTA ticket) lives in the fixed array below instead of the chunk's
// cudaMalloc'd buffers.
//
// The scratch is a file-scope __device__ array: every GPU that loads this
// library holds its kNoallocScratchBytes until the process exits.  All calls
// on a device share it and it keeps the last call's contents, so each call
// clears the ticket counter first, and calls that overlap on the GPU (two
// streams, or two host threads) race on it: the caller must order them.
// The array's device address is looked up on the first call on each device
// and kept for the life of the process, so a device must not be reset
// (cudaDeviceReset) while this library is loaded: after a reset the module
// reloads and the array may move.
#include <stdint.h>

#include "tl_internal.cuh"

namespace tl {
namespace {

// 1 MiB: a 256-byte header (the ticket counter) and one partial sum per
// 32 x 32 tile, i.e. up to 131040 tiles = 134 million cells (11584^2).
constexpr size_t kNoallocScratchBytes = 1u << 20;
constexpr size_t kNoallocHeader = 256;
constexpr int kNoallocMaxTiles = (int)((kNoallocScratchBytes - kNoallocHeader) / sizeof(double));
constexpr int kTileCols = 32, kTileRows = 32;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// device address of g_noalloc_scratch per device, looked up once per device
static void *g_scratch_addr[kMaxDevices];

// One CTA per 32x32 tile; 8 warps, a lane owns one column of four rows.  The
// tile's partial goes to scratch, and the last CTA to take a ticket sums the
// partials in tile order and writes *result.  No CTA waits for another.
__global__ void __launch_bounds__(256) k_dot_noalloc(const double *__restrict__ a,
                                                      const double *__restrict__ b, int nx, int ny,
                                                      long long pitch, int tiles_x, int tiles,
                                                      unsigned char *scratch,
                                                      double *__restrict__ result) {
    unsigned int *ticket = (unsigned int *)scratch;
    double *partials = (double *)(scratch + kNoallocHeader);
    __shared__ double sh[8];
    __shared__ int is_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int t = blockIdx.x;
    const int i = (t % tiles_x) * kTileCols + lane;
    const int j0 = (t / tiles_x) * kTileRows + warp * 4;
    double acc = 0.0;
    if (i < nx) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int j = j0 + k;
            if (j < ny) {
                const int64_t idx = (int64_t)i + (int64_t)j * pitch;
                acc = fma(a[idx], b[idx], acc);
            }
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (lane == 0) sh[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < 8; ++w) s += sh[w];
        partials[t] = s;
        __threadfence();
        is_last = atomicAdd(ticket, 1u) == (unsigned int)(tiles - 1);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double s = 0.0;
    for (int k = threadIdx.x; k < tiles; k += blockDim.x) s += __ldcg(&partials[k]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    __syncthreads();
    if (lane == 0) sh[warp] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < 8; ++w) tot += sh[w];
        *result = tot;
        *ticket = 0u;
    }
}

}  // namespace
}  // namespace tl

using namespace tl;

extern "C" int tl_dot_noalloc(const double *a, const double *b, int nx, int ny, long long pitch,
                              double *result, void *stream) {
    if (!a || !b || !result || nx < 1 || ny < 1 || pitch < nx) {
        set_error("tl_dot_noalloc: bad arguments (nx=%d ny=%d pitch=%lld)", nx, ny, pitch);
        return TL_ERR_ARG;
    }
    // widened before the sums: nx, ny near INT_MAX must not overflow
    const long long tiles_x = ((long long)nx + kTileCols - 1) / kTileCols;
    const long long tiles = tiles_x * (((long long)ny + kTileRows - 1) / kTileRows);
    if (tiles <= 0 || tiles > kNoallocMaxTiles) {
        set_error("tl_dot_noalloc: %d x %d cells need %lld scratch tiles; the fixed scratch holds "
                  "%d (at most %d cells)", nx, ny, tiles, kNoallocMaxTiles,
                  kNoallocMaxTiles * kTileCols * kTileRows);
        return TL_ERR_ARG;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "tl_dot_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("tl_dot_noalloc: device %d out of range", dev);
        return TL_ERR_ARG;
    }
    // first call on this device (made current by the caller): find the
    // scratch array's device address
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "tl_dot_noalloc: cudaGetSymbolAddress");
        g_scratch_addr[dev] = p;
    }
    unsigned char *scratch = (unsigned char *)g_scratch_addr[dev];
    cudaStream_t s = (cudaStream_t)stream;
    // the ticket must start at zero; the array keeps the last call's contents
    e = cudaMemsetAsync(scratch, 0, kNoallocHeader, s);
    if (e != cudaSuccess) return cuda_fail(e, "tl_dot_noalloc: clearing the ticket");
    k_dot_noalloc<<<(unsigned int)tiles, 256, 0, s>>>(a, b, nx, ny, pitch, (int)tiles_x, (int)tiles,
                                                      scratch, result);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "tl_dot_noalloc: launch");
    return TL_OK;
}

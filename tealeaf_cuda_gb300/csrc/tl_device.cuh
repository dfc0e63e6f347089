// tl_device.cuh -- device helpers shared by the FP64 kernels (tl_kernels.cu)
// and the mixed-precision ones (tl_mixed.cu).
#pragma once

#include <stdint.h>

namespace tl {

// block-Jacobi strip solve z = M^-1 x (tea_block_jacobi.cuknl:11-46)
__device__ __forceinline__ void strip_block_solve(const double *__restrict__ dg,
                                                  const double *__restrict__ ky,
                                                  const double *__restrict__ cp,
                                                  const double *__restrict__ bfp, int pitch,
                                                  int64_t base, int m, const double (&x)[4],
                                                  double (&z)[4]) {
    double dp[4];
    dp[0] = x[0] / dg[base];
#pragma unroll
    for (int k = 1; k < 4; ++k)
        if (k < m) {
            const int64_t i = base + (int64_t)k * pitch;
            dp[k] = fma(ky[i], dp[k - 1], x[k]) * bfp[i];
        }
#pragma unroll
    for (int k = 3; k >= 0; --k) {
        if (k == m - 1) {
            z[k] = dp[k];
        } else if (k < m - 1) {
            const int64_t i = base + (int64_t)k * pitch;
            z[k] = fma(-cp[i], z[k + 1], dp[k]);
        }
    }
}

}  // namespace tl

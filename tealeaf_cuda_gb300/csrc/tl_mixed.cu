// tl_mixed.cu -- mixed-precision solve: FP32 inner Krylov iterations inside
// an FP64 iterative-refinement loop.
#include "tl_internal.cuh"

namespace tl {

int solve_timestep_mixed(Chunk *c, tl_solve_info_t *info) {
    (void)c;
    (void)info;
    set_error("tl_precision mixed is not available in this build");
    return TL_ERR_ARG;
}

void mixed_free(Chunk *c) { (void)c; }

}  // namespace tl

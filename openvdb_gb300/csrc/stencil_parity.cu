// Parity-mode stencil kernels.  Built with -fmad=false in addition to the
// explicit round-to-nearest intrinsics of ParityArith, so that every FP32
// and FP64 operation is rounded exactly where the reference rounds it.
#include "stencil.h"
#include "stencil_ops.cuh"

namespace gbls {

void launch_rk_parity(const RkArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    rk_stage_kernel<ParityArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

void launch_norm_parity(const NormArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    normalize_kernel<ParityArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

}  // namespace gbls

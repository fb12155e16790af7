// PARITY-mode stencil kernels on the FP32 pipes (ExactArith): the same bits
// as the FP64 kernels of stencil_parity.cu, which stay available as
// GBLS_PARITY_FP64=1 for cross-checking.  Built with -fmad=false like the
// FP64 unit.
#include "stencil.h"
#include "filter_ops.cuh"
#include "morph_ops.cuh"
#include "stencil_ops.cuh"

namespace gbls {

void launch_rk_exact(const RkArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    rk_stage_kernel<ExactArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

void launch_norm_exact(const NormArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    normalize_kernel<ExactArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

void launch_morph_stage_exact(const MorphArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    morph_stage_kernel<ExactArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

void launch_filter_exact(const FilterArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    if (a.op >= FILTER_MEAN_CURVATURE)
        filter_full_kernel<ExactArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
    else
        filter_kernel<ExactArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

}  // namespace gbls

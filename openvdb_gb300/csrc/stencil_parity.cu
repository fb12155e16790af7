// Parity-mode stencil kernels.  Built with -fmad=false in addition to the
// explicit round-to-nearest intrinsics of ParityArith, so that every FP32
// and FP64 operation is rounded exactly where the reference rounds it.
#include "stencil.h"
#include "filter_ops.cuh"
#include "morph_ops.cuh"
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

void launch_morph_speed_parity(const MorphSpeedArgs& a, unsigned int* max_bits, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    morph_speed_kernel<ParityArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
    morph_reduce_kernel<<<1, 1024, 0, s>>>(a.part, a.nleaf, max_bits);
}

void launch_morph_stage_parity(const MorphArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    morph_stage_kernel<ParityArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

void launch_filter_parity(const FilterArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    if (a.op >= FILTER_MEAN_CURVATURE)
        filter_full_kernel<ParityArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
    else
        filter_kernel<ParityArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

}  // namespace gbls

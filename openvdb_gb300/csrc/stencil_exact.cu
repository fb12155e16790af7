// PARITY-mode stencil kernels on the FP32 pipes (ExactArith): the same bits
// as the FP64 kernels of stencil_parity.cu, which stay available as
// GBLS_PARITY_FP64=1 for cross-checking.  Built with -fmad=false like the
// FP64 unit.
#include "stencil.h"
#include "filter_ops.cuh"
#include "morph_ops.cuh"
#include "stencil_ops.cuh"

namespace gbls {

// min_ctas: the register budget as the minimum resident CTAs per SM given to
// the compiler (0: none, its own heuristic; 1: registers unconstrained; 14 or
// 16: at most 72 or 64 registers per thread).
void launch_rk_exact(const RkArgs& a, cudaStream_t s, int min_ctas) {
    if (a.nleaf <= 0) return;
    const unsigned g = unsigned(a.nleaf * (a.parts > 1 ? a.parts : 1));
    if (min_ctas == 16) rk_stage_kernel<ExactArith, 16><<<g, STENCIL_THREADS, 0, s>>>(a);
    else if (min_ctas == 14) rk_stage_kernel<ExactArith, 14><<<g, STENCIL_THREADS, 0, s>>>(a);
    else if (min_ctas == 1) rk_stage_kernel<ExactArith, 1><<<g, STENCIL_THREADS, 0, s>>>(a);
    else rk_stage_kernel<ExactArith><<<g, STENCIL_THREADS, 0, s>>>(a);
}

void launch_norm_exact(const NormArgs& a, cudaStream_t s, int min_ctas) {
    if (a.nleaf <= 0) return;
    const unsigned g = unsigned(a.nleaf);
    if (min_ctas == 16) normalize_kernel<ExactArith, 16><<<g, STENCIL_THREADS, 0, s>>>(a);
    else if (min_ctas == 14) normalize_kernel<ExactArith, 14><<<g, STENCIL_THREADS, 0, s>>>(a);
    else if (min_ctas == 1) normalize_kernel<ExactArith, 1><<<g, STENCIL_THREADS, 0, s>>>(a);
    else normalize_kernel<ExactArith><<<g, STENCIL_THREADS, 0, s>>>(a);
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

// The PARITY kernels' WENO5 on n operand quintuples v[5i..5i+4]: the
// double-word evaluation, FP64 where it leaves the rounding undecided.
__global__ void weno5_exact_kernel(const float* __restrict__ v, int64_t n, float* __restrict__ out,
                                   uint8_t* __restrict__ decided) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* q = v + 5 * i;
    float r;
    const bool ok = xw::weno5<float>(q[0], q[1], q[2], q[3], q[4], r) != 0u;
    out[i] = ok ? r : weno5_fp64(q[0], q[1], q[2], q[3], q[4]);
    if (decided) decided[i] = ok ? 1 : 0;
}

void launch_weno5_exact(const float* v, int64_t n, float* out, uint8_t* decided, cudaStream_t s) {
    if (n <= 0) return;
    weno5_exact_kernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(v, n, out, decided);
}

}  // namespace gbls

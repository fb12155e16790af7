// FP32 stencil kernels and the CFL reduction.
#include "stencil.h"
#include "stencil_ops.cuh"

namespace gbls {

void launch_rk_fast(const RkArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    rk_stage_kernel<FastArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

void launch_norm_fast(const NormArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    normalize_kernel<FastArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

// One CTA per leaf; Vec3f::lengthSqr (math/Vec3.h:212-218) is evaluated with
// non-contracting intrinsics so the maximum equals the reference's exactly.
__global__ void __launch_bounds__(128) cfl_max_kernel(const CflArgs a) {
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    const int s = a.slot[l];
    int ox, oy, oz;
    key_origin(a.keys[l], ox, oy, oz);
    float m = 0.0f;
    for (int v = threadIdx.x; v < LEAF_VOX; v += blockDim.x) {
        const uint64_t w = a.amask[size_t(s) * 8 + (v >> 6)];
        if (!((w >> (v & 63)) & 1)) continue;
        float vel[3];
        eval_field(a.field, ox + (v >> 6), oy + ((v >> 3) & 7), oz + (v & 7), a.t0, vel);
        const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(vel[0], vel[0]), __fmul_rn(vel[1], vel[1])),
                                   __fmul_rn(vel[2], vel[2]));
        m = ref_max(m, l2);
    }
    for (int o = 16; o > 0; o >>= 1) m = ref_max(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float wm[4];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float r = wm[0];
        for (int k = 1; k < int(blockDim.x >> 5); ++k) r = ref_max(r, wm[k]);
        atomicMax(a.max_bits, __float_as_uint(r));
    }
}

void launch_cfl(const CflArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    cfl_max_kernel<<<unsigned(a.nleaf), 128, 0, s>>>(a);
}

}  // namespace gbls

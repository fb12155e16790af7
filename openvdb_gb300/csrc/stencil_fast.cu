// FP32 stencil kernels and the CFL reduction.
#include "stencil.h"
#include "stencil_ops.cuh"
#include "stencil_fast2.cuh"

namespace gbls {

void launch_rk_fast(const RkArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    rk_stage_kernel_x2<<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

void launch_norm_fast(const NormArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    if (!a.copy_only && !a.has_phi)
        normalize_kernel_x2<<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
    else
        normalize_kernel<FastArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

// One CTA per leaf, thread t visits bit t of each active-mask word;
// Vec3f::lengthSqr (math/Vec3.h:212-218) is evaluated with non-contracting
// intrinsics so the maximum equals the reference's exactly.
__global__ void __launch_bounds__(64) cfl_max_kernel(const __grid_constant__ CflArgs a) {
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    const int s = a.slot[l];
    const int t = threadIdx.x;
    const uint64_t key = a.keys[l];
    uint32_t inst = 0;
    const FieldParams* fp = &a.field;
    float t0 = a.t0;
    if (a.inst_run) {
        inst = key_instance(key);
        if (!a.inst_run[inst]) return;
        fp = a.inst_field + inst;
        t0 = a.inst_t0[inst];
    }
    int ox, oy, oz;
    key_origin(key, ox, oy, oz);
    float m = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint64_t w = a.amask[size_t(s) * 8 + k];
        if (!((w >> t) & 1)) continue;
        float vel[3];
        eval_field(*fp, ox + k, oy + (t >> 3), oz + (t & 7), t0, vel);
        const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(vel[0], vel[0]), __fmul_rn(vel[1], vel[1])),
                                   __fmul_rn(vel[2], vel[2]));
        m = ref_max(m, l2);
    }
    for (int o = 16; o > 0; o >>= 1) m = ref_max(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float wm[2];
    if ((t & 31) == 0) wm[t >> 5] = m;
    __syncthreads();
    if (t == 0) atomicMax(a.max_bits + inst, __float_as_uint(ref_max(wm[0], wm[1])));
}

void launch_cfl(const CflArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    cfl_max_kernel<<<unsigned(a.nleaf), 64, 0, s>>>(a);
}

}  // namespace gbls

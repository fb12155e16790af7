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

// Each CTA covers CFL_LEAVES consecutive leaves, four at a time (64 threads
// per leaf, thread t visiting bit t of each active-mask word), with all
// keys, slots and mask words of its leaves loaded up front so that the
// loads overlap.  The maximum is published with one atomicMax per CTA (one
// per warp and instance met for batches, whose instances spread the
// atomics over many addresses), not one per leaf, which serialised on a
// single address.  Vec3f::lengthSqr (math/Vec3.h:212-218) is evaluated with
// non-contracting intrinsics so the maximum equals the reference's exactly
// (the maximum of non-negative floats does not depend on order).
constexpr int CFL_THREADS = 256;
constexpr int CFL_GROUPS = CFL_THREADS / 64;
constexpr int CFL_ROUNDS = 4;
constexpr int CFL_LEAVES = CFL_GROUPS * CFL_ROUNDS;

__device__ __forceinline__ float warp_max(float m) {
    for (int o = 16; o > 0; o >>= 1) m = ref_max(m, __shfl_xor_sync(0xffffffffu, m, o));
    return m;
}

__global__ void __launch_bounds__(CFL_THREADS) cfl_max_kernel(const __grid_constant__ CflArgs a) {
    const int64_t n = a.nleaf_dev ? min(a.nleaf, int64_t(*a.nleaf_dev)) : a.nleaf;
    const int t = threadIdx.x, g = t >> 6, b = t & 63;
    const int64_t base = int64_t(blockIdx.x) * CFL_LEAVES + g;
    uint64_t key[CFL_ROUNDS], w[CFL_ROUNDS][8];
    int slot[CFL_ROUNDS];
#pragma unroll
    for (int r = 0; r < CFL_ROUNDS; ++r) {
        const int64_t l = base + r * CFL_GROUPS;
        key[r] = l < n ? a.keys[l] : 0;
        slot[r] = l < n ? a.slot[l] : -1;
    }
#pragma unroll
    for (int r = 0; r < CFL_ROUNDS; ++r)
#pragma unroll
        for (int k = 0; k < 8; ++k) w[r][k] = slot[r] >= 0 ? a.amask[size_t(slot[r]) * 8 + k] : 0;
    float m = 0.0f;
    uint32_t cur = 0xffffffffu;  // batches: instance of the running maximum (uniform per warp)
#pragma unroll
    for (int r = 0; r < CFL_ROUNDS; ++r) {
        if (slot[r] < 0) continue;
        const FieldParams* fp = &a.field;
        float t0 = a.t0;
        if (a.inst_run) {
            const uint32_t inst = key_instance(key[r]);
            if (inst != cur) {
                if (cur != 0xffffffffu) {
                    const float wm = warp_max(m);
                    if ((t & 31) == 0) atomicMax(a.max_bits + cur, __float_as_uint(wm));
                }
                cur = inst;
                m = 0.0f;
            }
            if (!a.inst_run[inst]) continue;
            fp = a.inst_field + inst;
            t0 = a.inst_t0[inst];
        }
        int ox, oy, oz;
        key_origin(key[r], ox, oy, oz);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (!((w[r][k] >> b) & 1)) continue;
            float vel[3];
            eval_field(*fp, ox + k, oy + (b >> 3), oz + (b & 7), t0, vel);
            const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(vel[0], vel[0]), __fmul_rn(vel[1], vel[1])),
                                       __fmul_rn(vel[2], vel[2]));
            m = ref_max(m, l2);
        }
    }
    if (a.inst_run) {
        if (cur != 0xffffffffu) {
            const float wm = warp_max(m);
            if ((t & 31) == 0) atomicMax(a.max_bits + cur, __float_as_uint(wm));
        }
        return;
    }
    __shared__ float red[CFL_THREADS / 32];
    m = warp_max(m);
    if ((t & 31) == 0) red[t >> 5] = m;
    __syncthreads();
    if (t == 0) {
        float x = red[0];
        for (int i = 1; i < CFL_THREADS / 32; ++i) x = ref_max(x, red[i]);
        atomicMax(a.max_bits, __float_as_uint(x));
    }
}

void launch_cfl(const CflArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    cfl_max_kernel<<<unsigned((a.nleaf + CFL_LEAVES - 1) / CFL_LEAVES), CFL_THREADS, 0, s>>>(a);
}

}  // namespace gbls

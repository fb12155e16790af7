// FP32 stencil kernels and the CFL reduction.
#include "stencil.h"
#include "filter_ops.cuh"
#include "morph_ops.cuh"
#include "stencil_ops.cuh"
#include "stencil_fast2.cuh"

namespace gbls {

// The packed FP32x2 kernels evaluate HJ-WENO5; other schemes run the scalar ones.
void launch_rk_fast(const RkArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    if (a.spatial == 4)
        rk_stage_kernel_x2<<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
    else
        rk_stage_kernel<FastArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

void launch_norm_fast(const NormArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    if (!a.copy_only && !a.has_phi && a.spatial == 4)
        normalize_kernel_x2<<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
    else
        normalize_kernel<FastArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

// One CTA of 64 threads per leaf (thread t visits bit t of each active-mask
// word), the leaf's six sine rows of the deformation table staged in shared
// memory as in the RK kernel.  A single level set writes its leaf maxima to
// a partial array reduced by cfl_reduce_kernel (no same-address atomics);
// a batch publishes each leaf maximum with atomicMax on its instance's word
// (spread over the instances).  Vec3f::lengthSqr (math/Vec3.h:212-218) and
// the field use non-contracting intrinsics in eval_field's order, so the
// maximum equals the reference's exactly (the maximum of non-negative floats
// does not depend on order).
constexpr int CFL_THREADS = 64;

__global__ void __launch_bounds__(CFL_THREADS) cfl_max_kernel(const __grid_constant__ CflArgs a) {
    const int64_t n = a.nleaf_dev ? min(a.nleaf, int64_t(*a.nleaf_dev)) : a.nleaf;
    const int64_t l = blockIdx.x;
    const int t = threadIdx.x;
    __shared__ float vtab[6][8];
    __shared__ float wm[2];
    if (l >= n) {
        if (t == 0 && a.part) a.part[l] = 0.0f;
        return;
    }
    const uint64_t key = a.keys[l];
    const FieldParams* fp = &a.field;
    float t0 = a.t0;
    uint32_t inst = 0;
    if (a.inst_run) {
        inst = key_instance(key);
        if (!a.inst_run[inst]) return;
        fp = a.inst_field + inst;
        t0 = a.inst_t0[inst];
    }
    const int s = a.slot[l];
    int ox, oy, oz;
    key_origin(key, ox, oy, oz);
    const FieldParams& f = *fp;
    const bool tabbed = f.kind == 2 && f.tab && ox - f.tab_lo >= 0 && oy - f.tab_lo >= 0 && oz - f.tab_lo >= 0 &&
                        ox + 8 - f.tab_lo <= f.tab_n && oy + 8 - f.tab_lo <= f.tab_n && oz + 8 - f.tab_lo <= f.tab_n;
    if (tabbed) {  // block-uniform
        if (t < 48) {
            const int ax = t >> 4, fn = (t >> 3) & 1, q = t & 7;
            const int o = ax == 0 ? ox : ax == 1 ? oy : oz;
            vtab[ax * 2 + fn][q] = f.tab[2 * (o + q - f.tab_lo) + fn];
        }
        __syncthreads();
    }
    const int y = t >> 3, z = t & 7;
    float m = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uint64_t w = a.amask[size_t(s) * 8 + k];
        if (!((w >> t) & 1)) continue;
        float vel[3];
        if (tabbed) {  // eval_field's deformation branch with the staged sines
            const float sx = vtab[0][k], s2x = vtab[1][k], sy = vtab[2][y], s2y = vtab[3][y];
            const float sz = vtab[4][z], s2z = vtab[5][z];
            const float u = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(2.0f, sx), sx), s2y), s2z);
            const float v = __fmul_rn(__fmul_rn(__fmul_rn(s2x, sy), sy), s2z);
            const float ww = __fmul_rn(__fmul_rn(__fmul_rn(s2x, s2y), sz), sz);
            vel[0] = __fmul_rn(u, f.amp);
            vel[1] = -__fmul_rn(v, f.amp);
            vel[2] = -__fmul_rn(ww, f.amp);
        } else {
            eval_field(f, ox + k, oy + y, oz + z, t0, vel);
        }
        const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(vel[0], vel[0]), __fmul_rn(vel[1], vel[1])),
                                   __fmul_rn(vel[2], vel[2]));
        m = ref_max(m, l2);
    }
    for (int o = 16; o > 0; o >>= 1) m = ref_max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (a.inst_run) {
        if ((t & 31) == 0) atomicMax(a.max_bits + inst, __float_as_uint(m));
        return;
    }
    if ((t & 31) == 0) wm[t >> 5] = m;
    __syncthreads();
    if (t == 0) a.part[l] = ref_max(wm[0], wm[1]);
}

// Maximum of the per-leaf partials into max_bits[0] (one CTA).
__global__ void __launch_bounds__(1024) cfl_reduce_kernel(const float* part, int64_t n, unsigned int* max_bits) {
    float m = 0.0f;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) m = ref_max(m, part[i]);
    for (int o = 16; o > 0; o >>= 1) m = ref_max(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float wm[32];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float x = wm[0];
        for (int i = 1; i < 32; ++i) x = ref_max(x, wm[i]);
        atomicMax(max_bits, __float_as_uint(x));
    }
}

__global__ void __launch_bounds__(1024) morph_reduce_kernel(const float* part, int64_t n, unsigned int* max_bits) {
    float m = 0.0f;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) m = ref_max(m, part[i]);
    for (int o = 16; o > 0; o >>= 1) m = ref_max(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float wm[32];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float x = wm[0];
        for (int i = 1; i < 32; ++i) x = ref_max(x, wm[i]);
        atomicMax(max_bits, __float_as_uint(x));
    }
}

void launch_morph_speed_fast(const MorphSpeedArgs& a, unsigned int* max_bits, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    morph_speed_kernel<FastArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
    morph_reduce_kernel<<<1, 1024, 0, s>>>(a.part, a.nleaf, max_bits);
}

void launch_morph_stage_fast(const MorphArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    morph_stage_kernel<FastArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

void launch_cfl(const CflArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    cfl_max_kernel<<<unsigned(a.nleaf), CFL_THREADS, 0, s>>>(a);
    if (!a.inst_run) cfl_reduce_kernel<<<1, 1024, 0, s>>>(a.part, a.nleaf, a.max_bits);
}

void launch_filter_fast(const FilterArgs& a, cudaStream_t s) {
    if (a.nleaf <= 0) return;
    if (a.op >= FILTER_MEAN_CURVATURE)
        filter_full_kernel<FastArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
    else
        filter_kernel<FastArith><<<unsigned(a.nleaf), STENCIL_THREADS, 0, s>>>(a);
}

}  // namespace gbls

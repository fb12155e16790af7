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

// Eight threads per leaf, thread w visiting the set bits of active-mask word
// w (voxels x = w), 32 leaves per CTA of 256 threads: every leaf's chain of
// dependent loads (slot, then mask and key, then the field's sine rows) is
// in flight at once, which the reduction's few operations per voxel cannot
// hide otherwise.  The deformation field reads its per-coordinate sine table
// directly (L1-resident rows).  A single level set writes its leaf maxima to
// a partial array reduced by cfl_reduce_kernel (no same-address atomics); a
// batch publishes each leaf maximum with atomicMax on its instance's word.
// Vec3f::lengthSqr (math/Vec3.h:212-218) and the field use non-contracting
// intrinsics in eval_field's order, so the maximum equals the reference's
// exactly (the maximum of non-negative floats does not depend on order).
// LEAVES leaves per CTA, 8 threads per leaf (one per mask word)
template <int LEAVES>
__global__ void __launch_bounds__(LEAVES * 8) cfl_max_kernel(const __grid_constant__ CflArgs a) {
    const int64_t n = a.nleaf_dev ? min(a.nleaf, int64_t(*a.nleaf_dev)) : a.nleaf;
    const int64_t l = int64_t(blockIdx.x) * LEAVES + (threadIdx.x >> 3);
    const int w = threadIdx.x & 7;
    float m = 0.0f;
    uint32_t inst = 0;
    bool live = l < n && l < a.nleaf;
    if (live && a.inst_run) {
        inst = key_instance(a.keys[l]);
        live = a.inst_run[inst] != 0;
    }
    if (live) {
        const int s = a.slot[l];
        uint64_t bits = a.amask[size_t(s) * 8 + w];
        const uint64_t key = a.keys[l];
        const FieldParams& f = a.inst_run ? a.inst_field[inst] : a.field;
        const float t0 = a.inst_run ? a.inst_t0[inst] : a.t0;
        int ox, oy, oz;
        key_origin(key, ox, oy, oz);
        const bool tabbed = f.kind == 2 && f.tab && ox - f.tab_lo >= 0 && oy - f.tab_lo >= 0 &&
                            oz - f.tab_lo >= 0 && ox + 8 - f.tab_lo <= f.tab_n && oy + 8 - f.tab_lo <= f.tab_n &&
                            oz + 8 - f.tab_lo <= f.tab_n;
        float sx = 0.0f, s2x = 0.0f;
        if (tabbed) {
            const int ia = ox + w - f.tab_lo;
            sx = __ldg(f.tab + 2 * ia);
            s2x = __ldg(f.tab + 2 * ia + 1);
        }
        while (bits) {
            const int b = __ffsll(static_cast<long long>(bits)) - 1;
            bits &= bits - 1;
            const int y = b >> 3, z = b & 7;
            float vel[3];
            if (tabbed) {  // eval_field's deformation branch, sines from the table
                const int ja = oy + y - f.tab_lo, ka = oz + z - f.tab_lo;
                const float sy = __ldg(f.tab + 2 * ja), s2y = __ldg(f.tab + 2 * ja + 1);
                const float sz = __ldg(f.tab + 2 * ka), s2z = __ldg(f.tab + 2 * ka + 1);
                const float u = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(2.0f, sx), sx), s2y), s2z);
                const float v = __fmul_rn(__fmul_rn(__fmul_rn(s2x, sy), sy), s2z);
                const float ww = __fmul_rn(__fmul_rn(__fmul_rn(s2x, s2y), sz), sz);
                vel[0] = __fmul_rn(u, f.amp);
                vel[1] = -__fmul_rn(v, f.amp);
                vel[2] = -__fmul_rn(ww, f.amp);
            } else {
                eval_field(f, ox + w, oy + y, oz + z, t0, vel);
            }
            const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(vel[0], vel[0]), __fmul_rn(vel[1], vel[1])),
                                       __fmul_rn(vel[2], vel[2]));
            m = ref_max(m, l2);
        }
    }
    // maximum over the leaf's 8 lanes (groups of 8 consecutive lanes)
    for (int o = 4; o > 0; o >>= 1) m = ref_max(m, __shfl_xor_sync(0xffffffffu, m, o, 8));
    if (w != 0 || l >= a.nleaf) return;
    if (a.inst_run) {
        if (live) atomicMax(a.max_bits + inst, __float_as_uint(m));
        return;
    }
    a.part[l] = m;
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

template <int LEAVES>
void launch_cfl_shape(const CflArgs& a, cudaStream_t s) {
    cfl_max_kernel<LEAVES><<<unsigned((a.nleaf + LEAVES - 1) / LEAVES), LEAVES * 8, 0, s>>>(a);
}

void launch_cfl(const CflArgs& a, cudaStream_t s, int leaves_per_block) {
    if (a.nleaf <= 0) return;
    if (leaves_per_block == 8) launch_cfl_shape<8>(a, s);
    else if (leaves_per_block == 16) launch_cfl_shape<16>(a, s);
    else if (leaves_per_block == 64) launch_cfl_shape<64>(a, s);
    else launch_cfl_shape<32>(a, s);
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

// Kernels of LevelSetMorphing::advect (tools/LevelSetMorph.h), templated on
// the arithmetic policy like the advection stencils: PARITY instances are
// built in stencil_parity.cu (-fmad=false), FAST ones in stencil_fast.cu.
//
//   speed   s = phi(ijk) - target(ijk), times a(ijk) or 1 - a(ijk) with
//           a = SmoothUnitStep((mask(ijk) - min) / (max - min)) when an alpha
//           mask is set (sampleAlignedSpeed, LevelSetMorph.h:563-601), per
//           active voxel at the start of every CFL substep, with max |s|;
//   stage   v = phi - dt * s * invdx^2 * GodunovNormSqrd(HJ-WENO5)(phi),
//           out = N ? alpha * phi_n + beta * v : v, voxels with |s| <= 1e-8
//           keep their value (euler<N,D>, LevelSetMorph.h:617-648).
// The target and the mask are level sets resident on the device, looked up
// at the source voxel's own index (aligned transforms).
#pragma once

#include "stencil_ops.cuh"

namespace gbls {

// A device level set that values are looked up in.
struct LookupGrid {
    const uint64_t* keys;   // [nleaf] sorted leaf keys
    const int32_t* slot;    // [nleaf]
    int64_t nleaf;
    Layout layout;          // its current masks and packed values
    NodeTables nodes;
    float gamma;            // its background
};

struct MorphSpeedArgs {
    int64_t nleaf;
    const uint64_t* keys;
    const int32_t* slot;
    Layout src;             // the morphing level set
    float* speed;           // out: [slot*512 + rank] per active voxel
    float* part;            // out: [nleaf] max |s| of each leaf
    LookupGrid target;
    int has_mask, invert;
    LookupGrid mask;
    float mask_min, mask_inv_norm;
};

struct MorphArgs {
    int spatial;            // FIRST_BIAS or HJWENO5_BIAS
    int64_t nleaf;
    const int32_t* slot;
    const int32_t* nbr;
    Layout src;             // stage input
    const float* phin;      // phi_n (convex combination), packed like src
    const float* speed;
    float* out;
    float alpha, beta, dt, gamma, invdxdx;
    int has_phi;
};

// Per-CTA view of the lookup grid's leaf that has the same key as the
// source leaf: its masks, or the tile value when it has no such leaf.
struct LookupStage {
    uint64_t am[8], sm[8];
    const float* vp;
    float tile;
};

// All threads call; ends with a barrier.
__device__ inline void stage_lookup(LookupStage& st, const LookupGrid& g, uint64_t key) {
    __shared__ int64_t found;
    if (threadIdx.x == 0) {
        found = find_u64(g.keys, g.nleaf, key);
        if (found >= 0) {
            st.vp = g.layout.vals + size_t(g.slot[found]) * LEAF_VOX;
        } else {
            st.vp = nullptr;
            st.tile = tile_sign(g.nodes, key) ? -g.gamma : g.gamma;
        }
    }
    __syncthreads();
    if (threadIdx.x < 8 && found >= 0) {
        const size_t s = size_t(g.slot[found]);
        st.am[threadIdx.x] = g.layout.amask[s * 8 + threadIdx.x];
        st.sm[threadIdx.x] = g.layout.smask[s * 8 + threadIdx.x];
    }
    __syncthreads();
}

// ValueAccessor::getValue of voxel (word k, bit b) of the staged leaf.
__device__ __forceinline__ float lookup_value(const LookupStage& st, int k, int b, float gamma) {
    if (!st.vp) return st.tile;
    const uint64_t m = st.am[k];
    if ((m >> b) & 1) {
        int rank = __popcll(m & ((uint64_t(1) << b) - 1));
        for (int w = 0; w < k; ++w) rank += __popcll(st.am[w]);
        return st.vp[rank];
    }
    return ((st.sm[k] >> b) & 1) ? -gamma : gamma;
}

// math::SmoothUnitStep (math/Math.h:300-303).
template <class A>
__device__ __forceinline__ float smooth_unit_step(float x) {
    return x > 0.0f ? (x < 1.0f ? A::mul(A::mul(A::sub(3.0f, A::mul(2.0f, x)), x), x) : 1.0f) : 0.0f;
}

template <class A>
__global__ void __launch_bounds__(STENCIL_THREADS) morph_speed_kernel(const MorphSpeedArgs a) {
    __shared__ uint64_t am[8];
    __shared__ LookupStage tg, mk;
    __shared__ float wm[2];
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    const int s = a.slot[l];
    const uint64_t key = a.keys[l];
    const int t = threadIdx.x;
    if (t < 8) am[t] = a.src.amask[size_t(s) * 8 + t];
    stage_lookup(tg, a.target, key);
    if (a.has_mask) stage_lookup(mk, a.mask, key);
    const uint64_t below = (uint64_t(1) << t) - 1;
    float m = 0.0f;
    int base = 0;
#pragma unroll 1
    for (int k = 0; k < 8; ++k) {
        const uint64_t w = am[k];
        if ((w >> t) & 1) {
            const int rank = base + __popcll(w & below);
            float sp = A::sub(a.src.vals[size_t(s) * LEAF_VOX + rank], lookup_value(tg, k, t, a.target.gamma));
            if (a.has_mask) {
                const float al = smooth_unit_step<A>(
                    A::mul(A::sub(lookup_value(mk, k, t, a.mask.gamma), a.mask_min), a.mask_inv_norm));
                sp = A::mul(sp, a.invert ? A::sub(1.0f, al) : al);
            }
            a.speed[size_t(s) * LEAF_VOX + rank] = sp;
            m = ref_max(m, fabsf(sp));
        }
        base += __popcll(w);
    }
    for (int o = 16; o > 0; o >>= 1) m = ref_max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((t & 31) == 0) wm[t >> 5] = m;
    __syncthreads();
    if (t == 0) a.part[l] = ref_max(wm[0], wm[1]);
}

template <class A>
__global__ void __launch_bounds__(STENCIL_THREADS) morph_stage_kernel(const MorphArgs a) {
    __shared__ float tile[TILE_VOX];
    __shared__ LeafStage st;
    __shared__ uint16_t list[LEAF_VOX];
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    const int s = a.slot[l];
    stage_masks(st, a.src, s, a.nbr + 6 * l, nullptr, nullptr);
    load_tile(tile, st, a.gamma);
    const int n = build_list(list, st.am[0]);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += STENCIL_THREADS) {
        const int v = list[i];
        const int x = v >> 6, y = (v >> 3) & 7, z = v & 7;
        const float c = tile[tile_index(x, y, z)];
        const float sp = a.speed[size_t(s) * LEAF_VOX + i];
        float o = c;  // math::isApproxZero(speed): the voxel keeps its value
        if ((sp > 1e-8f) || (sp < -1e-8f)) {
            float up[3], down[3];
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                const Line7 L = tile_line(tile, x, y, z, ax);
                up[ax] = scheme_fd<A>(L, a.spatial);
                down[ax] = scheme_bd<A>(L, a.spatial);
            }
            const float g2 = A::mul(a.invdxdx, godunov<A>(c > 0.0f, down, up));
            const float vv = A::sub(c, A::mul(A::mul(a.dt, sp), g2));
            o = a.has_phi ? A::add(A::mul(a.alpha, a.phin[size_t(s) * LEAF_VOX + i]), A::mul(a.beta, vv)) : vv;
        }
        a.out[size_t(s) * LEAF_VOX + i] = o;
    }
}

// Max of the per-leaf speed maxima into *max_bits (one CTA).
__global__ void __launch_bounds__(1024) morph_reduce_kernel(const float* part, int64_t n, unsigned int* max_bits);

}  // namespace gbls

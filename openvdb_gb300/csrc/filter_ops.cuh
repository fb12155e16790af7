// Kernels of LevelSetFilter (tools/LevelSetFilter.h) on the device: one
// pass updates every active voxel from the staged 14^3 tile of its leaf
// (values of the previous pass), as the reference's Filter::cook does over
// its leaf buffers, and writes the result in the same packed layout:
//   LAPLACIAN  phi + dt * invdx2 * (sum of the six face neighbours - 6 phi)
//              (laplacianImpl :452-477, GradStencil::laplacian,
//              math/Stencils.h:1294-1299), dt = dx^2 / 6;
//   BOX        the mean of the 2w+1 values along one axis, summed in index
//              order and scaled by 1/(2w+1) (Filter::Avg :206-219, boxImpl
//              :327-349); w <= 3, the tile's halo;
//   OFFSET     phi + offset (offsetImpl :479-497).
// With an alpha mask (tools::AlphaMask, tools/Interpolation.h:545-579: a =
// SmoothUnitStep((mask(ijk) - min) / (max - min)), b = 1 - a, swapped when
// inverted) a voxel with a > 0 takes b * phi + a * filtered (OFFSET:
// phi + a * offset; FILLET: filtered = phi + min(0, dt * kappa)), the others
// keep their value (the reference leaves the copied buffer entry).
#pragma once

#include "morph_ops.cuh"
#include "stencil_ops.cuh"

namespace gbls {

enum FilterOp {
    FILTER_LAPLACIAN = 0,
    FILTER_BOX = 1,
    FILTER_OFFSET = 2,
    FILTER_MEAN_CURVATURE = 3,  // the passes below read the full 14^3 tile
    FILTER_FILLET = 4,
    FILTER_MEDIAN = 5
};

struct FilterArgs {
    int64_t nleaf;
    const int32_t* slot;
    const int32_t* nbr;
    Layout src;
    float* out;
    float gamma;
    int op, axis, width;
    float frac;        // BOX: 1 / (2w + 1)
    float dt, invdx2;  // LAPLACIAN, curvature filters (dt = dx^2/6 or dx^2/3)
    float inv2dx;      // curvature filters
    float offset;      // OFFSET
    // full-tile passes: the 26 neighbour leaves are found by key
    const uint64_t* keys;
    NodeTables nodes;
    // alpha mask: a device level set with the same transform, looked up at
    // each voxel's own index
    int has_mask, invert;
    LookupGrid mask;
    float mask_min, mask_inv_norm;  // min, 1 / (max - min)
};

// AlphaMask::operator() at voxel (word k, bit b) of the staged mask leaf:
// returns a > 0 with a, b.
template <class A>
__device__ __forceinline__ bool filter_alpha(const FilterArgs& f, const LookupStage& mk, int k, int bit, float& al,
                                             float& bl) {
    al = smooth_unit_step<A>(A::mul(A::sub(lookup_value(mk, k, bit, f.mask.gamma), f.mask_min), f.mask_inv_norm));
    bl = A::sub(1.0f, al);
    if (f.invert) {
        const float t = al;
        al = bl;
        bl = t;
    }
    return al > 0.0f;
}

template <class A>
__global__ void __launch_bounds__(STENCIL_THREADS) filter_kernel(const FilterArgs a) {
    __shared__ float tile[TILE_VOX];
    __shared__ LeafStage st;
    __shared__ uint16_t list[LEAF_VOX];
    __shared__ LookupStage mk;
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    const int s = a.slot[l];
    if (a.has_mask) stage_lookup(mk, a.mask, a.keys[l]);
    stage_masks(st, a.src, s, a.nbr + 6 * l, nullptr, nullptr);
    load_tile(tile, st, a.gamma);
    const int n = build_list(list, st.am[0]);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += STENCIL_THREADS) {
        const int v = list[i];
        const int x = v >> 6, y = (v >> 3) & 7, z = v & 7;
        const float c = tile[tile_index(x, y, z)];
        float r;
        if (a.op == FILTER_LAPLACIAN) {
            float sum = A::add(tile[tile_index(x - 1, y, z)], tile[tile_index(x + 1, y, z)]);
            sum = A::add(sum, tile[tile_index(x, y - 1, z)]);
            sum = A::add(sum, tile[tile_index(x, y + 1, z)]);
            sum = A::add(sum, tile[tile_index(x, y, z - 1)]);
            sum = A::add(sum, tile[tile_index(x, y, z + 1)]);
            const float lap = A::mul(a.invdx2, A::sub(sum, A::mul(6.0f, c)));
            r = A::add(c, A::mul(a.dt, lap));
        } else if (a.op == FILTER_BOX) {
            float sum = 0.0f;
            for (int k = -a.width; k <= a.width; ++k) {
                const int xx = x + (a.axis == 0 ? k : 0), yy = y + (a.axis == 1 ? k : 0),
                          zz = z + (a.axis == 2 ? k : 0);
                sum = A::add(sum, tile[tile_index(xx, yy, zz)]);
            }
            r = A::mul(sum, a.frac);
        } else {
            r = A::add(c, a.offset);
        }
        if (a.has_mask) {
            float al, bl;
            if (!filter_alpha<A>(a, mk, x, v & 63, al, bl)) r = c;
            else if (a.op == FILTER_OFFSET) r = A::add(c, A::mul(al, a.offset));
            else r = A::add(A::mul(bl, c), A::mul(al, r));
        }
        a.out[size_t(s) * LEAF_VOX + i] = r;
    }
}

// ---- full 14^3 tile: the 26 neighbour leaves (faces, edges, corners) ------
// Neighbour r = bx*9 + by*3 + bz for offsets (bx-1, by-1, bz-1) * 8; r = 13
// is the leaf itself.
struct FullStage {
    uint64_t am[27][8], sm[27][8];
    int preh[27][16];
    const float* vp[27];
    int32_t code[27];  // slot, or NBR_TILE_POS / NBR_TILE_NEG
};

// All threads call; ends with a barrier.
__device__ inline void stage_full(FullStage& st, const FilterArgs& a, int64_t l) {
    const int t = threadIdx.x;
    const uint64_t key = a.keys[l];
    if (t < 27) {
        int32_t code;
        if (t == 13) {
            code = a.slot[l];
        } else {
            int32_t x, y, z;
            key_origin(key, x, y, z);
            x += (t / 9 - 1) * 8;
            y += ((t / 3) % 3 - 1) * 8;
            z += (t % 3 - 1) * 8;
            if (x < -COORD_LIMIT || x >= COORD_LIMIT || y < -COORD_LIMIT || y >= COORD_LIMIT || z < -COORD_LIMIT ||
                z >= COORD_LIMIT) {
                code = NBR_TILE_POS;  // outside the key space: the background
            } else {
                const uint64_t nk = leaf_key(x, y, z) | (key & ~KEY_COORD_MASK);
                const int64_t j = find_u64(a.keys, a.nleaf, nk);
                code = j >= 0 ? a.slot[j] : (tile_sign(a.nodes, nk) ? NBR_TILE_NEG : NBR_TILE_POS);
            }
        }
        st.code[t] = code;
        st.vp[t] = code >= 0 ? a.src.vals + size_t(code) * LEAF_VOX : nullptr;
    }
    __syncthreads();
    for (int e = t; e < 27 * 8; e += blockDim.x) {
        const int r = e >> 3, w = e & 7;
        const int32_t code = st.code[r];
        st.am[r][w] = code >= 0 ? a.src.amask[size_t(code) * 8 + w] : 0;
        st.sm[r][w] = code >= 0 ? a.src.smask[size_t(code) * 8 + w] : (code == NBR_TILE_NEG ? ~uint64_t(0) : 0);
    }
    __syncthreads();
    if (t < 27) {
        int acc = 0;
        for (int w = 0; w < 8; ++w) {
            const uint64_t m = st.am[t][w];
            st.preh[t][2 * w] = acc;
            acc += __popc(uint32_t(m));
            st.preh[t][2 * w + 1] = acc;
            acc += __popc(uint32_t(m >> 32));
        }
    }
    __syncthreads();
}

// Fill every entry of the 14^3 tile from the staged leaves.  Ends with a barrier.
__device__ inline void load_full_tile(float* tile, const FullStage& st, float gamma) {
    for (int e = threadIdx.x; e < TILE_VOX; e += blockDim.x) {
        const int x = e / (TILE_DIM * TILE_DIM) - 3, y = (e / TILE_DIM) % TILE_DIM - 3, z = e % TILE_DIM - 3;
        const int bx = x < 0 ? 0 : (x > 7 ? 2 : 1), by = y < 0 ? 0 : (y > 7 ? 2 : 1), bz = z < 0 ? 0 : (z > 7 ? 2 : 1);
        const int r = bx * 9 + by * 3 + bz;
        const int lx = x - (bx - 1) * 8, ly = y - (by - 1) * 8, lz = z - (bz - 1) * 8;
        const int w = lx, b = (ly << 3) | lz, h = b >> 5, bb = b & 31;
        const uint32_t m = reinterpret_cast<const uint32_t*>(&st.am[r][w])[h];
        float v;
        if ((m >> bb) & 1) {
            v = st.vp[r][st.preh[r][2 * w + h] + __popc(m & ((1u << bb) - 1u))];
        } else {
            const uint32_t g = reinterpret_cast<const uint32_t*>(&st.sm[r][w])[h];
            v = ((g >> bb) & 1) ? -gamma : gamma;
        }
        tile[e] = v;
    }
    __syncthreads();
}

// math::CurvatureStencil (math/Stencils.h:1512-1747) at tile voxel (x, y, z):
// the unscaled central differences in double from float differences, in the
// reference's evaluation order.  Returns false when |grad|^2 <= 1e-15.
struct Curv {
    double Dx, Dy, Dz, Dx2, Dy2, Dz2, Dxx, Dyy, Dzz, Dxy, Dxz, Dyz, normGrad;
};
__device__ inline bool curvature_terms(const float* tile, int x, int y, int z, Curv& c) {
    auto T = [&](int dx, int dy, int dz) { return tile[tile_index(x + dx, y + dy, z + dz)]; };
    const float v0 = T(0, 0, 0);
    c.Dx = 0.5 * double(T(1, 0, 0) - T(-1, 0, 0));
    c.Dy = 0.5 * double(T(0, 1, 0) - T(0, -1, 0));
    c.Dz = 0.5 * double(T(0, 0, 1) - T(0, 0, -1));
    c.Dx2 = c.Dx * c.Dx;
    c.Dy2 = c.Dy * c.Dy;
    c.Dz2 = c.Dz * c.Dz;
    const double ng2 = c.Dx2 + c.Dy2 + c.Dz2;
    if (ng2 <= 1e-15) return false;
    c.Dxx = double(T(1, 0, 0) - 2 * v0 + T(-1, 0, 0));
    c.Dyy = double(T(0, 1, 0) - 2 * v0 + T(0, -1, 0));
    c.Dzz = double(T(0, 0, 1) - 2 * v0 + T(0, 0, -1));
    c.Dxy = 0.25 * double(T(1, 1, 0) - T(1, -1, 0) + T(-1, -1, 0) - T(-1, 1, 0));
    c.Dxz = 0.25 * double(T(1, 0, 1) - T(1, 0, -1) + T(-1, 0, -1) - T(-1, 0, 1));
    c.Dyz = 0.25 * double(T(0, 1, 1) - T(0, 1, -1) + T(0, -1, -1) - T(0, -1, 1));
    c.normGrad = sqrt(ng2);
    return true;
}

__device__ inline double alpha_mean(const Curv& c) {
    return c.Dx2 * (c.Dyy + c.Dzz) + c.Dy2 * (c.Dxx + c.Dzz) + c.Dz2 * (c.Dxx + c.Dyy) -
           2 * (c.Dx * (c.Dy * c.Dxy + c.Dz * c.Dxz) + c.Dy * c.Dz * c.Dyz);
}

__device__ inline double alpha_gauss(const Curv& c) {
    return c.Dx2 * (c.Dyy * c.Dzz - c.Dyz * c.Dyz) + c.Dy2 * (c.Dxx * c.Dzz - c.Dxz * c.Dxz) +
           c.Dz2 * (c.Dxx * c.Dyy - c.Dxy * c.Dxy) +
           2 * (c.Dy * c.Dz * (c.Dxy * c.Dxz - c.Dyz * c.Dxx) + c.Dx * c.Dz * (c.Dxy * c.Dyz - c.Dxz * c.Dyy) +
                c.Dx * c.Dy * (c.Dxz * c.Dyz - c.Dxy * c.Dzz));
}

// Median of the (2w+1)^3 window (DenseStencil::median, math/Stencils.h:121-132):
// the element of rank ((2w+1)^3 - 1) / 2, found by counting.
__device__ inline float window_median(const float* tile, int x, int y, int z, int w) {
    const int n = 2 * w + 1, total = n * n * n, k = (total - 1) >> 1;
    for (int i = 0; i < total; ++i) {
        const float vi = tile[tile_index(x - w + i / (n * n), y - w + (i / n) % n, z - w + i % n)];
        int less = 0, eq = 0;
        for (int j = 0; j < total; ++j) {
            const float vj = tile[tile_index(x - w + j / (n * n), y - w + (j / n) % n, z - w + j % n)];
            less += vj < vi;
            eq += vj == vi;
        }
        if (less <= k && k < less + eq) return vi;
    }
    return tile[tile_index(x, y, z)];  // not reached for ordered values
}

// LevelSetFilter passes that read edge and corner neighbours: meanCurvatureImpl
// (:376-403), filletImpl (:405-432), medianImpl (:499-525).
template <class A>
__global__ void __launch_bounds__(STENCIL_THREADS) filter_full_kernel(const FilterArgs a) {
    __shared__ float tile[TILE_VOX];
    __shared__ FullStage st;
    __shared__ uint16_t list[LEAF_VOX];
    __shared__ LookupStage mk;
    const int64_t l = blockIdx.x;
    if (l >= a.nleaf) return;
    const int s = a.slot[l];
    if (a.has_mask) stage_lookup(mk, a.mask, a.keys[l]);
    stage_full(st, a, l);
    load_full_tile(tile, st, a.gamma);
    const int n = build_list(list, st.am[13]);
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += STENCIL_THREADS) {
        const int v = list[i];
        const int x = v >> 6, y = (v >> 3) & 7, z = v & 7;
        const float c0 = tile[tile_index(x, y, z)];
        float r = c0;
        if (a.op == FILTER_MEDIAN) {
            r = window_median(tile, x, y, z, a.width);
        } else {
            Curv c;
            const bool ok = curvature_terms(tile, x, y, z, c);
            if (a.op == FILTER_MEAN_CURVATURE) {
                // meanCurvatureNormGrad: alpha * invDx2 / (2 |grad|^2), 0 without a gradient
                const float k = ok ? float(alpha_mean(c) * double(a.invdx2) / (2 * (c.normGrad * c.normGrad))) : 0.0f;
                r = A::add(c0, A::mul(a.dt, k));
            } else {  // FILLET: principalCurvatures().first (0 without a gradient)
                float k = 0.0f;
                if (ok) {
                    const double ng = c.normGrad;
                    const double mean = alpha_mean(c) * double(a.inv2dx) / (ng * ng * ng);
                    const double tmp =
                        sqrt(mean * mean - alpha_gauss(c) * double(a.invdx2) / ((ng * ng) * (ng * ng)));
                    k = float(mean - tmp);
                }
                if (a.has_mask) r = A::add(c0, ref_min(0.0f, A::mul(a.dt, k)));  // phi + Min(0, dt kappa)
                else if (k < 0.0f) r = A::add(c0, A::mul(a.dt, k));              // applied when negative
            }
        }
        if (a.has_mask) {
            float al, bl;
            r = filter_alpha<A>(a, mk, x, v & 63, al, bl) ? A::add(A::mul(bl, c0), A::mul(al, r)) : c0;
        }
        a.out[size_t(s) * LEAF_VOX + i] = r;
    }
}

}  // namespace gbls

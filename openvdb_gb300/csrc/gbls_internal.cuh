// Device-side data model of the GB300 narrow-band level-set library.
//
// A level set (OpenVDB Tree4<float,5,4,3>, tree/Tree.h:1125-1127) lives on
// the device as:
//
//   * a leaf list in reference tree order, held as 64-bit keys whose integer
//     order IS the tree order (root map order = lexicographic upper-node
//     origin, tree/RootNode.h:157 + math/Coord.h:157-162; then the upper-node
//     child offset; then the lower-node child offset);
//   * per leaf a storage slot: an active-voxel mask, a sign mask (bit set when
//     the voxel value is negative) and the active values packed in voxel
//     order at the start of a 512-float slot (OnIndex-style: value of active
//     voxel v = vals[slot*512 + rank(v)]).  Every inactive voxel of a narrow
//     band level set holds exactly +background or -background (signed flood
//     fill, tools/SignedFloodFill.h:111-139; trimming,
//     tools/LevelSetTracker.h:473-506; new leaves inherit a +-background tile,
//     tree/InternalNode.h:2874-2876), so the sign mask reproduces it exactly;
//   * node tables: sorted lower/upper node keys with one sign bit per child
//     slot (the +-background tile value of every slot that holds no child) and
//     a small sorted list of root tiles.  A key k has lower-node key k>>12 and
//     upper-node key k>>27.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gbls {

constexpr int LEAF_VOX = 512;
constexpr int LOWER_SLOTS = 4096;
constexpr int UPPER_SLOTS = 32768;
// Coordinates must lie in [-2^20, 2^20): 9 bits of root index per axis.
constexpr int32_t COORD_LIMIT = 1 << 20;
// Supported input range keeps leaves created by dilation inside the key space.
constexpr int32_t COORD_SAFE = COORD_LIMIT - 8192;
constexpr int KEY_INST_SHIFT = 54;
constexpr uint64_t KEY_COORD_MASK = (uint64_t(1) << KEY_INST_SHIFT) - 1;
constexpr int32_t NBR_TILE_POS = -1;  // missing neighbour: +background tile
constexpr int32_t NBR_TILE_NEG = -2;  // missing neighbour: -background tile

// Face order used by every per-leaf neighbour table: -x,+x,-y,+y,-z,+z.
__host__ __device__ inline void face_offset(int f, int& dx, int& dy, int& dz) {
    dx = (f == 0) ? -8 : (f == 1) ? 8 : 0;
    dy = (f == 2) ? -8 : (f == 3) ? 8 : 0;
    dz = (f == 4) ? -8 : (f == 5) ? 8 : 0;
}

__host__ __device__ inline uint64_t leaf_key(int32_t x, int32_t y, int32_t z) {
    const uint64_t rx = uint64_t((x >> 12) + 256), ry = uint64_t((y >> 12) + 256),
                   rz = uint64_t((z >> 12) + 256);
    const uint64_t ux = (x >> 7) & 31, uy = (y >> 7) & 31, uz = (z >> 7) & 31;
    const uint64_t lx = (x >> 3) & 15, ly = (y >> 3) & 15, lz = (z >> 3) & 15;
    return (((rx << 18) | (ry << 9) | rz) << 27) | (((ux << 10) | (uy << 5) | uz) << 12) |
           ((lx << 8) | (ly << 4) | lz);
}

__host__ __device__ inline void key_origin(uint64_t k, int32_t& x, int32_t& y, int32_t& z) {
    const int32_t lx = int32_t((k >> 8) & 15), ly = int32_t((k >> 4) & 15), lz = int32_t(k & 15);
    const int32_t ux = int32_t((k >> 22) & 31), uy = int32_t((k >> 17) & 31),
                  uz = int32_t((k >> 12) & 31);
    const int32_t rx = int32_t((k >> 45) & 511), ry = int32_t((k >> 36) & 511),
                  rz = int32_t((k >> 27) & 511);
    x = (rx - 256) * 4096 + ux * 128 + lx * 8;
    y = (ry - 256) * 4096 + uy * 128 + ly * 8;
    z = (rz - 256) * 4096 + uz * 128 + lz * 8;
}

__host__ __device__ inline uint32_t key_instance(uint64_t k) { return uint32_t(k >> KEY_INST_SHIFT); }

// Key of the face neighbour of leaf k (same instance).
__host__ __device__ inline uint64_t neighbour_key(uint64_t k, int f) {
    int32_t x, y, z, dx, dy, dz;
    key_origin(k, x, y, z);
    face_offset(f, dx, dy, dz);
    return leaf_key(x + dx, y + dy, z + dz) | (k & ~KEY_COORD_MASK);
}

// Lower bound in a sorted key array: first index with a[i] >= key.
__host__ __device__ inline int64_t lower_bound_u64(const uint64_t* a, int64_t n, uint64_t key) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__host__ __device__ inline int64_t find_u64(const uint64_t* a, int64_t n, uint64_t key) {
    const int64_t i = lower_bound_u64(a, n, key);
    return (i < n && a[i] == key) ? i : -1;
}

// Node tables (device pointers, counts).
struct NodeTables {
    const uint64_t* lower_keys;  // [nlower] sorted (leaf key >> 12)
    const uint64_t* lower_sign;  // [nlower * 64]
    const uint64_t* upper_keys;  // [nupper] sorted (leaf key >> 27)
    const uint64_t* upper_sign;  // [nupper * 512]
    const uint64_t* root_keys;   // [nroot] sorted (leaf key >> 27)
    const uint8_t* root_sign;    // [nroot]
    int64_t nlower, nupper, nroot;
};

// Sign (1 = -background) of the tile that covers the leaf-sized region with
// key k, following ValueAccessor::getValue through the node levels
// (tree/ValueAccessor.h:455): lower-node tile, else upper-node tile, else
// root tile, else the (positive) background.
__host__ __device__ inline int tile_sign(const NodeTables& nt, uint64_t k) {
    const int64_t li = find_u64(nt.lower_keys, nt.nlower, k >> 12);
    if (li >= 0) {
        const uint32_t n = uint32_t(k & 4095);
        return int((nt.lower_sign[li * 64 + (n >> 6)] >> (n & 63)) & 1);
    }
    const int64_t ui = find_u64(nt.upper_keys, nt.nupper, k >> 27);
    if (ui >= 0) {
        const uint32_t n = uint32_t((k >> 12) & 32767);
        return int((nt.upper_sign[ui * 512 + (n >> 6)] >> (n & 63)) & 1);
    }
    const int64_t ri = find_u64(nt.root_keys, nt.nroot, k >> 27);
    if (ri >= 0) return nt.root_sign[ri];
    return 0;
}

// A value layout: which voxels of a slot are stored, their packed values,
// and the signs of the others.
struct Layout {
    const uint64_t* amask;  // [slots * 8]
    const uint64_t* smask;  // [slots * 8]
    const float* vals;      // [slots * 512]
};

// ---- bit helpers ---------------------------------------------------------
__device__ __forceinline__ int popc64(uint64_t w) { return __popcll(w); }

// Position of the n-th (0-based) set bit of w (n < popcount(w)), by
// bisection on population counts; always returns a value in [0, 63].
__device__ __forceinline__ int select64(uint64_t w, int n) {
    int pos = 0;
#pragma unroll
    for (int width = 32; width >= 1; width >>= 1) {
        const uint64_t low = w & ((uint64_t(1) << width) - 1);
        const int c = __popcll(low);
        if (n >= c) {
            n -= c;
            w >>= width;
            pos += width;
        } else {
            w = low;
        }
    }
    return pos & 63;
}

// Voxel index of the i-th active voxel of mask m[8] with prefix counts pre[9].
__device__ __forceinline__ int select_voxel(const uint64_t* m, const int* pre, int i) {
    int w = 0;
#pragma unroll
    for (int k = 1; k < 8; ++k) w += (i >= pre[k]) ? 1 : 0;
    return (w << 6) | select64(m[w], i - pre[w]);
}

// ---- 14^3 stencil tile ---------------------------------------------------
// The 19-point stencil (math/Stencils.h:816-863) reaches +-3 voxels along
// each axis, so a leaf needs its 8^3 block plus three-voxel slabs of its six
// face neighbours; the 14^3 box corners are never read.
constexpr int TILE_DIM = 14;
constexpr int TILE_VOX = TILE_DIM * TILE_DIM * TILE_DIM;
constexpr int TILE_POINTS = 512 + 6 * 192;
__device__ __forceinline__ int tile_index(int x, int y, int z) {
    return (x + 3) * (TILE_DIM * TILE_DIM) + (y + 3) * TILE_DIM + (z + 3);
}

// Per-CTA staging of a leaf and its 6 face neighbours.
struct LeafStage {
    uint64_t am[1][8];     // active mask of the centre leaf
    uint64_t sm[1][8];     // sign mask of the centre leaf
    // One 16-byte record per staged leaf r (0 = centre, 1..6 = -x,+x,-y,+y,
    // -z,+z) and 32-bit half word: active half mask, sign half mask, rank of
    // the half's first voxel, and the offset slot*512 of the leaf's values
    // (0 for a tile).  A tile element is staged from one record load.
    uint4 rec[7][16];
    const float* vb;       // the layout's value array (rec offsets are relative to it)
    int slot[7];
};

// Stencil kernels run one leaf per CTA of STAGE_THREADS threads: thread t
// owns bit t of every 64-bit mask word, so the staging below is straight-line
// code with every load independent.
constexpr int STAGE_THREADS = 64;

// Stage the masks of a leaf (slot s) and of its face neighbours nb[6] from
// layout L as half-word records.  Threads 56..63
// load pm[8] (the processed-voxel mask of the centre) when pmask is given.
// Ends with a barrier.
__device__ inline void stage_masks(LeafStage& st, const Layout& L, int s, const int32_t* nb,
                                   const uint64_t* pmask, uint64_t* pm) {
    const int t = threadIdx.x;
    uint32_t clo = 0, c = 0;
    int sl = 0;
    uint64_t a = 0, g = 0;
    if (t < 56) {
        const int r = t >> 3, w = t & 7;
        sl = (r == 0) ? s : nb[r - 1];
        if (sl >= 0) {
            a = L.amask[size_t(sl) * 8 + w];
            g = L.smask[size_t(sl) * 8 + w];
        } else {
            a = 0;
            g = (sl == NBR_TILE_NEG) ? ~uint64_t(0) : uint64_t(0);
        }
        if (r == 0) {
            st.am[0][w] = a;
            st.sm[0][w] = g;
        }
        if (w == 0) st.slot[r] = sl;
        clo = uint32_t(__popc(uint32_t(a)));
        c = clo + uint32_t(__popc(uint32_t(a >> 32)));
    } else if (pmask) {
        pm[t - 56] = pmask[size_t(s) * 8 + (t - 56)];
    }
    // inclusive scan of the popcounts within each group of 8 lanes
    uint32_t v = c;
#pragma unroll
    for (int d = 1; d < 8; d <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, v, d, 8);
        if ((t & 7) >= d) v += u;
    }
    if (t < 56) {
        const int r = t >> 3, w = t & 7;
        const uint32_t base = sl >= 0 ? uint32_t(sl) * uint32_t(LEAF_VOX) : 0u;
        st.rec[r][2 * w] = make_uint4(uint32_t(a), uint32_t(g), v - c, base);
        st.rec[r][2 * w + 1] = make_uint4(uint32_t(a >> 32), uint32_t(g >> 32), v - c + clo, base);
    } else if (t == 56) {
        st.vb = L.vals;
    }
    __syncthreads();
}

// Value of bit bb of the half word whose record is q (packed value, else
// +-gamma by the sign bit).
__device__ __forceinline__ float record_load(const uint4 q, int bb, const float* vb, float gamma) {
    const float inactive = ((q.y >> bb) & 1) ? -gamma : gamma;
    if ((q.x >> bb) & 1) return __ldg(vb + (q.w + q.z + uint32_t(__popc(q.x & ((1u << bb) - 1u)))));
    return inactive;
}

// Fill the 14^3 tile (centre block + three-voxel face slabs).  Thread t
// handles bit t of each centre word and the (t>>3, t&7) column of every slab
// layer; all 26 loads of a thread are independent, and each reads its mask
// bits and rank from one 16-byte half-word record (18 distinct records per
// thread).  Requires blockDim.x == STAGE_THREADS.  No barrier at the end.
__device__ inline void load_tile(float* tile, const LeafStage& st, float gamma) {
    const int t = threadIdx.x;
    const int a = t >> 3, c = t & 7, h = t >> 5, bt = t & 31;
    const float* vb = st.vb;
    float cv[8], fv[18];
#pragma unroll
    for (int k = 0; k < 8; ++k) cv[k] = record_load(st.rec[0][2 * k + h], bt, vb, gamma);
    {
        // -y: bits (5+d)<<3|c of word a (high half); +y: bits d<<3|c (low half);
        // -z: bits c<<3|(5+d) and +z: bits c<<3|d (half c>>2)
        const uint4 qmy = st.rec[3][2 * a + 1], qpy = st.rec[4][2 * a];
        const uint4 qmz = st.rec[5][2 * a + (c >> 2)], qpz = st.rec[6][2 * a + (c >> 2)];
        const int zb = (c & 3) << 3;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            fv[0 * 3 + d] = record_load(st.rec[1][2 * (5 + d) + h], bt, vb, gamma);  // -x: (5+d, a, c)
            fv[1 * 3 + d] = record_load(st.rec[2][2 * d + h], bt, vb, gamma);        // +x: (d, a, c)
            fv[2 * 3 + d] = record_load(qmy, ((5 + d) << 3 | c) & 31, vb, gamma);     // -y: (a, 5+d, c)
            fv[3 * 3 + d] = record_load(qpy, (d << 3) | c, vb, gamma);                // +y: (a, d, c)
            fv[4 * 3 + d] = record_load(qmz, zb | (5 + d), vb, gamma);                // -z: (a, c, 5+d)
            fv[5 * 3 + d] = record_load(qpz, zb | d, vb, gamma);                      // +z: (a, c, d)
        }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) tile[tile_index(k, a, c)] = cv[k];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        tile[tile_index(-3 + d, a, c)] = fv[0 * 3 + d];
        tile[tile_index(8 + d, a, c)] = fv[1 * 3 + d];
        tile[tile_index(a, -3 + d, c)] = fv[2 * 3 + d];
        tile[tile_index(a, 8 + d, c)] = fv[3 * 3 + d];
        tile[tile_index(a, c, -3 + d)] = fv[4 * 3 + d];
        tile[tile_index(a, c, 8 + d)] = fv[5 * 3 + d];
    }
}

// ---- velocity fields (device form of gbls_field_desc) -------------------
struct FieldParams {
    int kind;
    // DEFORMATION: per-coordinate tables tab[2*(i-tab_lo)] = sin(pi i/domain),
    // tab[2*(i-tab_lo)+1] = sin(2 pi i/domain) (same function as the direct
    // evaluation, so identical bits) and the per-substep amplitude.
    const float* tab;
    int tab_lo, tab_n;
    float amp;
    float constant[3];
    int dense_origin[3];
    int dense_dims[3];
    const float* dense;  // device [nx][ny][nz][3]
    float dense_background[3];
    // DENSE with its own transform: world = ijk * ls_scale + ls_translation
    // (the level set's map), grid index = (world - vel_translation) *
    // vel_inv_scale (the velocity grid's inverse map), then trilinear.
    int xform;
    double ls_scale, ls_translation[3], vel_inv_scale, vel_translation[3];
    float domain, period, scale;
    float omega[3];
    float center[3];
    // HOST_SAMPLED: the velocity of active voxel `rank` of leaf l (leaf list
    // order) is sampled[3 * (prefix[l] + rank) ...]
    const float* sampled;
    const int64_t* prefix;
};

}  // namespace gbls

// NanoVDB buffers on the device; see nanovdb_device.h.  The node and leaf
// bytes are those of the host writer (nanovdb_export.cc, itself byte for
// byte nanovdb::tools::createNanoGrid, nanovdb/tools/CreateNanoGrid.h): one
// CTA per node, children found by key range, node statistics combined by one
// thread per node in tree order with the host's double operations (this unit
// is compiled without contraction).
#include "nanovdb_device.h"

#include <cub/cub.cuh>

#include <string>

#include "gbls_internal.cuh"

namespace gbls {
namespace {

using gbls_nano::BBox;
using gbls_nano::NodeStats;
using gbls_nano::put;

void check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return;
    gbls_nano::fail(e == cudaErrorMemoryAllocation ? GBLS_ERR_OUT_OF_MEMORY : GBLS_ERR_CUDA,
                    std::string(what) + ": " + cudaGetErrorString(e));
}

constexpr int LEAF_THREADS = 64;  // thread t owns bit t of every mask word
constexpr int NODE_THREADS = 256;

__device__ inline bool mask_bit(const uint64_t* m, int i) { return (m[i >> 6] >> (i & 63)) & 1; }

// Bounding box of the active voxels of a leaf at origin o.
__device__ inline BBox leaf_bbox(const uint64_t* m, const int32_t* o) {
    BBox b;
    for (int i = 0; i < 512; ++i) {
        if (!mask_bit(m, i)) continue;
        const int32_t c[3] = {o[0] + (i >> 6), o[1] + ((i >> 3) & 7), o[2] + (i & 7)};
        for (int k = 0; k < 3; ++k) {
            b.lo[k] = c[k] < b.lo[k] ? c[k] : b.lo[k];
            b.hi[k] = c[k] > b.hi[k] ? c[k] : b.hi[k];
        }
    }
    return b;
}

// NanoGrid<float> leaf f: bounding box (or origin), flags, value mask,
// statistics and the 512 dense values (inactive: +-background by the sign
// mask).
__global__ void __launch_bounds__(LEAF_THREADS)
k_leaf_float(const NanoDevTree t, int mode, uint8_t* out, size_t leaf_at, NodeStats* stats) {
    const int64_t f = blockIdx.x;
    const int tid = threadIdx.x;
    __shared__ uint64_t m[8], sg[8];
    const int s = t.slot[f];
    if (tid < 8) {
        m[tid] = t.am[size_t(s) * 8 + tid];
        sg[tid] = t.sm[size_t(s) * 8 + tid];
    }
    __syncthreads();
    uint8_t* L = out + leaf_at + gbls_nano::kLeafBytes * size_t(f);
    const float* pv = t.vals + size_t(s) * LEAF_VOX;
    float* V = reinterpret_cast<float*>(L + 96);
    const uint64_t below = (uint64_t(1) << tid) - 1;
    int base = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
        const uint64_t mw = m[w];
        V[w * 64 + tid] = ((mw >> tid) & 1) ? pv[base + __popcll(mw & below)]
                                            : (((sg[w] >> tid) & 1) ? -t.gamma : t.gamma);
        base += __popcll(mw);
    }
    if (tid < 8) reinterpret_cast<uint64_t*>(L + 16)[tid] = m[tid];
    if (tid != 0) return;
    int32_t o[3];
    key_origin(t.keys[f], o[0], o[1], o[2]);
    NodeStats ns;
    if (mode != gbls_nano::kStatsDisable) {
        ns.bbox = leaf_bbox(m, o);
        if (mode >= gbls_nano::kStatsMinMax)
            for (int r = 0; r < base; ++r) ns.stats.add(pv[r]);  // active values in index order
    }
    if (mode == gbls_nano::kStatsDisable || ns.bbox.empty()) {
        memcpy(L, o, 12);
    } else {
        memcpy(L, ns.bbox.lo, 12);
        for (int k = 0; k < 3; ++k) L[12 + k] = uint8_t(ns.bbox.hi[k] - ns.bbox.lo[k]);
        L[15] = 2;  // has a bounding box; rendering enabled
        gbls_nano::put_stats(L, 80, ns.stats, mode);
    }
    if (stats) stats[f] = ns;
}

// Child range [c0, c1) of node key nk among sorted child keys (the child's
// key >> key_shift is its parent's key).
__device__ inline void child_range(uint64_t nk, const uint64_t* child_keys, int64_t nchild, int key_shift,
                                   int64_t& c0, int64_t& c1) {
    c0 = lower_bound_u64(child_keys, nchild, nk << key_shift);
    c1 = lower_bound_u64(child_keys, nchild, (nk + 1) << key_shift);
}

// Child mask and child offsets of an internal node (slot n of a child is the
// low 3*LOG2 bits of its key); returns with the mask in cm after a barrier.
template <int LOG2>
__device__ inline void node_children(uint32_t* cm, uint8_t* N, size_t table_at, int64_t node_at,
                                     const uint64_t* child_keys, int64_t c0, int64_t c1, size_t child_base,
                                     size_t child_bytes) {
    constexpr int NV = 1 << (3 * LOG2);
    for (int w = threadIdx.x; w < NV / 32; w += blockDim.x) cm[w] = 0;
    __syncthreads();
    for (int64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        const int n = int(child_keys[c] & uint64_t(NV - 1));
        atomicOr(&cm[n >> 5], 1u << (n & 31));
        put<int64_t>(N, table_at + 8 * size_t(n), int64_t(child_base + child_bytes * size_t(c)) - node_at);
    }
    __syncthreads();
    for (int w = threadIdx.x; w < NV / 32; w += blockDim.x) put<uint32_t>(N, 32 + NV / 8 + 4 * size_t(w), cm[w]);
}

// NanoGrid<float> internal node i (lower: LOG2 4, children leaves; upper:
// LOG2 5, children lower nodes): child mask and offsets, +-background tile
// values, then origin (Disable) or bounding box, flags and statistics of the
// children combined in tree order.
template <int LOG2>
__global__ void __launch_bounds__(NODE_THREADS)
k_internal_float(const uint64_t* node_keys, const uint64_t* node_sign, int origin_shift, const uint64_t* child_keys,
                 int64_t nchild, int key_shift, size_t base_at, size_t node_bytes, size_t table_at, size_t child_base,
                 size_t child_bytes, const NodeStats* child_stats, NodeStats* out_stats, int mode, float gamma,
                 uint8_t* out) {
    constexpr int NV = 1 << (3 * LOG2);
    __shared__ uint32_t cm[NV / 32];
    const int64_t i = blockIdx.x;
    const uint64_t nk = node_keys[i];
    int64_t c0, c1;
    child_range(nk, child_keys, nchild, key_shift, c0, c1);
    const int64_t at = int64_t(base_at + node_bytes * size_t(i));
    uint8_t* N = out + at;
    node_children<LOG2>(cm, N, table_at, at, child_keys, c0, c1, child_base, child_bytes);
    const uint64_t* sg = node_sign + size_t(i) * (NV / 64);
    for (int n = threadIdx.x; n < NV; n += blockDim.x)
        if (!((cm[n >> 5] >> (n & 31)) & 1))
            put<float>(N, table_at + 8 * size_t(n), ((sg[n >> 6] >> (n & 63)) & 1) ? -gamma : gamma);
    if (threadIdx.x != 0) return;
    if (mode == gbls_nano::kStatsDisable) {
        int32_t o[3];
        key_origin(nk << origin_shift, o[0], o[1], o[2]);
        memcpy(N, o, 12);
        return;
    }
    const bool moments = mode == gbls_nano::kStatsAll;
    NodeStats total;
    for (int64_t c = c0; c < c1; ++c) {  // children are consecutive in tree order, which is their table order
        total.stats.add(child_stats[c].stats, moments);
        total.bbox.add(child_stats[c].bbox);
    }
    gbls_nano::put_bbox(N, 0, total.bbox);  // empty (max, min) when no child has active values
    if (total.bbox.empty()) {
        put<uint64_t>(N, 24, 1);  // no active values: skip rendering
    } else {
        put<uint64_t>(N, 24, 2);
        gbls_nano::put_stats(N, 32 + NV / 4, total.stats, mode);
    }
    out_stats[i] = total;
}

__device__ inline int leaf_active(const uint64_t* am, int s) {
    int n = 0;
    for (int w = 0; w < 8; ++w) n += __popcll(am[size_t(s) * 8 + w]);
    return n;
}

// Value counts per leaf (active + statistics slots), 0 after the last leaf.
__global__ void k_index_counts(const NanoDevTree t, uint64_t nstat, uint64_t* cnt) {
    const int64_t f = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (f < t.nf) cnt[f] = uint64_t(leaf_active(t.am, t.slot[f])) + nstat;
    else if (f == t.nf) cnt[f] = 0;
}

// NanoGrid<ValueOnIndex> leaf f: bounding box (or origin), flags, value mask,
// first value offset, 9-bit prefix sums; with a channel its active values
// and statistics slots.
__global__ void __launch_bounds__(LEAF_THREADS)
k_leaf_index(const NanoDevTree t, uint64_t nstat, uint64_t base, const uint64_t* off, uint8_t* out, size_t leaf_at,
             float* chan, BBox* boxes) {
    const int64_t f = blockIdx.x;
    const int tid = threadIdx.x;
    __shared__ uint64_t m[8];
    const int s = t.slot[f];
    if (tid < 8) m[tid] = t.am[size_t(s) * 8 + tid];
    __syncthreads();
    uint8_t* L = out + leaf_at + gbls_nano::kIndexLeafBytes * size_t(f);
    const uint64_t first = base + off[f];
    int na = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) na += __popcll(m[w]);
    if (chan) {
        const float* pv = t.vals + size_t(s) * LEAF_VOX;
        for (int r = tid; r < na; r += LEAF_THREADS) chan[first + uint64_t(r)] = pv[r];
        for (int k = tid; k < int(nstat); k += LEAF_THREADS) chan[first + uint64_t(na) + uint64_t(k)] = t.gamma;
    }
    if (tid < 8) reinterpret_cast<uint64_t*>(L + 16)[tid] = m[tid];
    if (tid != 0) return;
    int32_t o[3];
    key_origin(t.keys[f], o[0], o[1], o[2]);
    const BBox bx = leaf_bbox(m, o);
    uint8_t flags = nstat ? 16 : 0;
    if (!bx.empty()) {
        memcpy(L, bx.lo, 12);
        for (int k = 0; k < 3; ++k) L[12 + k] = uint8_t(bx.hi[k] - bx.lo[k]);
        flags |= 2;
    } else {
        memcpy(L, o, 12);
    }
    L[15] = flags;
    put<uint64_t>(L, 80, first);
    uint64_t sum = uint64_t(__popcll(m[0])), prefix = sum;
    for (int w = 1, sh = 9; w < 7; ++w, sh += 9) {
        sum += uint64_t(__popcll(m[w]));
        prefix |= sum << sh;
    }
    put<uint64_t>(L, 88, prefix);
    boxes[f] = bx;
}

// NanoGrid<ValueOnIndex> internal node i: child mask and offsets (tile slots
// stay 0), statistics slot offsets, bounding box of the children, flags.
template <int LOG2>
__global__ void __launch_bounds__(NODE_THREADS)
k_internal_index(const uint64_t* node_keys, const uint64_t* child_keys, int64_t nchild, int key_shift, size_t base_at,
                 size_t node_bytes, size_t table_at, size_t child_base, size_t child_bytes, const BBox* child_box,
                 BBox* out_box, int stat_slots, uint64_t first_slot, uint8_t* out) {
    constexpr int NV = 1 << (3 * LOG2);
    __shared__ uint32_t cm[NV / 32];
    const int64_t i = blockIdx.x;
    int64_t c0, c1;
    child_range(node_keys[i], child_keys, nchild, key_shift, c0, c1);
    const int64_t at = int64_t(base_at + node_bytes * size_t(i));
    uint8_t* N = out + at;
    node_children<LOG2>(cm, N, table_at, at, child_keys, c0, c1, child_base, child_bytes);
    if (threadIdx.x != 0) return;
    BBox box;
    for (int64_t c = c0; c < c1; ++c) box.add(child_box[c]);
    if (stat_slots)
        for (int k = 0; k < 4; ++k)
            put<uint64_t>(N, 32 + NV / 4 + 8 * size_t(k), first_slot + 4 * uint64_t(i) + uint64_t(k));
    gbls_nano::put_bbox(N, 0, box);
    put<uint64_t>(N, 24, box.empty() ? 1 : 2);
    out_box[i] = box;
}

// The background slot and the internal nodes' statistics slots of a channel.
__global__ void k_channel_head(float* chan, uint64_t n, float bg) {
    const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
    if (i < n) chan[i] = bg;
}

// CRC-32 of each 4 KiB block of p[0, n) (the last block takes the
// remainder), table-driven, one thread per block.
__global__ void k_crc_blocks(const uint8_t* p, size_t n, size_t blocks, uint32_t* sums) {
    __shared__ uint32_t lut[256];
    for (int j = threadIdx.x; j < 256; j += blockDim.x) {
        uint32_t c = uint32_t(j);
        for (int k = 0; k < 8; ++k) c = (c >> 1) ^ ((c & 1) ? 0xEDB88320u : 0u);
        lut[j] = c;
    }
    __syncthreads();
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= blocks) return;
    size_t len = size_t(1) << 12;
    if (i + 1 == blocks) len += n - (blocks << 12);
    const uint8_t* q = p + (i << 12);
    uint32_t crc = ~0u;
    size_t k = 0;
    for (; k + 16 <= len; k += 16) {
        const uint4 u = *reinterpret_cast<const uint4*>(q + k);
        const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int b = 0; b < 4; ++b) crc = lut[(crc ^ (w[j] >> (8 * b))) & 0xFF] ^ (crc >> 8);
    }
    for (; k < len; ++k) crc = lut[(crc ^ q[k]) & 0xFF] ^ (crc >> 8);
    sums[i] = ~crc;
}

__global__ void __launch_bounds__(LEAF_THREADS)
k_gather_leaves(const uint8_t* buf, const uint64_t* at, int64_t n, uint64_t* masks, float* values) {
    const int64_t i = blockIdx.x;
    if (i >= n) return;
    const uint8_t* L = buf + at[i];
    const int tid = threadIdx.x;
    if (tid < 8) masks[i * 8 + tid] = reinterpret_cast<const uint64_t*>(L + 16)[tid];
    const float4* v = reinterpret_cast<const float4*>(L + 96);
    float4* o = reinterpret_cast<float4*>(values + i * LEAF_VOX);
    for (int j = tid; j < LEAF_VOX / 4; j += LEAF_THREADS) o[j] = v[j];
}

// Bounds-checked reads of a probed buffer (any alignment).
struct NanoBytes {
    const uint8_t* b;
    uint64_t size;
    template <class T>
    __device__ bool get(uint64_t at, T& v) const {
        if (at > size || sizeof(T) > size - at) return false;
        memcpy(&v, b + at, sizeof(T));
        return true;
    }
    __device__ bool bit(uint64_t at, uint32_t n, bool& v) const {
        uint8_t byte = 0;
        const bool ok = get(at + (n >> 3), byte);
        v = (byte >> (n & 7)) & 1;
        return ok;
    }
};

// ReadAccessor::getValue / isActive of a NanoGrid<float> (type 1) or
// NanoGrid<ValueOnIndex> (type 20) at one index coordinate: root tiles
// searched in table order by key, internal nodes through their child masks
// and tables, the leaf's value (float) or its value index by the 9-bit
// prefix-sum decode (nanovdb/NanoVDB.h:4144-4170).  err bit 1: a read
// outside the buffer, bit 2: another grid type, bit 4: no output array for
// the type.
__global__ void k_probe(const uint8_t* buf, uint64_t size, const int32_t* ijk, int64_t n, float* fv, uint64_t* iv,
                        uint8_t* act, int* err) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const NanoBytes g{buf, size};
    uint32_t type = 0;
    if (!g.get(636, type)) { atomicOr(err, 1); return; }
    const bool isf = type == 1;
    if (!isf && type != 20) { atomicOr(err, 2); return; }
    if (isf ? !fv : !iv) { atomicOr(err, 4); return; }
    const int32_t x = ijk[3 * i], y = ijk[3 * i + 1], z = ijk[3 * i + 2];
    bool ok = true, active = false;
    float fval = 0.0f;
    uint64_t ival = 0;
    int64_t rel = 0;
    ok &= g.get(gbls_nano::kGridBytes + 24, rel);
    const uint64_t root = gbls_nano::kGridBytes + uint64_t(rel);
    uint32_t table = 0;
    ok &= g.get(root + 24, table);
    if (isf) ok &= g.get(root + 28, fval);  // background
    else ok &= g.get(root + 32, ival);
    const uint64_t tiles = root + (isf ? gbls_nano::kRootBytes : gbls_nano::kIndexRootBytes);
    const uint64_t key = uint64_t(uint32_t(z) >> 12) | (uint64_t(uint32_t(y) >> 12) << 21) |
                         (uint64_t(uint32_t(x) >> 12) << 42);
    uint64_t node = 0;
    for (uint32_t t = 0; ok && t < table; ++t) {
        const uint64_t at = tiles + gbls_nano::kTileBytes * t;
        uint64_t k = 0;
        ok &= g.get(at, k);
        if (k != key) continue;
        int64_t child = 0;
        ok &= g.get(at + 8, child);
        if (child) {
            node = root + uint64_t(child);
        } else {
            uint32_t state = 0;
            ok &= g.get(at + 16, state);
            active = state != 0;
            if (isf) ok &= g.get(at + 20, fval);
            else ok &= g.get(at + 24, ival);
        }
        break;
    }
    // upper (LOG2 5 over 7-bit children), then lower (LOG2 4 over leaves)
    for (int level = 0; ok && node && level < 2; ++level) {
        const int log2 = level == 0 ? 5 : 4, cshift = level == 0 ? 7 : 3;
        const uint32_t mask = (1u << (log2 + cshift)) - 1u, nv = 1u << (3 * log2);
        const uint32_t slot = (((uint32_t(x) & mask) >> cshift) << (2 * log2)) |
                              (((uint32_t(y) & mask) >> cshift) << log2) | ((uint32_t(z) & mask) >> cshift);
        const uint64_t tab = node + (level == 0 ? gbls_nano::kUpperTableAt : gbls_nano::kLowerTableAt);
        bool is_child = false;
        ok &= g.bit(node + 32 + nv / 8, slot, is_child);
        if (is_child) {
            int64_t off = 0;
            ok &= g.get(tab + 8 * uint64_t(slot), off);
            node += uint64_t(off);
            continue;
        }
        ok &= g.bit(node + 32, slot, active);
        if (isf) ok &= g.get(tab + 8 * uint64_t(slot), fval);
        else ok &= g.get(tab + 8 * uint64_t(slot), ival);
        node = 0;
    }
    if (ok && node) {  // a leaf
        const uint32_t v = ((uint32_t(x) & 7u) << 6) | ((uint32_t(y) & 7u) << 3) | (uint32_t(z) & 7u);
        uint64_t w = 0;
        ok &= g.get(node + 16 + 8 * uint64_t(v >> 6), w);
        const uint64_t bitm = uint64_t(1) << (v & 63u);
        active = (w & bitm) != 0;
        if (isf) {
            ok &= g.get(node + 96 + 4 * uint64_t(v), fval);
        } else if (!active) {
            ival = 0;  // the background's index
        } else {
            uint64_t offset = 0, prefix = 0;
            ok &= g.get(node + 80, offset);
            ok &= g.get(node + 88, prefix);
            uint32_t word = v >> 6;
            ival = offset + uint64_t(__popcll(w & (bitm - 1u)));
            if (word--) ival += (prefix >> (9u * word)) & 511u;
        }
    }
    if (!ok) {
        atomicOr(err, 1);
        return;
    }
    if (isf) fv[i] = fval;
    else iv[i] = ival;
    if (act) act[i] = active ? 1 : 0;
}

template <class T>
T* scratch(size_t n, cudaStream_t s) {
    void* p = nullptr;
    check(cudaMallocAsync(&p, (n ? n : 1) * sizeof(T), s), "cudaMallocAsync");
    return static_cast<T*>(p);
}

}  // namespace

void nano_float_nodes(const NanoDevTree& t, int mode, uint8_t* out, const gbls_nano::FloatLayout& L,
                      std::vector<NodeStats>& upper_stats, cudaStream_t s) {
    const bool st = mode != gbls_nano::kStatsDisable;
    NodeStats* ls = st ? scratch<NodeStats>(size_t(t.nf), s) : nullptr;
    NodeStats* los = st ? scratch<NodeStats>(size_t(t.nl), s) : nullptr;
    NodeStats* us = st ? scratch<NodeStats>(size_t(t.nu), s) : nullptr;
    if (t.nf) k_leaf_float<<<unsigned(t.nf), LEAF_THREADS, 0, s>>>(t, mode, out, L.leaf_at, ls);
    if (t.nl)
        k_internal_float<4><<<unsigned(t.nl), NODE_THREADS, 0, s>>>(
            t.lower_keys, t.lower_sign, 12, t.keys, t.nf, 12, L.lower_at, gbls_nano::kLowerBytes,
            gbls_nano::kLowerTableAt, L.leaf_at, gbls_nano::kLeafBytes, ls, los, mode, t.gamma, out);
    if (t.nu)
        k_internal_float<5><<<unsigned(t.nu), NODE_THREADS, 0, s>>>(
            t.upper_keys, t.upper_sign, 27, t.lower_keys, t.nl, 15, L.upper_at, gbls_nano::kUpperBytes,
            gbls_nano::kUpperTableAt, L.lower_at, gbls_nano::kLowerBytes, los, us, mode, t.gamma, out);
    check(cudaGetLastError(), "NanoGrid<float> node kernels");
    upper_stats.clear();
    if (st) {
        upper_stats.resize(size_t(t.nu));
        if (t.nu)
            check(cudaMemcpyAsync(upper_stats.data(), us, size_t(t.nu) * sizeof(NodeStats), cudaMemcpyDeviceToHost, s),
                  "upper statistics");
        check(cudaFreeAsync(ls, s), "cudaFreeAsync");
        check(cudaFreeAsync(los, s), "cudaFreeAsync");
        check(cudaFreeAsync(us, s), "cudaFreeAsync");
    }
    check(cudaStreamSynchronize(s), "NanoGrid<float> nodes");
}

uint64_t nano_index_offsets(const NanoDevTree& t, bool stats, bool tiles, uint64_t** leaf_off, cudaStream_t s) {
    const uint64_t nstat = stats ? 4 : 0;
    const int64_t n = t.nf + 1;
    uint64_t* cnt = scratch<uint64_t>(size_t(n), s);
    uint64_t* off = scratch<uint64_t>(size_t(n), s);
    k_index_counts<<<unsigned((n + 255) / 256), 256, 0, s>>>(t, nstat, cnt);
    check(cudaGetLastError(), "k_index_counts");
    size_t bytes = 0;
    check(cub::DeviceScan::ExclusiveSum(nullptr, bytes, cnt, off, int(n), s), "scan size");
    void* tmp = scratch<uint8_t>(bytes, s);
    check(cub::DeviceScan::ExclusiveSum(tmp, bytes, cnt, off, int(n), s), "scan");
    uint64_t last = 0;
    check(cudaMemcpyAsync(&last, off + t.nf, sizeof(last), cudaMemcpyDeviceToHost, s), "value count");
    check(cudaFreeAsync(tmp, s), "cudaFreeAsync");
    check(cudaFreeAsync(cnt, s), "cudaFreeAsync");
    check(cudaStreamSynchronize(s), "index offsets");
    *leaf_off = off;
    return gbls_nano::index_leaf_base(t.nu, t.nl, stats, tiles) + last;
}

void nano_index_nodes(const NanoDevTree& t, bool stats, bool tiles, int channels, const uint64_t* leaf_off,
                      uint8_t* out, const gbls_nano::IndexLayout& L, std::vector<BBox>& upper_box, cudaStream_t s) {
    const uint64_t nstat = stats ? 4 : 0;
    const uint64_t base = gbls_nano::index_leaf_base(t.nu, t.nl, stats, tiles);
    BBox* lb = scratch<BBox>(size_t(t.nf), s);
    BBox* lob = scratch<BBox>(size_t(t.nl), s);
    BBox* ub = scratch<BBox>(size_t(t.nu), s);
    float* chan = channels ? reinterpret_cast<float*>(out + L.blind_at) : nullptr;
    if (chan) k_channel_head<<<unsigned((base + 255) / 256), 256, 0, s>>>(chan, base, t.gamma);
    if (t.nf)
        k_leaf_index<<<unsigned(t.nf), LEAF_THREADS, 0, s>>>(t, nstat, base, leaf_off, out, L.leaf_at, chan, lb);
    const int slots = tiles && stats;
    if (t.nl)
        k_internal_index<4><<<unsigned(t.nl), NODE_THREADS, 0, s>>>(
            t.lower_keys, t.keys, t.nf, 12, L.lower_at, gbls_nano::kLowerBytes, gbls_nano::kLowerTableAt, L.leaf_at,
            gbls_nano::kIndexLeafBytes, lb, lob, slots, 1 + nstat + nstat * uint64_t(t.nu), out);
    if (t.nu)
        k_internal_index<5><<<unsigned(t.nu), NODE_THREADS, 0, s>>>(
            t.upper_keys, t.lower_keys, t.nl, 15, L.upper_at, gbls_nano::kUpperBytes, gbls_nano::kUpperTableAt,
            L.lower_at, gbls_nano::kLowerBytes, lob, ub, slots, 1 + nstat, out);
    check(cudaGetLastError(), "NanoGrid<ValueOnIndex> node kernels");
    upper_box.assign(size_t(t.nu), BBox());
    if (t.nu)
        check(cudaMemcpyAsync(upper_box.data(), ub, size_t(t.nu) * sizeof(BBox), cudaMemcpyDeviceToHost, s),
              "upper boxes");
    check(cudaFreeAsync(lb, s), "cudaFreeAsync");
    check(cudaFreeAsync(lob, s), "cudaFreeAsync");
    check(cudaFreeAsync(ub, s), "cudaFreeAsync");
    check(cudaStreamSynchronize(s), "NanoGrid<ValueOnIndex> nodes");
}

uint32_t nano_blocked_crc(const uint8_t* p, size_t n, cudaStream_t s) {
    const size_t blocks = gbls_nano::crc_blocks(n);
    std::vector<uint32_t> sums(blocks);
    if (blocks) {
        uint32_t* d = scratch<uint32_t>(blocks, s);
        k_crc_blocks<<<unsigned((blocks + 127) / 128), 128, 0, s>>>(p, n, blocks, d);
        check(cudaGetLastError(), "k_crc_blocks");
        check(cudaMemcpyAsync(sums.data(), d, blocks * 4, cudaMemcpyDeviceToHost, s), "block checksums");
        check(cudaFreeAsync(d, s), "cudaFreeAsync");
        check(cudaStreamSynchronize(s), "blocked CRC");
    }
    return gbls_nano::crc_of_blocks(sums, n);
}

void nano_gather_leaves(const uint8_t* buf, const uint64_t* at, int64_t n, uint64_t* masks, float* values,
                        cudaStream_t s) {
    if (n <= 0) return;
    k_gather_leaves<<<unsigned(n), LEAF_THREADS, 0, s>>>(buf, at, n, masks, values);
    check(cudaGetLastError(), "k_gather_leaves");
}

int nano_probe(const uint8_t* buf, uint64_t size, const int32_t* ijk, int64_t n, float* values, uint64_t* indices,
               uint8_t* active, cudaStream_t s) {
    int* err = scratch<int>(1, s);
    check(cudaMemsetAsync(err, 0, sizeof(int), s), "cudaMemsetAsync");
    if (n > 0) k_probe<<<unsigned((n + 127) / 128), 128, 0, s>>>(buf, size, ijk, n, values, indices, active, err);
    check(cudaGetLastError(), "k_probe");
    int e = 0;
    check(cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, s), "probe status");
    check(cudaFreeAsync(err, s), "cudaFreeAsync");
    check(cudaStreamSynchronize(s), "probe");
    return e;
}

}  // namespace gbls

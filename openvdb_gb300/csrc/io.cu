// Device side of the host exchange format; see io.h.
#include "io.h"

#include "gbls_internal.cuh"

namespace gbls {
namespace {

constexpr int PACK_THREADS = 64;   // thread t owns bit t of every mask word
constexpr int NODE_THREADS = 256;

__global__ void __launch_bounds__(PACK_THREADS)
k_pack_leaves(int64_t n, const int32_t* perm, const uint64_t* in_masks, const float* in_vals, float gamma,
              uint64_t* am, uint64_t* sm, float* vals, unsigned long long* err) {
    const int64_t l = blockIdx.x;
    if (l >= n) return;
    const int64_t src = perm ? int64_t(perm[l]) : l;
    const int t = threadIdx.x;
    __shared__ uint64_t m[8];
    __shared__ uint32_t neg[8][2];
    if (t < 8) m[t] = in_masks[src * 8 + t];
    __syncthreads();
    const uint64_t below = (uint64_t(1) << t) - 1;
    const float* v = in_vals + src * LEAF_VOX;
    float* out = vals + l * LEAF_VOX;
    int base = 0;
    bool bad = false;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
        const uint64_t mw = m[w];
        const float x = v[w * 64 + t];
        if ((mw >> t) & 1) out[base + __popcll(mw & below)] = x;
        else bad |= !(x == gamma || x == -gamma);
        // the sign mask records x < 0 for every voxel, active or not
        const uint32_t b = __ballot_sync(0xffffffffu, x < 0.0f);
        if ((t & 31) == 0) neg[w][t >> 5] = b;
        base += __popcll(mw);
    }
    if (bad) atomicOr(err, IO_ERR_LEAF_VALUE);
    __syncthreads();
    if (t < 8) {
        am[l * 8 + t] = m[t];
        sm[l * 8 + t] = uint64_t(neg[t][0]) | (uint64_t(neg[t][1]) << 32);
    }
}

__device__ __forceinline__ bool origin_ok(const int32_t* o) {
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) ok &= (o[a] % 8 == 0) && o[a] >= -COORD_SAFE && o[a] < COORD_SAFE;
    return ok;
}

__global__ void k_leaf_keys(int64_t n, const int32_t* orig, const uint64_t* lower_keys, int64_t nlower,
                            uint64_t* keys, int32_t* slot, unsigned long long* err) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const int32_t* o = orig + 3 * i;
    bool bad = !origin_ok(o);
    const uint64_t k = leaf_key(o[0], o[1], o[2]);
    if (i > 0) {
        const int32_t* q = o - 3;
        if (!(leaf_key(q[0], q[1], q[2]) < k)) bad = true;
    }
    if (find_u64(lower_keys, nlower, k >> 12) < 0) bad = true;
    keys[i] = k;
    slot[i] = int32_t(i);
    if (bad) atomicOr(err, IO_ERR_KEYS);
}

__global__ void k_free_slots(int64_t n, int32_t top, int32_t* free_slots) {
    const int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (j < n) free_slots[j] = int32_t(top - 1 - j);
}

// Child bitmap of node `nk` (one bit per slot) in shared memory.
__device__ void child_bitmap(uint32_t* bits, int nwords, uint64_t nk, int shift, const uint64_t* child_keys,
                             int64_t nchild) {
    __shared__ int64_t range[2];
    for (int i = threadIdx.x; i < nwords; i += blockDim.x) bits[i] = 0;
    if (threadIdx.x == 0) {
        range[0] = lower_bound_u64(child_keys, nchild, nk << shift);
        range[1] = lower_bound_u64(child_keys, nchild, (nk + 1) << shift);
    }
    __syncthreads();
    const uint64_t slot_mask = (uint64_t(1) << shift) - 1;
    for (int64_t j = range[0] + threadIdx.x; j < range[1]; j += blockDim.x) {
        const uint32_t q = uint32_t(child_keys[j] & slot_mask);
        atomicOr(bits + (q >> 5), 1u << (q & 31));
    }
    __syncthreads();
}

__global__ void __launch_bounds__(NODE_THREADS)
k_node_signs(int64_t n, int shift, const uint64_t* node_keys, const int32_t* perm, const float* tiles,
             const uint64_t* child_keys, int64_t nchild, float gamma, uint64_t* sign, unsigned long long* err,
             unsigned long long err_bit) {
    const int64_t i = blockIdx.x;
    if (i >= n) return;
    __shared__ uint32_t bits[UPPER_SLOTS / 32];
    const int slots = 1 << shift;
    child_bitmap(bits, slots / 32, node_keys[i], shift, child_keys, nchild);
    const float* tl = tiles + size_t(perm ? perm[i] : i) * size_t(slots);
    // 32-bit halves of the 64-bit sign words (little-endian word layout)
    uint32_t* out = reinterpret_cast<uint32_t*>(sign + i * (slots / 64));
    bool bad = false;
    for (int q0 = 0; q0 < slots; q0 += NODE_THREADS) {
        const int q = q0 + threadIdx.x;
        const bool child = (bits[q >> 5] >> (q & 31)) & 1;
        const float x = tl[q];
        if (!child) bad |= !(x == gamma || x == -gamma);
        const uint32_t b = __ballot_sync(0xffffffffu, !child && x < 0.0f);
        if ((threadIdx.x & 31) == 0) out[q >> 5] = b;
    }
    if (bad) atomicOr(err, err_bit);
}

__global__ void k_leaf_headers(int64_t n, const uint64_t* keys, const int32_t* slot, const uint64_t* am,
                               int32_t* origins, uint64_t* masks) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n * 8) return;
    const int64_t l = i >> 3;
    const int w = int(i & 7);
    masks[i] = am[size_t(slot[l]) * 8 + w];
    if (w < 3) {
        int32_t o[3];
        key_origin(keys[l], o[0], o[1], o[2]);
        origins[l * 3 + w] = o[w];
    }
}

__global__ void __launch_bounds__(NODE_THREADS)
k_node_tiles(int64_t n, int shift, const uint64_t* node_keys, const uint64_t* sign, const uint64_t* child_keys,
             int64_t nchild, float gamma, float* tiles) {
    const int64_t i = blockIdx.x;
    if (i >= n) return;
    __shared__ uint32_t bits[UPPER_SLOTS / 32];
    const int slots = 1 << shift;
    child_bitmap(bits, slots / 32, node_keys[i], shift, child_keys, nchild);
    const uint32_t* sg = reinterpret_cast<const uint32_t*>(sign + i * (slots / 64));
    float* out = tiles + size_t(i) * size_t(slots);
    for (int q = threadIdx.x; q < slots; q += NODE_THREADS) {
        const bool child = (bits[q >> 5] >> (q & 31)) & 1;
        out[q] = child ? 0.0f : (((sg[q >> 5] >> (q & 31)) & 1) ? -gamma : gamma);
    }
}

}  // namespace

void launch_leaf_keys(int64_t n, const int32_t* origins, const uint64_t* lower_keys, int64_t nlower,
                      uint64_t* keys, int32_t* slot, unsigned long long* err, cudaStream_t s) {
    if (n <= 0) return;
    k_leaf_keys<<<unsigned((n + 255) / 256), 256, 0, s>>>(n, origins, lower_keys, nlower, keys, slot, err);
}

void launch_free_slots(int64_t n, int32_t top, int32_t* free_slots, cudaStream_t s) {
    if (n <= 0) return;
    k_free_slots<<<unsigned((n + 255) / 256), 256, 0, s>>>(n, top, free_slots);
}

void launch_pack_leaves(int64_t n, const int32_t* perm, const uint64_t* in_masks, const float* in_vals,
                        float gamma, uint64_t* am, uint64_t* sm, float* vals, unsigned long long* err,
                        cudaStream_t s) {
    if (n > 0) k_pack_leaves<<<unsigned(n), PACK_THREADS, 0, s>>>(n, perm, in_masks, in_vals, gamma, am, sm, vals, err);
}

void launch_node_signs(int64_t n, int shift, const uint64_t* node_keys, const int32_t* perm, const float* tiles,
                       const uint64_t* child_keys, int64_t nchild, float gamma, uint64_t* sign,
                       unsigned long long* err, unsigned long long err_bit, cudaStream_t s) {
    if (n > 0)
        k_node_signs<<<unsigned(n), NODE_THREADS, 0, s>>>(n, shift, node_keys, perm, tiles, child_keys, nchild,
                                                            gamma, sign, err, err_bit);
}

void launch_leaf_headers(int64_t n, const uint64_t* keys, const int32_t* slot, const uint64_t* am,
                         int32_t* origins, uint64_t* masks, cudaStream_t s) {
    if (n > 0)
        k_leaf_headers<<<unsigned((n * 8 + 255) / 256), 256, 0, s>>>(n, keys, slot, am, origins, masks);
}

void launch_node_tiles(int64_t n, int shift, const uint64_t* node_keys, const uint64_t* sign,
                       const uint64_t* child_keys, int64_t nchild, float gamma, float* tiles, cudaStream_t s) {
    if (n > 0)
        k_node_tiles<<<unsigned(n), NODE_THREADS, 0, s>>>(n, shift, node_keys, sign, child_keys, nchild, gamma,
                                                            tiles);
}

}  // namespace gbls

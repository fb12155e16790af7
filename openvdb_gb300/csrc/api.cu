// C ABI of the GB300 narrow-band level-set library (include/gbls.h).
//
// Host orchestration of LevelSetAdvection::advect (tools/LevelSetAdvect.h:
// 338-418) and LevelSetTracker::track (tools/LevelSetTracker.h:302-315) over
// the device tree described in gbls_internal.cuh.
#include <cub/cub.cuh>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <functional>
#include <memory>
#include <cstdlib>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gbls.h"
#include "adjoint.h"
#include "cfl_clock.h"
#include "gbls_internal.cuh"
#include "filter_ops.cuh"
#include "io.h"
#include "morph_ops.cuh"
#include "host_grid.h"
#include "nanovdb_device.h"
#include "stencil.h"
#include "stencil_f64.h"
#include "stencil_ops.cuh"
#include "topology.cuh"
#include "volume.h"

using namespace gbls;

namespace {

thread_local std::string g_last_error;
thread_local int g_device = 0;

struct Error {
    int code;
    std::string msg;
};

[[noreturn]] void fail(int code, const std::string& msg) { throw Error{code, msg}; }

void cuda_check(cudaError_t e, const char* what, int line) {
    if (e != cudaSuccess) {
        if (e == cudaErrorMemoryAllocation)
            fail(GBLS_ERR_OUT_OF_MEMORY, std::string(what) + ": " + cudaGetErrorString(e));
        fail(GBLS_ERR_CUDA, std::string(what) + " (line " + std::to_string(line) + "): " +
                                cudaGetErrorString(e));
    }
}
#define CU(x) cuda_check((x), #x, __LINE__)

template <class F>
int guarded(F&& f) {
    try {
        f();
        return GBLS_OK;
    } catch (const Error& e) {
        g_last_error = e.msg;
        return e.code;
    } catch (const gbls_nano::ExportError& e) {
        g_last_error = e.msg;
        return e.code;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return GBLS_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return GBLS_ERR_RUNTIME;
    }
}

// Growable device array.
template <class T>
struct DevArray {
    T* p = nullptr;
    size_t cap = 0;
    DevArray() = default;
    DevArray(const DevArray&) = delete;
    DevArray& operator=(const DevArray&) = delete;
    ~DevArray() {
        if (p) cudaFree(p);
    }
    // Ensure room for n elements, keeping the first `keep` elements.
    void reserve(size_t n, cudaStream_t s, size_t keep = 0, double growth = 1.5) {
        if (n <= cap) return;
        size_t nc = std::max(n, size_t(double(cap) * growth));
        if (nc < 16) nc = 16;
        T* q = nullptr;
        CU(cudaMalloc(&q, nc * sizeof(T)));
        if (p && keep) CU(cudaMemcpyAsync(q, p, keep * sizeof(T), cudaMemcpyDeviceToDevice, s));
        if (p) {
            CU(cudaStreamSynchronize(s));
            CU(cudaFree(p));
        }
        p = q;
        cap = nc;
    }
    void upload(const T* h, size_t n, cudaStream_t s) {
        reserve(n, s);
        if (n) CU(cudaMemcpyAsync(p, h, n * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void download(T* h, size_t n, cudaStream_t s) const {
        if (n) CU(cudaMemcpyAsync(h, p, n * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
};

inline unsigned blocks_for(int64_t n, int threads) { return unsigned((n + threads - 1) / threads); }

// ---------------------------------------------------------------------------
// topology kernels
// ---------------------------------------------------------------------------

// Candidate leaves created by NN_FACE dilation: a missing face neighbour
// that would receive active bits.  Emits (key << 1) | tile sign.
__global__ void k_emit_candidates(int64_t n, const uint64_t* keys, const int32_t* slot,
                                  const int32_t* nbr, const uint64_t* am, uint64_t* cand,
                                  unsigned long long* count, const uint8_t* inst_run) {
    const int64_t l = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (l >= n) return;
    if (inst_run && !inst_run[key_instance(keys[l])]) return;
    const int32_t* nb = nbr + 6 * l;
    bool any_missing = false;
    for (int f = 0; f < 6; ++f) any_missing |= nb[f] < 0;
    if (!any_missing) return;
    uint64_t m[8];
    const int s = slot[l];
    for (int w = 0; w < 8; ++w) m[w] = am[size_t(s) * 8 + w];
    for (int f = 0; f < 6; ++f) {
        if (nb[f] >= 0) continue;
        if (!face_layer_nonzero(m, f)) continue;
        const uint64_t nk = neighbour_key(keys[l], f);
        if (!origin_in_range(nk)) continue;
        const unsigned long long at = atomicAdd(count, 1ull);
        cand[at] = (nk << 1) | uint64_t(nb[f] == NBR_TILE_NEG ? 1 : 0);
    }
}

// Give the sorted unique new leaves their slots; their masks start empty and
// every voxel takes the tile value (tree/InternalNode.h:2874-2876).
// The count is n, or *n_dev when n_dev is set (launched for a capacity).
__global__ void k_new_leaves(int64_t n, const unsigned long long* n_dev, const uint64_t* cand,
                             const int32_t* free_slots, int64_t nfree, uint64_t* new_keys, int32_t* new_slots,
                             uint64_t* am, uint64_t* sm) {
    const int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (n_dev) n = int64_t(*n_dev);
    if (j >= n) return;
    const uint64_t c = cand[j];
    const int32_t s = free_slots[nfree - 1 - j];
    new_keys[j] = c >> 1;
    new_slots[j] = s;
    const uint64_t fill = (c & 1) ? ~uint64_t(0) : uint64_t(0);
    for (int w = 0; w < 8; ++w) {
        am[size_t(s) * 8 + w] = 0;
        sm[size_t(s) * 8 + w] = fill;
    }
}

// Merge two sorted, disjoint key lists (with their slots) into tree order.
// nb is *nb_dev when nb_dev is set.
__global__ void k_merge(int64_t na, const uint64_t* ka, const int32_t* sa, int64_t nb,
                        const unsigned long long* nb_dev, const uint64_t* kb, const int32_t* sb, uint64_t* ko,
                        int32_t* so) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (nb_dev) nb = int64_t(*nb_dev);
    if (i < na) {
        const int64_t pos = i + lower_bound_u64(kb, nb, ka[i]);
        ko[pos] = ka[i];
        so[pos] = sa[i];
    } else if (i < na + nb) {
        const int64_t j = i - na;
        const int64_t pos = j + lower_bound_u64(ka, na, kb[j]);
        ko[pos] = kb[j];
        so[pos] = sb[j];
    }
}

// Face-neighbour table: slot of the neighbour leaf, else the sign of the
// tile covering it.
__global__ void k_build_nbr(int64_t n, const uint64_t* keys, const int32_t* slot, NodeTables nt,
                            int32_t* nbr) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n * 6) return;
    const int64_t l = i / 6;
    const int f = int(i - l * 6);
    const uint64_t nk = neighbour_key(keys[l], f);
    int32_t r;
    if (!origin_in_range(nk)) {
        r = NBR_TILE_POS;
    } else {
        const int64_t j = find_u64(keys, n, nk);
        r = (j >= 0) ? slot[j] : (tile_sign(nt, nk) ? NBR_TILE_NEG : NBR_TILE_POS);
    }
    nbr[i] = r;
}

// NN_FACE dilation of every leaf mask into dmask (8 threads per leaf).
__global__ void k_dilate(int64_t n, const int32_t* slot, const int32_t* nbr, const uint64_t* am,
                         uint64_t* dmask, const uint64_t* keys, const uint8_t* inst_run) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n * 8) return;
    const int64_t l = i >> 3;
    const int x = int(i & 7);
    const int s = slot[l];
    const int32_t* nb = nbr + 6 * l;
    const uint64_t* own = am + size_t(s) * 8;
    if (inst_run && !inst_run[key_instance(keys[l])]) {  // finished instance: unchanged
        dmask[size_t(s) * 8 + x] = own[x];
        return;
    }
    auto P = [&](int f) -> const uint64_t* { return nb[f] >= 0 ? am + size_t(nb[f]) * 8 : nullptr; };
    dmask[size_t(s) * 8 + x] = dilate_word(own, x, P(0), P(1), P(2), P(3), P(4), P(5));
}

// NN_FACE erosion of every leaf mask (tools/Morphology.h NodeMaskOp::erode6
// over 8-bit z rows; missing neighbours count as inactive, empty leaves stay
// empty).  8 threads per leaf.
__global__ void k_erode(int64_t n, const int32_t* slot, const int32_t* nbr, const uint64_t* in,
                        uint64_t* out) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n * 8) return;
    const int64_t l = i >> 3;
    const int x = int(i & 7);
    const int s = slot[l];
    const int32_t* nb = nbr + 6 * l;
    const uint64_t* own = in + size_t(s) * 8;
    auto W = [&](int f, int word) -> uint64_t { return nb[f] >= 0 ? in[size_t(nb[f]) * 8 + word] : 0; };
    const uint64_t w = own[x];
    uint64_t e = w;
    e &= ((w << 1) & 0xFEFEFEFEFEFEFEFEull) | ((W(4, x) >> 7) & 0x0101010101010101ull);
    e &= ((w >> 1) & 0x7F7F7F7F7F7F7F7Full) | ((W(5, x) << 7) & 0x8080808080808080ull);
    e &= (w << 8) | (W(2, x) >> 56);
    e &= (w >> 8) | (W(3, x) << 56);
    e &= (x > 0) ? own[x - 1] : W(0, 7);
    e &= (x < 7) ? own[x + 1] : W(1, 0);
    out[size_t(s) * 8 + x] = e;
}

// m[s] &= ~a[s] over the leaves (voxels activated by a dilation).
__global__ void k_andnot(int64_t n, const int32_t* slot, uint64_t* m, const uint64_t* a) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n * 8) return;
    const size_t k = size_t(slot[i >> 3]) * 8 + (i & 7);
    m[k] &= ~a[k];
}

// Lower nodes missing for new leaves (rare): append lower keys.
__global__ void k_missing_lower(int64_t n, const unsigned long long* n_dev, const uint64_t* new_keys,
                                const uint64_t* lower_keys, int64_t nlower, uint64_t* out,
                                unsigned long long* count) {
    const int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (n_dev) n = int64_t(*n_dev);
    if (j >= n) return;
    const uint64_t lk = new_keys[j] >> 12;
    if (find_u64(lower_keys, nlower, lk) >= 0) return;
    out[atomicAdd(count, 1ull)] = lk;
}

// Sorted distinct candidates of one dilation when there are at most
// SMALL_SORT_CAP of them (the usual case: the 64-sphere workload emits about
// 12k candidates, 6.6k distinct new leaves per substep): one CTA radix-sorts
// them in shared memory over the key bits that vary and compacts the
// distinct values, so the dilation needs no host read of the candidate
// count.  More candidates set st->overflow and leave the work to the
// device-wide sort.
constexpr int SMALL_SORT_THREADS = 1024;
constexpr int SMALL_SORT_ITEMS = 12;
constexpr int64_t SMALL_SORT_CAP = int64_t(SMALL_SORT_THREADS) * SMALL_SORT_ITEMS;
using SmallSort = cub::BlockRadixSort<uint64_t, SMALL_SORT_THREADS, SMALL_SORT_ITEMS>;
using SmallScan = cub::BlockScan<int, SMALL_SORT_THREADS>;
union SmallSortStorage {
    typename SmallSort::TempStorage sort;
    uint64_t keys[SMALL_SORT_CAP];
};
constexpr size_t SMALL_SORT_SMEM = sizeof(SmallSortStorage);

__global__ void __launch_bounds__(SMALL_SORT_THREADS) k_sort_unique_small(const uint64_t* cand, DevStatus* st,
                                                                          uint64_t* out, int64_t limit) {
    extern __shared__ __align__(16) unsigned char small_sort_smem[];
    SmallSortStorage& sm = *reinterpret_cast<SmallSortStorage*>(small_sort_smem);
    __shared__ typename SmallScan::TempStorage scan;
    __shared__ uint64_t red_or[SMALL_SORT_THREADS / 32], red_and[SMALL_SORT_THREADS / 32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int64_t n = int64_t(st->n_cand);
    if (n > SMALL_SORT_CAP || n > limit) {
        if (t == 0) {
            st->overflow = 1;
            st->n_unique = 0;
        }
        return;
    }
    uint64_t k[SMALL_SORT_ITEMS];
    uint64_t vor = 0, vand = ~uint64_t(0);
#pragma unroll
    for (int i = 0; i < SMALL_SORT_ITEMS; ++i) {
        const int64_t idx = int64_t(t) * SMALL_SORT_ITEMS + i;
        k[i] = idx < n ? cand[idx] : 0;
        if (idx < n) {
            vor |= k[i];
            vand &= k[i];
        }
    }
    // the bits in which the candidates differ
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        vor |= __shfl_xor_sync(0xffffffffu, vor, o);
        vand &= __shfl_xor_sync(0xffffffffu, vand, o);
    }
    if (lane == 0) {
        red_or[warp] = vor;
        red_and[warp] = vand;
    }
    __syncthreads();
    vor = 0;
    vand = ~uint64_t(0);
#pragma unroll 4
    for (int w = 0; w < SMALL_SORT_THREADS / 32; ++w) {
        vor |= red_or[w];
        vand &= red_and[w];
    }
    const uint64_t vary = vor ^ vand;
    const int end_bit = vary ? 64 - __clzll(static_cast<long long>(vary)) : 1;
    // padding sorts after every candidate on bits [0, end_bit): the common
    // high bits with every low bit set
    const uint64_t low = end_bit == 64 ? ~uint64_t(0) : ((uint64_t(1) << end_bit) - 1);
    const uint64_t pad = (vor & ~low) | low;
#pragma unroll
    for (int i = 0; i < SMALL_SORT_ITEMS; ++i)
        if (int64_t(t) * SMALL_SORT_ITEMS + i >= n) k[i] = pad;
    SmallSort(sm.sort).Sort(k, 0, end_bit);  // blocked arrangement in and out
    __syncthreads();
#pragma unroll
    for (int i = 0; i < SMALL_SORT_ITEMS; ++i) sm.keys[t * SMALL_SORT_ITEMS + i] = k[i];
    __syncthreads();
    // the first n sorted values are the candidates
    bool head[SMALL_SORT_ITEMS];
    int cnt = 0;
#pragma unroll
    for (int i = 0; i < SMALL_SORT_ITEMS; ++i) {
        const int idx = t * SMALL_SORT_ITEMS + i;
        head[i] = idx < n && (idx == 0 || sm.keys[idx] != sm.keys[idx - 1]);
        cnt += head[i] ? 1 : 0;
    }
    int off = 0, total = 0;
    SmallScan(scan).ExclusiveSum(cnt, off, total);
#pragma unroll
    for (int i = 0; i < SMALL_SORT_ITEMS; ++i)
        if (head[i]) out[off++] = k[i];
    if (t == 0) {
        st->n_unique = (unsigned long long)total;
        st->overflow = 0;
    }
}

// Processed-voxel mask of a masked renormalisation (Normalizer with a mask,
// tools/LevelSetTracker.h:661-670): for every leaf of the level set, the
// active voxels of the mask leaf with the same origin (found by key among the
// sorted mask keys), none without one.  A mask voxel that is inactive in the
// level set sets *err (the renormalised value of an inactive voxel has no
// place in the packed layout).
__global__ void k_mask_from_leaves(int64_t n, const uint64_t* keys, const int32_t* slot, const uint64_t* am,
                                   const uint64_t* mkeys, const uint64_t* mmasks, int64_t nm, uint64_t* pmask,
                                   unsigned long long* err) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n * 8) return;
    const int64_t l = i >> 3;
    const int w = int(i & 7);
    const int64_t j = find_u64(mkeys, nm, keys[l]);
    const uint64_t bits = j >= 0 ? mmasks[size_t(j) * 8 + w] : 0;
    const size_t s = size_t(slot[l]);
    pmask[s * 8 + w] = bits;
    if (bits & ~am[s * 8 + w]) atomicAdd(err, 1ull);
}

__global__ void k_keep_flags(int64_t n, const int32_t* cnt, int32_t* keep) {
    const int64_t l = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (l >= n) return;
    keep[l] = cnt[l] > 0 ? 1 : 0;
}

// Leaf-level prune (tools/Prune.h:305-312 with getTileValue :326-329): an
// inactive leaf becomes a lower-node tile of the sign of its first voxel;
// its slot returns to the free stack.
__global__ void k_prune_scatter(int64_t n, const uint64_t* keys, const int32_t* slot,
                                const int32_t* keep, const int32_t* idx, const uint64_t* sm,
                                uint64_t* ko, int32_t* so, int32_t* free_slots, int64_t nfree,
                                const uint64_t* lower_keys, int64_t nlower, uint64_t* lower_sign,
                                const int32_t* cnt, unsigned long long* nactive,
                                unsigned long long* nkept, unsigned long long* err,
                                unsigned long long* inst_active) {
    const int64_t l = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    // active voxels of the kept leaves: warp sum, one atomic per warp
    // (blockDim is a multiple of 32, every lane takes part)
    unsigned long long c = (l < n && keep[l]) ? (unsigned long long)cnt[l] : 0ull;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(nactive, c);
    if (l >= n) return;
    const int64_t k = idx[l];
    if (l == n - 1) *nkept = (unsigned long long)(k + keep[l]);
    if (keep[l]) {
        ko[k] = keys[l];
        so[k] = slot[l];
        if (inst_active) atomicAdd(inst_active + key_instance(keys[l]), (unsigned long long)cnt[l]);
        return;
    }
    const int s = slot[l];
    free_slots[nfree + (l - k)] = s;
    const uint64_t key = keys[l];
    const int64_t li = find_u64(lower_keys, nlower, key >> 12);
    if (li < 0) {
        atomicAdd(err, 1ull);
        return;
    }
    const uint32_t nbit = uint32_t(key & 4095);
    unsigned long long* word = reinterpret_cast<unsigned long long*>(lower_sign + li * 64 + (nbit >> 6));
    const unsigned long long bit = 1ull << (nbit & 63);
    if (sm[size_t(s) * 8] & 1) atomicOr(word, bit);
    else atomicAnd(word, ~bit);
}

// Lower nodes without leaves (pruned into upper-node tiles by the host).
// flag: 0 = keep, 1 = empty with a positive first value, 2 = empty negative.
__global__ void k_lower_status(int64_t nlower, const uint64_t* lower_keys, const uint64_t* lower_sign,
                               const uint64_t* keys, const unsigned long long* nleaf, uint8_t* flags,
                               unsigned long long* nempty) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= nlower) return;
    const int64_t n = int64_t(*nleaf);
    const uint64_t lk = lower_keys[i];
    const int64_t j = lower_bound_u64(keys, n, lk << 12);
    const bool has = j < n && (keys[j] >> 12) == lk;
    if (has) {
        flags[i] = 0;
    } else {
        flags[i] = (lower_sign[i * 64] & 1) ? 2 : 1;
        atomicAdd(nempty, 1ull);
    }
}

// Rebuild lower sign rows after node insertion/removal: row r copies old row
// src[r] >= 0, or is filled with the sign (-1 - src[r]).
__global__ void k_remap_rows(int64_t nrows, const int32_t* src, const uint64_t* old_sign, uint64_t* new_sign) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= nrows * 64) return;
    const int64_t r = i >> 6;
    const int w = int(i & 63);
    const int32_t s = src[r];
    new_sign[i] = (s >= 0) ? old_sign[int64_t(s) * 64 + w] : ((-1 - s) ? ~uint64_t(0) : uint64_t(0));
}

__global__ void k_count_active(int64_t n, const int32_t* slot, const uint64_t* am, unsigned long long* out) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    unsigned long long c = 0;
    if (i < n * 8) c = __popcll(am[size_t(slot[i >> 3]) * 8 + (i & 7)]);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// Active voxels per instance (one atomic per leaf).
__global__ void k_count_active_inst(int64_t n, const uint64_t* keys, const int32_t* slot, const uint64_t* am,
                                    unsigned long long* out) {
    const int64_t l = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (l >= n) return;
    unsigned long long c = 0;
    for (int w = 0; w < 8; ++w) c += __popcll(am[size_t(slot[l]) * 8 + w]);
    if (c) atomicAdd(out + key_instance(keys[l]), c);
}

// Active voxels per leaf, in leaf-list order.
__global__ void k_leaf_active(int64_t n, const int32_t* slot, const uint64_t* am, int64_t* cnt) {
    const int64_t l = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (l >= n) return;
    int64_t c = 0;
    for (int w = 0; w < 8; ++w) c += __popcll(am[size_t(slot[l]) * 8 + w]);
    cnt[l] = c;
}

// Index coordinates of the active voxels in the reference's velocity order
// (leaves in tree order, voxels in offset order): leaf l's active voxel of
// rank r goes to entry prefix[l] + r.  One CTA of 64 threads per leaf,
// thread t owning bit t of every mask word.
__global__ void __launch_bounds__(64) k_active_ijk(int64_t n, const uint64_t* keys, const int32_t* slot,
                                                  const uint64_t* am, const int64_t* prefix, int32_t* ijk) {
    const int64_t l = blockIdx.x;
    if (l >= n) return;
    const int t = threadIdx.x;
    int32_t ox, oy, oz;
    key_origin(keys[l], ox, oy, oz);
    const uint64_t low = (uint64_t(1) << t) - 1;
    int64_t base = prefix[l];
    for (int k = 0; k < 8; ++k) {
        const uint64_t w = am[size_t(slot[l]) * 8 + k];
        if ((w >> t) & 1) {
            const int v = (k << 6) | t;
            int32_t* q = ijk + 3 * (base + __popcll(w & low));
            q[0] = ox + (v >> 6);
            q[1] = oy + ((v >> 3) & 7);
            q[2] = oz + (v & 7);
        }
        base += __popcll(w);
    }
}

// Active voxels per leaf of a mask array indexed through slot (or
// directly), 0 for leaves with keep[l] == 0.
__global__ void k_mask_count(int64_t n, const int32_t* slot, const uint64_t* m, const int32_t* keep, int64_t* cnt) {
    const int64_t l = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (l >= n) return;
    const size_t s = size_t(slot ? slot[l] : int32_t(l));
    int64_t c = 0;
    if (!keep || keep[l])
        for (int w = 0; w < 8; ++w) c += __popcll(m[s * 8 + w]);
    cnt[l] = c;
}

// Packed per-leaf values (leaf storage s = slot[l] or l, [s*512 + rank]) to
// one array in leaf order (to_packed: packed[prefix[l] + rank]), or back
// (to leaf dst_leaf[l] when given, else s).  Leaves with keep[l] == 0 are
// skipped.  One CTA of 64 threads per leaf, thread t owning bit t of every
// mask word.
__global__ void __launch_bounds__(64) k_packed_move(int64_t n, const int32_t* slot, const int32_t* keep,
                                                   const int32_t* dst_leaf, const uint64_t* m,
                                                   const int64_t* prefix, const float* src, float* dst,
                                                   int to_packed) {
    const int64_t l = blockIdx.x;
    if (l >= n || (keep && !keep[l])) return;
    const size_t s = size_t(slot ? slot[l] : int32_t(l));
    const size_t d = dst_leaf ? size_t(dst_leaf[l]) : s;
    const int t = threadIdx.x;
    const uint64_t low = (uint64_t(1) << t) - 1;
    int base = 0;
    for (int w = 0; w < 8; ++w) {
        const uint64_t mw = m[s * 8 + w];
        if ((mw >> t) & 1) {
            const int r = base + __popcll(mw & low);
            if (to_packed) dst[prefix[l] + r] = src[s * LEAF_VOX + r];
            else dst[d * LEAF_VOX + r] = src[prefix[l] + r];
        }
        base += __popcll(mw);
    }
}

// dst[pairs[2i]] = pairs[2i + 1] for i < n (upper-node sign words changed
// in place on the host).
__global__ void k_scatter_words(int64_t n, const uint64_t* pairs, uint64_t* dst) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i < n) dst[pairs[2 * i]] = pairs[2 * i + 1];
}

// The sign mask records value < 0 for every voxel: refresh its active bits
// after new active values.
__global__ void __launch_bounds__(64) k_active_signs(int64_t n, const int32_t* slot, const uint64_t* am,
                                                    const float* vals, uint64_t* sm) {
    const int64_t l = blockIdx.x;
    if (l >= n) return;
    const size_t s = size_t(slot[l]);
    const int t = threadIdx.x;
    const uint64_t low = (uint64_t(1) << t) - 1;
    __shared__ uint32_t neg[8][2];
    int base = 0;
    for (int w = 0; w < 8; ++w) {
        const uint64_t mw = am[s * 8 + w];
        const bool on = (mw >> t) & 1;
        const bool old = (sm[s * 8 + w] >> t) & 1;
        const bool x = on ? vals[s * LEAF_VOX + base + __popcll(mw & low)] < 0.0f : old;
        const uint32_t b = __ballot_sync(0xffffffffu, x);
        if ((t & 31) == 0) neg[w][t >> 5] = b;
        base += __popcll(mw);
    }
    __syncthreads();
    if (t < 8) sm[s * 8 + t] = uint64_t(neg[t][0]) | (uint64_t(neg[t][1]) << 32);
}

// Pack leaf values into the slot layout (upload) / unpack (download).
__global__ void k_unpack(int64_t n, const int32_t* slot, const uint64_t* am, const uint64_t* sm,
                         const float* vals, float gamma, float* dense) {
    const int64_t l = blockIdx.x;
    if (l >= n) return;
    const int s = slot[l];
    __shared__ int pre[9];
    __shared__ uint64_t m[8];
    if (threadIdx.x < 8) m[threadIdx.x] = am[size_t(s) * 8 + threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int w = 0; w < 8; ++w) { pre[w] = acc; acc += __popcll(m[w]); }
        pre[8] = acc;
    }
    __syncthreads();
    for (int v = threadIdx.x; v < LEAF_VOX; v += blockDim.x) {
        const int w = v >> 6, b = v & 63;
        float val;
        if ((m[w] >> b) & 1) {
            val = vals[size_t(s) * LEAF_VOX + pre[w] + __popcll(m[w] & ((1ull << b) - 1))];
        } else {
            val = ((sm[size_t(s) * 8 + w] >> b) & 1) ? -gamma : gamma;
        }
        dense[l * LEAF_VOX + v] = val;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// handle
// ---------------------------------------------------------------------------

// One recorded CFL substep of the adjoint tape (leaf-index numbering).
struct TapeStep {
    // RK part on the substep's leaf list
    int64_t n = 0;
    DevArray<uint64_t> keys, am, sm;
    DevArray<int32_t> nbr;
    DevArray<float> phin, phi1, phi2;
    float dt = 0.0f, t0 = 0.0f;
    bool backward = false;
    // how dt was set (its derivative with respect to the velocity): max
    // |v|^2 at the substep's start and the clock's choices (CflClock)
    float maxv2 = 0.0f, open_lim = 0.0f;
    bool limited = false, opened = false, end_lim = false, first = false;
    // tracker part on the dilated (merged) list
    int64_t nm = 0;
    DevArray<uint64_t> keys_m, am3, sm3, pmask, fin;
    DevArray<int32_t> nbr_m, keep, idx;
    DevArray<float> phi3;
    float gamma = 0.0f;
};

struct gbls_field {
    gbls_field_desc desc{};
    int device = 0;
    DevArray<float> dense;
    DevArray<float> tab;  // DEFORMATION: sin(pi i/domain), sin(2 pi i/domain) per coordinate
    int tab_lo = 0, tab_n = 0;
};

struct gbls_handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    double voxel_size = 1.0;
    double translation[3] = {0, 0, 0};
    int map_type = GBLS_MAP_UNIFORM_SCALE;
    float gamma = 3.0f;
    // LevelSetTracker::State defaults (tools/LevelSetTracker.h:74-83)
    int tr_spatial = GBLS_HJWENO5_BIAS, tr_temporal = GBLS_TVD_RK1, norm_count = 3, grain = 1;
    int trim = GBLS_TRIM_ALL;
    int mode = GBLS_MODE_PARITY;
    gbls_interrupter intr{};
    bool has_intr = false;

    // leaves in tree order (double-buffered for merge / compaction)
    int64_t nleaf = 0;
    DevArray<uint64_t> keys[2];
    DevArray<int32_t> slot[2];
    int kc = 0;
    DevArray<int32_t> nbr, nbr_alt;  // face-neighbour table; a rebuild writes the other and swaps
    // slot storage: 3 mask sets, 3 value buffers, dilation mask
    int64_t slot_cap = 0;
    DevArray<uint64_t> am[3], sm[3];
    DevArray<float> vals[3];  // FP32 values, or (f64) 512 doubles per slot in the same arrays
    bool f64 = false;         // the FP64 instance (GBLS_MODE_FP64)
    DevArray<float> f32_view; // f64: the current values rounded to float (downloads)
    DevArray<unsigned long long> argk;
    DevArray<double> argv;
    DevArray<uint64_t> scatter;  // (index, word) pairs for in-place sign-table updates
    DevArray<uint64_t> dmask, emask;
    DevArray<int32_t> free_slots;
    int64_t nfree = 0;
    int mc = 0, vc = 0;  // current mask set / value buffer
    // node tables: device arrays + host mirrors of keys, upper signs, root tiles
    std::vector<uint64_t> lower_keys_h, upper_keys_h, upper_sign_h, root_keys_h;
    std::vector<uint8_t> root_sign_h;
    DevArray<uint64_t> lower_keys, lower_sign, lower_sign_spare, upper_keys, upper_sign, root_keys;
    DevArray<uint8_t> root_sign;
    bool nodes_checked = false;  // empty nodes of the input removed by a prune
    // scratch
    DevArray<uint64_t> cand, cand_sorted, new_keys, miss;
    DevArray<int32_t> new_slots, cnt, keep, idx, remap;
    DevArray<uint8_t> cub_tmp, flags;
    DevArray<int32_t> io_perm;   // upload: staged index of each leaf / lower / upper node
    DevArray<float> io_tiles;    // staged node tiles (upload and download)
    DevArray<int32_t> io_orig;   // download: leaf origins
    DevArray<float> cfl_part;    // CFL reduction: per-leaf maxima
    DevArray<float> morph_speed; // LevelSetMorphing: speed per active voxel, packed like the values
    DevStatus* st_d = nullptr;
    DevStatus* st_h = nullptr;
    DevArray<unsigned long long> u64s;
    unsigned long long* acc_d = nullptr;  // [2] normalize voxels processed / written
    // batches: instance id in key bits 54..62
    int ninst = 1;
    bool batch_run = false;  // kernels see the per-instance arrays below
    DevArray<uint8_t> inst_run;
    DevArray<float> inst_dt, inst_t0;
    DevArray<FieldParams> inst_field;
    DevArray<unsigned int> inst_max;
    DevArray<unsigned long long> inst_active;
    const uint8_t* run_ptr() const { return batch_run ? inst_run.p : nullptr; }
    // adjoint tape
    bool tape_on = false;
    std::vector<std::unique_ptr<TapeStep>> tape;
    TapeStep* tape_cur = nullptr;
    // steps of discarded tapes, kept with their device arrays: a re-recorded
    // forward pass of the same size allocates nothing
    std::vector<std::unique_ptr<TapeStep>> tape_pool;
    void discard_tape() {
        for (auto& t : tape) tape_pool.push_back(std::move(t));
        tape.clear();
        tape_cur = nullptr;
    }
    DevArray<int32_t> tape_inv;
    // work enqueued by the advection loop right before the read-back that
    // ends a tracker pass (the next substep's CFL reduction), so that one
    // synchronisation serves both
    std::function<void()> before_prune_sync;
    std::function<void()> after_normalize;  // called by track() after the renormalisation is enqueued
    // measurement
    gbls_stats stats{};
    int64_t nactive = -1;  // active voxels, -1 = unknown
    bool profiling = false;
    struct Pending {
        cudaEvent_t a, b;
        int kind;  // 0 rk, 1 norm
        double bytes;
    };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> event_pool;
    cudaEvent_t sync_ev = nullptr;
    // During advection the tracker's dilation runs on `side`, concurrently
    // with the RK stages of the same substep (they read values, the dilation
    // writes topology): ev_fork precedes the RK stages, ev_rk follows them,
    // ev_join ends the dilation.  on_side: `stream` is the side stream.
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_rk = nullptr, ev_join = nullptr, ev_norm = nullptr, ev_cfl = nullptr;
    // The next substep's CFL maximum, reduced on the side stream while the
    // main stream prunes: device word and its page-locked copy.
    unsigned int* cfl_d = nullptr;
    unsigned int* cfl_h = nullptr;
    bool overlap_dilation = false, on_side = false;
    bool small_sort_ready = false;  // dynamic shared memory of k_sort_unique_small set on this device
    // Candidates above this many take the device-wide sort (SMALL_SORT_CAP;
    // the environment variable GBLS_SMALL_SORT_LIMIT, read when the handle
    // is created, lowers it so tests can exercise that path).
    int64_t small_sort_limit = SMALL_SORT_CAP;
    // PARITY mode runs the ExactArith kernels (FP32 pipes, the same bits as
    // the FP64 kernels); GBLS_PARITY_FP64=1 when the handle is created
    // selects the FP64 kernels instead, for cross-checking.
    bool parity_fp64 = false;
    // launch shapes (gbls_set_launch_config; the autotuner's choices)
    int rk_min_ctas = 0, norm_min_ctas = 0, cfl_leaves = 32, rk_parts = 1;
    // a general FloatGrid volume (gbls_create_volume): any background, and
    // only volume operations
    bool volume = false;
    // HOST_SAMPLED fields: per-leaf active prefix, active voxel coordinates
    // and the sampled velocities of the current substep
    DevArray<int64_t> hs_count, hs_prefix;
    DevArray<int32_t> hs_ijk;
    DevArray<float> hs_vel;
    std::vector<int32_t> hs_ijk_h;
    std::vector<float> hs_vel_h;
    // CFL maximum of an analytic field at the end time of the last advect
    // call, reused by the next call that starts there with the same field
    // (any other operation on the level set clears it)
    struct {
        bool valid = false;
        float t = 0.0f, v2 = 0.0f;
        gbls_field_desc desc{};
    } cfl_cache;
    // alpha mask of the filter call in progress (gbls_filter_masked)
    struct {
        bool on = false;
        gbls_handle* grid = nullptr;
        float min = 0.0f, inv_norm = 1.0f;
        int invert = 0;
    } filter_mask;
    std::vector<uint8_t> flags_h;  // lower-node flags read back with the prune's status
    // Page-locked staging of the tracker's small node-table transfers, so
    // they are asynchronous copies; pin_ev marks the last copy issued from it.
    void* pin = nullptr;
    size_t pin_cap = 0, pin_off = 0;
    cudaEvent_t pin_ev = nullptr;
    bool pin_busy = false;

    ~gbls_handle() {
        if (st_d) cudaFree(st_d);
        if (st_h) cudaFreeHost(st_h);
        if (acc_d) cudaFree(acc_d);
        for (auto& p : pending) { event_pool.push_back(p.a); event_pool.push_back(p.b); }
        for (auto e : event_pool) cudaEventDestroy(e);
        if (sync_ev) cudaEventDestroy(sync_ev);
        if (pin_ev) cudaEventSynchronize(pin_ev), cudaEventDestroy(pin_ev);
        if (pin) cudaFreeHost(pin);
        if (side) cudaStreamSynchronize(side), cudaStreamDestroy(side);
        for (cudaEvent_t e : {ev_fork, ev_rk, ev_join, ev_norm, ev_cfl})
            if (e) cudaEventDestroy(e);
        if (cfl_d) cudaFree(cfl_d);
        if (cfl_h) cudaFreeHost(cfl_h);
    }

    // `bytes` of page-locked staging not read by a copy in flight: the next
    // free part of the staging, else all of it once its copies completed.
    void* pinned(size_t bytes) {
        bytes = (bytes + 15) & ~size_t(15);
        if (pin_busy && pin_off + bytes <= pin_cap) {
            void* r = static_cast<char*>(pin) + pin_off;
            pin_off += bytes;
            return r;
        }
        if (pin_busy) {
            CU(cudaEventSynchronize(pin_ev));
            pin_busy = false;
        }
        if (bytes > pin_cap) {
            if (pin) CU(cudaFreeHost(pin));
            pin = nullptr;
            const size_t nc = std::max<size_t>(std::max(bytes, pin_cap * 2), 65536);
            CU(cudaHostAlloc(&pin, nc, cudaHostAllocDefault));
            pin_cap = nc;
        }
        pin_off = bytes;
        return pin;
    }
    // Copies from the staging were enqueued: it is reused after they complete.
    void pinned_issued() {
        if (!pin_ev) CU(cudaEventCreateWithFlags(&pin_ev, cudaEventDisableTiming));
        CU(cudaEventRecord(pin_ev, stream));
        pin_busy = true;
    }
    // Copy n elements of a device array to host memory (waits for them).
    template <class T>
    void download_small(const DevArray<T>& d, T* out, size_t n) {
        if (!n) return;
        T* st = static_cast<T*>(pinned(n * sizeof(T)));
        CU(cudaMemcpyAsync(st, d.p, n * sizeof(T), cudaMemcpyDeviceToHost, stream));
        sync();
        std::memcpy(out, st, n * sizeof(T));
    }

    cudaEvent_t event() {
        if (event_pool.empty()) {
            cudaEvent_t e;
            CU(cudaEventCreate(&e));
            return e;
        }
        cudaEvent_t e = event_pool.back();
        event_pool.pop_back();
        return e;
    }
    // Accumulate the device time of completed profiled launches.
    void resolve_pending() {
        for (auto& p : pending) {
            float ms = 0.0f;
            CU(cudaEventElapsedTime(&ms, p.a, p.b));
            if (p.kind == 0) stats.rk_ms += ms;
            else stats.norm_ms += ms;
            event_pool.push_back(p.a);
            event_pool.push_back(p.b);
        }
        pending.clear();
    }

    NodeTables nodes() const {
        NodeTables t;
        t.lower_keys = lower_keys.p;
        t.lower_sign = lower_sign.p;
        t.upper_keys = upper_keys.p;
        t.upper_sign = upper_sign.p;
        t.root_keys = root_keys.p;
        t.root_sign = root_sign.p;
        t.nlower = int64_t(lower_keys_h.size());
        t.nupper = int64_t(upper_keys_h.size());
        t.nroot = int64_t(root_keys_h.size());
        return t;
    }
    uint64_t* K() { return keys[kc].p; }
    int32_t* S() { return slot[kc].p; }
    Layout layout(int m, int v) const { return Layout{am[m].p, sm[m].p, vals[v].p}; }

    // Wait for the stream.  The tracker's read-backs wait on a few small
    // kernels, so the host polls an event for up to 2 ms (a blocking wait
    // returns tens of microseconds after the work ends) and blocks after that.
    void sync() {
        if (!sync_ev) CU(cudaEventCreateWithFlags(&sync_ev, cudaEventDisableTiming));
        CU(cudaEventRecord(sync_ev, stream));
        const auto start = std::chrono::steady_clock::now();
        for (;;) {
            const cudaError_t e = cudaEventQuery(sync_ev);
            if (e == cudaSuccess) break;
            if (e != cudaErrorNotReady) CU(e);
            if (std::chrono::steady_clock::now() - start > std::chrono::milliseconds(2)) {
                CU(cudaEventSynchronize(sync_ev));
                break;
            }
        }
        if (!on_side) {  // the side stream's syncs leave the RK stages running
            pin_busy = false;  // every copy from the staging has completed
            pin_off = 0;
            if (!pending.empty()) resolve_pending();
        }
    }
    void read_status() {
        CU(cudaMemcpyAsync(st_h, st_d, sizeof(DevStatus), cudaMemcpyDeviceToHost, stream));
        sync();
        if (st_h->error) fail(GBLS_ERR_DEVICE_CHECK, "device-side tree consistency check failed");
    }
    void clear_status() { CU(cudaMemsetAsync(st_d, 0, sizeof(DevStatus), stream)); }

    bool leaf_cap_ok(int64_t n) const {
        const size_t u = size_t(n);
        return keys[0].cap >= u && keys[1].cap >= u && slot[0].cap >= u && slot[1].cap >= u &&
               nbr.cap >= 6 * u && nbr_alt.cap >= 6 * u && cnt.cap >= u && keep.cap >= u && idx.cap >= u;
    }
    void ensure_leaf_cap(int64_t n) {
        const size_t keep_n = size_t(nleaf);
        for (int b = 0; b < 2; ++b) {
            keys[b].reserve(n, stream, b == kc ? keep_n : 0);
            slot[b].reserve(n, stream, b == kc ? keep_n : 0);
        }
        nbr.reserve(size_t(n) * 6, stream, size_t(nleaf) * 6);
        nbr_alt.reserve(size_t(n) * 6, stream);
        cnt.reserve(n, stream);
        keep.reserve(n, stream);
        idx.reserve(n, stream);
    }

    // Make at least `need` free slots available.
    void ensure_free_slots(int64_t need) {
        if (nfree >= need) return;
        const int64_t old = slot_cap;
        int64_t nc = std::max(old + (need - nfree), int64_t(double(old) * 1.5) + 1024);
        // the stencil staging records address values by the 32-bit offset slot*512
        constexpr int64_t kMaxSlots = int64_t(1) << 23;
        if (old + (need - nfree) > kMaxSlots) fail(GBLS_ERR_OUT_OF_MEMORY, "more than 2^23 leaves in one handle");
        nc = std::min(nc, kMaxSlots);
        for (int b = 0; b < 3; ++b) {
            am[b].reserve(size_t(nc) * 8, stream, size_t(old) * 8, 1.0);
            sm[b].reserve(size_t(nc) * 8, stream, size_t(old) * 8, 1.0);
            const size_t vw = f64 ? 2 : 1;  // floats per value
            vals[b].reserve(size_t(nc) * LEAF_VOX * vw, stream, size_t(old) * LEAF_VOX * vw, 1.0);
        }
        dmask.reserve(size_t(nc) * 8, stream, size_t(old) * 8, 1.0);
        emask.reserve(size_t(nc) * 8, stream, 0, 1.0);
        free_slots.reserve(size_t(nc), stream, size_t(nfree), 1.0);
        // push the new slots below the existing free ones so that they are
        // used last: [new slots..., old free slots...]
        std::vector<int32_t> fresh;
        for (int64_t s = nc - 1; s >= old; --s) fresh.push_back(int32_t(s));
        const int64_t nnew = nc - old;
        DevArray<int32_t> tmp;
        tmp.reserve(size_t(nnew + nfree), stream);
        CU(cudaMemcpyAsync(tmp.p, fresh.data(), nnew * sizeof(int32_t), cudaMemcpyHostToDevice, stream));
        if (nfree)
            CU(cudaMemcpyAsync(tmp.p + nnew, free_slots.p, nfree * sizeof(int32_t),
                               cudaMemcpyDeviceToDevice, stream));
        CU(cudaMemcpyAsync(free_slots.p, tmp.p, (nnew + nfree) * sizeof(int32_t),
                           cudaMemcpyDeviceToDevice, stream));
        sync();
        nfree += nnew;
        slot_cap = nc;
    }

    // Upload the upper-node and root tables through the page-locked staging
    // (the host tables may change right after: the copies read the staging).
    void upload_upper_root() {
        const size_t b0 = upper_keys_h.size() * 8, b1 = upper_sign_h.size() * 8, b2 = root_keys_h.size() * 8,
                     b3 = root_sign_h.size();
        upper_keys.reserve(upper_keys_h.size(), stream);
        upper_sign.reserve(upper_sign_h.size(), stream);
        root_keys.reserve(root_keys_h.size(), stream);
        root_sign.reserve(root_sign_h.size(), stream);
        char* st = static_cast<char*>(pinned(b0 + b1 + b2 + b3 + 1));
        std::memcpy(st, upper_keys_h.data(), b0);
        std::memcpy(st + b0, upper_sign_h.data(), b1);
        std::memcpy(st + b0 + b1, root_keys_h.data(), b2);
        std::memcpy(st + b0 + b1 + b2, root_sign_h.data(), b3);
        if (b0) CU(cudaMemcpyAsync(upper_keys.p, st, b0, cudaMemcpyHostToDevice, stream));
        if (b1) CU(cudaMemcpyAsync(upper_sign.p, st + b0, b1, cudaMemcpyHostToDevice, stream));
        if (b2) CU(cudaMemcpyAsync(root_keys.p, st + b0 + b1, b2, cudaMemcpyHostToDevice, stream));
        if (b3) CU(cudaMemcpyAsync(root_sign.p, st + b0 + b1 + b2, b3, cudaMemcpyHostToDevice, stream));
        pinned_issued();
    }

    // Rebuild into the other table (kernels enqueued earlier keep reading
    // the current one) and make it current.
    void rebuild_nbr() {
        if (nleaf == 0) return;
        nbr_alt.reserve(size_t(nleaf) * 6, stream);
        k_build_nbr<<<blocks_for(nleaf * 6, 256), 256, 0, stream>>>(nleaf, K(), S(), nodes(), nbr_alt.p);
        ++stats.kernel_launches;
        CU(cudaGetLastError());
        std::swap(nbr.p, nbr_alt.p);
        std::swap(nbr.cap, nbr_alt.cap);
    }

    // Capacity for a dilation of the current leaves in the common case, taken
    // before the RK stages are enqueued so that the concurrent dilation
    // reallocates nothing they read.
    void prepare_dilation() {
        if (!side) {
            // highest priority: the dilation's small grids (a single-CTA sort)
            // are dispatched as soon as RK-stage CTAs retire
            int lo = 0, hi = 0;
            CU(cudaDeviceGetStreamPriorityRange(&lo, &hi));
            CU(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, hi));
            for (cudaEvent_t* e : {&ev_fork, &ev_rk, &ev_join, &ev_norm, &ev_cfl})
                CU(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
            CU(cudaMalloc(&cfl_d, sizeof(unsigned int)));
            CU(cudaHostAlloc(&cfl_h, sizeof(unsigned int), cudaHostAllocDefault));
        }
        const int64_t L = nleaf;
        const int64_t cap = std::min<int64_t>(L * 6, SMALL_SORT_CAP);
        ensure_free_slots(cap);
        ensure_leaf_cap(L + cap);
        cand.reserve(size_t(L) * 6, stream);
        cand_sorted.reserve(size_t(cap), stream);
        new_keys.reserve(size_t(cap), stream);
        new_slots.reserve(size_t(cap), stream);
        miss.reserve(size_t(cap), stream);
    }
};

namespace {

int other_of(int a, int b) {
    for (int i = 0; i < 3; ++i)
        if (i != a && i != b) return i;
    return -1;
}

// Remap lower-node rows: src[r] = old row or -1-sign for a new row.
// The new lower-node table: rows of the old table (src >= 0) or tiles of
// one sign (src = -1 - sign).  The rows are written into the spare table,
// which then becomes the current one (no allocation once the spare is
// large enough).
void remap_lower(gbls_handle& h, const std::vector<uint64_t>& new_keys, const std::vector<int32_t>& src) {
    const int64_t n = int64_t(new_keys.size());
    DevArray<uint64_t>& ns = h.lower_sign_spare;
    ns.reserve(size_t(std::max<int64_t>(n, 1)) * 64, h.stream);
    h.remap.reserve(size_t(std::max<int64_t>(n, 1)), h.stream);
    h.lower_keys.reserve(size_t(std::max<int64_t>(n, 1)), h.stream);
    if (n) {
        // stage keys and row sources in page-locked memory: asynchronous copies
        char* st = static_cast<char*>(h.pinned(size_t(n) * (sizeof(uint64_t) + sizeof(int32_t))));
        std::memcpy(st, new_keys.data(), size_t(n) * sizeof(uint64_t));
        std::memcpy(st + size_t(n) * sizeof(uint64_t), src.data(), size_t(n) * sizeof(int32_t));
        CU(cudaMemcpyAsync(h.lower_keys.p, st, size_t(n) * sizeof(uint64_t), cudaMemcpyHostToDevice, h.stream));
        CU(cudaMemcpyAsync(h.remap.p, st + size_t(n) * sizeof(uint64_t), size_t(n) * sizeof(int32_t),
                           cudaMemcpyHostToDevice, h.stream));
        h.pinned_issued();
        k_remap_rows<<<blocks_for(n * 64, 256), 256, 0, h.stream>>>(n, h.remap.p, h.lower_sign.p, ns.p);
        ++h.stats.kernel_launches;
    }
    CU(cudaGetLastError());
    std::swap(h.lower_sign.p, ns.p);
    std::swap(h.lower_sign.cap, ns.cap);
    h.lower_keys_h = new_keys;
}

int upper_bit(const gbls_handle& h, size_t ui, uint32_t slotn) {
    return int((h.upper_sign_h[ui * 512 + (slotn >> 6)] >> (slotn & 63)) & 1);
}

// Create the lower (and upper) nodes that new leaves need
// (tree/InternalNode.h:2868-2878, tree/RootNode.h:3255-3266): a new node's
// tiles take the value of the tile it replaces.
void insert_nodes(gbls_handle& h, std::vector<uint64_t> miss) {
    std::sort(miss.begin(), miss.end());
    miss.erase(std::unique(miss.begin(), miss.end()), miss.end());
    // upper nodes first
    std::vector<uint64_t> new_up;
    for (uint64_t lk : miss) {
        const uint64_t uk = lk >> 15;
        if (!std::binary_search(h.upper_keys_h.begin(), h.upper_keys_h.end(), uk)) new_up.push_back(uk);
    }
    std::sort(new_up.begin(), new_up.end());
    new_up.erase(std::unique(new_up.begin(), new_up.end()), new_up.end());
    if (!new_up.empty()) {
        std::vector<uint64_t> keys;
        std::vector<uint64_t> signs;
        size_t a = 0, b = 0;
        while (a < h.upper_keys_h.size() || b < new_up.size()) {
            if (b >= new_up.size() || (a < h.upper_keys_h.size() && h.upper_keys_h[a] < new_up[b])) {
                keys.push_back(h.upper_keys_h[a]);
                signs.insert(signs.end(), h.upper_sign_h.begin() + a * 512, h.upper_sign_h.begin() + (a + 1) * 512);
                ++a;
            } else {
                const uint64_t uk = new_up[b++];
                int sgn = 0;
                auto it = std::lower_bound(h.root_keys_h.begin(), h.root_keys_h.end(), uk);
                if (it != h.root_keys_h.end() && *it == uk) {
                    const size_t ri = size_t(it - h.root_keys_h.begin());
                    sgn = h.root_sign_h[ri];
                    h.root_keys_h.erase(h.root_keys_h.begin() + ri);
                    h.root_sign_h.erase(h.root_sign_h.begin() + ri);
                }
                keys.push_back(uk);
                signs.insert(signs.end(), 512, sgn ? ~uint64_t(0) : uint64_t(0));
            }
        }
        h.upper_keys_h.swap(keys);
        h.upper_sign_h.swap(signs);
        h.upload_upper_root();
    }
    // lower nodes
    std::vector<uint64_t> keys;
    std::vector<int32_t> src;
    size_t a = 0, b = 0;
    while (a < h.lower_keys_h.size() || b < miss.size()) {
        if (b >= miss.size() || (a < h.lower_keys_h.size() && h.lower_keys_h[a] < miss[b])) {
            keys.push_back(h.lower_keys_h[a]);
            src.push_back(int32_t(a));
            ++a;
        } else {
            const uint64_t lk = miss[b++];
            const uint64_t uk = lk >> 15;
            const size_t ui = size_t(std::lower_bound(h.upper_keys_h.begin(), h.upper_keys_h.end(), uk) -
                                     h.upper_keys_h.begin());
            keys.push_back(lk);
            src.push_back(-1 - upper_bit(h, ui, uint32_t(lk & 32767)));
        }
    }
    remap_lower(h, keys, src);
}

// Node-level part of pruneLevelSet (tools/Prune.h:305-322): lower nodes
// without leaves become upper tiles of the sign of their first value, upper
// nodes without lower nodes become root tiles; +background root tiles are
// erased (RootNode::eraseBackgroundTiles).
void prune_nodes(gbls_handle& h, bool lower_changed) {
    const int64_t nl = int64_t(h.lower_keys_h.size());
    std::vector<size_t> dirty;  // upper sign words changed in place (upper-node slots that became tiles)
    if (lower_changed && nl) {
        std::vector<uint8_t> fl;
        if (h.flags_h.size() == size_t(nl)) {
            fl.swap(h.flags_h);  // read back with the prune's status
        } else {
            fl.resize(static_cast<size_t>(nl));
            h.download_small(h.flags, fl.data(), size_t(nl));
        }
        h.flags_h.clear();
        std::vector<uint64_t> keys;
        std::vector<int32_t> src;
        for (int64_t i = 0; i < nl; ++i) {
            const uint64_t lk = h.lower_keys_h[size_t(i)];
            if (fl[size_t(i)] == 0) {
                keys.push_back(lk);
                src.push_back(int32_t(i));
                continue;
            }
            const uint64_t uk = lk >> 15;
            auto it = std::lower_bound(h.upper_keys_h.begin(), h.upper_keys_h.end(), uk);
            if (it == h.upper_keys_h.end() || *it != uk) fail(GBLS_ERR_DEVICE_CHECK, "lower node without upper node");
            const size_t ui = size_t(it - h.upper_keys_h.begin());
            const uint32_t n = uint32_t(lk & 32767);
            uint64_t& w = h.upper_sign_h[ui * 512 + (n >> 6)];
            if (fl[size_t(i)] == 2) w |= (uint64_t(1) << (n & 63));
            else w &= ~(uint64_t(1) << (n & 63));
            dirty.push_back(ui * 512 + (n >> 6));
        }
        remap_lower(h, keys, src);
    }
    // upper nodes without lower nodes (the tables are rebuilt only when one is)
    bool changed = false;
    std::vector<size_t> drop;
    for (size_t u = 0; u < h.upper_keys_h.size(); ++u) {
        const uint64_t uk = h.upper_keys_h[u];
        auto it = std::lower_bound(h.lower_keys_h.begin(), h.lower_keys_h.end(), uk << 15);
        if (!(it != h.lower_keys_h.end() && ((*it) >> 15) == uk)) drop.push_back(u);
    }
    if (!drop.empty()) {
        changed = true;
        std::vector<uint64_t> ukeys, usign;
        size_t d = 0;
        for (size_t u = 0; u < h.upper_keys_h.size(); ++u) {
            const uint64_t uk = h.upper_keys_h[u];
            if (d < drop.size() && drop[d] == u) {
                ++d;
                if (h.upper_sign_h[u * 512] & 1) {
                    auto rt = std::lower_bound(h.root_keys_h.begin(), h.root_keys_h.end(), uk);
                    const size_t ri = size_t(rt - h.root_keys_h.begin());
                    h.root_keys_h.insert(rt, uk);
                    h.root_sign_h.insert(h.root_sign_h.begin() + ri, 1);
                }
                continue;
            }
            ukeys.push_back(uk);
            usign.insert(usign.end(), h.upper_sign_h.begin() + u * 512, h.upper_sign_h.begin() + (u + 1) * 512);
        }
        h.upper_keys_h.swap(ukeys);
        h.upper_sign_h.swap(usign);
    }
    // eraseBackgroundTiles
    for (size_t r = 0; r < h.root_sign_h.size();) {
        if (h.root_sign_h[r] == 0) {
            h.root_keys_h.erase(h.root_keys_h.begin() + r);
            h.root_sign_h.erase(h.root_sign_h.begin() + r);
            changed = true;
        } else {
            ++r;
        }
    }
    if (changed) {
        h.upload_upper_root();
    } else if (!dirty.empty()) {
        // only sign words changed: send those words, not the whole tables
        const int64_t m = int64_t(dirty.size());
        uint64_t* st = static_cast<uint64_t*>(h.pinned(size_t(m) * 16));
        for (int64_t i = 0; i < m; ++i) {
            st[2 * i] = uint64_t(dirty[size_t(i)]);
            st[2 * i + 1] = h.upper_sign_h[dirty[size_t(i)]];
        }
        h.scatter.reserve(size_t(m) * 2, h.stream);
        CU(cudaMemcpyAsync(h.scatter.p, st, size_t(m) * 16, cudaMemcpyHostToDevice, h.stream));
        h.pinned_issued();
        k_scatter_words<<<blocks_for(m, 256), 256, 0, h.stream>>>(m, h.scatter.p, h.upper_sign.p);
        ++h.stats.kernel_launches;
        CU(cudaGetLastError());
    }
}

// ---- dilation: new leaves, node creation, neighbour table, dmask ----------
// While h.overlap_dilation is set the dilation runs on the side stream after
// ev_fork (concurrently with the RK stages that follow it on the main
// stream) and the main stream waits for it; growing an array first waits for
// the RK stages (ev_rk).
struct SideStreamScope {
    gbls_handle& h;
    bool on;
    explicit SideStreamScope(gbls_handle& h_) : h(h_), on(h_.overlap_dilation && h_.side) {
        if (!on) return;
        CU(cudaStreamWaitEvent(h.side, h.ev_fork, 0));
        std::swap(h.stream, h.side);
        h.on_side = true;
    }
    void wait_rk() {
        if (on) CU(cudaStreamWaitEvent(h.stream, h.ev_rk, 0));
    }
    ~SideStreamScope() {
        if (!on) return;
        cudaEventRecord(h.ev_join, h.stream);
        std::swap(h.stream, h.side);
        h.on_side = false;
        cudaStreamWaitEvent(h.stream, h.ev_join, 0);
    }
};

void dilate_topology(gbls_handle& h) {
    if (h.nleaf == 0) return;
    SideStreamScope scope(h);
    const int64_t L = h.nleaf;
    h.cand.reserve(size_t(L) * 6, h.stream);
    h.clear_status();
    k_emit_candidates<<<blocks_for(L, 128), 128, 0, h.stream>>>(L, h.K(), h.S(), h.nbr.p, h.am[h.mc].p,
                                                                 h.cand.p, &h.st_d->n_cand, h.run_ptr());
    ++h.stats.kernel_launches;
    CU(cudaGetLastError());
    // Common case: at most SMALL_SORT_CAP candidates.  Sort, new leaves,
    // merge and the missing-node search run on the device counts, and one
    // read-back returns every count.  (The kernels are sized for `cap`; the
    // ones after the sort read the distinct count on the device.)
    const int64_t cap = std::min<int64_t>(L * 6, SMALL_SORT_CAP);
    if (h.nfree < cap || !h.leaf_cap_ok(L + cap)) scope.wait_rk();  // not prepared: grow after the RK stages
    h.ensure_free_slots(cap);
    h.ensure_leaf_cap(L + cap);
    h.cand_sorted.reserve(size_t(cap), h.stream);
    h.new_keys.reserve(size_t(cap), h.stream);
    h.new_slots.reserve(size_t(cap), h.stream);
    h.miss.reserve(size_t(cap), h.stream);
    const int ko = 1 - h.kc;
    const unsigned long long* nu = &h.st_d->n_unique;
    if (!h.small_sort_ready) {
        CU(cudaFuncSetAttribute(k_sort_unique_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(SMALL_SORT_SMEM)));
        h.small_sort_ready = true;
    }
    k_sort_unique_small<<<1, SMALL_SORT_THREADS, SMALL_SORT_SMEM, h.stream>>>(h.cand.p, h.st_d, h.cand_sorted.p,
                                                                               h.small_sort_limit);
    k_new_leaves<<<blocks_for(cap, 128), 128, 0, h.stream>>>(0, nu, h.cand_sorted.p, h.free_slots.p, h.nfree,
                                                              h.new_keys.p, h.new_slots.p, h.am[h.mc].p,
                                                              h.sm[h.mc].p);
    k_merge<<<blocks_for(L + cap, 256), 256, 0, h.stream>>>(L, h.K(), h.S(), 0, nu, h.new_keys.p, h.new_slots.p,
                                                            h.keys[ko].p, h.slot[ko].p);
    k_missing_lower<<<blocks_for(cap, 128), 128, 0, h.stream>>>(0, nu, h.new_keys.p, h.lower_keys.p,
                                                                 int64_t(h.lower_keys_h.size()), h.miss.p,
                                                                 &h.st_d->n_lower_miss);
    h.stats.kernel_launches += 4;
    CU(cudaGetLastError());
    h.read_status();
    int64_t nnew = 0;
    if (!h.st_h->overflow) {
        nnew = int64_t(h.st_h->n_unique);
    } else {
        // device-wide sort of many candidates, then the same steps on host counts
        scope.wait_rk();
        const int64_t nc = int64_t(h.st_h->n_cand);
        h.cand_sorted.reserve(size_t(nc), h.stream);
        h.u64s.reserve(1, h.stream);
        size_t b1 = 0, b2 = 0;
        CU(cub::DeviceRadixSort::SortKeys(nullptr, b1, h.cand.p, h.cand_sorted.p, int(nc), 0, 64, h.stream));
        CU(cub::DeviceSelect::Unique(nullptr, b2, h.cand_sorted.p, h.cand.p, h.u64s.p, int(nc), h.stream));
        h.cub_tmp.reserve(std::max(b1, b2), h.stream);
        b1 = b2 = h.cub_tmp.cap;
        CU(cub::DeviceRadixSort::SortKeys(h.cub_tmp.p, b1, h.cand.p, h.cand_sorted.p, int(nc), 0, 64, h.stream));
        CU(cub::DeviceSelect::Unique(h.cub_tmp.p, b2, h.cand_sorted.p, h.cand.p, h.u64s.p, int(nc), h.stream));
        unsigned long long n_u = 0;
        CU(cudaMemcpyAsync(&n_u, h.u64s.p, sizeof(n_u), cudaMemcpyDeviceToHost, h.stream));
        h.sync();
        nnew = int64_t(n_u);
        if (nnew > 0) {
            h.ensure_free_slots(nnew);
            h.ensure_leaf_cap(L + nnew);
            h.new_keys.reserve(size_t(nnew), h.stream);
            h.new_slots.reserve(size_t(nnew), h.stream);
            h.miss.reserve(size_t(nnew), h.stream);
            k_new_leaves<<<blocks_for(nnew, 128), 128, 0, h.stream>>>(nnew, nullptr, h.cand.p, h.free_slots.p,
                                                                       h.nfree, h.new_keys.p, h.new_slots.p,
                                                                       h.am[h.mc].p, h.sm[h.mc].p);
            k_merge<<<blocks_for(L + nnew, 256), 256, 0, h.stream>>>(L, h.K(), h.S(), nnew, nullptr, h.new_keys.p,
                                                                     h.new_slots.p, h.keys[ko].p, h.slot[ko].p);
            h.clear_status();
            k_missing_lower<<<blocks_for(nnew, 128), 128, 0, h.stream>>>(
                nnew, nullptr, h.new_keys.p, h.lower_keys.p, int64_t(h.lower_keys_h.size()), h.miss.p,
                &h.st_d->n_lower_miss);
            h.stats.kernel_launches += 3;
            CU(cudaGetLastError());
            h.read_status();
        }
    }
    if (nnew > 0) {
        h.nfree -= nnew;
        h.kc = ko;
        h.nleaf = L + nnew;
        // lower / upper nodes for the new leaves
        const int64_t nm = int64_t(h.st_h->n_lower_miss);
        if (nm > 0) {
            std::vector<uint64_t> miss(static_cast<size_t>(nm));
            h.download_small(h.miss, miss.data(), size_t(nm));
            insert_nodes(h, miss);
        }
    }
    h.rebuild_nbr();
    k_dilate<<<blocks_for(h.nleaf * 8, 256), 256, 0, h.stream>>>(h.nleaf, h.S(), h.nbr.p, h.am[h.mc].p,
                                                                  h.dmask.p, h.K(), h.run_ptr());
    ++h.stats.kernel_launches;
    CU(cudaGetLastError());
}

// ---- normalize / trim passes ----------------------------------------------
void launch_norm(gbls_handle& h, const NormArgs& a0) {
    NormArgs a = a0;
    a.acc = h.acc_d;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (h.profiling) {
        e0 = h.event();
        e1 = h.event();
        CU(cudaEventRecord(e0, h.stream));
    }
    if (h.f64) {
        if (a.spatial != GBLS_HJWENO5_BIAS && !a.copy_only)
            fail(GBLS_ERR_UNSUPPORTED, "the FP64 instance renormalises with HJWENO5");
        // Normalizer's mDt and 1/dx with ValueType double (dx = double(float(voxel size)))
        const double dx = double(float(h.voxel_size));
        a.mdt64 = dx * double(h.tr_temporal == GBLS_TVD_RK1 ? 0.3f : h.tr_temporal == GBLS_TVD_RK2 ? 0.9f : 1.0f);
        a.invdx64 = 1.0 / dx;
        launch_norm_f64(a, h.stream);
    } else if (h.mode == GBLS_MODE_PARITY) {
        if (h.parity_fp64) launch_norm_parity(a, h.stream);
        else launch_norm_exact(a, h.stream, h.norm_min_ctas);
    } else {
        launch_norm_fast(a, h.stream);
    }
    CU(cudaGetLastError());
    if (h.profiling) {
        CU(cudaEventRecord(e1, h.stream));
        h.pending.push_back({e0, e1, 1, 0.0});
    }
    ++h.stats.norm_launches;
    ++h.stats.kernel_launches;
}

// ---- adjoint tape recording ----------------------------------------------
void tape_list(gbls_handle& h, int64_t n, DevArray<uint64_t>& keys, DevArray<int32_t>& nbr) {
    keys.reserve(size_t(std::max<int64_t>(n, 1)), h.stream);
    nbr.reserve(size_t(std::max<int64_t>(n, 1)) * 6, h.stream);
    if (n == 0) return;
    CU(cudaMemcpyAsync(keys.p, h.K(), size_t(n) * 8, cudaMemcpyDeviceToDevice, h.stream));
    h.tape_inv.reserve(size_t(h.slot_cap), h.stream);
    launch_nbr_to_index(n, h.S(), h.nbr.p, h.tape_inv.p, h.slot_cap, nbr.p, h.stream);
    CU(cudaGetLastError());
}

void tape_values(gbls_handle& h, int64_t n, int m, int v, DevArray<uint64_t>* am, DevArray<uint64_t>* sm,
                 DevArray<float>* vals) {
    if (am) am->reserve(size_t(std::max<int64_t>(n, 1)) * 8, h.stream);
    if (sm) sm->reserve(size_t(std::max<int64_t>(n, 1)) * 8, h.stream);
    if (vals) vals->reserve(size_t(std::max<int64_t>(n, 1)) * LEAF_VOX, h.stream);
    launch_tape_gather(n, h.S(), h.am[m].p, h.sm[m].p, v >= 0 ? h.vals[v].p : nullptr, am ? am->p : nullptr,
                       sm ? sm->p : nullptr, vals ? vals->p : nullptr, h.stream);
    CU(cudaGetLastError());
}

void tape_begin_substep(gbls_handle& h, float t0, float dt, bool backward) {
    if (h.tape_pool.empty()) {
        h.tape.emplace_back(new TapeStep);
    } else {
        h.tape.push_back(std::move(h.tape_pool.back()));
        h.tape_pool.pop_back();
    }
    TapeStep& st = *h.tape.back();
    st.nm = 0;
    st.limited = st.opened = st.end_lim = st.first = false;
    st.maxv2 = st.open_lim = 0.0f;
    h.tape_cur = &st;
    st.n = h.nleaf;
    st.dt = dt;
    st.t0 = t0;
    st.backward = backward;
    st.gamma = h.gamma;
    tape_list(h, st.n, st.keys, st.nbr);
    tape_values(h, st.n, h.mc, h.vc, &st.am, &st.sm, &st.phin);
}

void start_intr(gbls_handle& h, const char* msg) {
    if (h.has_intr && h.intr.start) h.intr.start(h.intr.user, msg);
}
void end_intr(gbls_handle& h) {
    if (h.has_intr && h.intr.end) h.intr.end(h.intr.user);
}
bool check_intr(gbls_handle& h) {
    if (h.has_intr && h.intr.was_interrupted) return h.intr.was_interrupted(h.intr.user, -1) == 0;
    return true;
}

// Normalizer::normalize (tools/LevelSetTracker.h:528-598) over the voxels of
// pmask, starting from the current layout; when `trim` is set the final
// stage also applies Trim.  With norm_count == 0 and trim set, a trim-only
// pass runs.  Leaves the result as the current layout and per-leaf counts
// in h.cnt.
void normalize_pass(gbls_handle& h, const uint64_t* pmask, int trim, int carry = 0) {
    if (h.nleaf == 0) return;
    const float dx = float(h.voxel_size);
    const float mdt = dx * (h.tr_temporal == GBLS_TVD_RK1 ? 0.3f : h.tr_temporal == GBLS_TVD_RK2 ? 0.9f : 1.0f);
    const float invdx = 1.0f / dx;
    NormArgs base{};
    base.spatial = h.tr_spatial;
    base.nleaf = h.nleaf;
    base.slot = h.S();
    base.nbr = h.nbr.p;
    base.pmask = pmask;
    base.gamma = h.gamma;
    base.mdt = mdt;
    base.invdx = invdx;
    base.out_count = h.cnt.p;
    base.carry = carry;
    base.keys = h.K();
    base.inst_run = h.run_ptr();
    const int iters = h.norm_count;
    if (iters <= 0) {
        if (!trim) return;
        NormArgs a = base;
        const int mo = other_of(h.mc, h.mc), vo = other_of(h.vc, h.vc);
        a.src = h.layout(h.mc, h.vc);
        a.copy_only = 1;
        a.trim = trim;
        a.out_vals = h.vals[vo].p;
        a.out_amask = h.am[mo].p;
        a.out_smask = h.sm[mo].p;
        start_intr(h, "Pruning Level Set");
        launch_norm(h, a);
        end_intr(h);
        h.mc = mo;
        h.vc = vo;
        return;
    }
    const int stages = h.tr_temporal == GBLS_TVD_RK1 ? 1 : h.tr_temporal == GBLS_TVD_RK2 ? 2 : 3;
    for (int it = 0; it < iters; ++it) {
        const int m0 = h.mc, v0 = h.vc;  // phi_n
        int ms = m0, vs = v0;           // current stencil source
        for (int st = 0; st < stages; ++st) {
            const bool last = (st == stages - 1);
            NormArgs a = base;
            a.src = h.layout(ms, vs);
            a.phi = h.layout(m0, v0);
            a.trim = (last && it == iters - 1) ? trim : 0;
            int mo, vo;
            if (st == 0) {
                mo = other_of(m0, m0);
                vo = other_of(v0, v0);
                a.has_phi = 0;
                a.alpha = 0.0f;
                a.beta = 1.0f;
            } else {
                // euler12 (1/2), euler34 (3/4), euler13 (1/3): Alpha = N/D, Beta = 1 - Alpha
                const float alpha = (stages == 2) ? 1.0f / 2.0f : (st == 1 ? 3.0f / 4.0f : 1.0f / 3.0f);
                a.has_phi = 1;
                a.alpha = alpha;
                a.beta = 1.0f - alpha;
                if (last) {  // may overwrite phi_n (read only at the own voxel)
                    mo = m0;
                    vo = v0;
                    if (mo == ms) mo = other_of(ms, m0);
                    if (vo == vs) vo = other_of(vs, v0);
                } else {
                    mo = other_of(ms, m0);
                    vo = other_of(vs, v0);
                }
            }
            a.out_vals = h.vals[vo].p;
            a.out_amask = h.am[mo].p;
            a.out_smask = h.sm[mo].p;
            start_intr(h, "Normalizing level set");
            launch_norm(h, a);
            end_intr(h);
            ms = mo;
            vs = vo;
        }
        h.mc = ms;
        h.vc = vs;
        if (!carry) {
            pmask = h.am[h.mc].p;  // later iterations update the (now current) active set
            base.pmask = pmask;
        }
    }
}

// Copy the current values into the layout of pmask (| the active set when
// `carry`), optionally trimming; records per-leaf counts in h.cnt.
void relayout(gbls_handle& h, const uint64_t* pmask, int carry, int trim) {
    if (h.nleaf == 0) return;
    NormArgs a{};
    a.nleaf = h.nleaf;
    a.slot = h.S();
    a.nbr = h.nbr.p;
    a.src = h.layout(h.mc, h.vc);
    a.pmask = pmask;
    a.copy_only = 1;
    a.carry = carry;
    a.trim = trim;
    a.gamma = h.gamma;
    a.out_count = h.cnt.p;
    const int mo = other_of(h.mc, h.mc), vo = other_of(h.vc, h.vc);
    a.out_vals = h.vals[vo].p;
    a.out_amask = h.am[mo].p;
    a.out_smask = h.sm[mo].p;
    launch_norm(h, a);
    h.mc = mo;
    h.vc = vo;
}

// Leaf + node prune after a trim pass (LevelSetTracker::prune,
// tools/LevelSetTracker.h:279-300).  Uses per-leaf counts in h.cnt.
void prune_compact(gbls_handle& h) {
    const int64_t L = h.nleaf;
    bool lower_changed = false;
    h.flags_h.clear();
    if (L > 0) {
        k_keep_flags<<<blocks_for(L, 256), 256, 0, h.stream>>>(L, h.cnt.p, h.keep.p);
        ++h.stats.kernel_launches;
        CU(cudaGetLastError());
        size_t bytes = 0;
        CU(cub::DeviceScan::ExclusiveSum(nullptr, bytes, h.keep.p, h.idx.p, int(L), h.stream));
        h.cub_tmp.reserve(bytes, h.stream);
        bytes = h.cub_tmp.cap;
        CU(cub::DeviceScan::ExclusiveSum(h.cub_tmp.p, bytes, h.keep.p, h.idx.p, int(L), h.stream));
        h.clear_status();
        if (h.batch_run) CU(cudaMemsetAsync(h.inst_active.p, 0, size_t(h.ninst) * sizeof(unsigned long long), h.stream));
        const int ko = 1 - h.kc;
        k_prune_scatter<<<blocks_for(L, 256), 256, 0, h.stream>>>(
            L, h.K(), h.S(), h.keep.p, h.idx.p, h.sm[h.mc].p, h.keys[ko].p, h.slot[ko].p, h.free_slots.p,
            h.nfree, h.lower_keys.p, int64_t(h.lower_keys_h.size()), h.lower_sign.p, h.cnt.p,
            &h.st_d->n_active, &h.st_d->n_cand, &h.st_d->error, h.batch_run ? h.inst_active.p : nullptr);
        ++h.stats.kernel_launches;
        CU(cudaGetLastError());
        h.kc = ko;
        const int64_t nl = int64_t(h.lower_keys_h.size());
        h.flags.reserve(size_t(std::max<int64_t>(nl, 1)), h.stream);
        if (nl) {
            k_lower_status<<<blocks_for(nl, 128), 128, 0, h.stream>>>(nl, h.lower_keys.p, h.lower_sign.p,
                                                                       h.K(), &h.st_d->n_cand, h.flags.p,
                                                                       &h.st_d->n_lower_empty);
            ++h.stats.kernel_launches;
        }
        CU(cudaGetLastError());
        // the lower-node flags come back with the status (one read-back)
        uint8_t* fl_pin = nullptr;
        if (nl) {
            fl_pin = static_cast<uint8_t*>(h.pinned(size_t(nl)));
            CU(cudaMemcpyAsync(fl_pin, h.flags.p, size_t(nl), cudaMemcpyDeviceToHost, h.stream));
            h.pinned_issued();
        }
        if (h.before_prune_sync) h.before_prune_sync();
        h.read_status();
        const int64_t kept = int64_t(h.st_h->n_cand);
        h.nfree += L - kept;
        h.nleaf = kept;
        h.nactive = int64_t(h.st_h->n_active);
        lower_changed = h.st_h->n_lower_empty > 0;
        if (lower_changed) h.flags_h.assign(fl_pin, fl_pin + nl);
    } else if (h.batch_run) {
        CU(cudaMemsetAsync(h.inst_active.p, 0, size_t(h.ninst) * sizeof(unsigned long long), h.stream));
    }
    if (L == 0 && !h.lower_keys_h.empty()) {
        // no leaves: every lower node is empty
        const int64_t nl = int64_t(h.lower_keys_h.size());
        h.flags.reserve(size_t(nl), h.stream);
        h.clear_status();
        k_lower_status<<<blocks_for(nl, 128), 128, 0, h.stream>>>(nl, h.lower_keys.p, h.lower_sign.p, h.K(),
                                                                   &h.st_d->n_cand, h.flags.p,
                                                                   &h.st_d->n_lower_empty);
        ++h.stats.kernel_launches;
        CU(cudaGetLastError());
        h.read_status();
        lower_changed = true;
        h.nactive = 0;
    }
    if (lower_changed || !h.nodes_checked || !h.root_keys_h.empty()) prune_nodes(h, lower_changed);
    h.nodes_checked = true;
    h.rebuild_nbr();
}

void track(gbls_handle& h) {
    dilate_topology(h);
    TapeStep* tp = h.tape_cur;
    if (tp) {
        tp->nm = h.nleaf;
        tape_list(h, tp->nm, tp->keys_m, tp->nbr_m);
        tape_values(h, tp->nm, h.mc, h.vc, &tp->am3, &tp->sm3, &tp->phi3);
        tp->pmask.reserve(size_t(std::max<int64_t>(tp->nm, 1)) * 8, h.stream);
        launch_mask_gather(tp->nm, h.S(), h.dmask.p, tp->pmask.p, h.stream);
        CU(cudaGetLastError());
    }
    normalize_pass(h, h.dmask.p, h.trim);
    if (h.after_normalize) h.after_normalize();
    if (tp) tape_values(h, tp->nm, h.mc, -1, &tp->fin, nullptr, nullptr);
    if (h.nleaf > 0 && h.norm_count <= 0 && !h.trim) {
        // no normalisation and no trimming: the dilated mask becomes active as is
        NormArgs a{};
        a.nleaf = h.nleaf;
        a.slot = h.S();
        a.nbr = h.nbr.p;
        a.src = h.layout(h.mc, h.vc);
        a.pmask = h.dmask.p;
        a.copy_only = 1;
        a.gamma = h.gamma;
        a.out_count = h.cnt.p;
        const int mo = other_of(h.mc, h.mc), vo = other_of(h.vc, h.vc);
        a.out_vals = h.vals[vo].p;
        a.out_amask = h.am[mo].p;
        a.out_smask = h.sm[mo].p;
        launch_norm(h, a);
        h.mc = mo;
        h.vc = vo;
    }
    if (tp) {  // prune_compact overwrites keep / idx only when the list is non-empty
        tp->keep.reserve(size_t(std::max<int64_t>(tp->nm, 1)), h.stream);
        tp->idx.reserve(size_t(std::max<int64_t>(tp->nm, 1)), h.stream);
    }
    start_intr(h, "Pruning Level Set");
    prune_compact(h);
    end_intr(h);
    if (tp && tp->nm > 0) {
        CU(cudaMemcpyAsync(tp->keep.p, h.keep.p, size_t(tp->nm) * 4, cudaMemcpyDeviceToDevice, h.stream));
        CU(cudaMemcpyAsync(tp->idx.p, h.idx.p, size_t(tp->nm) * 4, cudaMemcpyDeviceToDevice, h.stream));
    }
    h.tape_cur = nullptr;
}

void check_scheme(int spatial, int temporal) {
    if (spatial < GBLS_FIRST_BIAS || spatial > GBLS_HJWENO5_BIAS)
        fail(GBLS_ERR_VALUE, "Spatial difference scheme not supported!");
    if (temporal < GBLS_TVD_RK1 || temporal > GBLS_TVD_RK3)
        fail(GBLS_ERR_VALUE, "Temporal integration scheme not supported!");
}

// Device form of a field for level set h at time t.  A dense field whose
// transform differs from h's (the reference compares transforms,
// tools/LevelSetAdvect.h:437) is sampled trilinearly.
FieldParams field_params(const gbls_handle& h, const gbls_field* f, float t) {
    FieldParams p{};
    if (f->desc.kind == GBLS_FIELD_DEFORMATION && f->tab_n > 0) {
        p.tab = f->tab.p;
        p.tab_lo = f->tab_lo;
        p.tab_n = f->tab_n;
        // the amplitude factor of gbls_deformation, same float operations
        p.amp = gbls_cospi(f->desc.domain == 0.0f ? 0.0f : t / f->desc.period) * f->desc.scale;
    }
    const gbls_field_desc& d = f->desc;
    p.kind = d.kind;
    for (int i = 0; i < 3; ++i) {
        p.constant[i] = d.constant[i];
        p.dense_origin[i] = d.dense_origin[i];
        p.dense_dims[i] = d.dense_dims[i];
        p.dense_background[i] = d.dense_background[i];
        p.omega[i] = d.omega[i];
        p.center[i] = d.center[i];
    }
    p.dense = f->dense.p;
    if (d.kind == GBLS_FIELD_DENSE && d.dense_map_type != 0) {
        const int vmap = d.dense_map_type - 1;  // GBLS_MAP_* of the velocity grid
        const bool same = vmap == h.map_type && d.dense_voxel_size == h.voxel_size &&
                          d.dense_translation[0] == h.translation[0] && d.dense_translation[1] == h.translation[1] &&
                          d.dense_translation[2] == h.translation[2];
        if (!same) {
            p.xform = 1;
            // map.applyMap = ijk * scale + translation for the three linear
            // map kinds (scale 1 for a translation, translation 0 for a scale)
            p.ls_scale = h.map_type == GBLS_MAP_TRANSLATION ? 1.0 : h.voxel_size;
            p.vel_inv_scale = vmap == GBLS_MAP_TRANSLATION ? 1.0 : 1.0 / d.dense_voxel_size;
            for (int i = 0; i < 3; ++i) {
                p.ls_translation[i] = h.map_type == GBLS_MAP_UNIFORM_SCALE ? 0.0 : h.translation[i];
                p.vel_translation[i] = vmap == GBLS_MAP_UNIFORM_SCALE ? 0.0 : d.dense_translation[i];
            }
        }
    }
    p.domain = d.domain;
    p.period = d.period;
    p.scale = d.scale;
    if (d.kind == GBLS_FIELD_HOST_SAMPLED) {
        p.sampled = h.hs_vel.p;
        p.prefix = h.hs_prefix.p;
    }
    return p;
}

int64_t active_count(gbls_handle& h);

// Advect::sampleField for a HOST_SAMPLED field (tools/LevelSetAdvect.h:
// 426-464): the active voxels' index coordinates in the reference's order go
// to the caller's sampler, whose velocities are uploaded for the RK stages;
// returns max |v|^2 over them (Vec3f::lengthSqr in float, math::Max).
float host_sampled_max_speed_sqr(gbls_handle& h, const gbls_field* f, float t) {
    const int64_t L = h.nleaf;
    const int64_t n = h.nactive >= 0 ? h.nactive : active_count(h);
    h.nactive = n;
    h.hs_count.reserve(size_t(std::max<int64_t>(L, 1)), h.stream);
    h.hs_prefix.reserve(size_t(std::max<int64_t>(L, 1)), h.stream);
    h.hs_ijk.reserve(size_t(std::max<int64_t>(3 * n, 1)), h.stream);
    h.hs_vel.reserve(size_t(std::max<int64_t>(3 * n, 1)), h.stream);
    h.hs_ijk_h.resize(size_t(3 * n));
    h.hs_vel_h.assign(size_t(3 * n), 0.0f);
    if (L > 0) {
        k_leaf_active<<<blocks_for(L, 256), 256, 0, h.stream>>>(L, h.S(), h.am[h.mc].p, h.hs_count.p);
        size_t bytes = 0;
        CU(cub::DeviceScan::ExclusiveSum(nullptr, bytes, h.hs_count.p, h.hs_prefix.p, int(L), h.stream));
        h.cub_tmp.reserve(bytes, h.stream);
        bytes = h.cub_tmp.cap;
        CU(cub::DeviceScan::ExclusiveSum(h.cub_tmp.p, bytes, h.hs_count.p, h.hs_prefix.p, int(L), h.stream));
        k_active_ijk<<<unsigned(L), 64, 0, h.stream>>>(L, h.K(), h.S(), h.am[h.mc].p, h.hs_prefix.p, h.hs_ijk.p);
        h.stats.kernel_launches += 3;
        CU(cudaGetLastError());
        if (n > 0)
            CU(cudaMemcpyAsync(h.hs_ijk_h.data(), h.hs_ijk.p, size_t(3 * n) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                               h.stream));
    }
    h.sync();
    f->desc.host_sample(f->desc.host_user, n, h.hs_ijk_h.data(), t, h.hs_vel_h.data());
    float m = 0.0f;
    for (int64_t i = 0; i < n; ++i) {
        const float* v = h.hs_vel_h.data() + 3 * i;
        const float l2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        m = (m < l2) ? l2 : m;  // math::Max
    }
    if (n > 0)
        CU(cudaMemcpyAsync(h.hs_vel.p, h.hs_vel_h.data(), size_t(3 * n) * sizeof(float), cudaMemcpyHostToDevice,
                           h.stream));
    h.sync();  // the host copy may be refilled by the next substep's sampler
    return m;
}

// max |v|^2 over the active voxels at time t (sampleField, :447-455).
// Enqueue the CFL reduction (max |v|^2 over the active voxels at time t)
// into the status block, which the caller has cleared; the leaf count is
// read on the device when `nleaf_dev` is given (h.nleaf is then an upper
// bound).
void enqueue_max_speed(gbls_handle& h, const gbls_field* f, float t, const unsigned long long* nleaf_dev) {
    CflArgs a{};
    a.nleaf = h.nleaf;
    a.nleaf_dev = nleaf_dev;
    a.keys = h.K();
    a.slot = h.S();
    a.amask = h.am[h.mc].p;
    a.t0 = t;
    a.field = field_params(h, f, t);
    a.max_bits = &h.st_d->max_v2_bits;
    h.cfl_part.reserve(size_t(std::max<int64_t>(h.nleaf, 1)), h.stream);
    a.part = h.cfl_part.p;
    launch_cfl(a, h.stream, h.cfl_leaves);
    h.stats.kernel_launches += 2;
    CU(cudaGetLastError());
}

// The CFL maximum of the renormalised level set at time t on the side
// stream, concurrently with the prune on the main stream: the leaves before
// the prune have the same active voxels (a pruned leaf has none), so the
// maximum is the same.  Result in h.cfl_d; ev_cfl follows it.
void enqueue_max_speed_side(gbls_handle& h, const gbls_field* f, float t) {
    CU(cudaEventRecord(h.ev_norm, h.stream));
    CU(cudaStreamWaitEvent(h.side, h.ev_norm, 0));
    CflArgs a{};
    a.nleaf = h.nleaf;
    a.keys = h.K();
    a.slot = h.S();
    a.amask = h.am[h.mc].p;
    a.t0 = t;
    a.field = field_params(h, f, t);
    a.max_bits = h.cfl_d;
    h.cfl_part.reserve(size_t(std::max<int64_t>(h.nleaf, 1)), h.side);
    a.part = h.cfl_part.p;
    CU(cudaMemsetAsync(h.cfl_d, 0, sizeof(unsigned int), h.side));
    launch_cfl(a, h.side, h.cfl_leaves);
    h.stats.kernel_launches += 2;
    CU(cudaGetLastError());
    CU(cudaEventRecord(h.ev_cfl, h.side));
}

float status_max_speed(const gbls_handle& h) {
    float m;
    std::memcpy(&m, &h.st_h->max_v2_bits, 4);
    return m;
}

float max_speed_sqr(gbls_handle& h, const gbls_field* f, float t) {
    if (f->desc.kind == GBLS_FIELD_HOST_SAMPLED) return host_sampled_max_speed_sqr(h, f, t);
    if (f->desc.kind == GBLS_FIELD_CONSTANT) {
        const float* c = f->desc.constant;
        return c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
    }
    h.clear_status();
    enqueue_max_speed(h, f, t, nullptr);
    h.read_status();
    return status_max_speed(h);
}

void rk_stage(gbls_handle& h, const RkArgs& a) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (h.profiling) {
        e0 = h.event();
        e1 = h.event();
        CU(cudaEventRecord(e0, h.stream));
    }
    if (h.f64) {
        if (a.spatial != GBLS_HJWENO5_BIAS) fail(GBLS_ERR_UNSUPPORTED, "the FP64 instance advects with HJWENO5");
        if (a.inst_run) fail(GBLS_ERR_UNSUPPORTED, "the FP64 instance runs single level sets");
        launch_rk_f64(a, h.stream);
    } else if (h.mode == GBLS_MODE_PARITY) {
        if (h.parity_fp64) launch_rk_parity(a, h.stream);
        else {
            RkArgs b = a;
            b.parts = h.rk_parts;
            launch_rk_exact(b, h.stream, h.rk_min_ctas);
        }
    } else {
        launch_rk_fast(a, h.stream);
    }
    CU(cudaGetLastError());
    // FP32 values of the active voxels: stencil read + result write (+ phi_n read)
    const double bytes = double(h.nactive) * (a.has_phi ? 12.0 : 8.0);
    if (h.profiling) {
        CU(cudaEventRecord(e1, h.stream));
        h.pending.push_back({e0, e1, 0, bytes});
    }
    h.stats.rk_bytes += bytes;
    ++h.stats.rk_launches;
    ++h.stats.kernel_launches;
}

// The TVD-RK stages of one substep (tools/LevelSetAdvect.h:360-405).
void advect_stages(gbls_handle& h, const gbls_field* f, int spatial, int temporal, float t0, float dt, bool backward,
                   double dt64 = 0.0) {
    RkArgs base{};
    base.dt64 = dt64;
    base.spatial = spatial;
    base.nleaf = h.nleaf;
    base.keys = h.K();
    base.slot = h.S();
    base.nbr = h.nbr.p;
    base.dt = dt;
    base.gamma = h.gamma;
    base.t0 = t0;
    base.backward = backward ? 1 : 0;
    base.invdx = 1.0 / h.voxel_size;
    base.invdx_f = float(1.0 / h.voxel_size);
    if (f) base.field = field_params(h, f, t0);
    if (h.batch_run) {
        base.inst_run = h.inst_run.p;
        base.inst_dt = h.inst_dt.p;
        base.inst_t0 = h.inst_t0.p;
        base.inst_field = h.inst_field.p;
    }
    const int a0 = h.vc, b0 = (h.vc + 1) % 3, c0 = (h.vc + 2) % 3;
    auto stage = [&](int src, int phin, int out, float alpha, int has_phi, const char* msg) {
        RkArgs a = base;
        a.src = h.layout(h.mc, src);
        a.phin = h.vals[phin].p;
        a.out = h.vals[out].p;
        a.alpha = alpha;
        a.beta = 1.0f - alpha;
        a.has_phi = has_phi;
        start_intr(h, msg);
        rk_stage(h, a);
        end_intr(h);
    };
    if (temporal == GBLS_TVD_RK1) {
        base.copy_done = 1;  // the only stage writes the result buffer
        stage(a0, a0, b0, 0.0f, 0, "Advecting level set using TVD_RK1");
        h.vc = b0;
    } else if (temporal == GBLS_TVD_RK2) {
        stage(a0, a0, b0, 0.0f, 0, "Advecting level set using TVD_RK1 (step 1 of 2)");
        stage(b0, a0, a0, 1.0f / 2.0f, 1, "Advecting level set using TVD_RK1 (step 2 of 2)");
        h.vc = a0;
    } else {
        stage(a0, a0, b0, 0.0f, 0, "Advecting level set using TVD_RK3 (step 1 of 3)");
        if (h.tape_cur) tape_values(h, h.nleaf, h.mc, b0, nullptr, nullptr, &h.tape_cur->phi1);
        stage(b0, a0, c0, 3.0f / 4.0f, 1, "Advecting level set using TVD_RK3 (step 2 of 3)");
        if (h.tape_cur) tape_values(h, h.nleaf, h.mc, c0, nullptr, nullptr, &h.tape_cur->phi2);
        stage(c0, a0, a0, 1.0f / 3.0f, 1, "Advecting level set using TVD_RK3 (step 3 of 3)");
        h.vc = a0;
    }
}

// |v|^2 of the time step in double for the FP64 instance: (x*x + y*y) + z*z
// of the widened components at the first active voxel (leaf order, voxel
// order) whose Vec3f |v|^2 is the float maximum maxv2.
double max_speed_sqr_f64(gbls_handle& h, const gbls_field* f, float t, float maxv2) {
    if (f->desc.kind == GBLS_FIELD_CONSTANT) {
        const double x = f->desc.constant[0], y = f->desc.constant[1], z = f->desc.constant[2];
        return (x * x + y * y) + z * z;
    }
    h.argk.reserve(1, h.stream);
    h.argv.reserve(1, h.stream);
    launch_argmax_f64(h.nleaf, h.K(), h.S(), h.am[h.mc].p, field_params(h, f, t), t, maxv2, h.argk.p, h.argv.p,
                      h.stream);
    h.stats.kernel_launches += 2;
    CU(cudaGetLastError());
    double v = 0.0;
    CU(cudaMemcpyAsync(&v, h.argv.p, sizeof(double), cudaMemcpyDeviceToHost, h.stream));
    h.sync();
    if (!(v >= 0.0)) fail(GBLS_ERR_RUNTIME, "no active voxel holds the maximum speed");
    return v;
}

// LevelSetAdvection::advect (tools/LevelSetAdvect.h:338-418) for the FP64
// instance (the FloatGrid scheme with double values): time and substep
// lengths in double (the interval clock over double time), velocities
// sampled as Vec3f at float(t), the RK stages and the tracker on double
// values.
void advect_f64(gbls_handle& h, const gbls_field* field, int spatial, int temporal, float t0, float t1, float cfl,
                uint64_t& count, bool& interrupted) {
    if (spatial != GBLS_HJWENO5_BIAS || h.tr_spatial != GBLS_HJWENO5_BIAS)
        fail(GBLS_ERR_UNSUPPORTED, "the FP64 instance advects and tracks with HJWENO5");
    if (field->desc.kind == GBLS_FIELD_HOST_SAMPLED)
        fail(GBLS_ERR_UNSUPPORTED, "the FP64 instance samples fields the device evaluates");
    const bool forward = t0 < t1;
    CflClockT<double> clock(t0, t1, cfl, temporal, float(h.voxel_size));
    double t = t0;
    h.cfl_cache.valid = false;
    while (clock.running(t)) {
        if (!check_intr(h)) { interrupted = true; break; }
        if (h.nleaf == 0) break;  // sampleField returns 0 for an empty grid
        const float tf = float(t);
        start_intr(h, "Sampling advection field");
        const float maxv2 = max_speed_sqr(h, field, tf);
        end_intr(h);
        if (!(maxv2 > 1e-5f) && !(maxv2 < -1e-5f)) break;  // isApproxZero(maxAbsV, Delta)
        const double dt = clock.next(t, max_speed_sqr_f64(h, field, tf, maxv2));
        if (dt == 0.0) break;
        if (h.nactive < 0) h.nactive = active_count(h);
        h.stats.voxel_updates += uint64_t(h.nactive);
        ++h.stats.substeps;
        advect_stages(h, field, spatial, temporal, tf, float(dt), !forward, dt);
        clock.advance(t, dt);
        ++count;
        track(h);
    }
    h.sync();
}

// ---- LevelSetMorphing (tools/LevelSetMorph.h) -------------------------------
LookupGrid lookup_grid(gbls_handle& g) {
    LookupGrid L{};
    L.keys = g.K();
    L.slot = g.S();
    L.nleaf = g.nleaf;
    L.layout = g.layout(g.mc, g.vc);
    L.nodes = g.nodes();
    L.gamma = g.gamma;
    return L;
}

// The RK stages of one morphing substep (Morph::advect, LevelSetMorph.h:
// 479-510): euler01 / euler12 / euler34 / euler13 over the same buffers as
// the advection stages.
void morph_stages(gbls_handle& h, int spatial, int temporal, float dt) {
    if (h.f64) fail(GBLS_ERR_UNSUPPORTED, "the FP64 instance runs advection and tracking only");
    MorphArgs base{};
    base.spatial = spatial;
    base.nleaf = h.nleaf;
    base.slot = h.S();
    base.nbr = h.nbr.p;
    base.dt = dt;
    base.gamma = h.gamma;
    const double inv = 1.0 / h.voxel_size;  // map.getInvScaleSqr()[0]
    base.invdxdx = float(inv * inv);
    base.speed = h.morph_speed.p;
    const int a0 = h.vc, b0 = (h.vc + 1) % 3, c0 = (h.vc + 2) % 3;
    auto stage = [&](int src, int phin, int out, float alpha, int has_phi) {
        MorphArgs a = base;
        a.src = h.layout(h.mc, src);
        a.phin = h.vals[phin].p;
        a.out = h.vals[out].p;
        a.alpha = alpha;
        a.beta = 1.0f - alpha;
        a.has_phi = has_phi;
        start_intr(h, "Morphing level set");
        if (h.mode == GBLS_MODE_PARITY) (h.parity_fp64 ? launch_morph_stage_parity : launch_morph_stage_exact)(a, h.stream);
        else launch_morph_stage_fast(a, h.stream);
        CU(cudaGetLastError());
        ++h.stats.kernel_launches;
        end_intr(h);
    };
    if (temporal == GBLS_TVD_RK1) {
        stage(a0, a0, b0, 0.0f, 0);
        h.vc = b0;
    } else if (temporal == GBLS_TVD_RK2) {
        stage(a0, a0, b0, 0.0f, 0);
        stage(b0, a0, a0, 1.0f / 2.0f, 1);
        h.vc = a0;
    } else {
        stage(a0, a0, b0, 0.0f, 0);
        stage(b0, a0, c0, 3.0f / 4.0f, 1);
        stage(c0, a0, a0, 1.0f / 3.0f, 1);
        h.vc = a0;
    }
}

// Morph::sampleSpeed (LevelSetMorph.h:521-546): speed per active voxel and
// the maximum of 1e-6 and every |s|.
float morph_sample_speed(gbls_handle& h, gbls_handle& target, gbls_handle* mask, float mask_min, float inv_norm,
                         int invert) {
    h.cfl_part.reserve(size_t(std::max<int64_t>(h.nleaf, 1)), h.stream);
    h.morph_speed.reserve(size_t(h.slot_cap) * LEAF_VOX, h.stream);
    MorphSpeedArgs a{};
    a.nleaf = h.nleaf;
    a.keys = h.K();
    a.slot = h.S();
    a.src = h.layout(h.mc, h.vc);
    a.speed = h.morph_speed.p;
    a.part = h.cfl_part.p;
    a.target = lookup_grid(target);
    a.has_mask = mask ? 1 : 0;
    if (mask) a.mask = lookup_grid(*mask);
    a.mask_min = mask_min;
    a.mask_inv_norm = inv_norm;
    a.invert = invert;
    h.clear_status();
    if (h.mode == GBLS_MODE_PARITY) launch_morph_speed_parity(a, &h.st_d->max_v2_bits, h.stream);
    else launch_morph_speed_fast(a, &h.st_d->max_v2_bits, h.stream);
    CU(cudaGetLastError());
    h.stats.kernel_launches += 2;
    h.read_status();
    float m;
    std::memcpy(&m, &h.st_h->max_v2_bits, 4);
    return (1e-6f < m) ? m : 1e-6f;  // mMaxAbsS starts at mMinAbsS = 1e-6
}

// ---- LevelSetFilter (tools/LevelSetFilter.h) -------------------------------
// One Filter::cook pass: every active voxel from the current values into the
// free value buffer, which becomes current (swapLeafBuffer).
void filter_pass(gbls_handle& h, FilterArgs a, const char* msg) {
    if (h.f64) fail(GBLS_ERR_UNSUPPORTED, "the FP64 instance runs advection and tracking only");
    if (h.nleaf == 0) return;
    const int vo = other_of(h.vc, h.vc);
    a.nleaf = h.nleaf;
    a.slot = h.S();
    a.nbr = h.nbr.p;
    a.src = h.layout(h.mc, h.vc);
    a.out = h.vals[vo].p;
    a.gamma = h.gamma;
    a.keys = h.K();
    a.nodes = h.nodes();
    if (h.filter_mask.on) {
        a.has_mask = 1;
        a.mask = lookup_grid(*h.filter_mask.grid);
        a.mask_min = h.filter_mask.min;
        a.mask_inv_norm = h.filter_mask.inv_norm;
        a.invert = h.filter_mask.invert;
    }
    start_intr(h, msg);
    if (h.mode == GBLS_MODE_PARITY) (h.parity_fp64 ? launch_filter_parity : launch_filter_exact)(a, h.stream);
    else launch_filter_fast(a, h.stream);
    CU(cudaGetLastError());
    ++h.stats.kernel_launches;
    end_intr(h);
    h.vc = vo;
}

// Filter::box (:277-289): axis-0, axis-2 and axis-1 averages (the
// reference's boxX/boxY/boxZ bind Avg<0>, Avg<2>, Avg<1>), then track.
void filter_box(gbls_handle& h, int width) {
    width = std::max(1, width);
    if (width > 3) fail(GBLS_ERR_UNSUPPORTED, "box widths above 3 voxels exceed the device stencil halo");
    FilterArgs a{};
    a.op = FILTER_BOX;
    a.width = width;
    a.frac = 1.0f / float(2 * width + 1);
    for (int axis : {0, 2, 1}) {
        a.axis = axis;
        filter_pass(h, a, "Mean-value flow of level set");
    }
    track(h);
}

// ---- upload / download ------------------------------------------------------
bool is_pm_gamma(float v, float g) { return v == g || v == -g; }

// Upload n level sets (instance i from descs[i]; n == 1 for a plain handle).
// Upload n instances.  dev_leaves (a single level set): the leaf keys are
// computed and checked on the device; returns false, having changed only
// device scratch, when the leaves are not valid input in tree order, and the
// caller repeats the upload with host-side keys (which sorts or reports the
// error).
bool upload_impl(gbls_handle& h, const gbls_grid_desc* descs, int n, bool dev_leaves) {
    if (n < 1 || n > GBLS_MAX_INSTANCES) fail(GBLS_ERR_INVALID_ARGUMENT, "instance count out of range");
    const gbls_grid_desc* d0 = descs;
    if (!(d0->voxel_size > 0.0)) fail(GBLS_ERR_RUNTIME, "The transform must have uniform scale for the LevelSetTracker to function");
    if (!h.volume && !(d0->background > 0.0f))
        fail(GBLS_ERR_RUNTIME, "LevelSetTracker expected a level set (positive background)");
    if (d0->map_type < GBLS_MAP_UNIFORM_SCALE || d0->map_type > GBLS_MAP_TRANSLATION)
        fail(GBLS_ERR_VALUE, "MapType not supported!");
    h.voxel_size = d0->voxel_size;
    for (int i = 0; i < 3; ++i) h.translation[i] = d0->translation[i];
    h.map_type = d0->map_type;
    h.gamma = d0->background;
    h.ninst = n;
    const float g = d0->background;
    auto check_origin = [&](const int32_t* o, int align) {
        for (int a = 0; a < 3; ++a) {
            if (o[a] % align != 0) fail(GBLS_ERR_INVALID_ARGUMENT, "node origin not aligned");
            if (o[a] < -COORD_SAFE || o[a] >= COORD_SAFE) fail(GBLS_ERR_DOMAIN, "coordinate outside the supported range");
        }
    };
    // Keys of every node with its index in the staged (concatenated) input
    // arrays; inputs in tree order (the usual case) need no sort.
    struct Src { uint64_t key; int64_t idx; bool operator<(const Src& o) const { return key < o.key; } };
    std::vector<Src> lv, lo, up, rt;
    std::vector<int64_t> lv_base(size_t(n) + 1, 0), lo_base(size_t(n) + 1, 0), up_base(size_t(n) + 1, 0);
    for (int q = 0; q < n; ++q) {
        const gbls_grid_desc* d = descs + q;
        if (d->voxel_size != d0->voxel_size || d->background != d0->background)
            fail(GBLS_ERR_INVALID_ARGUMENT, "batch instances must share voxel size and background");
        if (d->leaf_count < 0 || d->lower_count < 0 || d->upper_count < 0 || d->root_tile_count < 0)
            fail(GBLS_ERR_INVALID_ARGUMENT, "negative count");
        if (d->leaf_count > 0 && (!d->leaf_origins || !d->leaf_masks || !d->leaf_values))
            fail(GBLS_ERR_INVALID_ARGUMENT, "null leaf arrays");
        if ((d->lower_count > 0 && (!d->lower_origins || !d->lower_tiles)) ||
            (d->upper_count > 0 && (!d->upper_origins || !d->upper_tiles)) ||
            (d->root_tile_count > 0 && (!d->root_tile_origins || !d->root_tile_values)))
            fail(GBLS_ERR_INVALID_ARGUMENT, "null node arrays");
        const uint64_t ib = uint64_t(q) << KEY_INST_SHIFT;
        lv_base[size_t(q) + 1] = lv_base[size_t(q)] + d->leaf_count;
        lo_base[size_t(q) + 1] = lo_base[size_t(q)] + d->lower_count;
        up_base[size_t(q) + 1] = up_base[size_t(q)] + d->upper_count;
        if (!dev_leaves) {
            lv.reserve(lv.size() + size_t(d->leaf_count));
            for (int64_t i = 0; i < d->leaf_count; ++i) {
                const int32_t* o = d->leaf_origins + 3 * i;
                check_origin(o, 8);
                lv.push_back({leaf_key(o[0], o[1], o[2]) | ib, lv_base[size_t(q)] + i});
            }
        }
        for (int64_t i = 0; i < d->lower_count; ++i) {
            const int32_t* o = d->lower_origins + 3 * i;
            check_origin(o, 128);
            lo.push_back({(leaf_key(o[0], o[1], o[2]) | ib) >> 12, lo_base[size_t(q)] + i});
        }
        for (int64_t i = 0; i < d->upper_count; ++i) {
            const int32_t* o = d->upper_origins + 3 * i;
            check_origin(o, 4096);
            up.push_back({(leaf_key(o[0], o[1], o[2]) | ib) >> 27, up_base[size_t(q)] + i});
        }
        for (int64_t i = 0; i < d->root_tile_count; ++i) {
            const int32_t* o = d->root_tile_origins + 3 * i;
            check_origin(o, 4096);
            rt.push_back({(leaf_key(o[0], o[1], o[2]) | ib) >> 27, int64_t(q) << 32 | i});
        }
    }
    auto order = [](std::vector<Src>& v, const char* dup) {
        if (!std::is_sorted(v.begin(), v.end())) std::sort(v.begin(), v.end());
        for (size_t i = 1; i < v.size(); ++i)
            if (v[i].key == v[i - 1].key) fail(GBLS_ERR_INVALID_ARGUMENT, dup);
    };
    order(lv, "duplicate leaf");
    order(lo, "duplicate lower node");
    order(up, "duplicate upper node");
    order(rt, "duplicate root tile");
    const int64_t L = dev_leaves ? d0->leaf_count : int64_t(lv.size()), NLO = int64_t(lo.size()),
                  NUP = int64_t(up.size());
    const int64_t pl = dev_leaves ? 0 : L;  // leaf part of perm (identity on the device path)
    std::vector<uint64_t> keys(static_cast<size_t>(pl)), lkeys(static_cast<size_t>(NLO)), ukeys(static_cast<size_t>(NUP));
    std::vector<int32_t> perm(static_cast<size_t>(pl + NLO + NUP));
    for (int64_t i = 0; i < pl; ++i) { keys[size_t(i)] = lv[size_t(i)].key; perm[size_t(i)] = int32_t(lv[size_t(i)].idx); }
    for (int64_t i = 0; i < NLO; ++i) { lkeys[size_t(i)] = lo[size_t(i)].key; perm[size_t(pl + i)] = int32_t(lo[size_t(i)].idx); }
    for (int64_t i = 0; i < NUP; ++i) { ukeys[size_t(i)] = up[size_t(i)].key; perm[size_t(pl + NLO + i)] = int32_t(up[size_t(i)].idx); }
    // every leaf under a lower node, every lower node under an upper node (sorted walks)
    auto parents = [](const std::vector<uint64_t>& child, int shift, const std::vector<uint64_t>& par, const char* msg) {
        size_t p = 0;
        for (uint64_t k : child) {
            const uint64_t pk = k >> shift;
            while (p < par.size() && par[p] < pk) ++p;
            if (p == par.size() || par[p] != pk) fail(GBLS_ERR_INVALID_ARGUMENT, msg);
        }
    };
    if (!dev_leaves) parents(keys, 12, lkeys, "leaf without lower node");
    parents(lkeys, 15, ukeys, "lower node without upper node");
    h.root_keys_h.clear();
    h.root_sign_h.clear();
    for (const Src& r : rt) {
        const float v = descs[r.idx >> 32].root_tile_values[r.idx & 0xffffffff];
        if (!is_pm_gamma(v, g)) fail(GBLS_ERR_UNSUPPORTED, "root tile other than +-background");
        if (std::binary_search(ukeys.begin(), ukeys.end(), r.key)) fail(GBLS_ERR_INVALID_ARGUMENT, "root tile overlaps an upper node");
        h.root_keys_h.push_back(r.key);
        h.root_sign_h.push_back(uint8_t(v < 0.0f ? 1 : 0));
    }
    // device state (nothing of a previous level set is kept)
    h.nleaf = 0;
    h.kc = 0;
    h.mc = 0;
    h.vc = 0;
    h.slot_cap = 0;
    h.nfree = 0;
    h.ensure_leaf_cap(std::max<int64_t>(L, 16) + L / 2);
    h.nleaf = L;
    const int64_t scap = L + L / 2 + 1024;
    for (int b = 0; b < 3; ++b) {
        h.am[b].reserve(size_t(scap) * 8, h.stream);
        h.sm[b].reserve(size_t(scap) * 8, h.stream);
        h.vals[b].reserve(size_t(scap) * LEAF_VOX, h.stream);
    }
    h.dmask.reserve(size_t(scap) * 8, h.stream);
    h.emask.reserve(size_t(scap) * 8, h.stream);
    h.free_slots.reserve(size_t(scap), h.stream);
    h.slot_cap = scap;
    h.nfree = scap - L;
    launch_free_slots(scap - L, int32_t(scap), h.free_slots.p, h.stream);
    if (!dev_leaves) {
        std::vector<int32_t> slots(static_cast<size_t>(L));
        for (int64_t i = 0; i < L; ++i) slots[size_t(i)] = int32_t(i);
        h.keys[0].upload(keys.data(), keys.size(), h.stream);
        h.slot[0].upload(slots.data(), slots.size(), h.stream);
    }
    h.io_perm.upload(perm.data(), perm.size(), h.stream);
    h.lower_keys_h = lkeys;
    h.lower_keys.upload(lkeys.data(), lkeys.size(), h.stream);
    h.upper_keys.upload(ukeys.data(), ukeys.size(), h.stream);
    h.lower_sign.reserve(size_t(std::max<int64_t>(NLO, 1)) * 64, h.stream);
    h.upper_sign.reserve(size_t(std::max<int64_t>(NUP, 1)) * 512, h.stream);
    h.io_tiles.reserve(size_t(std::max<int64_t>(NLO * LOWER_SLOTS + NUP * UPPER_SLOTS, 1)), h.stream);
    // stage the inputs (mask set 1 and value buffer 1 are free) and pack them
    float* lo_stage = h.io_tiles.p;
    float* up_stage = h.io_tiles.p + NLO * LOWER_SLOTS;
    for (int q = 0; q < n; ++q) {
        const gbls_grid_desc* d = descs + q;
        const size_t a = size_t(lv_base[size_t(q)]), b = size_t(lo_base[size_t(q)]), c = size_t(up_base[size_t(q)]);
        if (d->leaf_count) {
            // host or device arrays (a NanoVDB import gathers its leaves on the device)
            CU(cudaMemcpyAsync(h.am[1].p + a * 8, d->leaf_masks, size_t(d->leaf_count) * 64, cudaMemcpyDefault, h.stream));
            CU(cudaMemcpyAsync(h.vals[1].p + a * LEAF_VOX, d->leaf_values, size_t(d->leaf_count) * LEAF_VOX * 4,
                               cudaMemcpyDefault, h.stream));
        }
        if (d->lower_count)
            CU(cudaMemcpyAsync(lo_stage + b * LOWER_SLOTS, d->lower_tiles, size_t(d->lower_count) * LOWER_SLOTS * 4,
                               cudaMemcpyHostToDevice, h.stream));
        if (d->upper_count)
            CU(cudaMemcpyAsync(up_stage + c * UPPER_SLOTS, d->upper_tiles, size_t(d->upper_count) * UPPER_SLOTS * 4,
                               cudaMemcpyHostToDevice, h.stream));
    }
    h.clear_status();
    unsigned long long* err = &h.st_d->io_err;
    if (dev_leaves) {
        h.io_orig.reserve(size_t(L) * 3, h.stream);
        CU(cudaMemcpyAsync(h.io_orig.p, d0->leaf_origins, size_t(L) * 12, cudaMemcpyHostToDevice, h.stream));
        launch_leaf_keys(L, h.io_orig.p, h.lower_keys.p, NLO, h.keys[0].p, h.slot[0].p, err, h.stream);
        ++h.stats.kernel_launches;
    }
    launch_pack_leaves(L, dev_leaves ? nullptr : h.io_perm.p, h.am[1].p, h.vals[1].p, g, h.am[0].p, h.sm[0].p,
                       h.vals[0].p, err, h.stream);
    launch_node_signs(NLO, 12, h.lower_keys.p, h.io_perm.p + pl, lo_stage, h.keys[0].p, L, g, h.lower_sign.p, err,
                      IO_ERR_LOWER_TILE, h.stream);
    launch_node_signs(NUP, 15, h.upper_keys.p, h.io_perm.p + pl + NLO, up_stage, h.lower_keys.p, NLO, g,
                      h.upper_sign.p, err, IO_ERR_UPPER_TILE, h.stream);
    h.stats.kernel_launches += (L > 0) + (NLO > 0) + (NUP > 0);
    CU(cudaGetLastError());
    std::vector<uint64_t> usign(static_cast<size_t>(NUP) * 512);
    h.upper_sign.download(usign.data(), usign.size(), h.stream);
    h.read_status();
    const unsigned long long e = h.st_h->io_err;
    if (dev_leaves && (e & IO_ERR_KEYS)) return false;
    if (e & IO_ERR_LEAF_VALUE) fail(GBLS_ERR_UNSUPPORTED, "inactive leaf value other than +-background");
    if (e & IO_ERR_LOWER_TILE) fail(GBLS_ERR_UNSUPPORTED, "lower-node tile other than +-background");
    if (e & IO_ERR_UPPER_TILE) fail(GBLS_ERR_UNSUPPORTED, "upper-node tile other than +-background");
    h.upper_keys_h = ukeys;
    h.upper_sign_h.swap(usign);
    h.nodes_checked = false;
    h.upload_upper_root();
    h.rebuild_nbr();
    h.inst_run.reserve(size_t(n), h.stream);
    h.inst_dt.reserve(size_t(n), h.stream);
    h.inst_t0.reserve(size_t(n), h.stream);
    h.inst_field.reserve(size_t(n), h.stream);
    h.inst_max.reserve(size_t(n), h.stream);
    h.inst_active.reserve(size_t(n), h.stream);
    h.sync();
    h.nactive = -1;
    return true;
}

// The FP64 instance keeps 512 doubles per slot in the value arrays: widen
// the current FP32 values (exactly) into a new array twice the size, or
// round the current doubles back to FP32.  The other two buffers only
// change capacity: the RK stages and renormalisation write them in full.
void widen_values(gbls_handle& h) {
    const size_t n = size_t(h.slot_cap) * LEAF_VOX;
    DevArray<float> w;
    w.reserve(std::max<size_t>(2 * n, 32), h.stream);
    launch_widen(h.vals[h.vc].p, reinterpret_cast<double*>(w.p), n, h.stream);
    ++h.stats.kernel_launches;
    CU(cudaGetLastError());
    h.sync();
    std::swap(h.vals[h.vc].p, w.p);
    std::swap(h.vals[h.vc].cap, w.cap);
    for (int b = 0; b < 3; ++b)
        if (b != h.vc) h.vals[b].reserve(std::max<size_t>(2 * n, 32), h.stream);
}

void narrow_values(gbls_handle& h) {
    const size_t n = size_t(h.slot_cap) * LEAF_VOX;
    DevArray<float> w;
    w.reserve(std::max<size_t>(n, 16), h.stream);
    launch_narrow(reinterpret_cast<const double*>(h.vals[h.vc].p), w.p, n, h.stream);
    ++h.stats.kernel_launches;
    CU(cudaGetLastError());
    h.sync();
    std::swap(h.vals[h.vc].p, w.p);
    std::swap(h.vals[h.vc].cap, w.cap);
}

// The current values as FP32 (the FP64 instance's rounded into f32_view).
const float* current_f32(gbls_handle& h) {
    if (!h.f64) return h.vals[h.vc].p;
    const size_t n = size_t(h.slot_cap) * LEAF_VOX;
    h.f32_view.reserve(std::max<size_t>(n, 16), h.stream);
    launch_narrow(reinterpret_cast<const double*>(h.vals[h.vc].p), h.f32_view.p, n, h.stream);
    ++h.stats.kernel_launches;
    CU(cudaGetLastError());
    return h.f32_view.p;
}

void upload(gbls_handle& h, const gbls_grid_desc* descs, int n) {
    if (n == 1 && descs[0].leaf_count > 0 && descs[0].leaf_origins && descs[0].leaf_masks && descs[0].leaf_values &&
        upload_impl(h, descs, n, true)) {
        if (h.f64) widen_values(h);
        return;
    }
    upload_impl(h, descs, n, false);
    if (h.f64) widen_values(h);
}

// Index ranges [lo, hi) of instance `inst` in the leaf / lower / upper / root
// lists (all of them for inst < 0): instance bits are the top key bits, so
// every list is sorted by instance first.
struct InstRange {
    int64_t l0, l1, lo0, lo1, u0, u1, r0, r1;
};

InstRange inst_range(gbls_handle& h, const std::vector<uint64_t>& keys, int inst) {
    InstRange r{0, int64_t(keys.size()), 0, int64_t(h.lower_keys_h.size()), 0,
                int64_t(h.upper_keys_h.size()), 0, int64_t(h.root_keys_h.size())};
    if (inst < 0) return r;
    auto rng = [](const std::vector<uint64_t>& v, uint64_t a, uint64_t b, int64_t& x, int64_t& y) {
        x = int64_t(std::lower_bound(v.begin(), v.end(), a) - v.begin());
        y = int64_t(std::lower_bound(v.begin(), v.end(), b) - v.begin());
    };
    const uint64_t q = uint64_t(inst), q1 = uint64_t(inst + 1);
    rng(keys, q << KEY_INST_SHIFT, q1 << KEY_INST_SHIFT, r.l0, r.l1);
    rng(h.lower_keys_h, q << (KEY_INST_SHIFT - 12), q1 << (KEY_INST_SHIFT - 12), r.lo0, r.lo1);
    rng(h.upper_keys_h, q << (KEY_INST_SHIFT - 27), q1 << (KEY_INST_SHIFT - 27), r.u0, r.u1);
    rng(h.root_keys_h, q << (KEY_INST_SHIFT - 27), q1 << (KEY_INST_SHIFT - 27), r.r0, r.r1);
    return r;
}

std::vector<uint64_t> host_keys(gbls_handle& h) {
    std::vector<uint64_t> keys(static_cast<size_t>(h.nleaf));
    h.keys[h.kc].download(keys.data(), size_t(h.nleaf), h.stream);
    h.sync();
    return keys;
}

void download(gbls_handle& h, gbls_grid_desc* d, int inst) {
    InstRange R{0, h.nleaf, 0, int64_t(h.lower_keys_h.size()), 0, int64_t(h.upper_keys_h.size()), 0,
                int64_t(h.root_keys_h.size())};
    if (inst >= 0) R = inst_range(h, host_keys(h), inst);
    const int64_t L = R.l1 - R.l0, NLO = R.lo1 - R.lo0, NUP = R.u1 - R.u0;
    if (d->leaf_count != L || d->lower_count != NLO || d->upper_count != NUP || d->root_tile_count != R.r1 - R.r0)
        fail(GBLS_ERR_INVALID_ARGUMENT, "descriptor counts do not match gbls_get_counts");
    if ((L > 0 && (!d->leaf_origins || !d->leaf_masks || !d->leaf_values)) ||
        (NLO > 0 && (!d->lower_origins || !d->lower_tiles)) || (NUP > 0 && (!d->upper_origins || !d->upper_tiles)) ||
        (R.r1 > R.r0 && (!d->root_tile_origins || !d->root_tile_values)))
        fail(GBLS_ERR_INVALID_ARGUMENT, "null arrays in the download descriptor");
    d->voxel_size = h.voxel_size;
    for (int i = 0; i < 3; ++i) d->translation[i] = h.translation[i];
    d->map_type = h.map_type;
    d->background = h.gamma;
    const float g = h.gamma;
    // dense values, masks and origins are assembled in the free value
    // buffer / mask set, node tiles in the tile staging buffer
    if (L > 0) {
        float* dense = h.vals[other_of(h.vc, h.vc)].p;
        uint64_t* masks = h.am[other_of(h.mc, h.mc)].p;
        h.io_orig.reserve(size_t(L) * 3, h.stream);
        k_unpack<<<unsigned(L), 128, 0, h.stream>>>(L, h.S() + R.l0, h.am[h.mc].p, h.sm[h.mc].p, current_f32(h), g,
                                                     dense);
        launch_leaf_headers(L, h.K() + R.l0, h.S() + R.l0, h.am[h.mc].p, h.io_orig.p, masks, h.stream);
        h.stats.kernel_launches += 2;
        CU(cudaGetLastError());
        CU(cudaMemcpyAsync(d->leaf_values, dense, size_t(L) * LEAF_VOX * 4, cudaMemcpyDeviceToHost, h.stream));
        CU(cudaMemcpyAsync(d->leaf_masks, masks, size_t(L) * 64, cudaMemcpyDeviceToHost, h.stream));
        CU(cudaMemcpyAsync(d->leaf_origins, h.io_orig.p, size_t(L) * 12, cudaMemcpyDeviceToHost, h.stream));
    }
    if (NLO + NUP > 0) {
        h.io_tiles.reserve(size_t(NLO * LOWER_SLOTS + NUP * UPPER_SLOTS), h.stream);
        float* lt = h.io_tiles.p;
        float* ut = h.io_tiles.p + NLO * LOWER_SLOTS;
        launch_node_tiles(NLO, 12, h.lower_keys.p + R.lo0, h.lower_sign.p + R.lo0 * 64, h.K(), h.nleaf, g, lt,
                          h.stream);
        launch_node_tiles(NUP, 15, h.upper_keys.p + R.u0, h.upper_sign.p + R.u0 * 512, h.lower_keys.p,
                          int64_t(h.lower_keys_h.size()), g, ut, h.stream);
        h.stats.kernel_launches += (NLO > 0) + (NUP > 0);
        CU(cudaGetLastError());
        if (NLO) CU(cudaMemcpyAsync(d->lower_tiles, lt, size_t(NLO) * LOWER_SLOTS * 4, cudaMemcpyDeviceToHost, h.stream));
        if (NUP) CU(cudaMemcpyAsync(d->upper_tiles, ut, size_t(NUP) * UPPER_SLOTS * 4, cudaMemcpyDeviceToHost, h.stream));
    }
    auto origins = [](const std::vector<uint64_t>& k, int64_t a, int64_t b, int shift, int32_t* out) {
        for (int64_t i = a; i < b; ++i) {
            int32_t x, y, z;
            key_origin(k[size_t(i)] << shift, x, y, z);
            out[3 * (i - a)] = x;
            out[3 * (i - a) + 1] = y;
            out[3 * (i - a) + 2] = z;
        }
    };
    origins(h.lower_keys_h, R.lo0, R.lo1, 12, d->lower_origins);
    origins(h.upper_keys_h, R.u0, R.u1, 27, d->upper_origins);
    origins(h.root_keys_h, R.r0, R.r1, 27, d->root_tile_origins);
    for (int64_t i = R.r0; i < R.r1; ++i) d->root_tile_values[i - R.r0] = h.root_sign_h[size_t(i)] ? -g : g;
    h.sync();
}

int64_t active_count(gbls_handle& h) {
    if (h.nleaf == 0) return 0;
    h.u64s.reserve(1, h.stream);
    CU(cudaMemsetAsync(h.u64s.p, 0, sizeof(unsigned long long), h.stream));
    k_count_active<<<blocks_for(h.nleaf * 8, 256), 256, 0, h.stream>>>(h.nleaf, h.S(), h.am[h.mc].p, h.u64s.p);
    ++h.stats.kernel_launches;
    CU(cudaGetLastError());
    unsigned long long n = 0;
    CU(cudaMemcpyAsync(&n, h.u64s.p, sizeof(n), cudaMemcpyDeviceToHost, h.stream));
    h.sync();
    return int64_t(n);
}

struct DeviceGuard {
    int prev = 0;
    explicit DeviceGuard(int dev) {
        CU(cudaGetDevice(&prev));
        if (prev != dev) CU(cudaSetDevice(dev));
    }
    ~DeviceGuard() { cudaSetDevice(prev); }
};

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

// SMALL_SORT_CAP, or the smaller non-negative GBLS_SMALL_SORT_LIMIT.
static int64_t small_sort_limit_from_env() {
    const char* e = std::getenv("GBLS_SMALL_SORT_LIMIT");
    if (!e || !*e) return SMALL_SORT_CAP;
    const long long v = std::atoll(e);
    return v < 0 ? SMALL_SORT_CAP : std::min<int64_t>(int64_t(v), SMALL_SORT_CAP);
}

static bool parity_fp64_from_env() {
    const char* e = std::getenv("GBLS_PARITY_FP64");
    return e && *e && std::atoi(e) != 0;
}

// Every operation that changes a level set outside gbls_advect drops the
// cached CFL maximum.
static void touched(gbls_handle* h) {
    if (h) h->cfl_cache.valid = false;
}

int gbls_abi_version(void) { return GBLS_ABI_VERSION; }

const char* gbls_last_error(void) { return g_last_error.c_str(); }

int gbls_set_device(int device) {
    return guarded([&] {
        int n = 0;
        CU(cudaGetDeviceCount(&n));
        if (device < 0 || device >= n) fail(GBLS_ERR_INVALID_ARGUMENT, "no such CUDA device");
        g_device = device;
    });
}

static int create_handle(const gbls_grid_desc* desc, gbls_handle** out, bool volume) {
    if (!desc || !out) {
        g_last_error = "null argument";
        return GBLS_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    gbls_handle* h = nullptr;
    const int rc = guarded([&] {
        DeviceGuard g(g_device);
        h = new gbls_handle;
        h->device = g_device;
        h->volume = volume;
        h->small_sort_limit = small_sort_limit_from_env();
        h->parity_fp64 = parity_fp64_from_env();
        CU(cudaMalloc(&h->st_d, sizeof(DevStatus)));
        CU(cudaMallocHost(&h->st_h, sizeof(DevStatus)));
        CU(cudaMalloc(&h->acc_d, 2 * sizeof(unsigned long long)));
        CU(cudaMemset(h->acc_d, 0, 2 * sizeof(unsigned long long)));
        upload(*h, desc, 1);
    });
    if (rc != GBLS_OK) {
        delete h;
        return rc;
    }
    *out = h;
    return GBLS_OK;
}

int gbls_create(const gbls_grid_desc* desc, gbls_handle** out) { return create_handle(desc, out, false); }

int gbls_create_volume(const gbls_grid_desc* desc, gbls_handle** out) { return create_handle(desc, out, true); }

int gbls_upload(gbls_handle* h, const gbls_grid_desc* desc) {
    touched(h);
    if (!h || !desc) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        if (h->ninst != 1) fail(GBLS_ERR_INVALID_ARGUMENT, "batch handles take their level sets at creation");
        h->sync();
        h->discard_tape();
        try {
            upload(*h, desc, 1);
        } catch (...) {
            // a refused upload leaves an empty level set, not a partial one
            h->nleaf = 0;
            h->nactive = 0;
            h->lower_keys_h.clear();
            h->upper_keys_h.clear();
            h->upper_sign_h.clear();
            h->root_keys_h.clear();
            h->root_sign_h.clear();
            throw;
        }
    });
}

int gbls_destroy(gbls_handle* h) {
    if (!h) return GBLS_OK;
    return guarded([&] {
        DeviceGuard g(h->device);
        cudaStreamSynchronize(h->stream);
        delete h;
    });
}

int gbls_get_counts(gbls_handle* h, gbls_grid_counts* out) {
    if (!h || !out) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        out->leaf_count = h->nleaf;
        out->lower_count = int64_t(h->lower_keys_h.size());
        out->upper_count = int64_t(h->upper_keys_h.size());
        out->root_tile_count = int64_t(h->root_keys_h.size());
        out->active_voxel_count = active_count(*h);
        out->background = h->gamma;
    });
}

int gbls_download(gbls_handle* h, gbls_grid_desc* out) {
    if (!h || !out) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        download(*h, out, -1);
    });
}

int gbls_set_stream(gbls_handle* h, void* stream) {
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        CU(cudaStreamSynchronize(h->stream));
        h->stream = static_cast<cudaStream_t>(stream);
    });
}

int gbls_set_tracker_state(gbls_handle* h, int spatial, int temporal, int norm_count, int grain_size) {
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        if (spatial < GBLS_FIRST_BIAS || spatial > GBLS_HJWENO5_BIAS) fail(GBLS_ERR_VALUE, "Spatial difference scheme not supported!");
        if (temporal < GBLS_TVD_RK1 || temporal > GBLS_TVD_RK3) fail(GBLS_ERR_VALUE, "Temporal integration scheme not supported!");
        h->tr_spatial = spatial;
        h->tr_temporal = temporal;
        h->norm_count = norm_count;
        h->grain = grain_size;
    });
}

int gbls_get_tracker_state(gbls_handle* h, int* spatial, int* temporal, int* norm_count, int* grain_size) {
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    if (spatial) *spatial = h->tr_spatial;
    if (temporal) *temporal = h->tr_temporal;
    if (norm_count) *norm_count = h->norm_count;
    if (grain_size) *grain_size = h->grain;
    return GBLS_OK;
}

int gbls_set_trimming(gbls_handle* h, int trim_mode) {
    touched(h);
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    if (trim_mode < GBLS_TRIM_NONE || trim_mode > GBLS_TRIM_ALL) {
        g_last_error = "bad trim mode";
        return GBLS_ERR_VALUE;
    }
    h->trim = trim_mode;
    return GBLS_OK;
}

// ---- launch shapes ------------------------------------------------------------
static bool launch_config_ok(const gbls_launch_config* c) {
    auto ctas = [](int v) { return v == 0 || v == 1 || v == 14 || v == 16; };
    const int l = c->cfl_leaves_per_block, p = c->rk_ctas_per_leaf;
    return ctas(c->stencil_min_ctas_rk) && ctas(c->stencil_min_ctas_norm) && (l == 8 || l == 16 || l == 32 || l == 64) &&
           (p == 1 || p == 2 || p == 4);
}

int gbls_set_launch_config(gbls_handle* h, const gbls_launch_config* c) {
    if (!h || !c) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    if (!launch_config_ok(c)) { g_last_error = "launch configuration out of range"; return GBLS_ERR_VALUE; }
    h->rk_min_ctas = c->stencil_min_ctas_rk;
    h->norm_min_ctas = c->stencil_min_ctas_norm;
    h->cfl_leaves = c->cfl_leaves_per_block;
    h->rk_parts = c->rk_ctas_per_leaf;
    return GBLS_OK;
}

int gbls_get_launch_config(gbls_handle* h, gbls_launch_config* c) {
    if (!h || !c) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    c->stencil_min_ctas_rk = h->rk_min_ctas;
    c->stencil_min_ctas_norm = h->norm_min_ctas;
    c->cfl_leaves_per_block = h->cfl_leaves;
    c->rk_ctas_per_leaf = h->rk_parts;
    return GBLS_OK;
}

// One RK stage, one renormalisation stage over the active voxels and one CFL
// maximum of the current level set under configuration c, each launched
// reps times after one warm-up launch; mean milliseconds per launch in
// ms[0..2].  The results go to spare buffers: the level set is unchanged.
int gbls_time_launch_config(gbls_handle* h, const gbls_field* f, const gbls_launch_config* c, int reps,
                            float* ms) {
    touched(h);
    if (!h || !f || !c || !ms) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    if (!launch_config_ok(c)) { g_last_error = "launch configuration out of range"; return GBLS_ERR_VALUE; }
    return guarded([&] {
        DeviceGuard g(h->device);
        if (h->nleaf == 0) fail(GBLS_ERR_INVALID_ARGUMENT, "empty level set");
        if (h->f64) fail(GBLS_ERR_UNSUPPORTED, "launch shapes are tuned on FP32 level sets");
        if (f->desc.kind == GBLS_FIELD_HOST_SAMPLED) fail(GBLS_ERR_UNSUPPORTED, "timing takes a device-evaluated field");
        if (h->tape_on) fail(GBLS_ERR_UNSUPPORTED, "timing while the adjoint records");
        const int n = std::max(1, reps);
        const int rk0 = h->rk_min_ctas, nm0 = h->norm_min_ctas, cl0 = h->cfl_leaves, rp0 = h->rk_parts;
        const bool prof = h->profiling;
        h->profiling = false;
        h->rk_min_ctas = c->stencil_min_ctas_rk;
        h->norm_min_ctas = c->stencil_min_ctas_norm;
        h->cfl_leaves = c->cfl_leaves_per_block;
        h->rk_parts = c->rk_ctas_per_leaf;
        const int vo = other_of(h->vc, h->vc), mo = other_of(h->mc, h->mc);
        RkArgs r{};
        r.spatial = GBLS_HJWENO5_BIAS;
        r.nleaf = h->nleaf;
        r.keys = h->K();
        r.slot = h->S();
        r.nbr = h->nbr.p;
        r.dt = 0.25f;
        r.gamma = h->gamma;
        r.invdx = 1.0 / h->voxel_size;
        r.invdx_f = float(1.0 / h->voxel_size);
        r.field = field_params(*h, f, 0.0f);
        r.src = h->layout(h->mc, h->vc);
        r.phin = h->vals[h->vc].p;
        r.out = h->vals[vo].p;
        r.beta = 1.0f;
        NormArgs q{};
        q.spatial = GBLS_HJWENO5_BIAS;
        q.nleaf = h->nleaf;
        q.slot = h->S();
        q.nbr = h->nbr.p;
        q.pmask = h->am[h->mc].p;
        q.gamma = h->gamma;
        q.mdt = float(h->voxel_size) * 0.3f;
        q.invdx = float(1.0 / h->voxel_size);
        q.out_count = h->cnt.p;
        q.keys = h->K();
        q.src = h->layout(h->mc, h->vc);
        q.phi = q.src;
        q.beta = 1.0f;
        q.out_vals = h->vals[vo].p;
        q.out_amask = h->am[mo].p;
        q.out_smask = h->sm[mo].p;
        cudaEvent_t e0 = h->event(), e1 = h->event();
        auto timed = [&](const std::function<void()>& launch) {
            launch();
            CU(cudaEventRecord(e0, h->stream));
            for (int i = 0; i < n; ++i) launch();
            CU(cudaEventRecord(e1, h->stream));
            CU(cudaEventSynchronize(e1));
            float t = 0.0f;
            CU(cudaEventElapsedTime(&t, e0, e1));
            return t / float(n);
        };
        ms[0] = timed([&] { rk_stage(*h, r); });
        ms[1] = timed([&] { launch_norm(*h, q); });
        ms[2] = timed([&] {
            h->clear_status();
            enqueue_max_speed(*h, f, 0.0f, nullptr);
        });
        h->sync();
        h->event_pool.push_back(e0);
        h->event_pool.push_back(e1);
        h->stats.kernel_launches += uint64_t(3 * (n + 1));
        h->rk_min_ctas = rk0;
        h->norm_min_ctas = nm0;
        h->cfl_leaves = cl0;
        h->rk_parts = rp0;
        h->profiling = prof;
    });
}

int gbls_set_precision(gbls_handle* h, int mode) {
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    if (mode != GBLS_MODE_PARITY && mode != GBLS_MODE_FAST && mode != GBLS_MODE_FP64) {
        g_last_error = "bad precision mode";
        return GBLS_ERR_VALUE;
    }
    return guarded([&] {
        DeviceGuard g(h->device);
        const bool want = mode == GBLS_MODE_FP64;
        if (want && (h->ninst != 1 || h->volume))
            fail(GBLS_ERR_UNSUPPORTED, "the FP64 instance runs single level sets");
        if (want && h->tape_on) fail(GBLS_ERR_UNSUPPORTED, "the adjoint records FP32 level sets");
        if (want != h->f64) {
            h->sync();
            if (want) widen_values(*h);
            else narrow_values(*h);
            h->f64 = want;
            touched(h);
        }
        h->mode = mode;
    });
}

int gbls_set_interrupter(gbls_handle* h, const gbls_interrupter* intr) {
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    if (intr) {
        h->intr = *intr;
        h->has_intr = true;
    } else {
        h->intr = gbls_interrupter{};
        h->has_intr = false;
    }
    return GBLS_OK;
}

int gbls_track(gbls_handle* h) {
    if (h && h->volume) { g_last_error = "a volume handle takes volume operations only"; return GBLS_ERR_UNSUPPORTED; }
    touched(h);
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        check_scheme(h->tr_spatial, h->tr_temporal);
        track(*h);
        h->sync();
    });
}

int gbls_normalize(gbls_handle* h) {
    if (h && h->volume) { g_last_error = "a volume handle takes volume operations only"; return GBLS_ERR_UNSUPPORTED; }
    touched(h);
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        check_scheme(h->tr_spatial, h->tr_temporal);
        normalize_pass(*h, h->am[h->mc].p, 0);
        h->sync();
    });
}

// LevelSetTracker::normalize(mask) (tools/LevelSetTracker.h:94, 398-416,
// Normalizer :661-670): the renormalisation restricted to the active voxels
// of the mask leaves that share an origin with a leaf of the level set, the
// other active voxels unchanged.  The mask arrives as its leaves' origins and
// active masks (x<<6 | y<<3 | z bit order).
int gbls_normalize_masked(gbls_handle* h, int64_t mask_leaf_count, const int32_t* mask_leaf_origins,
                          const uint64_t* mask_leaf_masks) {
    if (h && h->volume) { g_last_error = "a volume handle takes volume operations only"; return GBLS_ERR_UNSUPPORTED; }
    touched(h);
    if (!h || mask_leaf_count < 0 || (mask_leaf_count > 0 && (!mask_leaf_origins || !mask_leaf_masks))) {
        g_last_error = "null argument or negative count";
        return GBLS_ERR_INVALID_ARGUMENT;
    }
    return guarded([&] {
        DeviceGuard g(h->device);
        check_scheme(h->tr_spatial, h->tr_temporal);
        if (h->ninst > 1) fail(GBLS_ERR_UNSUPPORTED, "masked normalisation works on single level sets");
        const int64_t nm = mask_leaf_count;
        std::vector<std::pair<uint64_t, int64_t>> mk(static_cast<size_t>(nm));
        for (int64_t i = 0; i < nm; ++i) {
            const int32_t* o = mask_leaf_origins + 3 * i;
            for (int a = 0; a < 3; ++a) {
                if (o[a] % 8 != 0) fail(GBLS_ERR_INVALID_ARGUMENT, "mask leaf origin not aligned");
                if (o[a] < -COORD_SAFE || o[a] >= COORD_SAFE) fail(GBLS_ERR_DOMAIN, "coordinate outside the supported range");
            }
            mk[size_t(i)] = {leaf_key(o[0], o[1], o[2]), i};
        }
        std::sort(mk.begin(), mk.end());
        for (size_t i = 1; i < mk.size(); ++i)
            if (mk[i].first == mk[i - 1].first) fail(GBLS_ERR_INVALID_ARGUMENT, "duplicate mask leaf");
        std::vector<uint64_t> keys(static_cast<size_t>(nm)), masks(static_cast<size_t>(nm) * 8);
        for (int64_t i = 0; i < nm; ++i) {
            keys[size_t(i)] = mk[size_t(i)].first;
            std::memcpy(&masks[size_t(i) * 8], mask_leaf_masks + mk[size_t(i)].second * 8, 64);
        }
        if (h->nleaf == 0) return;
        DevArray<uint64_t> dkeys, dmasks;
        dkeys.upload(keys.data(), keys.size(), h->stream);
        dmasks.upload(masks.data(), masks.size(), h->stream);
        h->clear_status();
        k_mask_from_leaves<<<blocks_for(h->nleaf * 8, 256), 256, 0, h->stream>>>(
            h->nleaf, h->K(), h->S(), h->am[h->mc].p, dkeys.p, dmasks.p, nm, h->emask.p, &h->st_d->n_cand);
        ++h->stats.kernel_launches;
        CU(cudaGetLastError());
        h->read_status();
        if (h->st_h->n_cand) fail(GBLS_ERR_UNSUPPORTED, "the mask covers voxels that are inactive in the level set");
        normalize_pass(*h, h->emask.p, 0, 1);
        h->nactive = -1;
        h->sync();
    });
}

int gbls_prune(gbls_handle* h) {
    if (h && h->volume) { g_last_error = "a volume handle takes volume operations only"; return GBLS_ERR_UNSUPPORTED; }
    touched(h);
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        start_intr(*h, "Pruning Level Set");
        relayout(*h, h->am[h->mc].p, 0, h->trim);  // Trim (records per-leaf counts)
        prune_compact(*h);
        end_intr(*h);
        h->sync();
    });
}

// LevelSetTracker::dilate (tools/LevelSetTracker.h:317-337): per iteration a
// NN_FACE dilation, the background grows by dx, and (normCount > 0) the
// newly activated voxels are renormalised with the others held fixed.
int gbls_dilate(gbls_handle* h, int iterations) {
    if (h && h->volume) { g_last_error = "a volume handle takes volume operations only"; return GBLS_ERR_UNSUPPORTED; }
    touched(h);
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        if (h->norm_count > 0) check_scheme(h->tr_spatial, h->tr_temporal);
        const float dx = float(h->voxel_size);
        for (int i = 0; i < iterations; ++i) {
            dilate_topology(*h);
            const int m_old = h->mc;
            relayout(*h, h->dmask.p, 0, 0);  // new voxels active with their old values
            h->gamma = dx + h->gamma;         // changeLevelSetBackground(mDx + background)
            h->nactive = -1;
            if (h->norm_count > 0 && h->nleaf > 0) {
                k_andnot<<<blocks_for(h->nleaf * 8, 256), 256, 0, h->stream>>>(h->nleaf, h->S(), h->dmask.p,
                                                                                h->am[m_old].p);
                ++h->stats.kernel_launches;
                CU(cudaGetLastError());
                normalize_pass(*h, h->dmask.p, 0, 1);
            }
        }
        h->sync();
    });
}

// LevelSetTracker::erode (tools/LevelSetTracker.h:339-349): NN_FACE erosion,
// pruneLevelSet, then the background shrinks by iterations * dx.
int gbls_erode(gbls_handle* h, int iterations) {
    if (h && h->volume) { g_last_error = "a volume handle takes volume operations only"; return GBLS_ERR_UNSUPPORTED; }
    touched(h);
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        if (iterations > 0 && h->nleaf > 0) {
            const uint64_t* in = h->am[h->mc].p;
            uint64_t* bufs[2] = {h->dmask.p, h->emask.p};
            for (int i = 0; i < iterations; ++i) {
                uint64_t* out = bufs[i & 1];
                k_erode<<<blocks_for(h->nleaf * 8, 256), 256, 0, h->stream>>>(h->nleaf, h->S(), h->nbr.p, in, out);
                ++h->stats.kernel_launches;
                CU(cudaGetLastError());
                in = out;
            }
            relayout(*h, in, 0, 0);
        } else if (h->nleaf > 0) {
            relayout(*h, h->am[h->mc].p, 1, 0);
        }
        prune_compact(*h);
        h->gamma = h->gamma - float(iterations) * float(h->voxel_size);
        h->sync();
    });
}

// LevelSetTracker::resize (tools/LevelSetTracker.h:351-364).
int gbls_resize(gbls_handle* h, uint32_t half_width, int* changed) {
    if (h && h->volume) { g_last_error = "a volume handle takes volume operations only"; return GBLS_ERR_UNSUPPORTED; }
    touched(h);
    if (changed) *changed = 0;
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    const int w_old = int(std::floor(h->gamma / float(h->voxel_size)));
    const int w_new = int(half_width);
    int rc = GBLS_OK;
    if (w_old < w_new) rc = gbls_dilate(h, w_new - w_old);
    else if (w_old > w_new) rc = gbls_erode(h, w_old - w_new);
    if (changed) *changed = (w_old != w_new) ? 1 : 0;
    return rc;
}

// ---- adjoint -----------------------------------------------------------------
int gbls_adjoint_record(gbls_handle* h, int enable) {
    if (h && h->f64 && enable) { g_last_error = "the adjoint records FP32 level sets"; return GBLS_ERR_UNSUPPORTED; }
    touched(h);
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        h->sync();
        h->discard_tape();
        if (!enable) h->tape_pool.clear();  // releases the tape's device memory
        h->tape_on = enable != 0;
    });
}

namespace {
// Active counts of the leaves of a recorded mask array (host).
std::vector<int> mask_counts(gbls_handle& h, const DevArray<uint64_t>& m, int64_t n) {
    std::vector<uint64_t> w(static_cast<size_t>(n) * 8);
    m.download(w.data(), w.size(), h.stream);
    h.sync();
    std::vector<int> c(static_cast<size_t>(n));
    for (int64_t l = 0; l < n; ++l) {
        int k = 0;
        for (int q = 0; q < 8; ++q) k += __builtin_popcountll(w[size_t(l) * 8 + q]);
        c[size_t(l)] = k;
    }
    return c;
}
}  // namespace

namespace {
// Leaf-order offsets of packed active values: cnt/pre over n leaves.
void packed_prefix(gbls_handle& h, int64_t n, const int32_t* slot, const uint64_t* m, const int32_t* keep,
                   DevArray<int64_t>& cnt, DevArray<int64_t>& pre) {
    cnt.reserve(size_t(std::max<int64_t>(n, 1)), h.stream);
    pre.reserve(size_t(std::max<int64_t>(n, 1)), h.stream);
    if (n <= 0) return;
    k_mask_count<<<blocks_for(n, 256), 256, 0, h.stream>>>(n, slot, m, keep, cnt.p);
    size_t bytes = 0;
    CU(cub::DeviceScan::ExclusiveSum(nullptr, bytes, cnt.p, pre.p, int(n), h.stream));
    h.cub_tmp.reserve(bytes, h.stream);
    bytes = h.cub_tmp.cap;
    CU(cub::DeviceScan::ExclusiveSum(h.cub_tmp.p, bytes, cnt.p, pre.p, int(n), h.stream));
    h.stats.kernel_launches += 2;
    CU(cudaGetLastError());
}
}  // namespace

int gbls_get_active_values_device(gbls_handle* h, float* out) {
    touched(h);
    if (!h || !out) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    if (h->f64) { g_last_error = "an FP64 level set: gbls_get_active_values_f64"; return GBLS_ERR_UNSUPPORTED; }
    return guarded([&] {
        DeviceGuard g(h->device);
        DevArray<int64_t> cnt, pre;
        packed_prefix(*h, h->nleaf, h->S(), h->am[h->mc].p, nullptr, cnt, pre);
        if (h->nleaf > 0)
            k_packed_move<<<unsigned(h->nleaf), 64, 0, h->stream>>>(h->nleaf, h->S(), nullptr, nullptr,
                                                                    h->am[h->mc].p, pre.p, h->vals[h->vc].p, out, 1);
        ++h->stats.kernel_launches;
        CU(cudaGetLastError());
        h->sync();
    });
}

int gbls_set_active_values_device(gbls_handle* h, const float* in) {
    touched(h);
    if (!h || !in) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    if (h->f64) { g_last_error = "the FP64 instance takes its values from gbls_upload"; return GBLS_ERR_UNSUPPORTED; }
    return guarded([&] {
        DeviceGuard g(h->device);
        if (h->tape_on && !h->tape.empty()) fail(GBLS_ERR_UNSUPPORTED, "values change under a recorded tape");
        DevArray<int64_t> cnt, pre;
        packed_prefix(*h, h->nleaf, h->S(), h->am[h->mc].p, nullptr, cnt, pre);
        if (h->nleaf > 0) {
            k_packed_move<<<unsigned(h->nleaf), 64, 0, h->stream>>>(h->nleaf, h->S(), nullptr, nullptr,
                                                                    h->am[h->mc].p, pre.p, in, h->vals[h->vc].p, 0);
            k_active_signs<<<unsigned(h->nleaf), 64, 0, h->stream>>>(h->nleaf, h->S(), h->am[h->mc].p,
                                                                     h->vals[h->vc].p, h->sm[h->mc].p);
        }
        h->stats.kernel_launches += 2;
        h->cfl_cache.valid = false;
        CU(cudaGetLastError());
        h->sync();
    });
}

int gbls_get_active_values_f64(gbls_handle* h, double* out) {
    if (!h || !out) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        if (h->ninst != 1) fail(GBLS_ERR_UNSUPPORTED, "single level sets only");
        DevArray<int64_t> cnt, pre;
        packed_prefix(*h, h->nleaf, h->S(), h->am[h->mc].p, nullptr, cnt, pre);
        if (h->nactive < 0) h->nactive = active_count(*h);
        const int64_t n = h->nactive;
        if (n == 0) return;
        if (h->f64) {
            DevArray<double> d;
            d.reserve(size_t(n), h->stream);
            launch_gather_active_f64(h->nleaf, h->S(), h->am[h->mc].p, pre.p,
                                     reinterpret_cast<const double*>(h->vals[h->vc].p), d.p, h->stream);
            ++h->stats.kernel_launches;
            CU(cudaGetLastError());
            CU(cudaMemcpyAsync(out, d.p, size_t(n) * 8, cudaMemcpyDeviceToHost, h->stream));
            h->sync();
        } else {
            DevArray<float> f;
            f.reserve(size_t(n), h->stream);
            k_packed_move<<<unsigned(h->nleaf), 64, 0, h->stream>>>(h->nleaf, h->S(), nullptr, nullptr,
                                                                    h->am[h->mc].p, pre.p, h->vals[h->vc].p, f.p, 1);
            ++h->stats.kernel_launches;
            CU(cudaGetLastError());
            std::vector<float> tmp(static_cast<size_t>(n));
            CU(cudaMemcpyAsync(tmp.data(), f.p, size_t(n) * 4, cudaMemcpyDeviceToHost, h->stream));
            h->sync();
            for (int64_t i = 0; i < n; ++i) out[i] = double(tmp[size_t(i)]);
        }
    });
}

int gbls_adjoint_sizes(gbls_handle* h, int64_t* n_initial, int64_t* n_final, int64_t* substeps) {
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        if (substeps) *substeps = int64_t(h->tape.size());
        if (n_final) *n_final = active_count(*h);
        if (n_initial) {
            if (h->tape.empty()) *n_initial = active_count(*h);
            else {
                const auto c = mask_counts(*h, h->tape[0]->am, h->tape[0]->n);
                int64_t t = 0;
                for (int x : c) t += x;
                *n_initial = t;
            }
        }
    });
}

// Reverse sweep over the tape: dL/dphi on the final active voxels (canonical
// order) -> dL/dphi on the initial active voxels and, for a DENSE field,
// dL/dvelocity on its grid.
// Reverse sweep over the tape.  dL/dv goes to host memory (zeroed first) or,
// with vel_on_device, is added into the caller's device array.
// dl_on_device: dl_final and dl_initial are device arrays (else host).
static int adjoint_backward(gbls_handle* h, const gbls_field* field, const float* dl_final, float* dl_initial,
                            float* dl_velocity, bool vel_on_device, bool dl_on_device = false) {
    if (!h || !field || !dl_final || !dl_initial) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        if (h->tape.empty()) fail(GBLS_ERR_INVALID_ARGUMENT, "no recorded substeps");
        const int S = int(h->tape.size());
        cudaStream_t st = h->stream;
        // final list = kept leaves of the last merged list, with masks fin
        TapeStep& last = *h->tape[size_t(S - 1)];
        DevArray<float> lam_next, lam4, lam3, lamA, lp2, lp1, lpn, dvel, part, halo;
        DevArray<int64_t> pcnt, ppre;
        if (dl_on_device) {
            lam_next.reserve(size_t(std::max<int64_t>(last.nm, 1)) * LEAF_VOX, st);
            packed_prefix(*h, last.nm, nullptr, last.fin.p, last.keep.p, pcnt, ppre);
            if (last.nm > 0)
                k_packed_move<<<unsigned(last.nm), 64, 0, st>>>(last.nm, nullptr, last.keep.p, last.idx.p, last.fin.p,
                                                                ppre.p, dl_final, lam_next.p, 0);
            ++h->stats.kernel_launches;
            CU(cudaGetLastError());
        } else {
            std::vector<int32_t> keep(static_cast<size_t>(last.nm));
            if (last.nm) last.keep.download(keep.data(), keep.size(), st);
            const auto finc = mask_counts(*h, last.fin, last.nm);
            std::vector<float> lam_h;
            int64_t nf = 0, off = 0;
            for (int64_t i = 0; i < last.nm; ++i) if (keep[size_t(i)]) ++nf;
            lam_h.assign(size_t(std::max<int64_t>(nf, 1)) * LEAF_VOX, 0.0f);
            int64_t j = 0;
            for (int64_t i = 0; i < last.nm; ++i) {
                if (!keep[size_t(i)]) continue;
                for (int r = 0; r < finc[size_t(i)]; ++r) lam_h[size_t(j) * LEAF_VOX + r] = dl_final[off + r];
                off += finc[size_t(i)];
                ++j;
            }
            lam_next.upload(lam_h.data(), lam_h.size(), st);
        }
        if (field_params(*h, field, 0.0f).xform)
            fail(GBLS_ERR_UNSUPPORTED, "the adjoint differentiates velocity grids aligned with the level set only");
        const bool want_vel = dl_velocity && field->desc.kind == GBLS_FIELD_DENSE;
        size_t nvel = 0;
        float* dv = nullptr;
        if (want_vel) {
            nvel = size_t(field->desc.dense_dims[0]) * field->desc.dense_dims[1] * field->desc.dense_dims[2] * 3;
            if (vel_on_device) {
                dv = dl_velocity;
            } else {
                dvel.reserve(nvel, st);
                CU(cudaMemsetAsync(dvel.p, 0, nvel * 4, st));
                dv = dvel.p;
            }
        }
        const float dx = float(h->voxel_size);
        const float mdt = dx * 0.3f, invdx = 1.0f / dx;
        // the time steps' dependence on the velocity: dL/d(dt) per substep
        // and the voxel holding each substep's maximum |v|^2
        DevArray<double> dt_part, gdt;
        DevArray<float> mbar_d;
        DevArray<unsigned long long> argkey;
        DevArray<int64_t> argcell;
        if (want_vel) {
            gdt.reserve(size_t(S), st);
            argkey.reserve(size_t(S), st);
            argcell.reserve(size_t(S), st);
            CU(cudaMemsetAsync(argkey.p, 0xff, size_t(S) * sizeof(unsigned long long), st));
        }
        for (int s = S - 1; s >= 0; --s) {
            TapeStep& tp = *h->tape[size_t(s)];
            const size_t nm = size_t(std::max<int64_t>(tp.nm, 1)) * LEAF_VOX, n = size_t(std::max<int64_t>(tp.n, 1)) * LEAF_VOX;
            lam4.reserve(nm, st);
            lam3.reserve(nm, st);
            CU(cudaMemsetAsync(lam3.p, 0, nm * 4, st));
            AdjExpandArgs ea{tp.nm, tp.pmask.p, tp.fin.p, tp.keep.p, tp.idx.p, lam_next.p, lam4.p};
            launch_adj_expand(ea, st);
            const size_t nmax = size_t(std::max<int64_t>(std::max(tp.nm, tp.n), 1));
            part.reserve(nmax * LEAF_VOX, st);
            halo.reserve(nmax * 6 * 192, st);
            AdjNormArgs na{};
            na.nleaf = tp.nm;
            na.nbr = tp.nbr_m.p;
            na.src = Layout{tp.am3.p, tp.sm3.p, tp.phi3.p};
            na.pmask = tp.pmask.p;
            na.lam4 = lam4.p;
            na.part = part.p;
            na.halo = halo.p;
            na.gamma = tp.gamma;
            na.mdt = mdt;
            na.invdx = invdx;
            launch_adj_norm(na, st);
            AdjCombineArgs ca{};
            ca.nleaf = tp.nm;
            ca.nbr = tp.nbr_m.p;
            ca.am = tp.am3.p;
            ca.part = part.p;
            ca.halo = halo.p;
            ca.lam = lam3.p;
            launch_adj_combine(ca, st);
            lamA.reserve(n, st);
            AdjMapArgs ma{tp.n, tp.keys.p, tp.am.p, tp.keys_m.p, tp.nm, lam3.p, lamA.p};
            launch_adj_map(ma, st);
            lp2.reserve(n, st);
            lp1.reserve(n, st);
            lpn.reserve(n, st);
            CU(cudaMemsetAsync(lp2.p, 0, n * 4, st));
            CU(cudaMemsetAsync(lp1.p, 0, n * 4, st));
            CU(cudaMemsetAsync(lpn.p, 0, n * 4, st));
            AdjRkArgs ra{};
            ra.nleaf = tp.n;
            ra.keys = tp.keys.p;
            ra.nbr = tp.nbr.p;
            ra.dt = tp.dt;
            ra.gamma = tp.gamma;
            ra.invdx = invdx;
            ra.t0 = tp.t0;
            ra.backward = tp.backward ? 1 : 0;
            ra.field = field_params(*h, field, tp.t0);
            ra.field.tab = nullptr;  // direct evaluation in the adjoint
            ra.dvel = dv;
            if (want_vel) {
                dt_part.reserve(size_t(std::max<int64_t>(tp.n, 1)), st);
                CU(cudaMemsetAsync(dt_part.p, 0, size_t(std::max<int64_t>(tp.n, 1)) * sizeof(double), st));
                ra.dt_part = dt_part.p;
            }
            ra.part = part.p;
            ra.halo = halo.p;
            AdjCombineArgs rc{};
            rc.nleaf = tp.n;
            rc.nbr = tp.nbr.p;
            rc.am = tp.am.p;
            rc.part = part.p;
            rc.halo = halo.p;
            auto stage = [&](const float* phi, float* lam_out, float* lam_in, float alpha) {
                ra.src = Layout{tp.am.p, tp.sm.p, phi};
                ra.lam_out = lam_out;
                ra.alpha = alpha;
                ra.beta = 1.0f - alpha;
                launch_adj_rk(ra, st);
                rc.lam = lam_in;
                rc.lam_out = lam_out;
                rc.lam_phin = lpn.p;
                rc.alpha = alpha;
                launch_adj_combine(rc, st);
            };
            stage(tp.phi2.p, lamA.p, lp2.p, 1.0f / 3.0f);  // phi3 = 1/3 phin + 2/3 (phi2 - dt v.grad phi2)
            stage(tp.phi1.p, lp2.p, lp1.p, 3.0f / 4.0f);   // phi2 = 3/4 phin + 1/4 (phi1 - dt v.grad phi1)
            stage(tp.phin.p, lp1.p, lpn.p, 0.0f);          // phi1 = phin - dt v.grad phin
            if (want_vel) {
                launch_adj_dt_reduce(dt_part.p, tp.n, gdt.p + s, st);
                AdjArgmaxArgs aa{};
                aa.nleaf = tp.n;
                aa.keys = tp.keys.p;
                aa.am = tp.am.p;
                aa.field = ra.field;
                aa.t0 = tp.t0;
                aa.maxv2 = tp.maxv2;
                aa.argkey = argkey.p + s;
                aa.argcell = argcell.p + s;
                launch_adj_argmax(aa, st);
                h->stats.kernel_launches += 3;
            }
            CU(cudaGetLastError());
            h->stats.kernel_launches += 10;
            std::swap(lam_next.p, lpn.p);
            std::swap(lam_next.cap, lpn.cap);
        }
        if (want_vel) {
            // reverse sweep of the substep clock (CflClock): tau_{k+1} =
            // tau_k + sgn dt_k; dt_k = CFL_ref dx / sqrt(m_k) when limited,
            // else sgn (E - tau_k) with E the interval's end, E = tau_o +
            // sgn lim_o (lim_o = cfl dx / sqrt(m_o)) for an interval opened
            // at substep o under an imposed CFL number, else t1 (fixed); the
            // first substep of a call starts at the caller's t0 (fixed).
            std::vector<double> G(static_cast<size_t>(S));
            gdt.download(G.data(), G.size(), st);
            h->sync();
            std::vector<float> mbar(static_cast<size_t>(S), 0.0f);
            double tb = 0.0, Eb = 0.0;
            for (int k = S - 1; k >= 0; --k) {
                const TapeStep& tk = *h->tape[size_t(k)];
                const double sg = tk.backward ? -1.0 : 1.0, m = double(tk.maxv2);
                const double dtb = G[size_t(k)] + sg * tb;
                double mb = 0.0;
                if (tk.limited) {
                    mb += dtb * (-double(tk.dt) / (2.0 * m));
                } else {
                    Eb += sg * dtb;
                    tb -= sg * dtb;
                }
                if (tk.opened) {
                    if (tk.end_lim) {
                        tb += Eb;
                        mb += sg * Eb * (-double(tk.open_lim) / (2.0 * m));
                    }
                    Eb = 0.0;
                }
                if (tk.first) tb = 0.0;
                mbar[size_t(k)] = float(mb);
            }
            mbar_d.upload(mbar.data(), mbar.size(), st);
            launch_adj_dt_scatter(S, argcell.p, mbar_d.p, field->dense.p, dv, st);
            CU(cudaGetLastError());
            h->stats.kernel_launches += 1;
        }
        // initial list: the first step's list and masks
        TapeStep& first = *h->tape[0];
        if (dl_on_device) {
            packed_prefix(*h, first.n, nullptr, first.am.p, nullptr, pcnt, ppre);
            if (first.n > 0)
                k_packed_move<<<unsigned(first.n), 64, 0, st>>>(first.n, nullptr, nullptr, nullptr, first.am.p, ppre.p,
                                                                lam_next.p, dl_initial, 1);
            ++h->stats.kernel_launches;
            CU(cudaGetLastError());
            h->sync();
            return;
        }
        const auto c0 = mask_counts(*h, first.am, first.n);
        std::vector<float> out(size_t(std::max<int64_t>(first.n, 1)) * LEAF_VOX);
        lam_next.download(out.data(), size_t(first.n) * LEAF_VOX, st);
        if (want_vel && !vel_on_device) dvel.download(dl_velocity, nvel, st);
        h->sync();
        int64_t off = 0;
        for (int64_t l = 0; l < first.n; ++l) {
            for (int r = 0; r < c0[size_t(l)]; ++r) dl_initial[off + r] = out[size_t(l) * LEAF_VOX + r];
            off += c0[size_t(l)];
        }
    });
}

int gbls_adjoint_backward(gbls_handle* h, const gbls_field* field, const float* dl_final, float* dl_initial,
                          float* dl_velocity) {
    touched(h);
    return adjoint_backward(h, field, dl_final, dl_initial, dl_velocity, false);
}

int gbls_adjoint_backward_device(gbls_handle* h, const gbls_field* field, const float* dl_final,
                                 float* dl_initial, float* dl_velocity) {
    touched(h);
    if (h) {
        for (const void* p : {static_cast<const void*>(dl_final), static_cast<const void*>(dl_initial),
                              static_cast<const void*>(dl_velocity)}) {
            if (!p) continue;
            cudaPointerAttributes at{};
            if (cudaPointerGetAttributes(&at, p) != cudaSuccess || at.type != cudaMemoryTypeDevice ||
                at.device != h->device) {
                cudaGetLastError();
                g_last_error = "gbls_adjoint_backward_device takes device memory of the handle's device";
                return GBLS_ERR_INVALID_ARGUMENT;
            }
        }
    }
    return adjoint_backward(h, field, dl_final, dl_initial, dl_velocity, true, true);
}

int gbls_adjoint_backward_accumulate(gbls_handle* h, const gbls_field* field, const float* dl_final,
                                     float* dl_initial, float* dl_velocity_device) {
    touched(h);
    if (h && dl_velocity_device) {
        cudaPointerAttributes at{};
        if (cudaPointerGetAttributes(&at, dl_velocity_device) != cudaSuccess || at.type != cudaMemoryTypeDevice ||
            at.device != h->device) {
            cudaGetLastError();
            g_last_error = "dl_velocity_device is not device memory of the handle's device";
            return GBLS_ERR_INVALID_ARGUMENT;
        }
    }
    return adjoint_backward(h, field, dl_final, dl_initial, dl_velocity_device, true);
}

int gbls_batch_create(int32_t n, const gbls_grid_desc* descs, gbls_handle** out) {
    if (!descs || !out) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    *out = nullptr;
    gbls_handle* h = nullptr;
    const int rc = guarded([&] {
        DeviceGuard g(g_device);
        h = new gbls_handle;
        h->small_sort_limit = small_sort_limit_from_env();
        h->parity_fp64 = parity_fp64_from_env();
        h->device = g_device;
        CU(cudaMalloc(&h->st_d, sizeof(DevStatus)));
        CU(cudaMallocHost(&h->st_h, sizeof(DevStatus)));
        CU(cudaMalloc(&h->acc_d, 2 * sizeof(unsigned long long)));
        CU(cudaMemset(h->acc_d, 0, 2 * sizeof(unsigned long long)));
        upload(*h, descs, int(n));
    });
    if (rc != GBLS_OK) {
        delete h;
        return rc;
    }
    *out = h;
    return GBLS_OK;
}

int gbls_batch_instances(gbls_handle* h, int32_t* n) {
    if (!h || !n) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    *n = h->ninst;
    return GBLS_OK;
}

int gbls_batch_get_counts(gbls_handle* h, int32_t instance, gbls_grid_counts* out) {
    if (!h || !out) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        if (instance < 0 || instance >= h->ninst) fail(GBLS_ERR_INVALID_ARGUMENT, "no such instance");
        DeviceGuard g(h->device);
        const std::vector<uint64_t> keys = host_keys(*h);
        const InstRange R = inst_range(*h, keys, instance);
        out->leaf_count = R.l1 - R.l0;
        out->lower_count = R.lo1 - R.lo0;
        out->upper_count = R.u1 - R.u0;
        out->root_tile_count = R.r1 - R.r0;
        out->active_voxel_count = 0;
        out->background = h->gamma;
        if (R.l1 > R.l0) {
            h->u64s.reserve(1, h->stream);
            CU(cudaMemsetAsync(h->u64s.p, 0, sizeof(unsigned long long), h->stream));
            k_count_active<<<blocks_for((R.l1 - R.l0) * 8, 256), 256, 0, h->stream>>>(R.l1 - R.l0, h->S() + R.l0,
                                                                                      h->am[h->mc].p, h->u64s.p);
            ++h->stats.kernel_launches;
            CU(cudaGetLastError());
            unsigned long long c = 0;
            CU(cudaMemcpyAsync(&c, h->u64s.p, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
            h->sync();
            out->active_voxel_count = int64_t(c);
        }
    });
}

int gbls_batch_download(gbls_handle* h, int32_t instance, gbls_grid_desc* out) {
    if (!h || !out) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        if (instance < 0 || instance >= h->ninst) fail(GBLS_ERR_INVALID_ARGUMENT, "no such instance");
        DeviceGuard g(h->device);
        download(*h, out, instance);
    });
}

// n independent LevelSetAdvection::advect loops (tools/LevelSetAdvect.h:338-418),
// one substep of every still-running instance per pass.
int gbls_batch_advect(gbls_handle* h, const gbls_field_desc* fields, int spatial, int temporal, float t0,
                      float t1, float cfl, uint64_t* substeps) {
    if (!h || !fields) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    const int n = h->ninst;
    std::vector<uint64_t> count(static_cast<size_t>(n), 0);
    bool interrupted = false;
    const int rc = guarded([&] {
        DeviceGuard g(h->device);
        check_scheme(spatial, temporal);
        check_scheme(h->tr_spatial, h->tr_temporal);
        std::vector<FieldParams> fp(static_cast<size_t>(n));
        bool all_constant = true;
        for (int i = 0; i < n; ++i) {
            const gbls_field_desc& d = fields[i];
            if (d.kind != GBLS_FIELD_CONSTANT && d.kind != GBLS_FIELD_ROTATION && d.kind != GBLS_FIELD_DEFORMATION)
                fail(GBLS_ERR_UNSUPPORTED, "batch fields must be CONSTANT, ROTATION or DEFORMATION");
            if (d.kind == GBLS_FIELD_DEFORMATION && !(d.domain > 0.0f && d.period != 0.0f))
                fail(GBLS_ERR_VALUE, "deformation field needs domain > 0 and period != 0");
            gbls_field tmp;
            tmp.desc = d;
            fp[size_t(i)] = field_params(*h, &tmp, t0);  // no tables: direct evaluation
            all_constant &= d.kind == GBLS_FIELD_CONSTANT;
        }
        h->inst_field.upload(fp.data(), fp.size(), h->stream);
        if (t0 - t1 == 0.0f) { h->sync(); return; }
        const bool forward = t0 < t1;
        std::vector<CflClock> clock(static_cast<size_t>(n), CflClock(t0, t1, cfl, temporal, float(h->voxel_size)));
        std::vector<float> t(static_cast<size_t>(n), t0), dt(static_cast<size_t>(n), 0.0f);
        std::vector<uint8_t> done(static_cast<size_t>(n), 0), run(static_cast<size_t>(n), 0);
        std::vector<unsigned long long> act(static_cast<size_t>(n), 0);
        std::vector<unsigned int> mx(static_cast<size_t>(n), 0);
        // active voxels per instance
        CU(cudaMemsetAsync(h->inst_active.p, 0, size_t(n) * sizeof(unsigned long long), h->stream));
        if (h->nleaf > 0) {
            k_count_active_inst<<<blocks_for(h->nleaf, 256), 256, 0, h->stream>>>(h->nleaf, h->K(), h->S(),
                                                                                   h->am[h->mc].p, h->inst_active.p);
            ++h->stats.kernel_launches;
            CU(cudaGetLastError());
        }
        h->inst_active.download(act.data(), size_t(n), h->stream);
        h->sync();
        h->batch_run = true;
        for (;;) {
            int nrun = 0;
            for (int i = 0; i < n; ++i) {
                run[size_t(i)] = !done[size_t(i)] && (forward ? t[size_t(i)] < t1 : t[size_t(i)] > t1);
                nrun += run[size_t(i)];
            }
            if (!nrun) break;
            if (!check_intr(*h)) { interrupted = true; break; }
            // sampleField per instance (:426-464)
            for (int i = 0; i < n; ++i) {
                if (!run[size_t(i)]) continue;
                if (act[size_t(i)] == 0) { run[size_t(i)] = 0; done[size_t(i)] = 1; }
            }
            h->inst_run.upload(run.data(), size_t(n), h->stream);
            h->inst_t0.upload(t.data(), size_t(n), h->stream);
            if (!all_constant) {
                CU(cudaMemsetAsync(h->inst_max.p, 0, size_t(n) * sizeof(unsigned int), h->stream));
                CflArgs a{};
                a.nleaf = h->nleaf;
                a.keys = h->K();
                a.slot = h->S();
                a.amask = h->am[h->mc].p;
                a.max_bits = h->inst_max.p;
                a.inst_run = h->inst_run.p;
                a.inst_t0 = h->inst_t0.p;
                a.inst_field = h->inst_field.p;
                launch_cfl(a, h->stream, h->cfl_leaves);
                ++h->stats.kernel_launches;
                CU(cudaGetLastError());
                h->inst_max.download(mx.data(), size_t(n), h->stream);
                h->sync();
            }
            uint64_t upd = 0;
            nrun = 0;
            for (int i = 0; i < n; ++i) {
                if (!run[size_t(i)]) continue;
                float maxv2;
                if (fields[i].kind == GBLS_FIELD_CONSTANT) {
                    const float* c = fields[i].constant;
                    maxv2 = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
                } else {
                    std::memcpy(&maxv2, &mx[size_t(i)], 4);
                }
                float d = 0.0f;
                if (maxv2 > 1e-5f || maxv2 < -1e-5f) d = clock[size_t(i)].next(t[size_t(i)], maxv2);
                if (d == 0.0f) {
                    run[size_t(i)] = 0;
                    done[size_t(i)] = 1;
                    continue;
                }
                dt[size_t(i)] = d;
                upd += act[size_t(i)];
                ++nrun;
            }
            if (!nrun) break;
            h->inst_run.upload(run.data(), size_t(n), h->stream);
            h->inst_dt.upload(dt.data(), size_t(n), h->stream);
            h->stats.voxel_updates += upd;
            h->stats.substeps += uint64_t(nrun);
            h->nactive = int64_t(upd);  // the RK stages' algorithmic bytes count the running instances
            // the dilation of this pass on the side stream beside the RK stages
            // (they read the masks it reads, and write none)
            h->prepare_dilation();
            CU(cudaEventRecord(h->ev_fork, h->stream));
            advect_stages(*h, nullptr, spatial, temporal, t0, 0.0f, !forward);
            CU(cudaEventRecord(h->ev_rk, h->stream));
            h->nactive = -1;
            for (int i = 0; i < n; ++i) {
                if (!run[size_t(i)]) continue;
                clock[size_t(i)].advance(t[size_t(i)], dt[size_t(i)]);
                ++count[size_t(i)];
            }
            h->overlap_dilation = true;
            struct Overlap {
                gbls_handle* h;
                ~Overlap() { h->overlap_dilation = false; }
            } overlap{h};
            track(*h);
            h->inst_active.download(act.data(), size_t(n), h->stream);
            h->sync();
        }
        h->batch_run = false;
        h->nactive = -1;
        h->sync();
    });
    h->batch_run = false;
    if (substeps)
        for (int i = 0; i < n; ++i) substeps[i] = count[size_t(i)];
    if (rc == GBLS_OK && interrupted) {
        g_last_error = "interrupted";
        return GBLS_ERR_INTERRUPTED;
    }
    return rc;
}

int gbls_get_stats(gbls_handle* h, gbls_stats* out) {
    if (!h || !out) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        h->sync();
        unsigned long long acc[2] = {0, 0};
        CU(cudaMemcpy(acc, h->acc_d, sizeof(acc), cudaMemcpyDeviceToHost));
        *out = h->stats;
        out->dilated_voxels = acc[0];
        out->norm_bytes = 4.0 * double(acc[0] + acc[1]);
        if (h->nactive < 0) h->nactive = active_count(*h);
        out->active_voxels = h->nactive;
        out->leaves = h->nleaf;
    });
}

int gbls_reset_stats(gbls_handle* h) {
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        h->sync();
        h->stats = gbls_stats{};
        CU(cudaMemsetAsync(h->acc_d, 0, 2 * sizeof(unsigned long long), h->stream));
        h->sync();
    });
}

int gbls_set_profiling(gbls_handle* h, int enable) {
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        h->sync();
        h->profiling = enable != 0;
    });
}

}  // extern "C"

namespace gbls {
int noalloc_count_active(int64_t nleaf, const int32_t* slot, const uint64_t* am, cudaStream_t stream,
                         int64_t* out, int* launches, std::string* err);
}

extern "C" {

// Active-voxel count that allocates nothing (see noalloc.cu for the scratch
// array, its size limit and its set-up).  Same result as the
// active_voxel_count of gbls_get_counts.
int gbls_count_active_noalloc(gbls_handle* h, int64_t* out) {
    if (!h || !out) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        std::string err;
        int launches = 0;
        const int rc = gbls::noalloc_count_active(h->nleaf, h->S(), h->am[h->mc].p, h->stream, out, &launches, &err);
        h->stats.kernel_launches += uint64_t(launches);
        if (rc == 1) fail(GBLS_ERR_INVALID_ARGUMENT, err);
        if (rc != 0) fail(GBLS_ERR_CUDA, err);
    });
}

int gbls_field_set_dense_device(gbls_field* f, const float* values, void* stream) {
    if (!f || !values) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        if (f->desc.kind != GBLS_FIELD_DENSE) fail(GBLS_ERR_INVALID_ARGUMENT, "not a DENSE field");
        DeviceGuard g(f->device);
        const size_t n = size_t(f->desc.dense_dims[0]) * f->desc.dense_dims[1] * f->desc.dense_dims[2] * 3;
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        CU(cudaMemcpyAsync(f->dense.p, values, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
        CU(cudaStreamSynchronize(s));
    });
}

int gbls_field_create(const gbls_field_desc* desc, gbls_field** out) {
    if (!desc || !out) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    *out = nullptr;
    gbls_field* f = nullptr;
    const int rc = guarded([&] {
        if (desc->kind < GBLS_FIELD_CONSTANT || desc->kind > GBLS_FIELD_HOST_SAMPLED)
            fail(GBLS_ERR_VALUE, "unknown field kind");
        if (desc->kind == GBLS_FIELD_HOST_SAMPLED && !desc->host_sample)
            fail(GBLS_ERR_INVALID_ARGUMENT, "HOST_SAMPLED field without a sampler");
        DeviceGuard g(g_device);
        f = new gbls_field;
        f->desc = *desc;
        f->device = g_device;
        if (desc->kind == GBLS_FIELD_DENSE) {
            const int64_t n = int64_t(desc->dense_dims[0]) * desc->dense_dims[1] * desc->dense_dims[2];
            if (n <= 0 || !desc->dense_values) fail(GBLS_ERR_INVALID_ARGUMENT, "empty dense field");
            if (desc->dense_map_type < 0 || desc->dense_map_type > GBLS_MAP_TRANSLATION + 1 ||
                (desc->dense_map_type != 0 && !(desc->dense_voxel_size > 0.0)))
                fail(GBLS_ERR_VALUE, "dense field transform must be a uniform scale and/or translation");
            f->dense.upload(desc->dense_values, size_t(n) * 3, nullptr);
            CU(cudaStreamSynchronize(nullptr));
        }
        f->desc.dense_values = nullptr;
        if (desc->kind == GBLS_FIELD_DEFORMATION) {
            if (!(desc->domain > 0.0f && desc->period != 0.0f))
                fail(GBLS_ERR_VALUE, "deformation field needs domain > 0 and period != 0");
            // per-coordinate sine tables over [-8192, domain + 8192): entries are
            // computed with the same functions as the direct evaluation
            const int lo = -8192;
            const int n = int(std::min(1.0e6f, std::ceil(desc->domain))) + 2 * 8192;
            std::vector<float> tab(size_t(n) * 2);
            for (int q = 0; q < n; ++q) {
                const float x = float(lo + q) / desc->domain;
                tab[size_t(q) * 2] = gbls_sinpi(x);
                tab[size_t(q) * 2 + 1] = gbls_sinpi(x * 2.0f);
            }
            f->tab.upload(tab.data(), tab.size(), nullptr);
            CU(cudaStreamSynchronize(nullptr));
            f->tab_lo = lo;
            f->tab_n = n;
        }
    });
    if (rc != GBLS_OK) {
        delete f;
        return rc;
    }
    *out = f;
    return GBLS_OK;
}

int gbls_field_destroy(gbls_field* f) {
    if (!f) return GBLS_OK;
    return guarded([&] {
        DeviceGuard g(f->device);
        delete f;
    });
}

int gbls_advect(gbls_handle* h, const gbls_field* field, int spatial, int temporal, float t0, float t1,
                float cfl, uint64_t* substeps) {
    if (h && h->volume) { g_last_error = "a volume handle takes volume operations only"; return GBLS_ERR_UNSUPPORTED; }
    if (substeps) *substeps = 0;
    if (!h || !field) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    uint64_t count = 0;
    bool interrupted = false;
    const int rc = guarded([&] {
        DeviceGuard g(h->device);
        check_scheme(spatial, temporal);
        check_scheme(h->tr_spatial, h->tr_temporal);
        if (t0 - t1 == 0.0f) return;  // math::isZero(time0 - time1)
        if (h->f64) {
            advect_f64(*h, field, spatial, temporal, t0, t1, cfl, count, interrupted);
            return;
        }
        const bool forward = t0 < t1;
        CflClock clock(t0, t1, cfl, temporal, float(h->voxel_size));
        // the CFL reduction of substep k+1 rides on the read-back that ends
        // the tracker pass of substep k; the first substep reuses the maximum
        // the previous call reduced for its end time when nothing else has
        // changed the level set since (analytic fields: the descriptor
        // determines the field)
        bool have_next = false;
        float next_v2 = 0.0f;
        const bool analytic = field->desc.kind == GBLS_FIELD_DEFORMATION || field->desc.kind == GBLS_FIELD_ROTATION;
        const bool cacheable = analytic && !h->batch_run && !h->tape_on;
        if (cacheable && h->cfl_cache.valid && h->cfl_cache.t == t0 &&
            std::memcmp(&h->cfl_cache.desc, &field->desc, sizeof(gbls_field_desc)) == 0) {
            have_next = true;
            next_v2 = h->cfl_cache.v2;
        }
        h->cfl_cache.valid = false;
        struct Reset {
            gbls_handle* h;
            ~Reset() {
                h->before_prune_sync = nullptr;
                h->after_normalize = nullptr;
                h->overlap_dilation = false;
            }
        } reset{h};
        while (forward ? t0 < t1 : t0 > t1) {
            if (!check_intr(*h)) { interrupted = true; break; }
            if (h->nleaf == 0) break;  // sampleField returns 0 for an empty grid
            start_intr(*h, "Sampling advection field");
            const float maxv2 = have_next ? next_v2 : max_speed_sqr(*h, field, t0);
            have_next = false;
            end_intr(*h);
            if (!(maxv2 > 1e-5f) && !(maxv2 < -1e-5f)) break;  // isApproxZero(maxAbsV, Delta)
            const float dt = clock.next(t0, maxv2);
            if (dt == 0.0f) break;
            if (h->nactive < 0) h->nactive = active_count(*h);
            h->stats.voxel_updates += uint64_t(h->nactive);
            ++h->stats.substeps;
            if (h->tape_on) {
                if (field->desc.kind == GBLS_FIELD_HOST_SAMPLED)
                    fail(GBLS_ERR_UNSUPPORTED, "the adjoint records fields the device evaluates, not HOST_SAMPLED");
                if (temporal != GBLS_TVD_RK3 || h->tr_temporal != GBLS_TVD_RK1 || h->norm_count != 1 ||
                    h->trim != GBLS_TRIM_ALL || spatial != GBLS_HJWENO5_BIAS || h->tr_spatial != GBLS_HJWENO5_BIAS)
                    fail(GBLS_ERR_UNSUPPORTED, "the adjoint records HJWENO5 TVD_RK3 advection with an HJWENO5 "
                                               "TVD_RK1 tracker, normCount 1 and full trimming");
                tape_begin_substep(*h, t0, dt, !forward);
                TapeStep& ts = *h->tape.back();
                ts.maxv2 = maxv2;
                ts.limited = clock.limited;
                ts.opened = clock.opened;
                ts.end_lim = clock.end_lim;
                ts.open_lim = clock.open_lim;
                ts.first = count == 0;
            }
            const bool overlap = true;  // dilation (and the next CFL maximum) on the side stream
            if (overlap) {
                h->prepare_dilation();
                CU(cudaEventRecord(h->ev_fork, h->stream));
            }
            advect_stages(*h, field, spatial, temporal, t0, dt, !forward);
            if (overlap) {
                CU(cudaEventRecord(h->ev_rk, h->stream));
                h->overlap_dilation = true;
            }
            clock.advance(t0, dt);
            ++count;
            const bool more = forward ? t0 < t1 : t0 > t1;
            bool queued = false;
            if ((more || cacheable) && field->desc.kind != GBLS_FIELD_CONSTANT &&
                field->desc.kind != GBLS_FIELD_HOST_SAMPLED) {
                const float tn = t0;
                if (overlap && !h->batch_run) {
                    // reduce on the side stream while the main stream prunes;
                    // the prune's read-back waits for it
                    h->after_normalize = [h, field, tn] { enqueue_max_speed_side(*h, field, tn); };
                    h->before_prune_sync = [h, &queued] {
                        CU(cudaStreamWaitEvent(h->stream, h->ev_cfl, 0));
                        CU(cudaMemcpyAsync(h->cfl_h, h->cfl_d, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                                           h->stream));
                        queued = true;
                    };
                } else {
                    h->before_prune_sync = [h, field, tn, &queued] {
                        enqueue_max_speed(*h, field, tn, &h->st_d->n_cand);
                        queued = true;
                    };
                }
            }
            track(*h);
            h->overlap_dilation = false;
            h->before_prune_sync = nullptr;
            h->after_normalize = nullptr;
            if (queued) {
                if (overlap && !h->batch_run) std::memcpy(&next_v2, h->cfl_h, sizeof(float));
                else next_v2 = status_max_speed(*h);
                have_next = true;
                if (!more) {  // the end time's maximum, for the next call
                    h->cfl_cache.valid = true;
                    h->cfl_cache.t = t0;
                    h->cfl_cache.v2 = next_v2;
                    h->cfl_cache.desc = field->desc;
                }
            }
        }
        h->sync();
    });
    if (substeps) *substeps = count;
    if (rc == GBLS_OK && interrupted) {
        g_last_error = "interrupted";
        return GBLS_ERR_INTERRUPTED;
    }
    return rc;
}

// LevelSetFilter (tools/LevelSetFilter.h:93-157): one filter, then the
// tracker pass with h's tracker state (the filter is a LevelSetTracker).
int gbls_filter(gbls_handle* h, int filter, int width, float value) {
    if (h && h->volume) { g_last_error = "a volume handle takes volume operations only"; return GBLS_ERR_UNSUPPORTED; }
    touched(h);
    if (!h) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    bool interrupted = false;
    const int rc = guarded([&] {
        DeviceGuard g(h->device);
        check_scheme(h->tr_spatial, h->tr_temporal);
        if (h->ninst > 1) fail(GBLS_ERR_UNSUPPORTED, "filters work on single level sets, not batches");
        if (h->tape_on) fail(GBLS_ERR_UNSUPPORTED, "the adjoint records advection only");
        const float dx = float(h->voxel_size);  // LevelSetTracker::voxelSize()
        switch (filter) {
        case GBLS_FILTER_LAPLACIAN: {  // Filter::laplacian :305-315, laplacianImpl :452-477
            FilterArgs a{};
            a.op = FILTER_LAPLACIAN;
            a.dt = (dx * dx) / 6.0f;
            const float inv2dx = float(0.5 / double(dx));  // GradStencil(grid, dx)
            a.invdx2 = float(4.0 * double(inv2dx) * double(inv2dx));
            filter_pass(*h, a, "Laplacian flow of level set");
            track(*h);
            break;
        }
        case GBLS_FILTER_MEAN:  // Filter::mean :257-263
            filter_box(*h, width);
            break;
        case GBLS_FILTER_GAUSSIAN:  // Filter::gaussian :265-271: four box filters
            for (int n = 0; n < 4; ++n) filter_box(*h, width);
            break;
        case GBLS_FILTER_OFFSET: {  // Filter::offset :317-334
            const float cfl = 0.5f * dx, offset = std::fabs(value);
            float dist = 0.0f;
            while (offset - dist > 0.001f * cfl) {
                if (!check_intr(*h)) { interrupted = true; break; }
                const float rest = offset - dist;
                const float delta = (cfl < rest) ? cfl : rest;  // math::Min
                dist += delta;
                FilterArgs a{};
                a.op = FILTER_OFFSET;
                a.offset = std::copysign(delta, value);
                filter_pass(*h, a, "Offsetting level set");
                track(*h);
            }
            break;
        }
        case GBLS_FILTER_MEAN_CURVATURE:  // Filter::meanCurvature :283-293
        case GBLS_FILTER_FILLET: {        // Filter::fillet :295-303
            FilterArgs a{};
            a.op = filter == GBLS_FILTER_FILLET ? FILTER_FILLET : FILTER_MEAN_CURVATURE;
            a.dt = (dx * dx) / 3.0f;
            a.inv2dx = float(0.5 / double(dx));  // CurvatureStencil(grid, dx)
            a.invdx2 = float(4.0 * double(a.inv2dx) * double(a.inv2dx));
            filter_pass(*h, a, filter == GBLS_FILTER_FILLET ? "Filleting level set" : "Mean-curvature flow of level set");
            track(*h);
            break;
        }
        case GBLS_FILTER_MEDIAN: {  // Filter::median :244-253
            FilterArgs a{};
            a.op = FILTER_MEDIAN;
            a.width = std::max(1, width);
            if (a.width > 3) fail(GBLS_ERR_UNSUPPORTED, "median widths above 3 voxels exceed the device stencil halo");
            filter_pass(*h, a, "Median-value flow of level set");
            track(*h);
            break;
        }
        default:
            fail(GBLS_ERR_VALUE, "unknown filter");
        }
        h->nactive = -1;
        h->sync();
    });
    if (rc == GBLS_OK && interrupted) {
        g_last_error = "interrupted";
        return GBLS_ERR_INTERRUPTED;
    }
    return rc;
}

// LevelSetFilter's filters with an alpha mask (tools/LevelSetFilter.h: the
// `mask` argument of every filter, setMaskRange :77-83, invertMask :89): the
// filter call of gbls_filter with the mask level set looked up at each
// voxel's index.
int gbls_filter_masked(gbls_handle* h, int filter, int width, float value, gbls_handle* alpha_mask,
                       float mask_min, float mask_max, int invert_mask) {
    if (h && h->volume) { g_last_error = "a volume handle takes volume operations only"; return GBLS_ERR_UNSUPPORTED; }
    if (!h || !alpha_mask) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    const int rc = guarded([&] {
        DeviceGuard g(h->device);
        if (!(mask_min < mask_max)) fail(GBLS_ERR_VALUE, "Invalid mask range (expects min < max)");
        if (alpha_mask == h) fail(GBLS_ERR_UNSUPPORTED, "the alpha mask must be another level set");
        if (alpha_mask->ninst > 1) fail(GBLS_ERR_UNSUPPORTED, "the alpha mask must be a single level set");
        if (alpha_mask->device != h->device || alpha_mask->voxel_size != h->voxel_size ||
            alpha_mask->map_type != h->map_type || alpha_mask->translation[0] != h->translation[0] ||
            alpha_mask->translation[1] != h->translation[1] || alpha_mask->translation[2] != h->translation[2])
            fail(GBLS_ERR_UNSUPPORTED, "the alpha mask must share the level set's device and transform "
                                       "(the trilinear sampling of non-aligned grids has no device form)");
        alpha_mask->sync();  // its tables are read on h's stream
    });
    if (rc != GBLS_OK) return rc;
    h->filter_mask.on = true;
    h->filter_mask.grid = alpha_mask;
    h->filter_mask.min = mask_min;
    h->filter_mask.inv_norm = 1.0f / (mask_max - mask_min);  // AlphaMask: mInvNorm(1/(max-min))
    h->filter_mask.invert = invert_mask ? 1 : 0;
    const int r = gbls_filter(h, filter, width, value);
    h->filter_mask.on = false;
    h->filter_mask.grid = nullptr;
    return r;
}

// LevelSetMorphing::advect (tools/LevelSetMorph.h:243-262, Morph::advect
// :479-510): CFL substeps from t0 towards t1 (forward time only), each with
// the speed sampled once, the RK stages and a tracker pass.
// ---- VolumeAdvection (tools/VolumeAdvect.h) ------------------------------------
namespace {
VolMap volume_map(const gbls_handle& h) {
    VolMap m{};
    m.scale = h.voxel_size;
    m.inv = 1.0 / h.voxel_size;
    for (int a = 0; a < 3; ++a) m.t[a] = h.translation[a];
    return m;
}

VolGrid live_grid(gbls_handle& h) {
    VolGrid g{};
    g.keys = h.K();
    g.slot = h.S();
    g.nleaf = h.nleaf;
    g.amask = h.am[h.mc].p;
    g.smask = h.sm[h.mc].p;
    g.vals = h.vals[h.vc].p;
    g.nodes = h.nodes();
    g.background = h.gamma;
    return g;
}

VolOut live_out(gbls_handle& h) {
    VolOut o{};
    o.nleaf = h.nleaf;
    o.keys = h.K();
    o.slot = h.S();
    o.amask = h.am[h.mc].p;
    return o;
}

// The grid as it is now, in arrays of its own (leaf-index numbering), so
// that it can be sampled while the handle's topology changes.
struct VolSnapshot {
    DevArray<uint64_t> keys, am, sm, lower_keys, lower_sign, upper_keys, upper_sign, root_keys;
    DevArray<uint8_t> root_sign;
    DevArray<float> vals;
    VolGrid grid{};

    void take(gbls_handle& h) {
        const int64_t n = h.nleaf;
        const size_t nn = size_t(std::max<int64_t>(n, 1));
        keys.reserve(nn, h.stream);
        am.reserve(nn * 8, h.stream);
        sm.reserve(nn * 8, h.stream);
        vals.reserve(nn * LEAF_VOX, h.stream);
        if (n > 0) CU(cudaMemcpyAsync(keys.p, h.K(), size_t(n) * 8, cudaMemcpyDeviceToDevice, h.stream));
        launch_tape_gather(n, h.S(), h.am[h.mc].p, h.sm[h.mc].p, h.vals[h.vc].p, am.p, sm.p, vals.p, h.stream);
        NodeTables t = h.nodes();
        auto copy = [&](auto& dst, const auto* src, int64_t count) {
            dst.reserve(size_t(std::max<int64_t>(count, 1)), h.stream);
            if (count > 0) CU(cudaMemcpyAsync(dst.p, src, size_t(count) * sizeof(*src), cudaMemcpyDeviceToDevice, h.stream));
        };
        copy(lower_keys, t.lower_keys, t.nlower);
        copy(lower_sign, t.lower_sign, t.nlower * 64);
        copy(upper_keys, t.upper_keys, t.nupper);
        copy(upper_sign, t.upper_sign, t.nupper * 512);
        copy(root_keys, t.root_keys, t.nroot);
        copy(root_sign, t.root_sign, t.nroot);
        CU(cudaGetLastError());
        grid = VolGrid{};
        grid.keys = keys.p;
        grid.slot = nullptr;
        grid.nleaf = n;
        grid.amask = am.p;
        grid.smask = sm.p;
        grid.vals = vals.p;
        grid.nodes = NodeTables{lower_keys.p, lower_sign.p, upper_keys.p, upper_sign.p, root_keys.p, root_sign.p,
                                t.nlower, t.nupper, t.nroot};
        grid.background = h.gamma;
    }
};
}  // namespace

// VolumeAdvection<Vec3fGrid, false>::advect<FloatGrid, Sampler<1, false>>
// (tools/VolumeAdvect.h:205-222, cook and Advect :270-560) on the handle's
// grid, in place.  integrator: Scheme::SemiLagrangian (SEMI, MID, RK3, RK4,
// MAC, BFECC); limiter: Scheme::Limiter (NO_LIMITER, CLAMP, REVERT).
int gbls_volume_advect(gbls_handle* h, const gbls_field* field, int integrator, int limiter, int substeps,
                       double time_step, double* max_velocity) {
    touched(h);
    if (!h || !field) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        if (integrator < 0 || integrator > 5) fail(GBLS_ERR_VALUE, "Spatial difference scheme not supported!");
        if (limiter < 0 || limiter > 2) fail(GBLS_ERR_VALUE, "unknown limiter");
        if (h->ninst != 1) fail(GBLS_ERR_UNSUPPORTED, "volume advection works on single grids, not batches");
        if (!h->volume) fail(GBLS_ERR_UNSUPPORTED, "volume advection takes a handle made by gbls_create_volume");
        if (h->tape_on) fail(GBLS_ERR_UNSUPPORTED, "the adjoint records level-set advection only");
        const gbls_field_desc& fd = field->desc;
        if (fd.kind != GBLS_FIELD_DENSE && fd.kind != GBLS_FIELD_CONSTANT)
            fail(GBLS_ERR_UNSUPPORTED, "volume advection samples a velocity grid: DENSE or CONSTANT fields");
        const int steps = std::max(1, substeps);  // setSubSteps clamps to 1
        const VolMap map = volume_map(*h);
        VolVelocity vel{};
        vel.kind = fd.kind == GBLS_FIELD_DENSE ? 1 : 0;
        for (int c = 0; c < 3; ++c) {
            vel.constant[c] = fd.constant[c];
            vel.background[c] = fd.kind == GBLS_FIELD_DENSE ? fd.dense_background[c] : fd.constant[c];
            vel.origin[c] = fd.dense_origin[c];
            vel.dims[c] = fd.dense_dims[c];
        }
        vel.dense = field->dense.p;
        if (fd.kind == GBLS_FIELD_DENSE && fd.dense_map_type != 0) {
            const int mt = fd.dense_map_type - 1;
            vel.map.scale = mt == GBLS_MAP_TRANSLATION ? 1.0 : fd.dense_voxel_size;
            vel.map.inv = 1.0 / vel.map.scale;
            for (int a = 0; a < 3; ++a) vel.map.t[a] = mt == GBLS_MAP_UNIFORM_SCALE ? 0.0 : fd.dense_translation[a];
        } else {
            vel.map = map;  // the velocity grid shares the volume's transform
        }
        // getMaxVelocity: max |v| over the velocity grid's values and its background
        auto len = [](const float* v) {
            const float s = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
            return double(float(std::sqrt(double(s))));
        };
        double vmax = len(vel.background);
        if (vel.kind == 1) {
            h->clear_status();
            launch_vol_max_speed(vel.dense, int64_t(vel.dims[0]) * vel.dims[1] * vel.dims[2],
                                 &h->st_d->max_v2_bits, h->stream);
            ++h->stats.kernel_launches;
            CU(cudaGetLastError());
            h->read_status();
            float m;
            std::memcpy(&m, &h->st_h->max_v2_bits, 4);
            vmax = std::max(vmax, double(m));
        }
        if (max_velocity) *max_velocity = vmax;
        const double dt = time_step / steps;
        const int n = int(std::ceil(vmax * std::fabs(dt) / h->voxel_size));  // getMaxDistance
        const float rdt = float(-dt);  // the method of characteristics backtracks
        const bool second = integrator == 4 || integrator == 5;
        const int order = second ? 1 : integrator == 0 ? 1 : integrator == 1 ? 2 : integrator == 2 ? 3 : 4;
        VolSnapshot snap;
        DevArray<float> out1;
        for (int step = 0; step < steps; ++step) {
            if (h->nleaf == 0) break;
            snap.take(*h);
            for (int i = 0; i < n; ++i) {  // dilateActiveValues(tree, n, NN_FACE, EXPAND_TILES)
                dilate_topology(*h);
                relayout(*h, h->dmask.p, 0, 0);  // new voxels active with their old values
            }
            h->nactive = -1;
            if (h->nleaf > 0) {
                VolRkArgs r{};
                r.out = live_out(*h);
                r.map = map;
                r.vel = vel;
                r.order = order;
                // forward: out0 = sample of the input along the characteristic
                r.dst = h->vals[h->vc].p;
                r.src = snap.grid;
                r.dt = rdt;
                launch_vol_rk(r, h->stream);
                ++h->stats.kernel_launches;
                if (second) {
                    out1.reserve(h->vals[h->vc].cap, h->stream);
                    VolCombineArgs c{};
                    c.out = r.out;
                    c.in = snap.grid;
                    // backward from the output: out1
                    r.src = live_grid(*h);
                    r.dst = out1.p;
                    r.dt = -rdt;
                    launch_vol_rk(r, h->stream);
                    c.out0 = h->vals[h->vc].p;
                    c.out1 = out1.p;
                    c.op = integrator == 4 ? VOL_COMBINE_MAC : VOL_COMBINE_BFECC;
                    launch_vol_combine(c, h->stream);
                    h->stats.kernel_launches += 2;
                    if (integrator == 5) {  // forward again from the corrected field, then out0 = out1
                        r.src = live_grid(*h);
                        r.dst = out1.p;
                        r.dt = rdt;
                        launch_vol_rk(r, h->stream);
                        ++h->stats.kernel_launches;
                        const size_t bytes = h->vals[h->vc].cap * sizeof(float);
                        CU(cudaMemcpyAsync(h->vals[h->vc].p, out1.p, bytes, cudaMemcpyDeviceToDevice, h->stream));
                    }
                }
                VolLimitArgs lm{};
                lm.out = live_out(*h);
                lm.vals = h->vals[h->vc].p;
                lm.keep = h->dmask.p;
                lm.in = snap.grid;
                lm.map = map;
                lm.vel = vel;
                lm.dt = rdt;
                lm.limiter = limiter;
                lm.do_limit = second && limiter != 0 ? 1 : 0;  // isLimiterOn
                lm.background = h->gamma;
                launch_vol_limit(lm, h->stream);
                ++h->stats.kernel_launches;
                CU(cudaGetLastError());
                relayout(*h, h->dmask.p, 0, 0);  // the kept voxels stay active
                prune_compact(*h);               // pruneInactive
            }
        }
        h->nactive = -1;
        h->cfl_cache.valid = false;
        h->sync();
    });
}

int gbls_morph(gbls_handle* h, gbls_handle* target, gbls_handle* alpha_mask, int spatial, int temporal, float t0,
               float t1, float mask_min, float mask_max, int invert_mask, uint64_t* substeps) {
    if (h && h->volume) { g_last_error = "a volume handle takes volume operations only"; return GBLS_ERR_UNSUPPORTED; }
    if ((h && h->f64) || (target && target->f64) || (alpha_mask && alpha_mask->f64)) {
        g_last_error = "the FP64 instance runs advection and tracking only";
        return GBLS_ERR_UNSUPPORTED;
    }
    touched(h);
    if (substeps) *substeps = 0;
    if (!h || !target) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    uint64_t count = 0;
    bool interrupted = false;
    const int rc = guarded([&] {
        DeviceGuard g(h->device);
        check_scheme(spatial, temporal);
        check_scheme(h->tr_spatial, h->tr_temporal);
        // LevelSetMorphing::advect accepts FIRST_BIAS and HJWENO5_BIAS only (:243-262)
        if (spatial != GBLS_FIRST_BIAS && spatial != GBLS_HJWENO5_BIAS)
            fail(GBLS_ERR_VALUE, "Spatial difference scheme not supported!");
        if (h->ninst > 1 || target->ninst > 1 || (alpha_mask && alpha_mask->ninst > 1))
            fail(GBLS_ERR_UNSUPPORTED, "morphing works on single level sets, not batches");
        if (h->tape_on) fail(GBLS_ERR_UNSUPPORTED, "the adjoint records advection only");
        auto same_device_and_map = [&](const gbls_handle* o) {
            return o->device == h->device && o->voxel_size == h->voxel_size && o->map_type == h->map_type &&
                   o->translation[0] == h->translation[0] && o->translation[1] == h->translation[1] &&
                   o->translation[2] == h->translation[2];
        };
        if (!same_device_and_map(target) || (alpha_mask && !same_device_and_map(alpha_mask)))
            fail(GBLS_ERR_UNSUPPORTED, "target and alpha mask must share the level set's device and transform "
                                       "(the trilinear sampling of non-aligned grids has no device form)");
        if (alpha_mask && !(mask_min < mask_max)) fail(GBLS_ERR_VALUE, "Invalid mask range (expects min < max)");
        const float delta = mask_max - mask_min;  // setMaskRange: mDeltaMask = max - min
        const float inv_norm = 1.0f / delta;
        const float C = (temporal == GBLS_TVD_RK1 ? 0.3f : temporal == GBLS_TVD_RK2 ? 0.9f : 1.0f) / std::sqrt(3.0f);
        const float dx = float(h->voxel_size);
        target->sync();
        if (alpha_mask) alpha_mask->sync();
        while (t0 < t1) {
            if (!check_intr(*h)) { interrupted = true; break; }
            if (h->nleaf == 0) break;  // sampleSpeed returns 0 for an empty grid
            const float max_s = morph_sample_speed(*h, *target, alpha_mask, mask_min, inv_norm, invert_mask ? 1 : 0);
            if (!(std::fabs(1e-6f - max_s) > 1e-8f)) break;  // isApproxEqual(mMinAbsS, mMaxAbsS): dt = 0
            const float span = std::fabs(t1 - t0);
            const float lim = C * dx / max_s;
            const float dt = (lim < span) ? lim : span;  // math::Min
            if (dt == 0.0f) break;
            if (h->nactive < 0) h->nactive = active_count(*h);
            h->stats.voxel_updates += uint64_t(h->nactive);
            ++h->stats.substeps;
            morph_stages(*h, spatial, temporal, dt);
            t0 += dt;
            ++count;
            track(*h);
        }
        h->sync();
    });
    if (substeps) *substeps = count;
    if (rc == GBLS_OK && interrupted) {
        g_last_error = "interrupted";
        return GBLS_ERR_INTERRUPTED;
    }
    return rc;
}

}  // extern "C"

// ---- NanoVDB on the device ----------------------------------------------------

namespace {

// The level set (or batch instance) of h as a device tree for the NanoVDB
// writers, and a host descriptor with its counts, map, upper-node origins
// and root tiles (the parts the host writes).
struct NanoExport {
    NanoDevTree t;
    gbls_grid_desc d{};
    std::vector<int32_t> upper_origins, root_origins;
    std::vector<float> root_values;
    int64_t voxels = 0;
};

NanoExport nano_export_view(gbls_handle& h, int instance) {
    if (h.f64) fail(GBLS_ERR_UNSUPPORTED, "NanoVDB export of an FP64 level set (NanoGrid<float> holds FP32 values)");
    if (h.ninst > 1 && (instance < 0 || instance >= h.ninst)) fail(GBLS_ERR_INVALID_ARGUMENT, "no such instance");
    if (h.ninst == 1 && instance > 0) fail(GBLS_ERR_INVALID_ARGUMENT, "no such instance");
    h.sync();
    const InstRange R = h.ninst > 1 ? inst_range(h, host_keys(h), instance)
                                    : InstRange{0, h.nleaf, 0, int64_t(h.lower_keys_h.size()), 0,
                                                int64_t(h.upper_keys_h.size()), 0, int64_t(h.root_keys_h.size())};
    NanoExport e;
    NanoDevTree& t = e.t;
    t.nf = R.l1 - R.l0;
    t.nl = R.lo1 - R.lo0;
    t.nu = R.u1 - R.u0;
    t.keys = h.K() + R.l0;
    t.slot = h.S() + R.l0;
    t.am = h.am[h.mc].p;
    t.sm = h.sm[h.mc].p;
    t.vals = h.vals[h.vc].p;
    t.gamma = h.gamma;
    t.lower_keys = h.lower_keys.p + R.lo0;
    t.lower_sign = h.lower_sign.p + R.lo0 * 64;
    t.upper_keys = h.upper_keys.p + R.u0;
    t.upper_sign = h.upper_sign.p + R.u0 * 512;
    for (int64_t i = R.u0; i < R.u1; ++i) {
        int32_t x, y, z;
        key_origin(h.upper_keys_h[size_t(i)] << 27, x, y, z);
        e.upper_origins.insert(e.upper_origins.end(), {x, y, z});
    }
    for (int64_t i = R.r0; i < R.r1; ++i) {
        int32_t x, y, z;
        key_origin(h.root_keys_h[size_t(i)] << 27, x, y, z);
        e.root_origins.insert(e.root_origins.end(), {x, y, z});
        e.root_values.push_back(h.root_sign_h[size_t(i)] ? -h.gamma : h.gamma);
    }
    gbls_grid_desc& d = e.d;
    d.voxel_size = h.voxel_size;
    for (int i = 0; i < 3; ++i) d.translation[i] = h.translation[i];
    d.map_type = h.map_type;
    d.background = h.gamma;
    d.leaf_count = t.nf;
    d.lower_count = t.nl;
    d.upper_count = t.nu;
    d.upper_origins = e.upper_origins.data();
    d.root_tile_count = R.r1 - R.r0;
    d.root_tile_origins = e.root_origins.data();
    d.root_tile_values = e.root_values.data();
    if (t.nf) {
        h.u64s.reserve(1, h.stream);
        CU(cudaMemsetAsync(h.u64s.p, 0, sizeof(unsigned long long), h.stream));
        k_count_active<<<blocks_for(t.nf * 8, 256), 256, 0, h.stream>>>(t.nf, t.slot, t.am, h.u64s.p);
        ++h.stats.kernel_launches;
        CU(cudaGetLastError());
        unsigned long long n = 0;
        CU(cudaMemcpyAsync(&n, h.u64s.p, sizeof(n), cudaMemcpyDeviceToHost, h.stream));
        h.sync();
        e.voxels = int64_t(n);
    }
    return e;
}

void check_device_out(const void* out, int64_t cap, int64_t size) {
    if (cap < size) fail(GBLS_ERR_INVALID_ARGUMENT, "output buffer too small");
    if (reinterpret_cast<uintptr_t>(out) % 32) fail(GBLS_ERR_INVALID_ARGUMENT, "output buffer not 32-byte aligned");
    cudaPointerAttributes a{};
    CU(cudaPointerGetAttributes(&a, out));
    if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)
        fail(GBLS_ERR_INVALID_ARGUMENT, "output buffer is not device memory");
}

// Grid and tree headers (and everything else host-written) are uploaded
// first; the checksum word covers them and, for Full, the device bytes.
void nano_finish(gbls_handle& h, uint8_t* out, std::vector<uint8_t>& top, size_t total, int checksum) {
    CU(cudaMemcpyAsync(out, top.data(), top.size(), cudaMemcpyHostToDevice, h.stream));
    if (checksum == 0) {
        h.sync();
        return;
    }
    const size_t head = gbls_nano::kGridBytes + gbls_nano::kTreeBytes;
    const uint32_t tail = checksum == 2 ? nano_blocked_crc(out + head, total - head, h.stream) : ~0u;
    const uint64_t word = gbls_nano::checksum_word(top.data(), checksum, tail);
    std::memcpy(top.data() + 8, &word, 8);
    CU(cudaMemcpyAsync(out + 8, top.data() + 8, 8, cudaMemcpyHostToDevice, h.stream));
    h.sync();
}

}  // namespace

extern "C" {

int gbls_nanovdb_export_device(gbls_handle* h, int32_t instance, const char* name, int32_t stats_mode,
                               int32_t checksum_mode, void* out, int64_t out_capacity, int64_t* size) {
    if (!h || !size) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        const std::string nm = name ? name : "";
        if (stats_mode < 0 || stats_mode > 3) fail(GBLS_ERR_INVALID_ARGUMENT, "statistics mode must be 0-3");
        if (checksum_mode < 0 || checksum_mode > 2) fail(GBLS_ERR_INVALID_ARGUMENT, "checksum mode must be 0-2");
        if (nm.size() >= 256) fail(GBLS_ERR_UNSUPPORTED, "grid names of 256 characters or more (blind-data names)");
        NanoExport e = nano_export_view(*h, instance);
        const gbls_nano::FloatLayout L(e.t.nu, e.t.nl, e.t.nf, e.d.root_tile_count);
        *size = int64_t(L.total);
        if (!out) return;
        check_device_out(out, out_capacity, *size);
        uint8_t* o = static_cast<uint8_t*>(out);
        CU(cudaMemsetAsync(o, 0, L.total, h->stream));
        std::vector<gbls_nano::NodeStats> upper_stats;
        nano_float_nodes(e.t, stats_mode, o, L, upper_stats, h->stream);
        h->stats.kernel_launches += (e.t.nf > 0) + (e.t.nl > 0) + (e.t.nu > 0);
        std::vector<uint8_t> top(L.upper_at, 0);
        gbls_nano::write_float_top(top.data(), e.d, nm, stats_mode, upper_stats, e.voxels);
        nano_finish(*h, o, top, L.total, checksum_mode);
    });
}

int gbls_nanovdb_export_index_device(gbls_handle* h, int32_t instance, const char* name, int32_t channels,
                                     int32_t include_stats, int32_t include_tiles, int32_t checksum_mode, void* out,
                                     int64_t out_capacity, int64_t* size) {
    if (!h || !size) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        DeviceGuard g(h->device);
        const std::string nm = name ? name : "";
        if (channels < 0) fail(GBLS_ERR_INVALID_ARGUMENT, "negative channel count");
        if (channels > 1) fail(GBLS_ERR_UNSUPPORTED, "more than one value channel");
        if (checksum_mode < 0 || checksum_mode > 2) fail(GBLS_ERR_INVALID_ARGUMENT, "checksum mode must be 0-2");
        if (nm.size() >= 256) fail(GBLS_ERR_UNSUPPORTED, "grid names of 256 characters or more (blind-data names)");
        const bool st = include_stats != 0, tiles = include_tiles != 0;
        NanoExport e = nano_export_view(*h, instance);
        uint64_t* leaf_off = nullptr;
        const uint64_t count = nano_index_offsets(e.t, st, tiles, &leaf_off, h->stream);
        struct OffGuard {
            uint64_t* p;
            cudaStream_t s;
            ~OffGuard() { if (p) cudaFreeAsync(p, s); }
        } og{leaf_off, h->stream};
        const gbls_nano::IndexLayout L(e.t.nu, e.t.nl, e.t.nf, e.d.root_tile_count, channels, count);
        *size = int64_t(L.total);
        if (!out) return;
        check_device_out(out, out_capacity, *size);
        uint8_t* o = static_cast<uint8_t*>(out);
        CU(cudaMemsetAsync(o, 0, L.total, h->stream));
        std::vector<gbls_nano::BBox> upper_box;
        nano_index_nodes(e.t, st, tiles, channels, leaf_off, o, L, upper_box, h->stream);
        h->stats.kernel_launches += (e.t.nf > 0) + (e.t.nl > 0) + (e.t.nu > 0) + (channels > 0);
        if (channels) {
            std::vector<uint8_t> meta(gbls_nano::kBlindMetaBytes * size_t(channels), 0);
            gbls_nano::write_index_meta(meta.data(), L, channels, count);
            CU(cudaMemcpyAsync(o + L.meta_at, meta.data(), meta.size(), cudaMemcpyHostToDevice, h->stream));
            h->sync();
        }
        std::vector<uint8_t> top(L.upper_at, 0);
        gbls_nano::write_index_top(top.data(), e.d, nm, channels, st, tiles, upper_box, e.voxels, count);
        nano_finish(*h, o, top, L.total, checksum_mode);
    });
}

int gbls_nanovdb_probe(const void* grid, int64_t size, const int32_t* ijk, int64_t n, float* values,
                       uint64_t* indices, uint8_t* active, void* stream) {
    if (!grid || size < 0 || n < 0 || (n > 0 && !ijk)) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        cudaPointerAttributes a{};
        CU(cudaPointerGetAttributes(&a, grid));
        if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged)
            fail(GBLS_ERR_INVALID_ARGUMENT, "the NanoVDB buffer is not device memory");
        const int e = nano_probe(static_cast<const uint8_t*>(grid), uint64_t(size), ijk, n, values, indices, active,
                                 static_cast<cudaStream_t>(stream));
        if (e & 2) fail(GBLS_ERR_UNSUPPORTED, "neither a NanoGrid<float> nor a NanoGrid<ValueOnIndex>");
        if (e & 4) fail(GBLS_ERR_INVALID_ARGUMENT, "no output array for the grid's value type");
        if (e & 1) fail(GBLS_ERR_RUNTIME, "truncated or corrupt NanoVDB buffer");
    });
}

int gbls_weno5_exact_device(const float* v, int64_t n, float* out, uint8_t* decided, void* stream) {
    if (n < 0 || (n > 0 && (!v || !out))) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    return guarded([&] {
        const cudaStream_t s = static_cast<cudaStream_t>(stream);
        launch_weno5_exact(v, n, out, decided, s);
        CU(cudaGetLastError());
        CU(cudaStreamSynchronize(s));
    });
}

int gbls_create_from_nanovdb(const void* buffer, int64_t size, gbls_handle** out) {
    if (!buffer || !out || size < 0) { g_last_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    *out = nullptr;
    gbls_host_grid* hg = nullptr;
    uint64_t* d_at = nullptr;
    uint64_t* d_masks = nullptr;
    float* d_vals = nullptr;
    gbls_grid_desc desc{};
    int rc = guarded([&] {
        DeviceGuard g(g_device);
        cudaPointerAttributes a{};
        CU(cudaPointerGetAttributes(&a, buffer));
        const uint8_t* b = static_cast<const uint8_t*>(buffer);
        if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) {
            const gbls_nano::ByteReader read = [b](size_t at, size_t n, uint8_t* dst) { std::memcpy(dst, b + at, n); };
            hg = gbls_nano::import_float(read, size, nullptr);
            if (gbls_host_grid_view(hg, &desc) != GBLS_OK) fail(GBLS_ERR_RUNTIME, "host grid view");
            return;
        }
        if (reinterpret_cast<uintptr_t>(buffer) % 32)
            fail(GBLS_ERR_INVALID_ARGUMENT, "device NanoVDB buffer not 32-byte aligned");
        const gbls_nano::ByteReader read = [b](size_t at, size_t n, uint8_t* dst) {
            CU(cudaMemcpy(dst, b + at, n, cudaMemcpyDeviceToHost));
        };
        std::vector<uint64_t> leaf_at;
        hg = gbls_nano::import_float(read, size, &leaf_at);
        for (uint64_t at : leaf_at)
            if (at % 32) fail(GBLS_ERR_UNSUPPORTED, "NanoVDB leaf not 32-byte aligned");
        if (gbls_host_grid_view(hg, &desc) != GBLS_OK) fail(GBLS_ERR_RUNTIME, "host grid view");
        const int64_t n = int64_t(leaf_at.size());
        if (n) {
            CU(cudaMalloc(&d_at, size_t(n) * 8));
            CU(cudaMalloc(&d_masks, size_t(n) * 64));
            CU(cudaMalloc(&d_vals, size_t(n) * LEAF_VOX * 4));
            CU(cudaMemcpy(d_at, leaf_at.data(), size_t(n) * 8, cudaMemcpyHostToDevice));
            nano_gather_leaves(b, d_at, n, d_masks, d_vals, 0);
            CU(cudaDeviceSynchronize());
        }
        desc.leaf_count = n;
        desc.leaf_masks = d_masks;
        desc.leaf_values = d_vals;
    });
    if (rc == GBLS_OK) rc = create_handle(&desc, out, false);
    cudaFree(d_at);
    cudaFree(d_masks);
    cudaFree(d_vals);
    if (hg) gbls_host_grid_free(hg);
    return rc;
}

}  // extern "C"

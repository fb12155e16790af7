// Topology kernels of the tracker pass: NN_FACE dilation with leaf creation,
// merge of new leaves into tree order, neighbour tables, and the level-set
// prune (leaf removal with the tile sign rule).
#pragma once

#include "gbls_internal.cuh"

namespace gbls {

// Device-side status words read back by the host after a topology phase.
struct DevStatus {
    unsigned long long n_cand;         // candidate new leaves (with duplicates)
    unsigned long long n_lower_miss;   // new leaves whose lower node is missing
    unsigned long long n_lower_empty;  // lower nodes left without leaves
    unsigned long long error;          // device-side consistency check failures
    unsigned int max_v2_bits;          // CFL reduction
    unsigned int pad;
    unsigned long long n_active;       // active voxels of the kept leaves
    unsigned long long io_err;         // upload value checks (IO_ERR_* bits of io.h)
    unsigned long long n_unique;       // distinct candidates (single-CTA sort)
    unsigned long long overflow;       // candidates beyond the single-CTA sort's capacity
};

// Face layer of a leaf mask that a missing neighbour on face f would receive.
__device__ __forceinline__ bool face_layer_nonzero(const uint64_t* m, int f) {
    switch (f) {
    case 0: return m[0] != 0;
    case 1: return m[7] != 0;
    default: break;
    }
    uint64_t sel = (f == 2) ? 0x00000000000000FFull
                 : (f == 3) ? 0xFF00000000000000ull
                 : (f == 4) ? 0x0101010101010101ull
                            : 0x8080808080808080ull;
    uint64_t acc = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) acc |= m[w] & sel;
    return acc != 0;
}

__device__ __forceinline__ bool origin_in_range(uint64_t k) {
    int32_t x, y, z;
    key_origin(k, x, y, z);
    return x > -COORD_LIMIT && y > -COORD_LIMIT && z > -COORD_LIMIT && x < COORD_LIMIT - 8 &&
           y < COORD_LIMIT - 8 && z < COORD_LIMIT - 8;
}

// NN_FACE dilation of leaf l: own mask shifted in-leaf plus the facing layers
// of its six neighbours (tools/Morphology.h:786-812 dilate6 semantics).
__device__ __forceinline__ uint64_t dilate_word(const uint64_t* own, int x, const uint64_t* nmx,
                                                const uint64_t* npx, const uint64_t* nmy,
                                                const uint64_t* npy, const uint64_t* nmz,
                                                const uint64_t* npz) {
    const uint64_t w = own[x];
    uint64_t d = w | ((w << 1) & 0xFEFEFEFEFEFEFEFEull) | ((w >> 1) & 0x7F7F7F7F7F7F7F7Full) |
                 (w << 8) | (w >> 8);
    d |= (x > 0) ? own[x - 1] : (nmx ? nmx[7] : 0);
    d |= (x < 7) ? own[x + 1] : (npx ? npx[0] : 0);
    if (nmy) d |= nmy[x] >> 56;
    if (npy) d |= npy[x] << 56;
    if (nmz) d |= (nmz[x] >> 7) & 0x0101010101010101ull;
    if (npz) d |= (npz[x] << 7) & 0x8080808080808080ull;
    return d;
}

}  // namespace gbls

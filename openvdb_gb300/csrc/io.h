// Device side of the host exchange format (gbls_grid_desc): packing of
// uploaded leaves and node tiles into the slot layout with validation, and
// the reverse assembly for downloads.  The host only builds and checks keys;
// every per-voxel and per-tile loop runs here.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gbls {

// Bits of the upload error word.
constexpr unsigned long long IO_ERR_LEAF_VALUE = 1;   // inactive leaf value other than +-background
constexpr unsigned long long IO_ERR_LOWER_TILE = 2;   // lower-node tile other than +-background
constexpr unsigned long long IO_ERR_UPPER_TILE = 4;   // upper-node tile other than +-background
constexpr unsigned long long IO_ERR_KEYS = 8;         // leaf origins not aligned, in range, in tree order and
                                                      // unique, each under a lower node (host path decides)

// Keys (and identity slots) of n leaves from their origins, checked on the
// device: sets IO_ERR_KEYS when an origin is misaligned or out of range, the
// keys are not strictly increasing, or a leaf has no lower node.
void launch_leaf_keys(int64_t n, const int32_t* origins, const uint64_t* lower_keys, int64_t nlower,
                      uint64_t* keys, int32_t* slot, unsigned long long* err, cudaStream_t s);
// free[j] = top - 1 - j for j < n (the free-slot stack after an upload).
void launch_free_slots(int64_t n, int32_t top, int32_t* free_slots, cudaStream_t s);

// Leaf l (tree order) takes the dense values and mask of staged leaf
// perm[l]: writes am/sm/vals of slot l.  Sets IO_ERR_LEAF_VALUE in *err.
void launch_pack_leaves(int64_t n, const int32_t* perm, const uint64_t* in_masks, const float* in_vals,
                        float gamma, uint64_t* am, uint64_t* sm, float* vals, unsigned long long* err,
                        cudaStream_t s);
// Sign bits of the tiles of node i (tree order) from staged tiles perm[i];
// child slots (a key of the child list under the node) get bit 0.
// `shift` = 12 for lower nodes (children: leaf keys), 15 for upper nodes
// (children: lower keys).
void launch_node_signs(int64_t n, int shift, const uint64_t* node_keys, const int32_t* perm, const float* tiles,
                       const uint64_t* child_keys, int64_t nchild, float gamma, uint64_t* sign,
                       unsigned long long* err, unsigned long long err_bit, cudaStream_t s);
// Download: tree-order origins and masks of leaves [0, n) (slots slot[]).
void launch_leaf_headers(int64_t n, const uint64_t* keys, const int32_t* slot, const uint64_t* am,
                         int32_t* origins, uint64_t* masks, cudaStream_t s);
// Download: dense tiles of nodes [0, n): 0 at child slots, else +-gamma.
void launch_node_tiles(int64_t n, int shift, const uint64_t* node_keys, const uint64_t* sign,
                       const uint64_t* child_keys, int64_t nchild, float gamma, float* tiles, cudaStream_t s);

}  // namespace gbls

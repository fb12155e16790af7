// NanoVDB buffers written and read on the device, straight from / into the
// device tree: the node and leaf parts of the NanoGrid<float> and
// NanoGrid<ValueOnIndex> writers (the headers and the root come from the
// shared host writer in nanovdb_layout.h), the blocked CRC-32, and the leaf
// gather of a NanoGrid<float> import.
#pragma once

#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "nanovdb_layout.h"

namespace gbls {

// A device tree in tree order (device pointers): leaves with their slots
// and masks and packed values, lower and upper nodes by key with their tile
// sign bits.
struct NanoDevTree {
    int64_t nf, nl, nu;
    const uint64_t* keys;        // [nf] leaf keys
    const int32_t* slot;         // [nf]
    const uint64_t* am;          // [slot * 8] active masks
    const uint64_t* sm;          // [slot * 8] sign masks
    const float* vals;           // [slot * 512] packed active values
    float gamma;                 // background
    const uint64_t* lower_keys;  // [nl] (leaf key >> 12)
    const uint64_t* lower_sign;  // [nl * 64]
    const uint64_t* upper_keys;  // [nu] (leaf key >> 27)
    const uint64_t* upper_sign;  // [nu * 512]
};

// Writes the upper nodes, lower nodes and leaves of the NanoGrid<float> of
// `t` into out[upper_at, total) (out zero-filled) with statistics mode
// `mode`, and returns the upper nodes' statistics (empty for Disable).
// Scratch is allocated on the stream.  out must be 32-byte aligned.
void nano_float_nodes(const NanoDevTree& t, int mode, uint8_t* out, const gbls_nano::FloatLayout& L,
                      std::vector<gbls_nano::NodeStats>& upper_stats, cudaStream_t s);

// Value offsets of the index grid's leaves: leaf_off[f] (f < nf) and the
// value count, computed on the device.  leaf_off is allocated on the stream
// and owned by the caller (cudaFreeAsync).
uint64_t nano_index_offsets(const NanoDevTree& t, bool stats, bool tiles, uint64_t** leaf_off, cudaStream_t s);

// Writes the nodes, leaves and (channels == 1) the value channel of the
// NanoGrid<ValueOnIndex> into out (zero-filled); returns the upper nodes'
// bounding boxes.
void nano_index_nodes(const NanoDevTree& t, bool stats, bool tiles, int channels, const uint64_t* leaf_off,
                      uint8_t* out, const gbls_nano::IndexLayout& L, std::vector<gbls_nano::BBox>& upper_box,
                      cudaStream_t s);

// Blocked CRC-32 of p[0, n) (p 16-byte aligned): the CRC of each 4 KiB block
// on the device, combined on the host.
uint32_t nano_blocked_crc(const uint8_t* p, size_t n, cudaStream_t s);

// Import: gathers the origin-ordered leaves at byte offsets at[i] of the
// device buffer `buf` (NanoGrid<float> leaves) into masks[i * 8] and dense
// values[i * 512].
void nano_gather_leaves(const uint8_t* buf, const uint64_t* at, int64_t n, uint64_t* masks, float* values,
                        cudaStream_t s);

// ReadAccessor::getValue / isActive of a NanoGrid<float> or
// NanoGrid<ValueOnIndex> device buffer at n index coordinates (device
// arrays): values for a float grid, indices for an index grid, active flags
// when given.  Returns the kernel's error bits (1: a read outside the
// buffer, 2: another grid type, 4: no output array for the type).
int nano_probe(const uint8_t* buf, uint64_t size, const int32_t* ijk, int64_t n, float* values, uint64_t* indices,
               uint8_t* active, cudaStream_t s);

}  // namespace gbls

// NanoVDB 32.9 buffer layout and the pieces of its writer shared by the host
// exporter (nanovdb_export.cc) and the device exporter (nanovdb_device.cu):
// sizes and offsets of the breadth-first NanoGrid<float> and
// NanoGrid<ValueOnIndex> buffers (nanovdb/NanoVDB.h:1944-2000 GridData,
// 2393-2400 TreeData, 2621-2700 RootData, 3181-3215 InternalData, the leaf
// data of float and ValueOnIndex), running statistics (nanovdb::tools::
// Stats<float, 0>, tools/GridStats.h), the index-to-world map
// (NanoVDB.h:1418-1573) and the CRC-32 checksums (tools/GridChecksum.h).
//
// The statistics are written over NV_HD so the device exporter combines them
// with the same double operations in the same order; both sides compile
// without floating-point contraction.
#pragma once

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "../../include/gbls.h"

#if defined(__CUDACC__)
#define NV_HD __host__ __device__
#else
#define NV_HD
#endif

namespace gbls_nano {

constexpr uint64_t kMagicGrid = 0x314244566f6e614eULL;  // "NanoVDB1"
constexpr uint32_t kVersion = (32u << 21) | (9u << 10) | 2u;
constexpr size_t kGridBytes = 672, kTreeBytes = 64, kRootBytes = 64, kIndexRootBytes = 96, kTileBytes = 32;
constexpr size_t kUpperBytes = 270400, kLowerBytes = 33856, kLeafBytes = 2144, kIndexLeafBytes = 96;
constexpr size_t kUpperTableAt = 8256, kLowerTableAt = 1088;
constexpr size_t kBlindMetaBytes = 288;
enum : uint32_t { kHasBBox = 2, kHasMinMax = 4, kHasAverage = 8, kHasStdDeviation = 16, kIsBreadthFirst = 32 };
enum { kStatsDisable = 0, kStatsBBox = 1, kStatsMinMax = 2, kStatsAll = 3 };

// Running extrema, mean and variance (nanovdb::tools::Stats<float, 0>).
struct Stats {
    float mn = FLT_MAX, mx = -FLT_MAX;
    uint64_t n = 0;
    double avg = 0.0, aux = 0.0;
    NV_HD void add(float v) {
        if (v < mn) mn = v;
        if (v > mx) mx = v;
        n += 1;
        const double delta = double(v) - avg;
        avg += delta / double(n);
        aux += delta * (double(v) - avg);
    }
    NV_HD void add(const Stats& o, bool moments) {
        if (!moments) {  // Extrema::add(Extrema)
            if (o.mn < mn) mn = o.mn;
            if (o.mx > mx) mx = o.mx;
            return;
        }
        if (o.n == 0) return;
        const double denom = 1.0 / double(n + o.n);
        const double delta = o.avg - avg;
        avg += denom * delta * double(o.n);
        aux += o.aux + denom * delta * delta * double(n) * double(o.n);
        if (o.mn < mn) mn = o.mn;
        if (o.mx > mx) mx = o.mx;
        n += o.n;
    }
    NV_HD double dev() const { return sqrt(n < 2 ? 0.0 : aux / double(n)); }
};

struct BBox {
    int32_t lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
    NV_HD bool empty() const { return lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]; }
    NV_HD void add(const BBox& o) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = lo[k] < o.lo[k] ? lo[k] : o.lo[k];
            hi[k] = hi[k] > o.hi[k] ? hi[k] : o.hi[k];
        }
    }
};

struct NodeStats {
    Stats stats;
    BBox bbox;
};

template <class T> NV_HD inline void put(uint8_t* b, size_t at, const T& v) { memcpy(b + at, &v, sizeof(T)); }

// Writes min / max / average / standard deviation at `at` in the statistics
// mode's extent (tools/GridStats.h:541-557).
NV_HD inline void put_stats(uint8_t* b, size_t at, const Stats& s, int mode) {
    if (mode >= kStatsMinMax) {
        put<float>(b, at, s.mn);
        put<float>(b, at + 4, s.mx);
    }
    if (mode == kStatsAll) {
        put<float>(b, at + 8, float(s.avg));
        put<float>(b, at + 12, float(s.dev()));
    }
}

NV_HD inline void put_bbox(uint8_t* b, size_t at, const BBox& x) {
    memcpy(b + at, x.lo, 12);
    memcpy(b + at + 12, x.hi, 12);
}

inline uint64_t root_key(const int32_t* o) {
    return uint64_t(uint32_t(o[2]) >> 12) | (uint64_t(uint32_t(o[1]) >> 12) << 21) |
           (uint64_t(uint32_t(o[0]) >> 12) << 42);
}

// Offsets of the NanoGrid<float> buffer of a grid with these node counts.
struct FloatLayout {
    size_t table, tree_at, root_at, upper_at, lower_at, leaf_at, total;
    FloatLayout(int64_t nu, int64_t nl, int64_t nf, int64_t nt) {
        table = size_t(nu + nt);
        tree_at = kGridBytes;
        root_at = tree_at + kTreeBytes;
        upper_at = root_at + kRootBytes + kTileBytes * table;
        lower_at = upper_at + kUpperBytes * size_t(nu);
        leaf_at = lower_at + kLowerBytes * size_t(nl);
        total = leaf_at + kLeafBytes * size_t(nf);
    }
};

// Offsets of the NanoGrid<ValueOnIndex> buffer; `count` is the value count.
struct IndexLayout {
    size_t table, tree_at, root_at, upper_at, lower_at, leaf_at, meta_at, blind_at, channel_bytes, total;
    IndexLayout(int64_t nu, int64_t nl, int64_t nf, int64_t nt, int channels, uint64_t count) {
        table = size_t(nu + nt);
        tree_at = kGridBytes;
        root_at = tree_at + kTreeBytes;
        upper_at = root_at + kIndexRootBytes + kTileBytes * table;
        lower_at = upper_at + kUpperBytes * size_t(nu);
        leaf_at = lower_at + kLowerBytes * size_t(nl);
        meta_at = leaf_at + kIndexLeafBytes * size_t(nf);
        blind_at = meta_at + kBlindMetaBytes * size_t(channels);
        channel_bytes = (count * 4 + 31) / 32 * 32;
        total = blind_at + channel_bytes * size_t(channels);
    }
};

// First value offset of the leaves and of the internal nodes' statistics
// slots of an index grid: 0 is the background, then (with tiles) four
// statistics slots of the root, every upper and every lower node.
inline uint64_t index_leaf_base(int64_t nu, int64_t nl, bool stats, bool tiles) {
    const uint64_t nstat = stats ? 4 : 0;
    return 1 + (tiles ? nstat * uint64_t(1 + nu + nl) : 0);
}

// CRC-32 (the reflected 0xEDB88320 polynomial) of n bytes.
inline uint32_t crc32(const uint8_t* p, size_t n) {
    uint32_t lut[256];
    for (uint32_t i = 0; i < 256; ++i) {
        uint32_t c = i;
        for (int k = 0; k < 8; ++k) c = (c >> 1) ^ ((c & 1) ? 0xEDB88320u : 0u);
        lut[i] = c;
    }
    uint32_t crc = ~0u;
    for (size_t i = 0; i < n; ++i) crc = lut[(crc ^ p[i]) & 0xFF] ^ (crc >> 8);
    return ~crc;
}

// Number of 4 KiB blocks of a blocked CRC over n bytes (the last block takes
// the remainder) and the CRC of the block checksums
// (util::blockedCrc32, tools/GridChecksum.h:172-185).
inline size_t crc_blocks(size_t n) { return n >> 12; }
inline uint32_t crc_of_blocks(const std::vector<uint32_t>& sums, size_t n) {
    if (n == 0) return ~0u;
    return crc32(reinterpret_cast<const uint8_t*>(sums.data()), 4 * sums.size());
}

// The checksum word: head CRC of the grid and tree headers (bytes 16-735),
// and for CheckMode::Full the blocked CRC of everything after them
// (tools/GridChecksum.h:206-230, 280-300).
inline uint64_t checksum_word(const uint8_t* head, int mode, uint32_t tail) {
    const uint32_t h = crc32(head + 16, kGridBytes + kTreeBytes - 16);
    return (uint64_t(mode == 2 ? tail : ~0u) << 32) | h;
}

// nanovdb Map (NanoVDB.h:1418-1573) of a uniform scale + translation.
struct MapD {
    double mat[9], inv[9], vec[3];
    void apply(const double xyz[3], double out[3]) const {  // math::matMult with fma
        for (int r = 0; r < 3; ++r)
            out[r] = std::fma(xyz[0], mat[3 * r], std::fma(xyz[1], mat[3 * r + 1], std::fma(xyz[2], mat[3 * r + 2], vec[r])));
    }
};

// Thrown by the writers; the C entry points turn it into an error code.
struct ExportError {
    int code;
    std::string msg;
};
[[noreturn]] inline void fail(int code, const std::string& msg) { throw ExportError{code, msg}; }

MapD make_map(const gbls_grid_desc& d);
void put_map(uint8_t* b, size_t at, const MapD& m);

// The grid header, tree header and root (header + tile table) of a
// NanoGrid<float>, written into b[0, upper_at): everything above the
// internal nodes.  Uses the descriptor's counts, upper-node origins, root
// tiles, map and background; upper_stats are the statistics of the upper
// nodes in tree order (empty when mode is Disable).  No checksum.
void write_float_top(uint8_t* b, const gbls_grid_desc& d, const std::string& name, int mode,
                     const std::vector<NodeStats>& upper_stats, int64_t voxels);

// The same for a NanoGrid<ValueOnIndex> into b[0, upper_at): upper_box are
// the bounding boxes of the upper nodes.
void write_index_top(uint8_t* b, const gbls_grid_desc& d, const std::string& name, int channels, bool stats,
                     bool tiles, const std::vector<BBox>& upper_box, int64_t voxels, uint64_t count);

// Reads n bytes at offset `at` of a NanoVDB buffer into dst.
using ByteReader = std::function<void(size_t at, size_t n, uint8_t* dst)>;

// A NanoGrid<float> read through `read` (size bytes) as a host grid in the
// exchange layout.  With leaf_at, the leaves are not read: their origins are
// filled in and their byte offsets appended to *leaf_at (tree order), the
// leaf masks and values stay empty.
gbls_host_grid* import_float(const ByteReader& read, int64_t size, std::vector<uint64_t>* leaf_at);

// The blind-data metadata of the value channels, into m[0, 288 * channels)
// (the bytes at layout.meta_at).
void write_index_meta(uint8_t* m, const IndexLayout& L, int channels, uint64_t count);

}  // namespace gbls_nano

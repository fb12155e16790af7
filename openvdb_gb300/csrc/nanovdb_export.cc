// NanoVDB export of a level set, on the host.
//
// gbls_nanovdb_export stands in for nanovdb::tools::createNanoGrid applied
// to an openvdb::FloatGrid (nanovdb/tools/CreateNanoGrid.h:162-168): the
// breadth-first NanoGrid<float> buffer of NanoVDB 32.9 --
//   GridData (672 B) | TreeData (64 B) | RootData (64 B) + root tiles (32 B
//   each, in the source root's Coord order) | upper nodes (270,400 B) |
//   lower nodes (33,856 B) | leaves (2,144 B), nodes in tree order
// (CreateNanoGrid.h:930-957 offsets, 1188-1221 leaves, 1481-1527 internal
// nodes, 1589-1614 root, 1660-1733 tree and grid; NanoVDB.h:1418-1573 Map,
// 1944-2000 GridData, 2393-2400 TreeData, 2621-2700 RootData,
// 3181-3215 InternalData).  The index-to-world map is the one CreateNanoGrid
// derives from the grid's affine matrix and its inverse (openvdb/math/
// Mat4.h:485-560 for a scale + translate matrix).  Statistics follow
// nanovdb::tools::updateGridStats (tools/GridStats.h:244-442, 577-760):
// per-node active bounding boxes, extrema, and the running mean / variance
// combined child by child in tree order (the serial form of the reduction),
// in double precision.  Checksums: the CRC-32 of the grid and tree headers
// (CheckMode::Partial) and the blocked CRC of the nodes (CheckMode::Full),
// tools/GridChecksum.h:172-230, 280-323.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "host_grid.h"
#include "nanovdb_layout.h"

namespace gbls_nano {

inline bool bit(const uint64_t* m, int i) { return (m[i >> 6] >> (i & 63)) & 1u; }

namespace {

// Gauss-Jordan elimination with partial pivoting on a 4x4 matrix (rows
// scaled by division, elimination below then above the pivots), the form
// openvdb::math::Mat4::invert takes (openvdb/math/Mat4.h) when the 3x3
// determinant is too small for the cofactor inverse.
void gauss_jordan(const double a[4][4], double inv[4][4]) {
    double t[4][4];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            t[r][c] = a[r][c];
            inv[r][c] = r == c ? 1.0 : 0.0;
        }
    for (int i = 0; i < 4; ++i) {
        int row = i;
        double mx = std::fabs(t[i][i]);
        for (int k = i + 1; k < 4; ++k)
            if (std::fabs(t[k][i]) > mx) {
                row = k;
                mx = std::fabs(t[k][i]);
            }
        if (mx == 0.0) fail(GBLS_ERR_RUNTIME, "singular index-to-world matrix");
        if (row != i)
            for (int k = 0; k < 4; ++k) {
                std::swap(t[row][k], t[i][k]);
                std::swap(inv[row][k], inv[i][k]);
            }
        const double pivot = t[i][i];
        for (int k = 0; k < 4; ++k) {
            t[i][k] /= pivot;
            inv[i][k] /= pivot;
        }
        for (int j = i + 1; j < 4; ++j) {
            const double f = t[j][i];
            if (f == 0.0) continue;
            for (int k = 0; k < 4; ++k) {
                t[j][k] -= t[i][k] * f;
                inv[j][k] -= inv[i][k] * f;
            }
        }
    }
    for (int i = 3; i > 0; --i)
        for (int j = 0; j < i; ++j) {
            const double f = t[j][i];
            if (f == 0.0) continue;
            for (int k = 0; k < 4; ++k) inv[j][k] -= inv[i][k] * f;
        }
}

}  // namespace

MapD make_map(const gbls_grid_desc& d) {
    MapD m{};
    const double s = d.map_type == GBLS_MAP_TRANSLATION ? 1.0 : d.voxel_size;
    double vec[3];
    for (int k = 0; k < 3; ++k) vec[k] = d.map_type == GBLS_MAP_UNIFORM_SCALE ? 0.0 : d.translation[k];
    for (int k = 0; k < 9; ++k) m.mat[k] = m.inv[k] = 0.0;
    for (int k = 0; k < 3; ++k) {
        m.mat[4 * k] = s;
        m.vec[k] = vec[k];
    }
    // Mat4d::inverse of diag(s, s, s, 1) with the translation in its last
    // row: 1/det(A) times the cofactors, or Gauss-Jordan when |det(A)| <= 1e-8
    const double det = s * s * s;
    if (std::fabs(det) <= 1e-8) {
        const double a[4][4] = {{s, 0, 0, 0}, {0, s, 0, 0}, {0, 0, s, 0}, {vec[0], vec[1], vec[2], 1.0}};
        double inv[4][4];
        gauss_jordan(a, inv);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) m.inv[3 * r + c] = inv[c][r];  // stored transposed
    } else {
        const double inv = (1.0 / det) * (s * s);
        for (int k = 0; k < 3; ++k) m.inv[4 * k] = inv;
    }
    return m;
}

void put_map(uint8_t* b, size_t at, const MapD& m) {
    for (int k = 0; k < 9; ++k) put<float>(b, at + 4 * k, float(m.mat[k]));
    for (int k = 0; k < 9; ++k) put<float>(b, at + 36 + 4 * k, float(m.inv[k]));
    for (int k = 0; k < 3; ++k) put<float>(b, at + 72 + 4 * k, float(m.vec[k]));
    put<float>(b, at + 84, 1.0f);
    for (int k = 0; k < 9; ++k) put<double>(b, at + 88 + 8 * k, m.mat[k]);
    for (int k = 0; k < 9; ++k) put<double>(b, at + 160 + 8 * k, m.inv[k]);
    for (int k = 0; k < 3; ++k) put<double>(b, at + 232 + 8 * k, m.vec[k]);
    put<double>(b, at + 256, 1.0);
}

namespace {

// Blocked CRC of n bytes (util::blockedCrc32, tools/GridChecksum.h:172-185).
uint32_t blocked_crc32(const uint8_t* p, size_t n) {
    const size_t blocks = crc_blocks(n);
    std::vector<uint32_t> sums(blocks);
    for (size_t i = 0; i < blocks; ++i) {
        size_t len = size_t(1) << 12;
        if (i + 1 == blocks) len += n - (blocks << 12);
        sums[i] = crc32(p + (i << 12), len);
    }
    return crc_of_blocks(sums, n);
}

void put_checksum(std::vector<uint8_t>& b, int mode) {
    if (mode == 0) return;
    const size_t head = kGridBytes + kTreeBytes;
    const uint32_t tail = mode == 2 ? blocked_crc32(b.data() + head, b.size() - head) : ~0u;
    put<uint64_t>(b.data(), 8, checksum_word(b.data(), mode, tail));
}

// Root entries of a grid: its upper nodes and root tiles merged in Coord
// order, as (index, is child).
std::vector<std::pair<int64_t, bool>> root_entries(const gbls_grid_desc& d) {
    std::vector<std::pair<int64_t, bool>> entries;
    for (int64_t i = 0; i < d.upper_count; ++i) entries.push_back({i, true});
    for (int64_t i = 0; i < d.root_tile_count; ++i) entries.push_back({i, false});
    auto origin_of = [&](const std::pair<int64_t, bool>& e) {
        return e.second ? d.upper_origins + 3 * e.first : d.root_tile_origins + 3 * e.first;
    };
    std::stable_sort(entries.begin(), entries.end(), [&](const auto& a, const auto& c) {
        const int32_t *p = origin_of(a), *q = origin_of(c);
        return std::lexicographical_compare(p, p + 3, q, q + 3);
    });
    return entries;
}

const int32_t* entry_origin(const gbls_grid_desc& d, const std::pair<int64_t, bool>& e) {
    return e.second ? d.upper_origins + 3 * e.first : d.root_tile_origins + 3 * e.first;
}

// World-space bounding box of an index bounding box (corners through the
// map) into grid bytes 560-607, and the voxel size at 608-631.
void put_world_bbox(uint8_t* b, const MapD& map, const BBox& box, bool valid) {
    double wlo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, whi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    if (valid) {
        const int32_t lo[3] = {box.lo[0], box.lo[1], box.lo[2]};
        const int32_t hi[3] = {box.hi[0] + 1, box.hi[1] + 1, box.hi[2] + 1};
        for (int corner = 0; corner < 8; ++corner) {
            const double p[3] = {double((corner & 4) ? hi[0] : lo[0]), double((corner & 2) ? hi[1] : lo[1]),
                                 double((corner & 1) ? hi[2] : lo[2])};
            double w[3];
            map.apply(p, w);
            for (int k = 0; k < 3; ++k) {
                wlo[k] = std::min(wlo[k], w[k]);
                whi[k] = std::max(whi[k], w[k]);
            }
        }
    }
    for (int k = 0; k < 3; ++k) {
        put<double>(b, 560 + 8 * k, wlo[k]);
        put<double>(b, 584 + 8 * k, whi[k]);
    }
    const double one[3] = {1.0, 1.0, 1.0}, zero[3] = {0.0, 0.0, 0.0};
    double a1[3], a0[3];
    map.apply(one, a1);
    map.apply(zero, a0);
    for (int k = 0; k < 3; ++k) put<double>(b, 608 + 8 * k, a1[k] - a0[k]);
}

void put_tree(uint8_t* b, size_t tree_at, size_t root_at, size_t upper_at, size_t lower_at, size_t leaf_at,
              int64_t nu, int64_t nl, int64_t nf, int64_t voxels) {
    put<int64_t>(b, tree_at, nf ? int64_t(leaf_at - tree_at) : 0);
    put<int64_t>(b, tree_at + 8, nl ? int64_t(lower_at - tree_at) : 0);
    put<int64_t>(b, tree_at + 16, nu ? int64_t(upper_at - tree_at) : 0);
    put<int64_t>(b, tree_at + 24, int64_t(root_at - tree_at));
    put<uint32_t>(b, tree_at + 32, uint32_t(nf));
    put<uint32_t>(b, tree_at + 36, uint32_t(nl));
    put<uint32_t>(b, tree_at + 40, uint32_t(nu));
    put<uint64_t>(b, tree_at + 56, uint64_t(voxels));
}

void check_desc(const gbls_grid_desc& d) {
    if (d.leaf_count < 0 || d.lower_count < 0 || d.upper_count < 0 || d.root_tile_count < 0)
        fail(GBLS_ERR_INVALID_ARGUMENT, "negative count in grid descriptor");
}

}  // namespace

void write_float_top(uint8_t* b, const gbls_grid_desc& d, const std::string& name, int mode,
                     const std::vector<NodeStats>& upper_stats, int64_t voxels) {
    const FloatLayout L(d.upper_count, d.lower_count, d.leaf_count, d.root_tile_count);
    const bool minmax = mode >= kStatsMinMax, moments = mode == kStatsAll;
    // root: children and tiles merged in Coord order
    const auto entries = root_entries(d);
    NodeStats root_total;
    for (size_t t = 0; t < entries.size(); ++t) {
        const size_t at = L.root_at + kRootBytes + kTileBytes * t;
        put<uint64_t>(b, at, root_key(entry_origin(d, entries[t])));
        if (entries[t].second) {
            put<int64_t>(b, at + 8, int64_t(L.upper_at + kUpperBytes * size_t(entries[t].first)) - int64_t(L.root_at));
            root_total.stats.add(upper_stats.empty() ? Stats() : upper_stats[size_t(entries[t].first)].stats, moments);
            if (!upper_stats.empty()) root_total.bbox.add(upper_stats[size_t(entries[t].first)].bbox);
        } else {
            put<float>(b, at + 20, d.root_tile_values[entries[t].first]);
        }
    }
    put<uint32_t>(b, L.root_at + 24, uint32_t(L.table));
    put<float>(b, L.root_at + 28, d.background);
    BBox root_bbox;
    if (L.table == 0 || mode == kStatsDisable) {
        put<float>(b, L.root_at + 32, d.background);
        put<float>(b, L.root_at + 36, d.background);
    } else {
        root_bbox = root_total.bbox;
        if (mode == kStatsBBox) {
            put<float>(b, L.root_at + 32, d.background);
            put<float>(b, L.root_at + 36, d.background);
        } else {
            put_stats(b, L.root_at + 32, root_total.stats, mode);
        }
    }
    put_bbox(b, L.root_at, root_bbox);
    put_tree(b, L.tree_at, L.root_at, L.upper_at, L.lower_at, L.leaf_at, d.upper_count, d.lower_count, d.leaf_count,
             voxels);
    // grid
    const MapD map = make_map(d);
    put<uint64_t>(b, 0, kMagicGrid);
    put<uint64_t>(b, 8, ~uint64_t(0));
    put<uint32_t>(b, 16, kVersion);
    uint32_t flags = kIsBreadthFirst;
    if (mode != kStatsDisable) {
        if (!root_bbox.empty()) flags |= kHasBBox;
        if (minmax) flags |= kHasMinMax;
        if (moments) flags |= kHasAverage | kHasStdDeviation;
    }
    put<uint32_t>(b, 20, flags);
    put<uint32_t>(b, 28, 1);  // grid count
    put<uint64_t>(b, 32, uint64_t(L.total));
    std::memcpy(b + 40, name.data(), name.size());
    put_map(b, 296, map);
    put_world_bbox(b, map, root_bbox, mode != kStatsDisable && !root_bbox.empty());
    put<uint32_t>(b, 632, 1);  // GridClass::LevelSet
    put<uint32_t>(b, 636, 1);  // GridType::Float
    put<int64_t>(b, 640, int64_t(L.total));  // no blind data
}

void write_index_top(uint8_t* b, const gbls_grid_desc& d, const std::string& name, int channels, bool stats,
                     bool tiles, const std::vector<BBox>& upper_box, int64_t voxels, uint64_t count) {
    const IndexLayout L(d.upper_count, d.lower_count, d.leaf_count, d.root_tile_count, channels, count);
    const auto entries = root_entries(d);
    BBox root_box;
    for (size_t t = 0; t < entries.size(); ++t) {
        const size_t at = L.root_at + kIndexRootBytes + kTileBytes * t;
        put<uint64_t>(b, at, root_key(entry_origin(d, entries[t])));
        if (entries[t].second) {
            put<int64_t>(b, at + 8, int64_t(L.upper_at + kUpperBytes * size_t(entries[t].first)) - int64_t(L.root_at));
            root_box.add(upper_box[size_t(entries[t].first)]);
        }
    }
    put_bbox(b, L.root_at, root_box);
    put<uint32_t>(b, L.root_at + 24, uint32_t(L.table));
    if (tiles && stats && L.table > 0)  // the statistics pass resets an empty root's slots to 0
        for (int k = 0; k < 4; ++k) put<uint64_t>(b, L.root_at + 40 + 8 * size_t(k), uint64_t(k + 1));
    put_tree(b, L.tree_at, L.root_at, L.upper_at, L.lower_at, L.leaf_at, d.upper_count, d.lower_count, d.leaf_count,
             voxels);
    const MapD map = make_map(d);
    put<uint64_t>(b, 0, kMagicGrid);
    put<uint64_t>(b, 8, ~uint64_t(0));
    put<uint32_t>(b, 16, kVersion);
    put<uint32_t>(b, 20, kIsBreadthFirst | (root_box.empty() ? 0u : kHasBBox));
    put<uint32_t>(b, 28, 1);
    put<uint64_t>(b, 32, uint64_t(L.total));
    std::memcpy(b + 40, name.data(), name.size());
    put_map(b, 296, map);
    put_world_bbox(b, map, root_box, !root_box.empty());
    put<uint32_t>(b, 632, 8);   // GridClass::IndexGrid
    put<uint32_t>(b, 636, 20);  // GridType::OnIndex
    put<int64_t>(b, 640, channels ? int64_t(L.meta_at) : int64_t(L.total));
    put<uint32_t>(b, 648, uint32_t(channels));
    put<uint64_t>(b, 656, count);
}

void write_index_meta(uint8_t* m, const IndexLayout& L, int channels, uint64_t count) {
    for (int ch = 0; ch < channels; ++ch) {
        const size_t mat = L.meta_at + kBlindMetaBytes * size_t(ch), dat = L.blind_at + L.channel_bytes * size_t(ch);
        const size_t at = kBlindMetaBytes * size_t(ch);
        put<int64_t>(m, at, int64_t(dat) - int64_t(mat));
        put<uint64_t>(m, at + 8, count);
        put<uint32_t>(m, at + 16, 4);
        put<uint32_t>(m, at + 20, 10);  // GridBlindDataSemantic::LevelSet
        put<uint32_t>(m, at + 24, 4);   // GridBlindDataClass::ChannelArray
        put<uint32_t>(m, at + 28, 1);   // GridType::Float
        const std::string cn = "channel_" + std::to_string(ch);
        std::memcpy(m + at + 32, cn.data(), cn.size());
    }
}

namespace {

std::vector<uint8_t> build(const gbls_grid_desc& d, const std::string& name, int mode, int checksum) {
    check_desc(d);
    if (mode < kStatsDisable || mode > kStatsAll) fail(GBLS_ERR_INVALID_ARGUMENT, "statistics mode must be 0-3");
    if (checksum < 0 || checksum > 2) fail(GBLS_ERR_INVALID_ARGUMENT, "checksum mode must be 0-2");
    if (name.size() >= 256) fail(GBLS_ERR_UNSUPPORTED, "grid names of 256 characters or more (blind-data names)");
    const int64_t nu = d.upper_count, nl = d.lower_count, nf = d.leaf_count;
    const FloatLayout L(nu, nl, nf, d.root_tile_count);
    std::vector<uint8_t> b(L.total, 0);
    const bool minmax = mode >= kStatsMinMax, moments = mode == kStatsAll;

    // leaves
    std::vector<NodeStats> leaf_stats(static_cast<size_t>(nf));
    int64_t voxels = 0;
    for (int64_t f = 0; f < nf; ++f) {
        const size_t at = L.leaf_at + kLeafBytes * size_t(f);
        const int32_t* o = d.leaf_origins + 3 * f;
        const uint64_t* m = d.leaf_masks + 8 * f;
        const float* v = d.leaf_values + 512 * f;
        for (int w = 0; w < 8; ++w) voxels += __builtin_popcountll(m[w]);
        std::memcpy(b.data() + at, o, 12);
        std::memcpy(b.data() + at + 16, m, 64);
        std::memcpy(b.data() + at + 96, v, 2048);
        if (mode == kStatsDisable) continue;
        NodeStats& ns = leaf_stats[size_t(f)];
        bool any = false;
        for (int i = 0; i < 512; ++i) {
            if (!bit(m, i)) continue;
            const int32_t c[3] = {o[0] + (i >> 6), o[1] + ((i >> 3) & 7), o[2] + (i & 7)};
            for (int k = 0; k < 3; ++k) {
                ns.bbox.lo[k] = std::min(ns.bbox.lo[k], c[k]);
                ns.bbox.hi[k] = std::max(ns.bbox.hi[k], c[k]);
            }
            if (minmax) ns.stats.add(v[i]);
            any = true;
        }
        if (!any) continue;
        std::memcpy(b.data() + at, ns.bbox.lo, 12);
        for (int k = 0; k < 3; ++k) b[at + 12 + k] = uint8_t(ns.bbox.hi[k] - ns.bbox.lo[k]);
        b[at + 15] = 2;  // has a bounding box; rendering enabled
        put_stats(b.data(), at + 80, ns.stats, mode);
    }

    // internal nodes: child offsets, tile values, then statistics from the children
    auto internal = [&](int64_t count, size_t base, size_t bytes, size_t table_at, int log2, const int32_t* origins,
                        const float* tiles, int64_t child_count, const int32_t* child_origins, size_t child_base,
                        size_t child_bytes, int child_log2, const std::vector<NodeStats>& child_stats,
                        std::vector<NodeStats>& out_stats) {
        const int dim = 1 << log2, nvals = 1 << (3 * log2), child_shift = child_log2;
        out_stats.assign(size_t(count), NodeStats());
        int64_t c = 0;
        for (int64_t i = 0; i < count; ++i) {
            const size_t at = base + bytes * size_t(i);
            const int32_t* o = origins + 3 * i;
            std::memcpy(b.data() + at, o, 12);
            const int64_t c0 = c;
            std::vector<uint8_t> is_child(size_t(nvals), 0);
            for (; c < child_count; ++c) {
                const int32_t* co = child_origins + 3 * c;
                const int32_t span = dim << child_shift;
                if ((co[0] & ~(span - 1)) != o[0] || (co[1] & ~(span - 1)) != o[1] || (co[2] & ~(span - 1)) != o[2]) break;
                const int n = ((((co[0] - o[0]) >> child_shift) << (2 * log2)) | (((co[1] - o[1]) >> child_shift) << log2) |
                               ((co[2] - o[2]) >> child_shift));
                if (is_child[size_t(n)]) fail(GBLS_ERR_INVALID_ARGUMENT, "grid descriptor is not in tree order");
                is_child[size_t(n)] = 1;
                b[at + 32 + size_t(nvals / 8) + size_t(n >> 3)] |= uint8_t(1u << (n & 7));  // child mask
                put<int64_t>(b.data(), at + table_at + 8 * size_t(n),
                             int64_t(child_base + child_bytes * size_t(c)) - int64_t(at));
            }
            for (int n = 0; n < nvals; ++n)
                if (!is_child[size_t(n)])
                    put<float>(b.data(), at + table_at + 8 * size_t(n), tiles[size_t(i) * size_t(nvals) + size_t(n)]);
            if (mode == kStatsDisable) continue;
            NodeStats& total = out_stats[size_t(i)];
            // children are consecutive in tree order, which is their table order
            for (int64_t k = c0; k < c; ++k) {
                total.stats.add(child_stats[size_t(k)].stats, moments);
                total.bbox.add(child_stats[size_t(k)].bbox);
            }
            put_bbox(b.data(), at, total.bbox);  // empty (max, min) when no child has active values
            if (total.bbox.empty()) {
                put<uint64_t>(b.data(), at + 24, 1);  // no active values: skip rendering
                continue;
            }
            put<uint64_t>(b.data(), at + 24, 2);
            put_stats(b.data(), at + 32 + size_t(nvals / 4), total.stats, mode);
        }
        if (c != child_count) fail(GBLS_ERR_INVALID_ARGUMENT, "grid descriptor is not in tree order (orphan child node)");
    };
    std::vector<NodeStats> lower_stats, upper_stats;
    internal(nl, L.lower_at, kLowerBytes, kLowerTableAt, 4, d.lower_origins, d.lower_tiles, nf, d.leaf_origins,
             L.leaf_at, kLeafBytes, 3, leaf_stats, lower_stats);
    internal(nu, L.upper_at, kUpperBytes, kUpperTableAt, 5, d.upper_origins, d.upper_tiles, nl, d.lower_origins,
             L.lower_at, kLowerBytes, 7, lower_stats, upper_stats);
    if (mode == kStatsDisable) upper_stats.clear();
    write_float_top(b.data(), d, name, mode, upper_stats, voxels);
    put_checksum(b, checksum);
    return b;
}

// NanoGrid<ValueOnIndex> (CreateNanoGrid.h:184-190, 1099-1186 value counts,
// 1228-1267 leaves, 1531-1585 internal nodes, 1618-1656 root, 1796-1880
// value channel): nodes hold offsets into a value array -- 0 the background,
// then (with tiles) four statistics slots of the root and of every internal
// node (the background value: an OpenVDB source has no statistics), then per
// leaf its active values in index order followed (with stats) by four
// background slots.  Leaves carry their first offset and the 9-bit prefix
// sums of active voxels over their mask words.  `channels` copies of the value
// array follow as blind data ("channel_<i>", ChannelArray, level-set
// semantic).  Node statistics are bounding boxes only (updateGridStats with
// StatsMode::BBox, as the converter does for index grids).
std::vector<uint8_t> build_index(const gbls_grid_desc& d, const std::string& name, int channels, bool stats,
                                 bool tiles, int checksum) {
    check_desc(d);
    if (channels < 0) fail(GBLS_ERR_INVALID_ARGUMENT, "negative channel count");
    // The converter fills channel i > 0 from (its own start - value count),
    // which reads across the previous channel's alignment padding: only 0 or 1
    // channels have well-defined contents.
    if (channels > 1) fail(GBLS_ERR_UNSUPPORTED, "more than one value channel");
    if (checksum < 0 || checksum > 2) fail(GBLS_ERR_INVALID_ARGUMENT, "checksum mode must be 0-2");
    if (name.size() >= 256) fail(GBLS_ERR_UNSUPPORTED, "grid names of 256 characters or more (blind-data names)");
    const int64_t nu = d.upper_count, nl = d.lower_count, nf = d.leaf_count;
    const uint64_t nstat = stats ? 4 : 0;
    // value offsets (countValues / countTileValues)
    uint64_t count = 1;
    std::vector<uint64_t> upper_off(static_cast<size_t>(nu)), lower_off(static_cast<size_t>(nl)),
        leaf_off(static_cast<size_t>(nf));
    if (tiles) {
        count += nstat;  // root statistics (a level set has no active root tiles)
        for (int64_t i = 0; i < nu; ++i) upper_off[size_t(i)] = count, count += nstat;
        for (int64_t i = 0; i < nl; ++i) lower_off[size_t(i)] = count, count += nstat;
    }
    std::vector<int> active(static_cast<size_t>(nf));
    for (int64_t f = 0; f < nf; ++f) {
        int a = 0;
        for (int w = 0; w < 8; ++w) a += __builtin_popcountll(d.leaf_masks[8 * f + w]);
        active[size_t(f)] = a;
        leaf_off[size_t(f)] = count;
        count += uint64_t(a) + nstat;
    }
    const IndexLayout L(nu, nl, nf, d.root_tile_count, channels, count);
    std::vector<uint8_t> b(L.total, 0);

    // leaves: origin, mask, offset, prefix sums; bounding boxes
    std::vector<BBox> leaf_box(static_cast<size_t>(nf));
    for (int64_t f = 0; f < nf; ++f) {
        const size_t at = L.leaf_at + kIndexLeafBytes * size_t(f);
        const int32_t* o = d.leaf_origins + 3 * f;
        const uint64_t* m = d.leaf_masks + 8 * f;
        std::memcpy(b.data() + at, o, 12);
        std::memcpy(b.data() + at + 16, m, 64);
        put<uint64_t>(b.data(), at + 80, leaf_off[size_t(f)]);
        uint64_t sum = uint64_t(__builtin_popcountll(m[0])), prefix = sum;
        for (int w = 1, sh = 9; w < 7; ++w, sh += 9) {
            sum += uint64_t(__builtin_popcountll(m[w]));
            prefix |= sum << sh;
        }
        put<uint64_t>(b.data(), at + 88, prefix);
        uint8_t flags = stats ? 16 : 0;
        BBox& bx = leaf_box[size_t(f)];
        for (int i = 0; i < 512; ++i) {
            if (!bit(m, i)) continue;
            const int32_t c[3] = {o[0] + (i >> 6), o[1] + ((i >> 3) & 7), o[2] + (i & 7)};
            for (int k = 0; k < 3; ++k) {
                bx.lo[k] = std::min(bx.lo[k], c[k]);
                bx.hi[k] = std::max(bx.hi[k], c[k]);
            }
        }
        if (!bx.empty()) {
            std::memcpy(b.data() + at, bx.lo, 12);
            for (int k = 0; k < 3; ++k) b[at + 12 + k] = uint8_t(bx.hi[k] - bx.lo[k]);
            flags |= 2;
        }
        b[at + 15] = flags;
    }
    // internal nodes: child offsets (tile slots 0: no active tiles), stats offsets, boxes
    auto internal = [&](int64_t cnt, size_t base, size_t bytes, size_t table_at, int log2, const int32_t* origins,
                        const std::vector<uint64_t>& offs, int64_t child_count, const int32_t* child_origins,
                        size_t child_base, size_t child_bytes, int child_shift, const std::vector<BBox>& child_box,
                        std::vector<BBox>& out_box) {
        const int nvals = 1 << (3 * log2);
        out_box.assign(size_t(cnt), BBox());
        int64_t c = 0;
        for (int64_t i = 0; i < cnt; ++i) {
            const size_t at = base + bytes * size_t(i);
            const int32_t* o = origins + 3 * i;
            const int32_t span = (1 << log2) << child_shift;
            for (; c < child_count; ++c) {
                const int32_t* co = child_origins + 3 * c;
                if ((co[0] & ~(span - 1)) != o[0] || (co[1] & ~(span - 1)) != o[1] || (co[2] & ~(span - 1)) != o[2]) break;
                const int n = ((((co[0] - o[0]) >> child_shift) << (2 * log2)) | (((co[1] - o[1]) >> child_shift) << log2) |
                               ((co[2] - o[2]) >> child_shift));
                b[at + 32 + size_t(nvals / 8) + size_t(n >> 3)] |= uint8_t(1u << (n & 7));
                put<int64_t>(b.data(), at + table_at + 8 * size_t(n), int64_t(child_base + child_bytes * size_t(c)) - int64_t(at));
                out_box[size_t(i)].add(child_box[size_t(c)]);
            }
            if (tiles && stats)
                for (int k = 0; k < 4; ++k)
                    put<uint64_t>(b.data(), at + 32 + size_t(nvals / 4) + 8 * size_t(k), offs[size_t(i)] + uint64_t(k));
            put_bbox(b.data(), at, out_box[size_t(i)]);
            put<uint64_t>(b.data(), at + 24, out_box[size_t(i)].empty() ? 1 : 2);
        }
        if (c != child_count) fail(GBLS_ERR_INVALID_ARGUMENT, "grid descriptor is not in tree order (orphan child node)");
    };
    std::vector<BBox> lower_box, upper_box;
    internal(nl, L.lower_at, kLowerBytes, kLowerTableAt, 4, d.lower_origins, lower_off, nf, d.leaf_origins, L.leaf_at,
             kIndexLeafBytes, 3, leaf_box, lower_box);
    internal(nu, L.upper_at, kUpperBytes, kUpperTableAt, 5, d.upper_origins, upper_off, nl, d.lower_origins,
             L.lower_at, kLowerBytes, 7, lower_box, upper_box);
    int64_t voxels = 0;
    for (int a : active) voxels += a;
    write_index_top(b.data(), d, name, channels, stats, tiles, upper_box, voxels, count);
    // value channels
    write_index_meta(b.data() + L.meta_at, L, channels, count);
    for (int ch = 0; ch < channels; ++ch) {
        float* v = reinterpret_cast<float*>(b.data() + L.blind_at + L.channel_bytes * size_t(ch));
        const float bg = d.background;
        v[0] = bg;
        if (tiles && stats) {
            for (int k = 0; k < 4; ++k) v[1 + k] = bg;
            for (int64_t i = 0; i < nu; ++i) for (int k = 0; k < 4; ++k) v[upper_off[size_t(i)] + uint64_t(k)] = bg;
            for (int64_t i = 0; i < nl; ++i) for (int k = 0; k < 4; ++k) v[lower_off[size_t(i)] + uint64_t(k)] = bg;
        }
        for (int64_t f = 0; f < nf; ++f) {
            uint64_t o = leaf_off[size_t(f)];
            const uint64_t* m = d.leaf_masks + 8 * f;
            for (int i = 0; i < 512; ++i)
                if (bit(m, i)) v[o++] = d.leaf_values[512 * f + i];
            for (uint64_t k = 0; k < nstat; ++k) v[o++] = bg;
        }
    }
    put_checksum(b, checksum);
    return b;
}

}  // namespace

// NanoGrid<float> -> exchange layout (the direction of
// nanovdb::tools::nanoToOpenVDB, nanovdb/tools/NanoToOpenVDB.h): the tree is
// walked through its links -- root table in Coord order, then child masks in
// slot order -- so the result is in tree order whatever the buffer's node
// layout; node origins come from the root keys and the slot indices.  The
// walk reads whole records (headers, root tiles, nodes, leaves) through
// `read`, so a device buffer is downloaded node by node and its leaves are
// never read on the host when leaf_at is given.
gbls_host_grid* import_float(const ByteReader& read, int64_t size, std::vector<uint64_t>* leaf_at) {
    auto need = [&](size_t at, size_t n) {
        if (at > size_t(size) || n > size_t(size) - at) fail(GBLS_ERR_RUNTIME, "truncated NanoVDB buffer");
    };
    std::vector<uint8_t> rec;
    auto fetch = [&](size_t at, size_t n) -> const uint8_t* {
        need(at, n);
        rec.resize(n + 1);
        if (n) read(at, n, rec.data());
        return rec.data();
    };
    auto get = [](const uint8_t* p, size_t at, auto v) {
        std::memcpy(&v, p + at, sizeof(v));
        return v;
    };
    const uint8_t* b = fetch(0, kGridBytes + kTreeBytes);
    const uint64_t magic = get(b, 0, uint64_t());
    if (magic != kMagicGrid && magic != 0x304244566f6e614eULL) fail(GBLS_ERR_RUNTIME, "not a NanoVDB grid");
    if ((get(b, 16, uint32_t()) >> 21) != 32) fail(GBLS_ERR_UNSUPPORTED, "NanoVDB major version other than 32");
    if (get(b, 636, uint32_t()) != 1) fail(GBLS_ERR_UNSUPPORTED, "not a NanoGrid<float>");
    double mat[9], vec[3];
    for (int k = 0; k < 9; ++k) mat[k] = get(b, 296 + 88 + 8 * k, double());
    for (int k = 0; k < 3; ++k) vec[k] = get(b, 296 + 232 + 8 * k, double());
    if (mat[1] != 0 || mat[2] != 0 || mat[3] != 0 || mat[5] != 0 || mat[6] != 0 || mat[7] != 0)
        fail(GBLS_ERR_UNSUPPORTED, "rotated or sheared NanoVDB map");
    if (!(mat[0] == mat[4] && mat[4] == mat[8]) || !(mat[0] > 0))
        fail(GBLS_ERR_RUNTIME, "The transform must have uniform scale for the LevelSetTracker to function");
    const size_t root_at = kGridBytes + size_t(get(b, kGridBytes + 24, int64_t()));
    auto* g = new gbls_host_grid;
    try {
        g->voxel_size = mat[0];
        for (int k = 0; k < 3; ++k) g->translation[k] = vec[k];
        g->map_type = (vec[0] == 0 && vec[1] == 0 && vec[2] == 0) ? GBLS_MAP_UNIFORM_SCALE
                                                                 : GBLS_MAP_UNIFORM_SCALE_TRANSLATE;
        b = fetch(root_at, kRootBytes);
        const uint32_t table = get(b, 24, uint32_t());
        g->background = get(b, 28, float());
        b = fetch(root_at + kRootBytes, size_t(table) * kTileBytes);
        struct Entry {
            int32_t o[3];
            int64_t child;
            float value;
        };
        std::vector<Entry> entries(table);
        for (uint32_t t = 0; t < table; ++t) {
            const size_t at = kTileBytes * t;
            const uint64_t key = get(b, at, uint64_t());
            Entry& e = entries[t];
            e.o[0] = int32_t(uint32_t(((key >> 42) & 0x1FFFFF) << 12));
            e.o[1] = int32_t(uint32_t(((key >> 21) & 0x1FFFFF) << 12));
            e.o[2] = int32_t(uint32_t((key & 0x1FFFFF) << 12));
            e.child = get(b, at + 8, int64_t());
            if (!e.child && get(b, at + 16, uint32_t())) fail(GBLS_ERR_UNSUPPORTED, "active root tile in a level set");
            e.value = get(b, at + 20, float());
        }
        std::sort(entries.begin(), entries.end(), [](const Entry& x, const Entry& y) {
            return std::lexicographical_compare(x.o, x.o + 3, y.o, y.o + 3);
        });
        // one internal node: its tile values, and its children as (address, origin) in slot order
        struct Child {
            size_t at;
            int32_t o[3];
        };
        auto node = [&](size_t at, int log2, size_t bytes, size_t table_at, const int32_t* origin, int child_shift,
                        std::vector<float>& tiles, std::vector<Child>& children) {
            const uint8_t* nb = fetch(at, bytes);
            const int nvals = 1 << (3 * log2), dim = 1 << log2;
            const uint8_t* vmask = nb + 32;
            const uint8_t* cmask = vmask + nvals / 8;
            const size_t base = tiles.size();
            tiles.resize(base + size_t(nvals), 0.0f);
            for (int n = 0; n < nvals; ++n) {
                if ((vmask[n >> 3] >> (n & 7)) & 1) fail(GBLS_ERR_UNSUPPORTED, "active tile in a level set");
                if ((cmask[n >> 3] >> (n & 7)) & 1) {
                    Child c;
                    c.at = size_t(int64_t(at) + get(nb, table_at + 8 * size_t(n), int64_t()));
                    c.o[0] = origin[0] + (((n >> (2 * log2)) & (dim - 1)) << child_shift);
                    c.o[1] = origin[1] + (((n >> log2) & (dim - 1)) << child_shift);
                    c.o[2] = origin[2] + ((n & (dim - 1)) << child_shift);
                    children.push_back(c);
                } else {
                    tiles[base + size_t(n)] = get(nb, table_at + 8 * size_t(n), float());
                }
            }
        };
        for (const Entry& e : entries) {
            if (!e.child) {
                g->root_tile_origins.insert(g->root_tile_origins.end(), e.o, e.o + 3);
                g->root_tile_values.push_back(e.value);
                continue;
            }
            g->upper_origins.insert(g->upper_origins.end(), e.o, e.o + 3);
            std::vector<Child> lowers;
            node(size_t(int64_t(root_at) + e.child), 5, kUpperBytes, kUpperTableAt, e.o, 7, g->upper_tiles, lowers);
            for (const Child& lo : lowers) {
                g->lower_origins.insert(g->lower_origins.end(), lo.o, lo.o + 3);
                std::vector<Child> leaves;
                node(lo.at, 4, kLowerBytes, kLowerTableAt, lo.o, 3, g->lower_tiles, leaves);
                for (const Child& lf : leaves) {
                    g->leaf_origins.insert(g->leaf_origins.end(), lf.o, lf.o + 3);
                    if (leaf_at) {
                        need(lf.at, kLeafBytes);
                        leaf_at->push_back(uint64_t(lf.at));
                        continue;
                    }
                    const uint8_t* lb = fetch(lf.at, kLeafBytes);
                    const size_t f = g->leaf_origins.size() / 3 - 1;
                    g->leaf_masks.resize(8 * (f + 1));
                    std::memcpy(g->leaf_masks.data() + 8 * f, lb + 16, 64);
                    g->leaf_values.resize(512 * (f + 1));
                    std::memcpy(g->leaf_values.data() + 512 * f, lb + 96, 2048);
                }
            }
        }
        return g;
    } catch (...) {
        delete g;
        throw;
    }
}

namespace {
}  // namespace
}  // namespace gbls_nano

using namespace gbls_nano;

extern "C" {

int gbls_nanovdb_export(const gbls_grid_desc* desc, const char* name, int32_t stats_mode, int32_t checksum_mode,
                        uint8_t* out, int64_t out_capacity, int64_t* size) {
    try {
        if (!desc || !size) fail(GBLS_ERR_INVALID_ARGUMENT, "null argument");
        std::vector<uint8_t> b = build(*desc, name ? name : "", stats_mode, checksum_mode);
        *size = int64_t(b.size());
        if (out) {
            if (out_capacity < *size) fail(GBLS_ERR_INVALID_ARGUMENT, "output buffer too small");
            std::memcpy(out, b.data(), b.size());
        }
        return GBLS_OK;
    } catch (const ExportError& e) {
        gbls_host::set_error(e.msg);
        return e.code;
    } catch (const std::bad_alloc&) {
        gbls_host::set_error("out of host memory");
        return GBLS_ERR_OUT_OF_MEMORY;
    }
}

int gbls_nanovdb_export_index(const gbls_grid_desc* desc, const char* name, int32_t channels, int32_t include_stats,
                              int32_t include_tiles, int32_t checksum_mode, uint8_t* out, int64_t out_capacity,
                              int64_t* size) {
    try {
        if (!desc || !size) fail(GBLS_ERR_INVALID_ARGUMENT, "null argument");
        std::vector<uint8_t> b = build_index(*desc, name ? name : "", channels, include_stats != 0, include_tiles != 0,
                                             checksum_mode);
        *size = int64_t(b.size());
        if (out) {
            if (out_capacity < *size) fail(GBLS_ERR_INVALID_ARGUMENT, "output buffer too small");
            std::memcpy(out, b.data(), b.size());
        }
        return GBLS_OK;
    } catch (const ExportError& e) {
        gbls_host::set_error(e.msg);
        return e.code;
    } catch (const std::bad_alloc&) {
        gbls_host::set_error("out of host memory");
        return GBLS_ERR_OUT_OF_MEMORY;
    }
}

int gbls_nanovdb_import(const uint8_t* buffer, int64_t size, gbls_host_grid** out) {
    try {
        if (!buffer || !out || size < 0) fail(GBLS_ERR_INVALID_ARGUMENT, "null argument");
        const ByteReader read = [buffer](size_t at, size_t n, uint8_t* dst) { std::memcpy(dst, buffer + at, n); };
        *out = import_float(read, size, nullptr);
        return GBLS_OK;
    } catch (const ExportError& e) {
        gbls_host::set_error(e.msg);
        return e.code;
    } catch (const std::bad_alloc&) {
        gbls_host::set_error("out of host memory");
        return GBLS_ERR_OUT_OF_MEMORY;
    }
}

}  // extern "C"

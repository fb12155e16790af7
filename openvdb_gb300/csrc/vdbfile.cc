// .vdb files of level-set FloatGrids, on the host.
//
// gbls_vdb_write stands in for io::File::write (io/File.h:130) and
// gbls_vdb_read for io::File::open + readGrid (io/File.h:107) for the grids
// the device path holds: Tree_float_5_4_3 narrow-band level sets with a
// uniform-scale / translate transform and inactive tiles.  The bytes follow
// OpenVDB's file format 225:
//   header                 io/Archive.cc:940-1080 (magic, format and library
//                          versions, grid-offsets flag, 36-character UUID)
//   file metadata, grids   io/Archive.cc:1261-1450 (grid count, then per grid
//                          io/GridDescriptor.cc:47-100 name / type / instance
//                          parent and three stream offsets, the grid's
//                          compression flags, MetaMap.cc:52-108 metadata,
//                          math/Transform.cc:67-94 transform, topology, buffers)
//   topology               tree/Tree.h:1144-1158 buffer count,
//                          tree/RootNode.h:2348-2425 background, tiles and
//                          children in Coord order, tree/InternalNode.h:
//                          2393-2460 child mask, value mask, node values,
//                          tree/LeafNode.h:1327-1337 leaf value masks
//   buffers                tree/LeafNode.h:1363-1470 value mask + values
//   node values            io/Compression.h:69-170 (MaskCompress), 465-590
//                          (readCompressedValues), 647-753
//                          (writeCompressedValues): a record-kind byte,
//                          at most two inactive values, an optional selection
//                          mask, then the active values only.
// Data compression is COMPRESS_ACTIVE_MASK alone (what a build without
// Blosc and zlib writes): no Blosc or zlib blocks are written, and files
// that hold them are rejected with GBLS_ERR_UNSUPPORTED.  Files stored with
// half floats (`_HalfFloat` grid types) are read and widened exactly.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <random>
#include <string>
#include <vector>

#include "host_grid.h"

namespace {

constexpr int64_t kMagic = 0x56444220;             // "VDB " (io/Archive.cc: OPENVDB_MAGIC)
constexpr uint32_t kFileVersion = 225;            // OPENVDB_FILE_VERSION (half-float grids)
constexpr uint32_t kNodeMaskCompressionVersion = 222;
constexpr uint32_t kLibraryMajor = 13, kLibraryMinor = 0;
constexpr uint32_t kCompressZip = 0x1, kCompressActiveMask = 0x2, kCompressBlosc = 0x4;
const char* const kTreeType = "Tree_float_5_4_3";
const char* const kHalfSuffix = "_HalfFloat";
const char kNameSeparator = '\x1e';  // io/GridDescriptor.cc: unique-name suffix separator

// Per-node record kinds of the active-mask compression (io/Compression.h:69-77).
enum : int8_t {
    kNoMaskOrInactiveVals = 0,   // inactive values all +background
    kNoMaskAndMinusBg = 1,       // inactive values all -background
    kNoMaskAndOneInactiveVal = 2,
    kMaskAndNoInactiveVals = 3,  // selection mask between -background and +background
    kMaskAndOneInactiveVal = 4,
    kMaskAndTwoInactiveVals = 5,
    kNoMaskAndAllVals = 6
};

struct VdbError {
    int code;
    std::string msg;
};
[[noreturn]] void fail(int code, const std::string& msg) { throw VdbError{code, msg}; }

inline bool bit(const uint64_t* m, int i) { return (m[i >> 6] >> (i & 63)) & 1u; }
inline void set_bit(uint64_t* m, int i) { m[i >> 6] |= uint64_t(1) << (i & 63); }
inline int popcount(const uint64_t* m, int words) {
    int n = 0;
    for (int w = 0; w < words; ++w) n += __builtin_popcountll(m[w]);
    return n;
}

// Same key as the device tree: integer order = tree order.
inline uint64_t tree_key(const int32_t* o) {
    const uint64_t rx = uint64_t((o[0] >> 12) + 256), ry = uint64_t((o[1] >> 12) + 256),
                   rz = uint64_t((o[2] >> 12) + 256);
    const uint64_t ux = (o[0] >> 7) & 31, uy = (o[1] >> 7) & 31, uz = (o[2] >> 7) & 31;
    const uint64_t lx = (o[0] >> 3) & 15, ly = (o[1] >> 3) & 15, lz = (o[2] >> 3) & 15;
    return (((rx << 18) | (ry << 9) | rz) << 27) | (((ux << 10) | (uy << 5) | uz) << 12) |
           ((lx << 8) | (ly << 4) | lz);
}

// ---- byte streams -----------------------------------------------------------

struct Out {
    std::vector<char> b;
    void raw(const void* p, size_t n) {
        const char* c = static_cast<const char*>(p);
        b.insert(b.end(), c, c + n);
    }
    template <class T> void put(const T& v) { raw(&v, sizeof(T)); }
    void str(const std::string& s) {
        put<uint32_t>(uint32_t(s.size()));
        raw(s.data(), s.size());
    }
    size_t pos() const { return b.size(); }
    template <class T> void patch(size_t at, const T& v) { std::memcpy(b.data() + at, &v, sizeof(T)); }
};

struct In {
    const char* p = nullptr;
    size_t n = 0;
    size_t at = 0;
    void need(size_t k) const {
        if (k > n - at) fail(GBLS_ERR_RUNTIME, "truncated VDB file");
    }
    void raw(void* dst, size_t k) {
        need(k);
        std::memcpy(dst, p + at, k);
        at += k;
    }
    template <class T> T get() {
        T v;
        raw(&v, sizeof(T));
        return v;
    }
    std::string str() {
        const uint32_t k = get<uint32_t>();
        need(k);
        std::string s(p + at, k);
        at += k;
        return s;
    }
    void skip(size_t k) {
        need(k);
        at += k;
    }
};

// IEEE binary16 -> binary32 (exact for every input).
inline float half_to_float(uint16_t h) {
    const uint32_t sign = uint32_t(h >> 15) << 31, exp = (h >> 10) & 31, man = h & 1023;
    uint32_t f;
    if (exp == 31) {
        f = sign | 0x7f800000u | (man << 13);
    } else if (exp == 0) {
        const float v = std::ldexp(float(man), -24);
        return sign ? -v : v;
    } else {
        f = sign | ((exp + 112) << 23) | (man << 13);
    }
    float out;
    std::memcpy(&out, &f, 4);
    return out;
}

// ---- node values ------------------------------------------------------------

struct MaskCompress {
    int8_t kind = kNoMaskAndAllVals;
    float inactive[2];
};

// io/Compression.h:79-166: the first (up to three) distinct values at
// inactive, non-child positions, in index order, choose the record kind.
MaskCompress classify(const uint64_t* vmask, const uint64_t* cmask, const float* src, int count, float bg) {
    MaskCompress m;
    m.inactive[0] = m.inactive[1] = bg;
    int unique = 0;
    for (int i = 0; i < count && unique < 3; ++i) {
        if (bit(vmask, i) || (cmask && bit(cmask, i))) continue;
        const float v = src[i];
        const bool seen = (unique > 0 && v == m.inactive[0]) || (unique > 1 && v == m.inactive[1]);
        if (!seen) {
            if (unique < 2) m.inactive[unique] = v;
            ++unique;
        }
    }
    const float nbg = -bg;
    m.kind = kNoMaskOrInactiveVals;
    if (unique == 1) {
        if (!(m.inactive[0] == bg))
            m.kind = (m.inactive[0] == nbg) ? kNoMaskAndMinusBg : kNoMaskAndOneInactiveVal;
    } else if (unique == 2) {
        if (!(m.inactive[0] == bg) && !(m.inactive[1] == bg)) {
            m.kind = kMaskAndTwoInactiveVals;
        } else if (m.inactive[1] == bg) {
            m.kind = (m.inactive[0] == nbg) ? kMaskAndNoInactiveVals : kMaskAndOneInactiveVal;
        } else if (m.inactive[0] == bg) {
            m.kind = (m.inactive[1] == nbg) ? kMaskAndNoInactiveVals : kMaskAndOneInactiveVal;
            std::swap(m.inactive[0], m.inactive[1]);
        }
    } else if (unique > 2) {
        m.kind = kNoMaskAndAllVals;
    }
    return m;
}

// writeCompressedValues with COMPRESS_ACTIVE_MASK and full floats.  `cmask`
// (internal nodes) excludes child slots from the inactive-value census; the
// selection mask, as in the reference, covers every inactive position.
void write_values(Out& o, const float* src, int count, const uint64_t* vmask, const uint64_t* cmask, float bg) {
    const MaskCompress m = classify(vmask, cmask, src, count, bg);
    o.put<int8_t>(m.kind);
    if (m.kind == kNoMaskAndOneInactiveVal || m.kind == kMaskAndOneInactiveVal || m.kind == kMaskAndTwoInactiveVals) {
        o.put<float>(m.inactive[0]);
        if (m.kind == kMaskAndTwoInactiveVals) o.put<float>(m.inactive[1]);
    }
    if (m.kind == kNoMaskAndAllVals) {
        o.raw(src, sizeof(float) * size_t(count));
        return;
    }
    if (m.kind == kMaskAndNoInactiveVals || m.kind == kMaskAndOneInactiveVal || m.kind == kMaskAndTwoInactiveVals) {
        std::vector<uint64_t> sel(static_cast<size_t>(count) / 64, 0);
        for (int i = 0; i < count; ++i)
            if (!bit(vmask, i) && src[i] == m.inactive[1]) set_bit(sel.data(), i);
        o.raw(sel.data(), sel.size() * 8);
    }
    for (int i = 0; i < count; ++i)
        if (bit(vmask, i)) o.put<float>(src[i]);
}

// readCompressedValues (format >= 222).
void read_values(In& in, float* dst, int count, const uint64_t* vmask, float bg, uint32_t compression, bool half) {
    const int8_t kind = in.get<int8_t>();
    if (kind < 0 || kind > kNoMaskAndAllVals) fail(GBLS_ERR_RUNTIME, "corrupt node record in VDB file");
    float inactive1 = bg;
    float inactive0 = (kind == kNoMaskOrInactiveVals) ? bg : -bg;
    if (kind == kNoMaskAndOneInactiveVal || kind == kMaskAndOneInactiveVal || kind == kMaskAndTwoInactiveVals) {
        inactive0 = in.get<float>();
        if (kind == kMaskAndTwoInactiveVals) inactive1 = in.get<float>();
    }
    std::vector<uint64_t> sel(static_cast<size_t>(count) / 64, 0);
    if (kind == kMaskAndNoInactiveVals || kind == kMaskAndOneInactiveVal || kind == kMaskAndTwoInactiveVals)
        in.raw(sel.data(), sel.size() * 8);
    const bool mask_compressed = (compression & kCompressActiveMask) != 0;
    const int n = (mask_compressed && kind != kNoMaskAndAllVals) ? popcount(vmask, count / 64) : count;
    std::vector<float> tmp(static_cast<size_t>(n));
    if (half) {
        std::vector<uint16_t> h(static_cast<size_t>(n));
        in.raw(h.data(), 2 * size_t(n));
        for (int i = 0; i < n; ++i) tmp[i] = half_to_float(h[i]);
    } else {
        in.raw(tmp.data(), 4 * size_t(n));
    }
    if (n == count) {
        std::memcpy(dst, tmp.data(), 4 * size_t(count));
        return;
    }
    for (int i = 0, k = 0; i < count; ++i)
        dst[i] = bit(vmask, i) ? tmp[k++] : (bit(sel.data(), i) ? inactive1 : inactive0);
}

// ---- transforms ---------------------------------------------------------------

// ScaleMap's stored fields (math/Maps.h:665-677, 813-829): scale, voxel size,
// 1/scale, 1/scale^2, 1/(2 scale).
void write_scale_fields(Out& o, double s) {
    const double inv = 1.0 / s;
    const double f[5] = {s, std::abs(s), inv, inv * inv, inv / 2};
    for (double v : f)
        for (int k = 0; k < 3; ++k) o.put<double>(v);
}

void write_transform(Out& o, const gbls_grid_desc& d) {
    if (d.map_type == GBLS_MAP_TRANSLATION) {
        o.str("TranslationMap");
        for (int k = 0; k < 3; ++k) o.put<double>(d.translation[k]);
    } else if (d.map_type == GBLS_MAP_UNIFORM_SCALE) {
        o.str("UniformScaleMap");
        write_scale_fields(o, d.voxel_size);
    } else {
        o.str("UniformScaleTranslateMap");
        for (int k = 0; k < 3; ++k) o.put<double>(d.translation[k]);
        write_scale_fields(o, d.voxel_size);
    }
}

// The map as the C++ drop-in's exportTransform sees it: UniformScaleMap and
// TranslationMap keep their kind, every other uniform linear map becomes
// scale + translate; the voxel size must be uniform.
void read_transform(In& in, gbls_host_grid& g) {
    const std::string type = in.str();
    double t[3] = {0.0, 0.0, 0.0}, f[15];
    auto scale_fields = [&]() {
        in.raw(f, sizeof(f));
        if (!(f[3] == f[4] && f[4] == f[5]))
            fail(GBLS_ERR_RUNTIME, "The transform must have uniform scale for the LevelSetTracker to function");
        g.voxel_size = f[3];
    };
    if (type == "UniformScaleMap" || type == "ScaleMap") {
        scale_fields();
        g.map_type = type == "UniformScaleMap" ? GBLS_MAP_UNIFORM_SCALE : GBLS_MAP_UNIFORM_SCALE_TRANSLATE;
    } else if (type == "UniformScaleTranslateMap" || type == "ScaleTranslateMap") {
        in.raw(t, sizeof(t));
        scale_fields();
        g.map_type = GBLS_MAP_UNIFORM_SCALE_TRANSLATE;
    } else if (type == "TranslationMap") {
        in.raw(t, sizeof(t));
        g.voxel_size = 1.0;
        g.map_type = GBLS_MAP_TRANSLATION;
    } else if (type == "AffineMap") {
        double m[16];  // Mat4d, row-vector convention: translation in the last row
        in.raw(m, sizeof(m));
        const bool diagonal = m[1] == 0 && m[2] == 0 && m[4] == 0 && m[6] == 0 && m[8] == 0 && m[9] == 0 &&
                              m[3] == 0 && m[7] == 0 && m[11] == 0 && m[15] == 1;
        if (!diagonal) fail(GBLS_ERR_UNSUPPORTED, "rotated, sheared or projective AffineMap");
        if (!(m[0] == m[5] && m[5] == m[10]) || !(m[0] > 0))
            fail(GBLS_ERR_RUNTIME, "The transform must have uniform scale for the LevelSetTracker to function");
        g.voxel_size = m[0];
        t[0] = m[12];
        t[1] = m[13];
        t[2] = m[14];
        g.map_type = GBLS_MAP_UNIFORM_SCALE_TRANSLATE;
    } else {
        fail(GBLS_ERR_UNSUPPORTED, "transform map '" + type + "' is not a uniform scale / translate map");
    }
    for (int k = 0; k < 3; ++k) g.translation[k] = t[k];
}

// ---- metadata -------------------------------------------------------------------

void meta_string(Out& o, const char* name, const std::string& v) {
    o.str(name);
    o.str("string");
    o.put<uint32_t>(uint32_t(v.size()));
    o.raw(v.data(), v.size());
}
void meta_vec3i(Out& o, const char* name, const int32_t v[3]) {
    o.str(name);
    o.str("vec3i");
    o.put<uint32_t>(12);
    o.raw(v, 12);
}
void meta_int64(Out& o, const char* name, int64_t v) {
    o.str(name);
    o.str("int64");
    o.put<uint32_t>(8);
    o.put<int64_t>(v);
}

struct GridMeta {
    std::string grid_class, name;
};

GridMeta read_meta(In& in) {
    GridMeta m;
    const uint32_t count = in.get<uint32_t>();
    for (uint32_t i = 0; i < count; ++i) {
        const std::string name = in.str(), type = in.str();
        const uint32_t size = in.get<uint32_t>();
        in.need(size);
        if (type == "string" && (name == "class" || name == "name"))
            (name == "class" ? m.grid_class : m.name).assign(in.p + in.at, size);
        in.at += size;
    }
    return m;
}

// ---- grids ----------------------------------------------------------------------

void check_desc(const gbls_grid_desc& d) {
    if (d.leaf_count < 0 || d.lower_count < 0 || d.upper_count < 0 || d.root_tile_count < 0)
        fail(GBLS_ERR_INVALID_ARGUMENT, "negative count in grid descriptor");
    if ((d.leaf_count && (!d.leaf_origins || !d.leaf_masks || !d.leaf_values)) ||
        (d.lower_count && (!d.lower_origins || !d.lower_tiles)) ||
        (d.upper_count && (!d.upper_origins || !d.upper_tiles)) ||
        (d.root_tile_count && (!d.root_tile_origins || !d.root_tile_values)))
        fail(GBLS_ERR_INVALID_ARGUMENT, "null array in grid descriptor");
    if (!(d.voxel_size > 0.0) && d.map_type != GBLS_MAP_TRANSLATION)
        fail(GBLS_ERR_RUNTIME, "voxel size must be positive");
    if (d.map_type < GBLS_MAP_UNIFORM_SCALE || d.map_type > GBLS_MAP_TRANSLATION)
        fail(GBLS_ERR_INVALID_ARGUMENT, "unknown map type");
}

// One grid record (io/Archive.cc:1366-1450) for descriptor `d`.
void write_grid(Out& o, const gbls_grid_desc& d, const std::string& unique_name, const std::string& grid_name) {
    check_desc(d);
    const float bg = d.background;
    o.str(unique_name);
    o.str(kTreeType);
    o.str("");
    const size_t offsets_at = o.pos();
    for (int k = 0; k < 3; ++k) o.put<int64_t>(0);
    const int64_t grid_pos = int64_t(o.pos());
    o.put<uint32_t>(kCompressActiveMask);

    // metadata, in name order (MetaMap is a std::map)
    int64_t active = 0;
    int32_t bmin[3] = {INT_MAX, INT_MAX, INT_MAX}, bmax[3] = {INT_MIN, INT_MIN, INT_MIN};
    for (int64_t f = 0; f < d.leaf_count; ++f) {
        const uint64_t* m = d.leaf_masks + 8 * f;
        const int32_t* lo = d.leaf_origins + 3 * f;
        for (int i = 0; i < 512; ++i) {
            if (!bit(m, i)) continue;
            ++active;
            const int32_t c[3] = {lo[0] + (i >> 6), lo[1] + ((i >> 3) & 7), lo[2] + (i & 7)};
            for (int k = 0; k < 3; ++k) {
                bmin[k] = std::min(bmin[k], c[k]);
                bmax[k] = std::max(bmax[k], c[k]);
            }
        }
    }
    o.put<uint32_t>(6);
    meta_string(o, "class", "level set");
    meta_vec3i(o, "file_bbox_max", bmax);
    meta_vec3i(o, "file_bbox_min", bmin);
    meta_string(o, "file_compression", "active values");
    meta_int64(o, "file_voxel_count", active);
    meta_string(o, "name", grid_name);
    write_transform(o, d);

    // topology: the root's tiles in Coord order, then its children
    o.put<int32_t>(1);
    o.put<float>(bg);
    std::vector<int64_t> tiles(static_cast<size_t>(d.root_tile_count));
    for (int64_t i = 0; i < d.root_tile_count; ++i) tiles[size_t(i)] = i;
    std::sort(tiles.begin(), tiles.end(), [&](int64_t a, int64_t b) {
        const int32_t *p = d.root_tile_origins + 3 * a, *q = d.root_tile_origins + 3 * b;
        return std::lexicographical_compare(p, p + 3, q, q + 3);
    });
    o.put<uint32_t>(uint32_t(d.root_tile_count));
    o.put<uint32_t>(uint32_t(d.upper_count));
    for (int64_t i : tiles) {
        o.raw(d.root_tile_origins + 3 * i, 12);
        o.put<float>(d.root_tile_values[i]);
        o.put<uint8_t>(0);
    }
    uint64_t prev_upper = 0, prev_lower = 0, prev_leaf = 0;
    auto in_order = [&](uint64_t& prev, const int32_t* origin, int64_t idx) {
        const uint64_t k = tree_key(origin);
        if (idx > 0 && k <= prev) fail(GBLS_ERR_INVALID_ARGUMENT, "grid descriptor is not in tree order");
        prev = k;
    };
    std::vector<uint64_t> ucm(512), lcm(64), zeros(512, 0);
    std::vector<float> vals(32768);
    int64_t li = 0, fi = 0;
    for (int64_t u = 0; u < d.upper_count; ++u) {
        const int32_t* uo = d.upper_origins + 3 * u;
        if ((uo[0] & 4095) || (uo[1] & 4095) || (uo[2] & 4095))
            fail(GBLS_ERR_INVALID_ARGUMENT, "upper node origin not aligned to 4096");
        in_order(prev_upper, uo, u);
        o.raw(uo, 12);
        const int64_t l0 = li;
        std::fill(ucm.begin(), ucm.end(), 0);
        for (; li < d.lower_count; ++li) {
            const int32_t* lo = d.lower_origins + 3 * li;
            if ((lo[0] & ~4095) != uo[0] || (lo[1] & ~4095) != uo[1] || (lo[2] & ~4095) != uo[2]) break;
            if ((lo[0] & 127) || (lo[1] & 127) || (lo[2] & 127))
                fail(GBLS_ERR_INVALID_ARGUMENT, "lower node origin not aligned to 128");
            in_order(prev_lower, lo, li);
            set_bit(ucm.data(), (((lo[0] & 4095) >> 7) << 10) | (((lo[1] & 4095) >> 7) << 5) | ((lo[2] & 4095) >> 7));
        }
        o.raw(ucm.data(), 4096);
        o.raw(zeros.data(), 4096);
        std::memcpy(vals.data(), d.upper_tiles + 32768 * u, 4 * 32768);
        for (int n = 0; n < 32768; ++n)
            if (bit(ucm.data(), n)) vals[n] = 0.0f;
        write_values(o, vals.data(), 32768, zeros.data(), ucm.data(), bg);
        for (int64_t l = l0; l < li; ++l) {
            const int32_t* lo = d.lower_origins + 3 * l;
            const int64_t f0 = fi;
            std::fill(lcm.begin(), lcm.end(), 0);
            for (; fi < d.leaf_count; ++fi) {
                const int32_t* fo = d.leaf_origins + 3 * fi;
                if ((fo[0] & ~127) != lo[0] || (fo[1] & ~127) != lo[1] || (fo[2] & ~127) != lo[2]) break;
                if ((fo[0] & 7) || (fo[1] & 7) || (fo[2] & 7))
                    fail(GBLS_ERR_INVALID_ARGUMENT, "leaf origin not aligned to 8");
                in_order(prev_leaf, fo, fi);
                set_bit(lcm.data(), (((fo[0] & 127) >> 3) << 8) | (((fo[1] & 127) >> 3) << 4) | ((fo[2] & 127) >> 3));
            }
            o.raw(lcm.data(), 512);
            o.raw(zeros.data(), 512);
            std::memcpy(vals.data(), d.lower_tiles + 4096 * l, 4 * 4096);
            for (int n = 0; n < 4096; ++n)
                if (bit(lcm.data(), n)) vals[n] = 0.0f;
            write_values(o, vals.data(), 4096, zeros.data(), lcm.data(), bg);
            for (int64_t f = f0; f < fi; ++f) o.raw(d.leaf_masks + 8 * f, 64);
        }
    }
    if (li != d.lower_count || fi != d.leaf_count)
        fail(GBLS_ERR_INVALID_ARGUMENT, "grid descriptor is not in tree order (orphan lower node or leaf)");
    const int64_t block_pos = int64_t(o.pos());
    for (int64_t f = 0; f < d.leaf_count; ++f) {
        o.raw(d.leaf_masks + 8 * f, 64);
        write_values(o, d.leaf_values + 512 * f, 512, d.leaf_masks + 8 * f, nullptr, bg);
    }
    const int64_t end_pos = int64_t(o.pos());
    o.patch<int64_t>(offsets_at, grid_pos);
    o.patch<int64_t>(offsets_at + 8, block_pos);
    o.patch<int64_t>(offsets_at + 16, end_pos);
}

// Topology and buffers of one Tree_float_5_4_3 (the stream is positioned
// after the transform).
void read_tree(In& in, gbls_host_grid& g, uint32_t compression, bool half) {
    if (in.get<int32_t>() != 1) fail(GBLS_ERR_UNSUPPORTED, "multi-buffer trees are not supported");
    const float bg = in.get<float>();
    g.background = bg;
    const uint32_t ntiles = in.get<uint32_t>(), nchildren = in.get<uint32_t>();
    for (uint32_t i = 0; i < ntiles; ++i) {
        int32_t o[3];
        in.raw(o, 12);
        const float v = in.get<float>();
        if (in.get<uint8_t>() != 0) fail(GBLS_ERR_UNSUPPORTED, "active root tile in a level set");
        g.root_tile_origins.insert(g.root_tile_origins.end(), o, o + 3);
        g.root_tile_values.push_back(v);
    }
    std::vector<uint64_t> ucm(512), uvm(512), lcm(64), lvm(64);
    uint64_t prev = 0;
    for (uint32_t c = 0; c < nchildren; ++c) {
        int32_t uo[3];
        in.raw(uo, 12);
        const uint64_t k = tree_key(uo);
        if ((uo[0] & 4095) || (uo[1] & 4095) || (uo[2] & 4095) || (c > 0 && k <= prev))
            fail(GBLS_ERR_RUNTIME, "corrupt root node in VDB file");
        prev = k;
        in.raw(ucm.data(), 4096);
        in.raw(uvm.data(), 4096);
        if (popcount(uvm.data(), 512)) fail(GBLS_ERR_UNSUPPORTED, "active tile in a level set");
        g.upper_origins.insert(g.upper_origins.end(), uo, uo + 3);
        const size_t ub = g.upper_tiles.size();
        g.upper_tiles.resize(ub + 32768);
        float* ut = g.upper_tiles.data() + ub;
        read_values(in, ut, 32768, uvm.data(), bg, compression, half);
        for (int n = 0; n < 32768; ++n) {
            if (!bit(ucm.data(), n)) continue;
            ut[n] = 0.0f;
        }
        for (int n = 0; n < 32768; ++n) {
            if (!bit(ucm.data(), n)) continue;
            const int32_t lo[3] = {uo[0] + ((n >> 10) & 31) * 128, uo[1] + ((n >> 5) & 31) * 128,
                                   uo[2] + (n & 31) * 128};
            in.raw(lcm.data(), 512);
            in.raw(lvm.data(), 512);
            if (popcount(lvm.data(), 64)) fail(GBLS_ERR_UNSUPPORTED, "active tile in a level set");
            g.lower_origins.insert(g.lower_origins.end(), lo, lo + 3);
            const size_t lb = g.lower_tiles.size();
            g.lower_tiles.resize(lb + 4096);
            float* lt = g.lower_tiles.data() + lb;
            read_values(in, lt, 4096, lvm.data(), bg, compression, half);
            for (int m = 0; m < 4096; ++m) {
                if (!bit(lcm.data(), m)) continue;
                lt[m] = 0.0f;
                const int32_t fo[3] = {lo[0] + ((m >> 8) & 15) * 8, lo[1] + ((m >> 4) & 15) * 8, lo[2] + (m & 15) * 8};
                g.leaf_origins.insert(g.leaf_origins.end(), fo, fo + 3);
                const size_t mb = g.leaf_masks.size();
                g.leaf_masks.resize(mb + 8);
                in.raw(g.leaf_masks.data() + mb, 64);
            }
        }
    }
    // buffers: each leaf repeats its value mask (skipped, as a seekable
    // io::File read does) before its values
    const size_t nleaf = g.leaf_origins.size() / 3;
    g.leaf_values.resize(nleaf * 512);
    for (size_t f = 0; f < nleaf; ++f) {
        in.skip(64);
        read_values(in, g.leaf_values.data() + 512 * f, 512, g.leaf_masks.data() + 8 * f, bg, compression, half);
    }
}

struct FileHeader {
    uint32_t version = 0;
    bool has_offsets = false;
    int32_t grid_count = 0;
};

FileHeader read_header(In& in) {
    FileHeader h;
    if (in.n < 8 || in.get<int64_t>() != kMagic) fail(GBLS_ERR_RUNTIME, "not a VDB file");
    h.version = in.get<uint32_t>();
    if (h.version < kNodeMaskCompressionVersion)
        fail(GBLS_ERR_UNSUPPORTED, "VDB file format " + std::to_string(h.version) + " predates node-mask compression (222)");
    in.get<uint32_t>();  // library major
    in.get<uint32_t>();  // library minor
    h.has_offsets = in.get<char>() != 0;
    in.skip(36);         // UUID
    read_meta(in);       // file-level metadata
    h.grid_count = in.get<int32_t>();
    if (h.grid_count < 0) fail(GBLS_ERR_RUNTIME, "corrupt grid count in VDB file");
    return h;
}

struct GridRecord {
    std::string unique_name, grid_name, type, parent, grid_class;
    bool half = false;
};

inline std::string strip_suffix(const std::string& s) {
    const size_t i = s.find(kNameSeparator);
    return i == std::string::npos ? s : s.substr(0, i);
}

// Walks the grid records; `visit(record, in)` is called with the stream
// positioned after the record's offsets and returns true to stop (having
// consumed the grid), false to have the grid skipped.
template <class Visit>
void walk_grids(In& in, const FileHeader& h, Visit&& visit) {
    for (int32_t i = 0; i < h.grid_count; ++i) {
        GridRecord r;
        r.unique_name = in.str();
        r.grid_name = strip_suffix(r.unique_name);
        r.type = in.str();
        const size_t hl = std::strlen(kHalfSuffix);
        if (r.type.size() > hl && r.type.compare(r.type.size() - hl, hl, kHalfSuffix) == 0) {
            r.half = true;
            r.type.resize(r.type.size() - hl);
        }
        r.parent = in.str();
        in.get<int64_t>();
        in.get<int64_t>();
        const int64_t end_pos = in.get<int64_t>();
        const size_t body = in.at;
        if (visit(r, in, i)) return;
        if (h.has_offsets && end_pos > 0) {
            if (uint64_t(end_pos) > in.n || size_t(end_pos) < body) fail(GBLS_ERR_RUNTIME, "corrupt grid offsets in VDB file");
            in.at = size_t(end_pos);
        } else {
            fail(GBLS_ERR_UNSUPPORTED, "skipping a grid needs the grid offsets of a seekable VDB file");
        }
    }
}

std::vector<char> read_file(const char* path) {
    std::FILE* f = std::fopen(path, "rb");
    if (!f) fail(GBLS_ERR_RUNTIME, std::string("could not open file \"") + path + "\" for reading");
    std::vector<char> buf;
    char chunk[1 << 16];
    size_t k;
    while ((k = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + k);
    const bool err = std::ferror(f) != 0;
    std::fclose(f);
    if (err) fail(GBLS_ERR_RUNTIME, std::string("read error on \"") + path + "\"");
    return buf;
}

template <class F>
int guarded(F&& f) {
    try {
        f();
        return GBLS_OK;
    } catch (const VdbError& e) {
        gbls_host::set_error(e.msg);
        return e.code;
    } catch (const std::bad_alloc&) {
        gbls_host::set_error("out of host memory");
        return GBLS_ERR_OUT_OF_MEMORY;
    } catch (const std::exception& e) {
        gbls_host::set_error(e.what());
        return GBLS_ERR_RUNTIME;
    }
}

void copy_out(const std::string& s, char* dst, int64_t cap) {
    if (!dst || cap <= 0) return;
    const size_t n = std::min(s.size(), size_t(cap - 1));
    std::memcpy(dst, s.data(), n);
    dst[n] = 0;
}

}  // namespace

extern "C" {

int gbls_vdb_write(const char* path, int32_t count, const gbls_grid_desc* grids, const char* const* names) {
    return guarded([&] {
        if (!path || count < 0 || (count > 0 && !grids)) fail(GBLS_ERR_INVALID_ARGUMENT, "null argument");
        Out o;
        o.put<int64_t>(kMagic);
        o.put<uint32_t>(kFileVersion);
        o.put<uint32_t>(kLibraryMajor);
        o.put<uint32_t>(kLibraryMinor);
        o.put<char>(1);  // seekable: grid offsets are filled in
        std::random_device rd;
        std::string uuid;
        for (int i = 0; i < 32; ++i) {
            if (i == 8 || i == 12 || i == 16 || i == 20) uuid.push_back('-');
            uuid.push_back("0123456789ABCDEF"[rd() & 15]);
        }
        o.raw(uuid.data(), 36);
        o.put<uint32_t>(0);  // no file-level metadata
        o.put<int32_t>(count);
        // unique names as io::Archive::write makes them (io/Archive.cc:1296-1330)
        std::vector<std::string> base(static_cast<size_t>(count));
        std::vector<std::string> unique;
        for (int32_t i = 0; i < count; ++i) base[size_t(i)] = (names && names[i]) ? names[i] : "";
        for (int32_t i = 0; i < count; ++i) {
            const std::string& b = base[size_t(i)];
            std::string name = b;
            if (name.empty() || std::count(base.begin(), base.end(), b) > 1)
                name = b + kNameSeparator + "0";
            for (int n = 1; std::find(unique.begin(), unique.end(), name) != unique.end(); ++n)
                name = b + kNameSeparator + std::to_string(n);
            unique.push_back(name);
            write_grid(o, grids[i], name, b);
        }
        std::FILE* f = std::fopen(path, "wb");
        if (!f) fail(GBLS_ERR_RUNTIME, std::string("could not open file \"") + path + "\" for writing");
        const size_t w = std::fwrite(o.b.data(), 1, o.b.size(), f);
        const int rc = std::fclose(f);
        if (w != o.b.size() || rc != 0) fail(GBLS_ERR_RUNTIME, std::string("write error on \"") + path + "\"");
    });
}

int gbls_vdb_grid_count(const char* path, int32_t* count) {
    return guarded([&] {
        if (!path || !count) fail(GBLS_ERR_INVALID_ARGUMENT, "null argument");
        const std::vector<char> buf = read_file(path);
        In in{buf.data(), buf.size()};
        *count = read_header(in).grid_count;
    });
}

int gbls_vdb_grid_info(const char* path, int32_t index, char* name, int64_t name_cap, char* grid_type,
                       int64_t type_cap, char* grid_class, int64_t class_cap) {
    return guarded([&] {
        if (!path) fail(GBLS_ERR_INVALID_ARGUMENT, "null argument");
        const std::vector<char> buf = read_file(path);
        In in{buf.data(), buf.size()};
        const FileHeader h = read_header(in);
        if (index < 0 || index >= h.grid_count) fail(GBLS_ERR_INVALID_ARGUMENT, "grid index out of range");
        walk_grids(in, h, [&](GridRecord& r, In& s, int32_t i) {
            if (i != index) return false;
            std::string cls;
            if (r.parent.empty()) {
                const uint32_t c = s.get<uint32_t>();
                (void)c;
                cls = read_meta(s).grid_class;
            }
            copy_out(r.unique_name, name, name_cap);
            copy_out(r.type + (r.half ? kHalfSuffix : ""), grid_type, type_cap);
            copy_out(cls, grid_class, class_cap);
            return true;
        });
    });
}

int gbls_vdb_read(const char* path, const char* name, int32_t index, gbls_host_grid** out) {
    return guarded([&] {
        if (!path || !out) fail(GBLS_ERR_INVALID_ARGUMENT, "null argument");
        *out = nullptr;
        const std::vector<char> buf = read_file(path);
        In in{buf.data(), buf.size()};
        const FileHeader h = read_header(in);
        gbls_host_grid* g = nullptr;
        // io::File::readGrid(name): the unique name first, then the grid name
        int32_t want = -1;
        if (name) {
            In scan = in;
            int32_t by_grid_name = -1;
            walk_grids(scan, h, [&](GridRecord& r, In&, int32_t i) {
                if (r.unique_name == name) {
                    want = i;
                    return true;
                }
                if (by_grid_name < 0 && r.grid_name == name) by_grid_name = i;
                return false;
            });
            if (want < 0) want = by_grid_name;
            if (want < 0) fail(GBLS_ERR_INVALID_ARGUMENT, std::string("no grid named \"") + name + "\"");
        } else {
            if (index < 0 || index >= h.grid_count) fail(GBLS_ERR_INVALID_ARGUMENT, "grid index out of range");
            want = index;
        }
        walk_grids(in, h, [&](GridRecord& r, In& s, int32_t i) {
            if (i != want) return false;
            if (!r.parent.empty())
                fail(GBLS_ERR_UNSUPPORTED, "grid \"" + r.unique_name + "\" is an instance of another grid's tree");
            if (r.type != kTreeType)
                fail(GBLS_ERR_UNSUPPORTED, "grid type " + r.type + ": the device path holds " + kTreeType + " level sets");
            const uint32_t compression = s.get<uint32_t>();
            if (compression & (kCompressBlosc | kCompressZip))
                fail(GBLS_ERR_UNSUPPORTED, "Blosc/zlib-compressed grid data (this library reads active-mask compression only)");
            read_meta(s);
            auto* hg = new gbls_host_grid;
            try {
                read_transform(s, *hg);
                read_tree(s, *hg, compression, r.half);
            } catch (...) {
                delete hg;
                throw;
            }
            g = hg;
            return true;
        });
        *out = g;
    });
}

}  // extern "C"

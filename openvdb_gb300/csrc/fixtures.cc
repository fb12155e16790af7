// Host construction of narrow-band level sets in the gbls_grid_desc format.
//
// gbls_host_sphere follows tools::createLevelSetSphere
// (tools/LevelSetSphere.h:127-199, 219-230): createLevelSet's background
// (Grid.h:1772-1783), the float distance rasterisation with leapfrogging in
// k over i in [imin, imax), then tools::signedFloodFill
// (tools/SignedFloodFill.h:82-215) bottom-up over leaves, lower nodes, upper
// nodes and the root.  Built with -ffp-contract=off so its float arithmetic
// matches the reference on every host.
//
// gbls_host_union_of_spheres rasterises the union directly: a voxel inside
// any sphere's band takes the minimum of all sphere distances (same float
// formula), is active when that minimum lies inside the band, and the result
// is signed-flood-filled the same way.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "host_grid.h"

namespace {

thread_local std::string g_fix_error;

// Same key as the device tree: integer order = tree order.
inline uint64_t key_of(int32_t x, int32_t y, int32_t z) {
    const uint64_t rx = uint64_t((x >> 12) + 256), ry = uint64_t((y >> 12) + 256), rz = uint64_t((z >> 12) + 256);
    const uint64_t ux = (x >> 7) & 31, uy = (y >> 7) & 31, uz = (z >> 7) & 31;
    const uint64_t lx = (x >> 3) & 15, ly = (y >> 3) & 15, lz = (z >> 3) & 15;
    return (((rx << 18) | (ry << 9) | rz) << 27) | (((ux << 10) | (uy << 5) | uz) << 12) | ((lx << 8) | (ly << 4) | lz);
}
inline void origin_of(uint64_t k, int32_t& x, int32_t& y, int32_t& z) {
    x = (int32_t((k >> 45) & 511) - 256) * 4096 + int32_t((k >> 22) & 31) * 128 + int32_t((k >> 8) & 15) * 8;
    y = (int32_t((k >> 36) & 511) - 256) * 4096 + int32_t((k >> 17) & 31) * 128 + int32_t((k >> 4) & 15) * 8;
    z = (int32_t((k >> 27) & 511) - 256) * 4096 + int32_t((k >> 12) & 31) * 128 + int32_t(k & 15) * 8;
}

struct Leaf {
    uint64_t mask[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    float v[512];
};

using LeafMap = std::unordered_map<uint64_t, Leaf>;

void set_voxel(LeafMap& m, int32_t i, int32_t j, int32_t k, float val, float bg) {
    const uint64_t key = key_of(i & ~7, j & ~7, k & ~7);
    auto it = m.find(key);
    if (it == m.end()) {
        Leaf L;
        std::fill(L.v, L.v + 512, bg);
        it = m.emplace(key, L).first;
    }
    const int n = ((i & 7) << 6) | ((j & 7) << 3) | (k & 7);
    it->second.v[n] = val;
    it->second.mask[n >> 6] |= uint64_t(1) << (n & 63);
}

inline float pow2(float x) { return x * x; }

struct Sphere {
    float r0, cx, cy, cz;
};

// Distance in voxel units exactly as rasterSphere computes it.
inline float sphere_dist(const Sphere& s, int32_t i, int32_t j, int32_t k) {
    const float x2 = pow2(float(i) - s.cx);
    const float x2y2 = pow2(float(j) - s.cy) + x2;
    return std::sqrt(x2y2 + pow2(float(k) - s.cz)) - s.r0;
}

// Enumerate the band voxels of one sphere as rasterSphere does (i < imax).
template <class F>
void sphere_band(const Sphere& s, float w, int32_t ilo, int32_t ihi, F&& emit) {
    const float rmax = s.r0 + w;
    const int jmin = int(std::floor(s.cy - rmax)), jmax = int(std::ceil(s.cy + rmax));
    const int kmin = int(std::floor(s.cz - rmax)), kmax = int(std::ceil(s.cz + rmax));
    for (int32_t i = ilo; i < ihi; ++i) {
        const float x2 = pow2(float(i) - s.cx);
        for (int32_t j = jmin; j <= jmax; ++j) {
            const float x2y2 = pow2(float(j) - s.cy) + x2;
            int m = 1;
            for (int32_t k = kmin; k <= kmax; k += m) {
                m = 1;
                const float v = std::sqrt(x2y2 + pow2(float(k) - s.cz)) - s.r0;
                const float d = std::fabs(v);
                if (d < w) emit(i, j, k, v);
                else m += int(std::floor(d - w));
            }
        }
    }
}

// ---- signed flood fill over an explicit node hierarchy -------------------
struct Tree {
    float bg;
    std::map<uint64_t, Leaf> leaves;                  // by key (tree order)
    std::map<uint64_t, std::vector<float>> lowers;    // lower key -> 4096 tiles
    std::map<uint64_t, std::vector<float>> uppers;    // upper key -> 32768 tiles
    std::map<uint64_t, float> root_tiles;             // upper key -> value
};

void build_nodes(Tree& t) {
    for (auto& kv : t.leaves) {
        const uint64_t lk = kv.first >> 12, uk = kv.first >> 27;
        if (!t.lowers.count(lk)) t.lowers.emplace(lk, std::vector<float>(4096, t.bg));
        if (!t.uppers.count(uk)) t.uppers.emplace(uk, std::vector<float>(32768, t.bg));
    }
}

void flood_leaf(Leaf& L, float inside, float outside) {
    auto on = [&](int n) { return (L.mask[n >> 6] >> (n & 63)) & 1; };
    int first = -1;
    for (int n = 0; n < 512; ++n)
        if (on(n)) { first = n; break; }
    if (first >= 0) {
        bool xIn = L.v[first] < 0, yIn = xIn, zIn = xIn;
        for (int x = 0; x < 8; ++x) {
            const int x00 = x << 6;
            if (on(x00)) xIn = L.v[x00] < 0;
            yIn = xIn;
            for (int y = 0; y < 8; ++y) {
                const int xy0 = x00 + (y << 3);
                if (on(xy0)) yIn = L.v[xy0] < 0;
                zIn = yIn;
                for (int z = 0; z < 8; ++z) {
                    const int xyz = xy0 + z;
                    if (on(xyz)) zIn = L.v[xyz] < 0;
                    else L.v[xyz] = zIn ? inside : outside;
                }
            }
        }
    } else {
        const float f = L.v[0] < 0 ? inside : outside;
        std::fill(L.v, L.v + 512, f);
    }
}

// Internal node flood fill with child first/last value callbacks.
template <class HasChild, class First, class Last>
void flood_internal(std::vector<float>& table, int log2dim, HasChild has, First firstv, Last lastv,
                    float inside, float outside) {
    const int dim = 1 << log2dim, nv = 1 << (3 * log2dim);
    int first = -1;
    for (int n = 0; n < nv; ++n)
        if (has(n)) { first = n; break; }
    if (first >= 0) {
        bool xIn = firstv(first) < 0, yIn = xIn, zIn = xIn;
        for (int x = 0; x < dim; ++x) {
            const int x00 = x << (2 * log2dim);
            if (has(x00)) xIn = lastv(x00) < 0;
            yIn = xIn;
            for (int y = 0; y < dim; ++y) {
                const int xy0 = x00 + (y << log2dim);
                if (has(xy0)) yIn = lastv(xy0) < 0;
                zIn = yIn;
                for (int z = 0; z < dim; ++z) {
                    const int xyz = xy0 + z;
                    if (has(xyz)) zIn = lastv(xyz) < 0;
                    else table[xyz] = zIn ? inside : outside;
                }
            }
        }
    } else {
        const float v = table[0] < 0 ? inside : outside;
        std::fill(table.begin(), table.end(), v);
    }
}

void signed_flood_fill(Tree& t) {
    const float outside = std::fabs(t.bg), inside = -outside;
    for (auto& kv : t.leaves) flood_leaf(kv.second, inside, outside);
    // lower nodes: children are leaves
    auto lower_first = [&](uint64_t lk) -> float {
        auto it = t.leaves.find(lk << 12);
        return it != t.leaves.end() ? it->second.v[0] : t.lowers.at(lk)[0];
    };
    auto lower_last = [&](uint64_t lk) -> float {
        auto it = t.leaves.find((lk << 12) | 4095);
        return it != t.leaves.end() ? it->second.v[511] : t.lowers.at(lk)[4095];
    };
    for (auto& kv : t.lowers) {
        const uint64_t lk = kv.first;
        auto has = [&](int n) { return t.leaves.count((lk << 12) | uint64_t(n)) != 0; };
        auto fv = [&](int n) { return t.leaves.at((lk << 12) | uint64_t(n)).v[0]; };
        auto lv = [&](int n) { return t.leaves.at((lk << 12) | uint64_t(n)).v[511]; };
        flood_internal(kv.second, 4, has, fv, lv, inside, outside);
    }
    for (auto& kv : t.uppers) {
        const uint64_t uk = kv.first;
        auto has = [&](int n) { return t.lowers.count((uk << 15) | uint64_t(n)) != 0; };
        auto fv = [&](int n) { return lower_first((uk << 15) | uint64_t(n)); };
        auto lv = [&](int n) { return lower_last((uk << 15) | uint64_t(n)); };
        flood_internal(kv.second, 5, has, fv, lv, inside, outside);
    }
    // root: z-scanline between consecutive children (map order = key order)
    auto upper_first = [&](uint64_t uk) -> float {
        return t.lowers.count(uk << 15) ? lower_first(uk << 15) : t.uppers.at(uk)[0];
    };
    auto upper_last = [&](uint64_t uk) -> float {
        const uint64_t lk = (uk << 15) | 32767;
        return t.lowers.count(lk) ? lower_last(lk) : t.uppers.at(uk)[32767];
    };
    std::vector<uint64_t> ukeys;
    for (auto& kv : t.uppers) ukeys.push_back(kv.first);
    for (size_t n = 1; n < ukeys.size(); ++n) {
        int32_t ax, ay, az, bx, by, bz;
        origin_of(ukeys[n - 1] << 27, ax, ay, az);
        origin_of(ukeys[n] << 27, bx, by, bz);
        if (bx != ax || by != ay || bz - az == 4096) continue;
        if (!(upper_last(ukeys[n - 1]) < 0) || !(upper_first(ukeys[n]) < 0)) continue;
        for (int32_t z = az + 4096; z != bz; z += 4096) t.root_tiles[key_of(ax, ay, z) >> 27] = inside;
    }
}

gbls_host_grid* export_tree(const Tree& t, double voxel_size) {
    auto* g = new gbls_host_grid;
    g->voxel_size = voxel_size;
    g->background = t.bg;
    for (auto& kv : t.leaves) {
        int32_t x, y, z;
        origin_of(kv.first, x, y, z);
        g->leaf_origins.insert(g->leaf_origins.end(), {x, y, z});
        g->leaf_masks.insert(g->leaf_masks.end(), kv.second.mask, kv.second.mask + 8);
        g->leaf_values.insert(g->leaf_values.end(), kv.second.v, kv.second.v + 512);
    }
    for (auto& kv : t.lowers) {
        int32_t x, y, z;
        origin_of(kv.first << 12, x, y, z);
        g->lower_origins.insert(g->lower_origins.end(), {x, y, z});
        std::vector<float> tiles = kv.second;
        for (int n = 0; n < 4096; ++n)
            if (t.leaves.count((kv.first << 12) | uint64_t(n))) tiles[size_t(n)] = 0.0f;
        g->lower_tiles.insert(g->lower_tiles.end(), tiles.begin(), tiles.end());
    }
    for (auto& kv : t.uppers) {
        int32_t x, y, z;
        origin_of(kv.first << 27, x, y, z);
        g->upper_origins.insert(g->upper_origins.end(), {x, y, z});
        std::vector<float> tiles = kv.second;
        for (int n = 0; n < 32768; ++n)
            if (t.lowers.count((kv.first << 15) | uint64_t(n))) tiles[size_t(n)] = 0.0f;
        g->upper_tiles.insert(g->upper_tiles.end(), tiles.begin(), tiles.end());
    }
    for (auto& kv : t.root_tiles) {
        int32_t x, y, z;
        origin_of(kv.first << 27, x, y, z);
        g->root_tile_origins.insert(g->root_tile_origins.end(), {x, y, z});
        g->root_tile_values.push_back(kv.second);
    }
    return g;
}

// Rasterise in parallel over x-slabs aligned to leaves (each leaf belongs to
// exactly one worker), then merge.
template <class Band>
void raster_parallel(int32_t imin, int32_t imax, Band&& band, std::map<uint64_t, Leaf>& out) {
    if (imax <= imin) return;
    unsigned nt = std::max(1u, std::thread::hardware_concurrency());
    const int32_t lo = imin & ~7;
    const int32_t nslabs = (imax - lo + 7) / 8;
    nt = std::min<unsigned>(nt, unsigned(std::max(1, nslabs)));
    std::vector<LeafMap> parts(nt);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t) {
        th.emplace_back([&, t] {
            const int32_t s0 = lo + 8 * int32_t((int64_t(nslabs) * t) / nt);
            const int32_t s1 = lo + 8 * int32_t((int64_t(nslabs) * (t + 1)) / nt);
            band(std::max(s0, imin), std::min(s1, imax), parts[t]);
        });
    }
    for (auto& x : th) x.join();
    for (auto& p : parts)
        for (auto& kv : p) out.emplace(kv.first, kv.second);
}

}  // namespace

namespace gbls_host {
void set_error(const std::string& msg) { g_fix_error = msg; }
}  // namespace gbls_host

extern "C" {

int gbls_host_sphere(float radius, const float center[3], float voxel_size, float half_width,
                     gbls_host_grid** out) {
    if (!out || !center) { g_fix_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    *out = nullptr;
    if (radius <= 0) { g_fix_error = "radius must be positive"; return GBLS_ERR_VALUE; }
    if (!(voxel_size > 0.0f)) { g_fix_error = "voxel size must be positive"; return GBLS_ERR_VALUE; }
    if (!(half_width > 1)) { g_fix_error = "half-width must be larger than one"; return GBLS_ERR_VALUE; }
    try {
        Tree t;
        t.bg = static_cast<float>(double(voxel_size) * double(half_width));
        const float dx = voxel_size, w = half_width;
        Sphere s;
        s.r0 = radius / dx;
        s.cx = center[0] / dx;
        s.cy = center[1] / dx;
        s.cz = center[2] / dx;
        if (!(s.r0 < 1.5f)) {
            const float rmax = s.r0 + w;
            const int imin = int(std::floor(s.cx - rmax)), imax = int(std::ceil(s.cx + rmax));
            const float bg = t.bg;
            raster_parallel(imin, imax, [&](int32_t a, int32_t b, LeafMap& m) {
                sphere_band(s, w, a, b, [&](int32_t i, int32_t j, int32_t k, float v) { set_voxel(m, i, j, k, dx * v, bg); });
            }, t.leaves);
        }
        build_nodes(t);
        signed_flood_fill(t);
        *out = export_tree(t, voxel_size);
        return GBLS_OK;
    } catch (const std::bad_alloc&) {
        g_fix_error = "out of host memory";
        return GBLS_ERR_OUT_OF_MEMORY;
    }
}

int gbls_host_union_of_spheres(int64_t n, const float* centers, const float* radii, float voxel_size,
                               float half_width, gbls_host_grid** out) {
    if (!out || (n > 0 && (!centers || !radii))) { g_fix_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    *out = nullptr;
    if (!(voxel_size > 0.0f)) { g_fix_error = "voxel size must be positive"; return GBLS_ERR_VALUE; }
    if (!(half_width > 1)) { g_fix_error = "half-width must be larger than one"; return GBLS_ERR_VALUE; }
    try {
        Tree t;
        t.bg = static_cast<float>(double(voxel_size) * double(half_width));
        const float dx = voxel_size, w = half_width;
        std::vector<Sphere> sp;
        std::vector<int32_t> lo, hi;  // bounding boxes (voxel units) of the bands
        for (int64_t q = 0; q < n; ++q) {
            if (radii[q] <= 0) { g_fix_error = "radius must be positive"; return GBLS_ERR_VALUE; }
            Sphere s;
            s.r0 = radii[q] / dx;
            s.cx = centers[3 * q] / dx;
            s.cy = centers[3 * q + 1] / dx;
            s.cz = centers[3 * q + 2] / dx;
            if (s.r0 < 1.5f) continue;
            sp.push_back(s);
            const float rmax = s.r0 + w;
            lo.insert(lo.end(), {int(std::floor(s.cx - rmax)), int(std::floor(s.cy - rmax)), int(std::floor(s.cz - rmax))});
            hi.insert(hi.end(), {int(std::ceil(s.cx + rmax)), int(std::ceil(s.cy + rmax)), int(std::ceil(s.cz + rmax))});
        }
        if (!sp.empty()) {
            int32_t imin = lo[0], imax = hi[0];
            for (size_t q = 0; q < sp.size(); ++q) {
                imin = std::min(imin, lo[3 * q]);
                imax = std::max(imax, hi[3 * q]);
            }
            const float bg = t.bg;
            raster_parallel(imin, imax, [&](int32_t a, int32_t b, LeafMap& m) {
                for (size_t q = 0; q < sp.size(); ++q) {
                    const int32_t a2 = std::max(a, lo[3 * q]), b2 = std::min(b, hi[3 * q]);
                    if (a2 >= b2) continue;
                    // A voxel whose union distance lies in the band lies in the
                    // band of the sphere attaining the minimum, so enumerating
                    // every sphere's band visits every active voxel.
                    sphere_band(sp[q], w, a2, b2, [&](int32_t i, int32_t j, int32_t k, float vq) {
                        float v = vq;
                        for (size_t r = 0; r < sp.size(); ++r) {
                            if (r == q) continue;
                            const float d = sphere_dist(sp[r], i, j, k);
                            if (d < v) v = d;
                        }
                        if (std::fabs(v) < w) set_voxel(m, i, j, k, dx * v, bg);
                    });
                }
            }, t.leaves);
        }
        build_nodes(t);
        signed_flood_fill(t);
        *out = export_tree(t, voxel_size);
        return GBLS_OK;
    } catch (const std::bad_alloc&) {
        g_fix_error = "out of host memory";
        return GBLS_ERR_OUT_OF_MEMORY;
    }
}

// Torus around the y axis through `center`: major radius R, tube radius r
// (voxel units after dividing by dx), rasterised over its bounding box with
// the leapfrogging of tools/LevelSetSphere.h:154-173 (the distance is exact,
// so skipping floor(d - w) voxels never misses the band), then signed flood
// filled.
int gbls_host_torus(float major_radius, float minor_radius, const float center[3], float voxel_size,
                    float half_width, gbls_host_grid** out) {
    if (!out || !center) { g_fix_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    *out = nullptr;
    if (!(major_radius > 0) || !(minor_radius > 0) || !(minor_radius < major_radius)) {
        g_fix_error = "torus radii must satisfy 0 < minor < major";
        return GBLS_ERR_VALUE;
    }
    if (!(voxel_size > 0.0f)) { g_fix_error = "voxel size must be positive"; return GBLS_ERR_VALUE; }
    if (!(half_width > 1)) { g_fix_error = "half-width must be larger than one"; return GBLS_ERR_VALUE; }
    try {
        Tree t;
        t.bg = static_cast<float>(double(voxel_size) * double(half_width));
        const float dx = voxel_size, w = half_width;
        const float R = major_radius / dx, r = minor_radius / dx;
        const float cx = center[0] / dx, cy = center[1] / dx, cz = center[2] / dx;
        const float ext = R + r + w, exty = r + w;
        const int imin = int(std::floor(cx - ext)), imax = int(std::ceil(cx + ext));
        const int jmin = int(std::floor(cy - exty)), jmax = int(std::ceil(cy + exty));
        const int kmin = int(std::floor(cz - ext)), kmax = int(std::ceil(cz + ext));
        const float bg = t.bg;
        raster_parallel(imin, imax + 1, [&](int32_t a, int32_t b, LeafMap& m) {
            for (int32_t i = a; i < b; ++i) {
                const float x = float(i) - cx;
                for (int32_t j = jmin; j <= jmax; ++j) {
                    const float y2 = pow2(float(j) - cy);
                    int step = 1;
                    for (int32_t k = kmin; k <= kmax; k += step) {
                        step = 1;
                        const float q = std::sqrt(x * x + pow2(float(k) - cz)) - R;
                        const float v = std::sqrt(q * q + y2) - r;
                        const float d = std::fabs(v);
                        if (d < w) set_voxel(m, i, j, k, dx * v, bg);
                        else step += int(std::floor(d - w));
                    }
                }
            }
        }, t.leaves);
        build_nodes(t);
        signed_flood_fill(t);
        *out = export_tree(t, voxel_size);
        return GBLS_OK;
    } catch (const std::bad_alloc&) {
        g_fix_error = "out of host memory";
        return GBLS_ERR_OUT_OF_MEMORY;
    }
}

int gbls_host_grid_view(gbls_host_grid* g, gbls_grid_desc* d) {
    if (!g || !d) { g_fix_error = "null argument"; return GBLS_ERR_INVALID_ARGUMENT; }
    std::memset(d, 0, sizeof(*d));
    d->voxel_size = g->voxel_size;
    for (int i = 0; i < 3; ++i) d->translation[i] = g->translation[i];
    d->map_type = g->map_type;
    d->background = g->background;
    d->leaf_count = int64_t(g->leaf_origins.size() / 3);
    d->leaf_origins = g->leaf_origins.data();
    d->leaf_masks = g->leaf_masks.data();
    d->leaf_values = g->leaf_values.data();
    d->lower_count = int64_t(g->lower_origins.size() / 3);
    d->lower_origins = g->lower_origins.data();
    d->lower_tiles = g->lower_tiles.data();
    d->upper_count = int64_t(g->upper_origins.size() / 3);
    d->upper_origins = g->upper_origins.data();
    d->upper_tiles = g->upper_tiles.data();
    d->root_tile_count = int64_t(g->root_tile_origins.size() / 3);
    d->root_tile_origins = g->root_tile_origins.data();
    d->root_tile_values = g->root_tile_values.data();
    return GBLS_OK;
}

int gbls_host_grid_free(gbls_host_grid* g) {
    delete g;
    return GBLS_OK;
}

const char* gbls_host_last_error(void) { return g_fix_error.c_str(); }

}  // extern "C"

// The oracle's restatement of the benchmark input: the union of narrow-band
// sphere level sets (test infrastructure; included by levelset_port.cc after
// key_of / origin_of).
//
// Follows tools::createLevelSetSphere (tools/LevelSetSphere.h:127-199,
// 219-230: the float distance sqrt((i-cx)^2 + (j-cy)^2 + (k-cz)^2) - r in
// voxel units, band |d| < w, k advanced by 1 + floor(d - w) outside the
// band, i over [floor(cx - r - w), ceil(cx + r + w))), combined by
// tools::csgUnion (tools/Composite.h:886): a voxel in the band of the union
// takes the minimum of the sphere distances, which lies in the band of the
// sphere attaining it, so visiting every sphere's band visits every active
// voxel.  Then tools::signedFloodFill (tools/SignedFloodFill.h:82-215):
// inactive leaf voxels, lower- and upper-node tiles by scanlines in x, y, z
// from the signs of their neighbours, root tiles between two upper nodes on
// one z column whose facing ends are both inside.  Pinned by the golden
// digest of the 64-sphere input, which came from the reference itself.
#pragma once

namespace fixture {

struct Ball {
    float r, cx, cy, cz;  // voxel units
};

inline float sq(float x) { return x * x; }
inline float ball_distance(const Ball& b, int32_t i, int32_t j, int32_t k) {
    return std::sqrt((sq(float(j) - b.cy) + sq(float(i) - b.cx)) + sq(float(k) - b.cz)) - b.r;
}

struct Node {
    uint64_t mask[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    float v[512];
};

// Scanline fill of one node level (dim^3 slots): slots without a child take
// the sign of the last child boundary value met along x, then y, then z;
// a node without children takes the sign of its slot 0.
template <class Has, class First, class Last, class Set>
void scan_fill(int log2dim, Has has, First first_v, Last last_v, Set set, float slot0) {
    const int dim = 1 << log2dim, count = 1 << (3 * log2dim);
    int first = -1;
    for (int n = 0; n < count && first < 0; ++n)
        if (has(n)) first = n;
    if (first < 0) {
        for (int n = 0; n < count; ++n) set(n, slot0 < 0);
        return;
    }
    bool xin = first_v(first) < 0;
    for (int x = 0; x < dim; ++x) {
        const int nx = x << (2 * log2dim);
        if (has(nx)) xin = last_v(nx) < 0;
        bool yin = xin;
        for (int y = 0; y < dim; ++y) {
            const int ny = nx | (y << log2dim);
            if (has(ny)) yin = last_v(ny) < 0;
            bool zin = yin;
            for (int z = 0; z < dim; ++z) {
                const int n = ny | z;
                if (has(n)) zin = last_v(n) < 0;
                else set(n, zin);
            }
        }
    }
}

// Builds the union in the exchange layout (vectors owned by the caller).
struct Union {
    float background;
    std::map<uint64_t, Node> leaves;
    std::map<uint64_t, std::vector<float>> lowers, uppers;
    std::map<uint64_t, float> root;
    std::vector<int32_t> leaf_origins, lower_origins, upper_origins, root_origins;
    std::vector<uint64_t> leaf_masks;
    std::vector<float> leaf_values, lower_tiles, upper_tiles, root_values;

    void build(int64_t n, const float* centers, const float* radii, float dx, float w, int threads) {
        background = float(double(dx) * double(w));
        std::vector<Ball> balls;
        for (int64_t q = 0; q < n; ++q) {
            const Ball b{radii[q] / dx, centers[3 * q] / dx, centers[3 * q + 1] / dx, centers[3 * q + 2] / dx};
            if (!(b.r < 1.5f)) balls.push_back(b);  // createLevelSetSphere leaves smaller spheres empty
        }
        // rasterise per sphere over x-slabs of whole leaves, one map per thread
        int32_t lo = 0, hi = 0;
        for (size_t q = 0; q < balls.size(); ++q) {
            const float ext = balls[q].r + w;
            const int32_t a = int32_t(std::floor(balls[q].cx - ext)), b = int32_t(std::ceil(balls[q].cx + ext));
            lo = q ? std::min(lo, a) : a;
            hi = q ? std::max(hi, b) : b;
        }
        const int32_t base = lo & ~7, slabs = std::max(0, (hi - base + 7) / 8);
        const int nt = std::max(1, std::min(threads, int(slabs)));
        std::vector<std::unordered_map<uint64_t, Node>> part(static_cast<size_t>(nt));
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t) {
            pool.emplace_back([&, t] {
                const int32_t s0 = base + 8 * int32_t(int64_t(slabs) * t / nt);
                const int32_t s1 = base + 8 * int32_t(int64_t(slabs) * (t + 1) / nt);
                for (size_t q = 0; q < balls.size(); ++q) raster(balls, q, w, dx, std::max(s0, lo), std::min(s1, hi), part[size_t(t)]);
            });
        }
        for (auto& th : pool) th.join();
        for (auto& p : part)
            for (auto& kv : p) leaves.emplace(kv.first, kv.second);
        flood();
        export_arrays();
    }

    void raster(const std::vector<Ball>& balls, size_t q, float w, float dx, int32_t i0, int32_t i1,
                std::unordered_map<uint64_t, Node>& out) const {
        const Ball& b = balls[q];
        const float ext = b.r + w;
        i0 = std::max(i0, int32_t(std::floor(b.cx - ext)));
        i1 = std::min(i1, int32_t(std::ceil(b.cx + ext)));
        const int32_t j0 = int32_t(std::floor(b.cy - ext)), j1 = int32_t(std::ceil(b.cy + ext));
        const int32_t k0 = int32_t(std::floor(b.cz - ext)), k1 = int32_t(std::ceil(b.cz + ext));
        for (int32_t i = i0; i < i1; ++i) {
            const float xx = sq(float(i) - b.cx);
            for (int32_t j = j0; j <= j1; ++j) {
                const float xy = sq(float(j) - b.cy) + xx;
                for (int32_t k = k0; k <= k1;) {
                    const float d = std::sqrt(xy + sq(float(k) - b.cz)) - b.r;
                    if (std::fabs(d) < w) {
                        float m = d;
                        for (size_t r = 0; r < balls.size(); ++r)
                            if (r != q) m = std::min(m, ball_distance(balls[r], i, j, k));
                        if (std::fabs(m) < w) put(out, i, j, k, dx * m);
                        k += 1;
                    } else {
                        k += 1 + int32_t(std::floor(std::fabs(d) - w));
                    }
                }
            }
        }
    }

    void put(std::unordered_map<uint64_t, Node>& out, int32_t i, int32_t j, int32_t k, float value) const {
        auto it = out.find(key_of(i & ~7, j & ~7, k & ~7));
        if (it == out.end()) {
            Node nd;
            std::fill(nd.v, nd.v + 512, background);
            it = out.emplace(key_of(i & ~7, j & ~7, k & ~7), nd).first;
        }
        const int n = ((i & 7) << 6) | ((j & 7) << 3) | (k & 7);
        it->second.v[n] = value;
        it->second.mask[n >> 6] |= uint64_t(1) << (n & 63);
    }

    void flood() {
        const float out = std::fabs(background), in = -out;
        for (auto& kv : leaves) {
            Node& L = kv.second;
            auto on = [&](int n) { return ((L.mask[n >> 6] >> (n & 63)) & 1) != 0; };
            scan_fill(3, on, [&](int n) { return L.v[n]; }, [&](int n) { return L.v[n]; },
                      [&](int n, bool inside) { L.v[n] = inside ? in : out; }, L.v[0]);
        }
        for (auto& kv : leaves) {
            lowers.emplace(kv.first >> 12, std::vector<float>(4096, background));
            uppers.emplace(kv.first >> 27, std::vector<float>(32768, background));
        }
        auto leaf_at = [&](uint64_t k) -> const Node* {
            auto it = leaves.find(k);
            return it == leaves.end() ? nullptr : &it->second;
        };
        for (auto& kv : lowers) {
            const uint64_t lk = kv.first;
            std::vector<float>& tab = kv.second;
            scan_fill(4, [&](int n) { return leaf_at((lk << 12) | uint64_t(n)) != nullptr; },
                      [&](int n) { return leaf_at((lk << 12) | uint64_t(n))->v[0]; },
                      [&](int n) { return leaf_at((lk << 12) | uint64_t(n))->v[511]; },
                      [&](int n, bool inside) { tab[size_t(n)] = inside ? in : out; }, tab[0]);
        }
        // first / last value of a lower node: its first / last child, else tile
        auto lower_end = [&](uint64_t lk, bool last) -> float {
            const Node* L = leaf_at((lk << 12) | (last ? 4095u : 0u));
            return L ? L->v[last ? 511 : 0] : lowers.at(lk)[last ? 4095 : 0];
        };
        for (auto& kv : uppers) {
            const uint64_t uk = kv.first;
            std::vector<float>& tab = kv.second;
            auto has = [&](int n) { return lowers.count((uk << 15) | uint64_t(n)) != 0; };
            scan_fill(5, has, [&](int n) { return lower_end((uk << 15) | uint64_t(n), false); },
                      [&](int n) { return lower_end((uk << 15) | uint64_t(n), true); },
                      [&](int n, bool inside) { tab[size_t(n)] = inside ? in : out; }, tab[0]);
        }
        auto upper_end = [&](uint64_t uk, bool last) -> float {
            const uint64_t lk = (uk << 15) | (last ? 32767u : 0u);
            return lowers.count(lk) ? lower_end(lk, last) : uppers.at(uk)[last ? 32767 : 0];
        };
        uint64_t prev = 0;
        bool have = false;
        for (auto& kv : uppers) {
            if (have) {
                int32_t ax, ay, az, bx, by, bz;
                origin_of(prev << 27, ax, ay, az);
                origin_of(kv.first << 27, bx, by, bz);
                if (ax == bx && ay == by && bz - az != 4096 && upper_end(prev, true) < 0 && upper_end(kv.first, false) < 0)
                    for (int32_t z = az + 4096; z != bz; z += 4096) root[key_of(ax, ay, z) >> 27] = in;
            }
            prev = kv.first;
            have = true;
        }
    }

    void export_arrays() {
        for (auto& kv : leaves) {
            int32_t x, y, z;
            origin_of(kv.first, x, y, z);
            leaf_origins.insert(leaf_origins.end(), {x, y, z});
            leaf_masks.insert(leaf_masks.end(), kv.second.mask, kv.second.mask + 8);
            leaf_values.insert(leaf_values.end(), kv.second.v, kv.second.v + 512);
        }
        for (auto& kv : lowers) {
            int32_t x, y, z;
            origin_of(kv.first << 12, x, y, z);
            lower_origins.insert(lower_origins.end(), {x, y, z});
            for (int n = 0; n < 4096; ++n)
                lower_tiles.push_back(leaves.count((kv.first << 12) | uint64_t(n)) ? 0.0f : kv.second[size_t(n)]);
        }
        for (auto& kv : uppers) {
            int32_t x, y, z;
            origin_of(kv.first << 27, x, y, z);
            upper_origins.insert(upper_origins.end(), {x, y, z});
            for (int n = 0; n < 32768; ++n)
                upper_tiles.push_back(lowers.count((kv.first << 15) | uint64_t(n)) ? 0.0f : kv.second[size_t(n)]);
        }
        for (auto& kv : root) {
            int32_t x, y, z;
            origin_of(kv.first << 27, x, y, z);
            root_origins.insert(root_origins.end(), {x, y, z});
            root_values.push_back(kv.second);
        }
    }

    gbls_grid_desc view(double dx) {
        gbls_grid_desc d{};
        d.voxel_size = dx;
        d.map_type = GBLS_MAP_UNIFORM_SCALE;
        d.background = background;
        d.leaf_count = int64_t(leaf_origins.size() / 3);
        d.leaf_origins = leaf_origins.data();
        d.leaf_masks = leaf_masks.data();
        d.leaf_values = leaf_values.data();
        d.lower_count = int64_t(lower_origins.size() / 3);
        d.lower_origins = lower_origins.data();
        d.lower_tiles = lower_tiles.data();
        d.upper_count = int64_t(upper_origins.size() / 3);
        d.upper_origins = upper_origins.data();
        d.upper_tiles = upper_tiles.data();
        d.root_tile_count = int64_t(root_origins.size() / 3);
        d.root_tile_origins = root_origins.data();
        d.root_tile_values = root_values.data();
        return d;
    }
};

}  // namespace fixture

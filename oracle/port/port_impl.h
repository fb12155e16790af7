// Implementation of the oracle's restatement, compiled once per value type
// (Real = float: bit-identical to the reference; Real = double: the same
// scheme and constants evaluated in FP64).  Included by levelset_port.cc
// inside a namespace that defines Real; not a standalone header.
struct Leaf {
    uint64_t key;
    uint64_t mask[8];
    Real buf[3][512];  // buffer 0 = the tree's values; 1, 2 = RK auxiliaries
};

inline bool on(const uint64_t* m, int n) { return (m[n >> 6] >> (n & 63)) & 1; }
inline void set_on(uint64_t* m, int n) { m[n >> 6] |= uint64_t(1) << (n & 63); }
inline void set_off(uint64_t* m, int n) { m[n >> 6] &= ~(uint64_t(1) << (n & 63)); }

// ---- arithmetic of the reference (math/FiniteDifference.h:301-321) -------
// weno5_r: the C++ expression of the reference with ValueType Real (for
// float it mixes float and double exactly as the reference does); for the
// tangent-linear Real, the same value plus its FP64 derivative.
inline Real weno5(Real v1, Real v2, Real v3, Real v4, Real v5) { return weno5_r(v1, v2, v3, v4, v5); }
// D1<FD_HJWENO5>::difference(xp3, xp2, xp1, xp0, xm1, xm2)
inline Real hj_fd(Real xp3, Real xp2, Real xp1, Real xp0, Real xm1, Real xm2) {
    return weno5(xp3 - xp2, xp2 - xp1, xp1 - xp0, xp0 - xm1, xm1 - xm2);
}
// D1<BD_HJWENO5>::difference(xm3, xm2, xm1, xm0, xp1, xp2) = -FD(...)
inline Real hj_bd(Real xm3, Real xm2, Real xm1, Real xm0, Real xp1, Real xp2) {
    return -hj_fd(xm3, xm2, xm1, xm0, xp1, xp2);
}
inline Real fmaxr(Real a, Real b) { return (a < b) ? b : a; }  // std::max
inline Real fminr(Real a, Real b) { return (b < a) ? b : a; }  // std::min

// ---- the level set ---------------------------------------------------------
struct Grid {
    Real gamma = 3.0f;
    double voxel_size = 1.0;
    double translation[3] = {0, 0, 0};
    int map_type = GBLS_MAP_UNIFORM_SCALE;
    std::vector<Leaf*> leaves;                       // tree order
    std::unordered_map<uint64_t, Leaf*> index;       // key -> leaf
    std::map<uint64_t, std::vector<uint64_t>> lower; // lower key -> 64 sign words
    std::map<uint64_t, std::vector<uint64_t>> upper; // upper key -> 512 sign words
    std::map<uint64_t, uint8_t> root;                // upper key -> tile sign
    Pool pool;
    TopoTape* topo = nullptr;                        // trim record / replay (tests)

    ~Grid() { for (Leaf* l : leaves) delete l; }

    // sign of the tile covering leaf-sized region k (ValueAccessor::getValue)
    int tile_sign(uint64_t k) const {
        auto li = lower.find(k >> 12);
        if (li != lower.end()) { const uint32_t n = uint32_t(k & 4095); return int((li->second[n >> 6] >> (n & 63)) & 1); }
        auto ui = upper.find(k >> 27);
        if (ui != upper.end()) { const uint32_t n = uint32_t((k >> 12) & 32767); return int((ui->second[n >> 6] >> (n & 63)) & 1); }
        auto ri = root.find(k >> 27);
        return ri != root.end() ? ri->second : 0;
    }
    Leaf* probe(uint64_t k) const {
        auto it = index.find(k);
        return it == index.end() ? nullptr : it->second;
    }
    void rebuild_order() {
        std::sort(leaves.begin(), leaves.end(), [](const Leaf* a, const Leaf* b) { return a->key < b->key; });
    }
    size_t active_count() const {
        size_t n = 0;
        for (const Leaf* l : leaves) for (int w = 0; w < 8; ++w) n += size_t(__builtin_popcountll(l->mask[w]));
        return n;
    }
};

inline uint64_t nkey(uint64_t k, int f) {
    int32_t x, y, z;
    origin_of(k, x, y, z);
    if (f == 0) x -= 8; else if (f == 1) x += 8; else if (f == 2) y -= 8; else if (f == 3) y += 8; else if (f == 4) z -= 8; else z += 8;
    return key_of(x, y, z);
}

// 14^3 view of buffer `b` around a leaf: centre values and three-voxel face
// slabs (NineteenPointStencil, math/Stencils.h:816-863, reads only these).
struct Tile {
    Real v[14 * 14 * 14];
    Real& at(int x, int y, int z) { return v[(x + 3) * 196 + (y + 3) * 14 + (z + 3)]; }
    Real at(int x, int y, int z) const { return v[(x + 3) * 196 + (y + 3) * 14 + (z + 3)]; }
};

void gather(const Grid& g, const Leaf* L, int b, Tile& t) {
    for (int n = 0; n < 512; ++n) t.at(n >> 6, (n >> 3) & 7, n & 7) = L->buf[b][n];
    for (int f = 0; f < 6; ++f) {
        const uint64_t k = nkey(L->key, f);
        const Leaf* N = g.probe(k);
        const Real tv = N ? Real(0) : (g.tile_sign(k) ? -g.gamma : g.gamma);
        for (int d = 0; d < 3; ++d)
            for (int a = 0; a < 8; ++a)
                for (int c = 0; c < 8; ++c) {
                    int x, y, z, nx, ny, nz;
                    switch (f) {
                    case 0: x = -3 + d; y = a; z = c; nx = 5 + d; ny = a; nz = c; break;
                    case 1: x = 8 + d; y = a; z = c; nx = d; ny = a; nz = c; break;
                    case 2: x = a; y = -3 + d; z = c; nx = a; ny = 5 + d; nz = c; break;
                    case 3: x = a; y = 8 + d; z = c; nx = a; ny = d; nz = c; break;
                    case 4: x = a; y = c; z = -3 + d; nx = a; ny = c; nz = 5 + d; break;
                    default: x = a; y = c; z = 8 + d; nx = a; ny = c; nz = d; break;
                    }
                    t.at(x, y, z) = N ? N->buf[b][(nx << 6) | (ny << 3) | nz] : tv;
                }
    }
}

struct Field {
    gbls_field_desc d{};
    std::vector<float> dense;
    // a dense grid with its own transform (tools/LevelSetAdvect.h:482-483):
    // world = ijk * ls_scale + ls_t, grid index = (world - vel_t) * vel_inv
    bool xform = false;
    double ls_scale = 1, ls_t[3] = {0, 0, 0}, vel_inv = 1, vel_t[3] = {0, 0, 0};

    // Sampling setup for a level set with map (map_type, voxel_size, translation).
    void set_level_set_map(int map_type, double voxel_size, const double* translation) {
        xform = false;
        if (d.kind != GBLS_FIELD_DENSE || d.dense_map_type == 0) return;
        const int vmap = d.dense_map_type - 1;
        if (vmap == map_type && d.dense_voxel_size == voxel_size && d.dense_translation[0] == translation[0] &&
            d.dense_translation[1] == translation[1] && d.dense_translation[2] == translation[2])
            return;  // same transform: the aligned lookup
        xform = true;
        ls_scale = map_type == GBLS_MAP_TRANSLATION ? 1.0 : voxel_size;
        vel_inv = vmap == GBLS_MAP_TRANSLATION ? 1.0 : 1.0 / d.dense_voxel_size;
        for (int a = 0; a < 3; ++a) {
            ls_t[a] = map_type == GBLS_MAP_UNIFORM_SCALE ? 0.0 : translation[a];
            vel_t[a] = vmap == GBLS_MAP_UNIFORM_SCALE ? 0.0 : d.dense_translation[a];
        }
    }
    void grid_value(int i, int j, int k, float out[3]) const {
        const int a = i - d.dense_origin[0], b = j - d.dense_origin[1], c = k - d.dense_origin[2];
        if (a >= 0 && b >= 0 && c >= 0 && a < d.dense_dims[0] && b < d.dense_dims[1] && c < d.dense_dims[2]) {
            const float* p = dense.data() + 3 * ((size_t(a) * d.dense_dims[1] + b) * d.dense_dims[2] + c);
            out[0] = p[0]; out[1] = p[1]; out[2] = p[2];
        } else {
            out[0] = d.dense_background[0]; out[1] = d.dense_background[1]; out[2] = d.dense_background[2];
        }
    }
    // BoxSampler (tools/Interpolation.h:714-762): a + float(double(b - a) * w)
    static float lerp(float a, float b, double w) { return a + float(double(b - a) * w); }
    void trilinear(int i, int j, int k, float out[3]) const {
        const int ijk[3] = {i, j, k};
        int i0[3];
        double uvw[3];
        for (int a = 0; a < 3; ++a) {
            const double w = double(ijk[a]) * ls_scale + ls_t[a];
            const double q = (w - vel_t[a]) * vel_inv;
            i0[a] = int(std::floor(q));
            uvw[a] = q - double(i0[a]);
        }
        float v[2][2][2][3];
        for (int x = 0; x < 2; ++x)
            for (int y = 0; y < 2; ++y)
                for (int z = 0; z < 2; ++z) grid_value(i0[0] + x, i0[1] + y, i0[2] + z, v[x][y][z]);
        for (int c = 0; c < 3; ++c) {
            const float a0 = lerp(lerp(v[0][0][0][c], v[0][0][1][c], uvw[2]), lerp(v[0][1][0][c], v[0][1][1][c], uvw[2]), uvw[1]);
            const float a1 = lerp(lerp(v[1][0][0][c], v[1][0][1][c], uvw[2]), lerp(v[1][1][0][c], v[1][1][1][c], uvw[2]), uvw[1]);
            out[c] = lerp(a0, a1, uvw[0]);
        }
    }
    // Tangent run: derivatives of the aligned dense velocity values along
    // the probe directions ([kLanes][nx][ny][nz][3], empty when the velocity
    // is held fixed); out[component][lane].
    std::vector<double> dense_tangent;
    void eval_tangent(int i, int j, int k, double out[3][kLanes]) const {
        for (int c = 0; c < 3; ++c)
            for (int q = 0; q < kLanes; ++q) out[c][q] = 0.0;
        if (dense_tangent.empty() || d.kind != GBLS_FIELD_DENSE || xform) return;
        const int a = i - d.dense_origin[0], b = j - d.dense_origin[1], c = k - d.dense_origin[2];
        if (a >= 0 && b >= 0 && c >= 0 && a < d.dense_dims[0] && b < d.dense_dims[1] && c < d.dense_dims[2]) {
            const size_t lane = size_t(3) * d.dense_dims[0] * d.dense_dims[1] * d.dense_dims[2];
            const size_t at = 3 * ((size_t(a) * d.dense_dims[1] + b) * d.dense_dims[2] + c);
            if (dense_tangent.size() < lane * kLanes) return;
            for (int q = 0; q < kLanes; ++q)
                for (int e = 0; e < 3; ++e) out[e][q] = dense_tangent[q * lane + at + e];
        }
    }
    void eval(int i, int j, int k, float t, float out[3]) const {
        switch (d.kind) {
        case GBLS_FIELD_CONSTANT: out[0] = d.constant[0]; out[1] = d.constant[1]; out[2] = d.constant[2]; break;
        case GBLS_FIELD_DENSE:
            if (xform) trilinear(i, j, k, out);
            else grid_value(i, j, k, out);
            break;
        case GBLS_FIELD_DEFORMATION: gbls_deformation(i, j, k, t, d.domain, d.period, d.scale, out); break;
        default: gbls_rotation(i, j, k, d.constant, d.omega, d.center, out); break;
        }
    }
};

struct Tracker {
    int spatial = GBLS_HJWENO5_BIAS, temporal = GBLS_TVD_RK1, norm_count = 3, trim = GBLS_TRIM_ALL;
};

// ---- Normalizer (tools/LevelSetTracker.h:511-676) --------------------------
// One stage: result[n] = N ? alpha*phi[n] + beta*v : v over the voxels of the
// process set (the active set, or `mask` when given).
void norm_stage(Grid& g, const Tracker& tr, int phiBuf, int resBuf, Real alpha, bool hasPhi,
                const std::unordered_map<uint64_t, std::vector<uint64_t>>* mask) {
    const Real dx = Real(float(g.voxel_size));
    const Real mDt = dx * Real(tr.temporal == GBLS_TVD_RK1 ? 0.3f : tr.temporal == GBLS_TVD_RK2 ? 0.9f : 1.0f);
    const Real mInvDx = Real(1) / dx;
    const Real beta = Real(1) - alpha;
    g.pool.run(g.leaves.size(), [&](size_t a, size_t b) {
        Tile t;
        for (size_t li = a; li < b; ++li) {
            Leaf* L = g.leaves[li];
            const uint64_t* pm = L->mask;
            if (mask) {
                auto it = mask->find(L->key);
                if (it == mask->end()) continue;
                pm = it->second.data();
            }
            gather(g, L, 0, t);
            for (int n = 0; n < 512; ++n) {
                if (!on(pm, n)) continue;
                const int x = n >> 6, y = (n >> 3) & 7, z = n & 7;
                auto S = [&](int dx_, int dy_, int dz_) { return t.at(x + dx_, y + dy_, z + dz_); };
                const Real up[3] = {hj_fd(S(3, 0, 0), S(2, 0, 0), S(1, 0, 0), S(0, 0, 0), S(-1, 0, 0), S(-2, 0, 0)),
                                     hj_fd(S(0, 3, 0), S(0, 2, 0), S(0, 1, 0), S(0, 0, 0), S(0, -1, 0), S(0, -2, 0)),
                                     hj_fd(S(0, 0, 3), S(0, 0, 2), S(0, 0, 1), S(0, 0, 0), S(0, 0, -1), S(0, 0, -2))};
                const Real dn[3] = {hj_bd(S(-3, 0, 0), S(-2, 0, 0), S(-1, 0, 0), S(0, 0, 0), S(1, 0, 0), S(2, 0, 0)),
                                     hj_bd(S(0, -3, 0), S(0, -2, 0), S(0, -1, 0), S(0, 0, 0), S(0, 1, 0), S(0, 2, 0)),
                                     hj_bd(S(0, 0, -3), S(0, 0, -2), S(0, 0, -1), S(0, 0, 0), S(0, 0, 1), S(0, 0, 2))};
                const Real phi0 = S(0, 0, 0);
                // GodunovsNormSqrd(phi0 > 0, down, up) (math/FiniteDifference.h:324-357)
                Real nsq;
                if (phi0 > 0) {
                    nsq = fmaxr(fmaxr(dn[0], 0) * fmaxr(dn[0], 0), fminr(up[0], 0) * fminr(up[0], 0));
                    nsq += fmaxr(fmaxr(dn[1], 0) * fmaxr(dn[1], 0), fminr(up[1], 0) * fminr(up[1], 0));
                    nsq += fmaxr(fmaxr(dn[2], 0) * fmaxr(dn[2], 0), fminr(up[2], 0) * fminr(up[2], 0));
                } else {
                    nsq = fmaxr(fminr(dn[0], 0) * fminr(dn[0], 0), fmaxr(up[0], 0) * fmaxr(up[0], 0));
                    nsq += fmaxr(fminr(dn[1], 0) * fminr(dn[1], 0), fmaxr(up[1], 0) * fmaxr(up[1], 0));
                    nsq += fmaxr(fminr(dn[2], 0) * fminr(dn[2], 0), fmaxr(up[2], 0) * fmaxr(up[2], 0));
                }
                // eval (tools/LevelSetTracker.h:623-643)
                Real v = phi0 / (sqrt_r(phi0 * phi0 + nsq) + Real(1e-8f));
                v = phi0 - mDt * v * (sqrt_r(nsq) * mInvDx - Real(1));
                L->buf[resBuf][n] = hasPhi ? alpha * L->buf[phiBuf][n] + beta * v : v;
            }
        }
    });
}

void copy_aux(Grid& g, int nAux) {
    g.pool.run(g.leaves.size(), [&](size_t a, size_t b) {
        for (size_t i = a; i < b; ++i)
            for (int k = 1; k <= nAux; ++k) std::memcpy(g.leaves[i]->buf[k], g.leaves[i]->buf[0], sizeof(Real) * 512);
    });
}
void swap_buf(Grid& g, int k) {
    for (Leaf* L : g.leaves) {
        Real tmp[512];
        std::memcpy(tmp, L->buf[0], sizeof(tmp));
        std::memcpy(L->buf[0], L->buf[k], sizeof(tmp));
        std::memcpy(L->buf[k], tmp, sizeof(tmp));
    }
}

// Normalizer::normalize (:528-598)
void normalize(Grid& g, const Tracker& tr, const std::unordered_map<uint64_t, std::vector<uint64_t>>* mask) {
    copy_aux(g, tr.temporal == GBLS_TVD_RK3 ? 2 : 1);
    for (int n = 0; n < tr.norm_count; ++n) {
        if (tr.temporal == GBLS_TVD_RK1) {
            norm_stage(g, tr, 0, 1, Real(0), false, mask); swap_buf(g, 1);
        } else if (tr.temporal == GBLS_TVD_RK2) {
            norm_stage(g, tr, 0, 1, Real(0), false, mask); swap_buf(g, 1);
            norm_stage(g, tr, 1, 1, Real(1.0f / 2.0f), true, mask); swap_buf(g, 1);
        } else {
            norm_stage(g, tr, 0, 1, Real(0), false, mask); swap_buf(g, 1);
            norm_stage(g, tr, 1, 2, Real(3.0f / 4.0f), true, mask); swap_buf(g, 2);
            norm_stage(g, tr, 1, 2, Real(1.0f / 3.0f), true, mask); swap_buf(g, 2);
        }
    }
}

// Create a leaf at key k filled with its tile value, creating the lower and
// upper nodes it needs with the value of the tile they replace.
Leaf* touch_leaf(Grid& g, uint64_t k) {
    const Real tv = g.tile_sign(k) ? -g.gamma : g.gamma;
    const uint64_t lk = k >> 12, uk = k >> 27;
    if (!g.upper.count(uk)) {
        uint8_t s = 0;
        auto r = g.root.find(uk);
        if (r != g.root.end()) { s = r->second; g.root.erase(r); }
        g.upper[uk] = std::vector<uint64_t>(512, s ? ~uint64_t(0) : 0);
    }
    if (!g.lower.count(lk)) {
        const uint32_t n = uint32_t(lk & 32767);
        const int s = int((g.upper[uk][n >> 6] >> (n & 63)) & 1);
        g.lower[lk] = std::vector<uint64_t>(64, s ? ~uint64_t(0) : 0);
    }
    Leaf* L = new Leaf;
    L->key = k;
    std::memset(L->mask, 0, sizeof(L->mask));
    for (int b = 0; b < 3; ++b) std::fill(L->buf[b], L->buf[b] + 512, tv);
    g.leaves.push_back(L);
    g.index[k] = L;
    return L;
}

// dilateActiveValues(NN_FACE, IGNORE_TILES), one iteration (tools/Morphology.h:612-812)
void dilate1(Grid& g) {
    const size_t n0 = g.leaves.size();
    // new leaves: missing face neighbours that receive active voxels
    std::vector<uint64_t> cand;
    for (size_t i = 0; i < n0; ++i) {
        const Leaf* L = g.leaves[i];
        const uint64_t* m = L->mask;
        uint64_t any[6];
        any[0] = m[0]; any[1] = m[7];
        uint64_t ym = 0, yp = 0, zm = 0, zp = 0;
        for (int w = 0; w < 8; ++w) {
            ym |= m[w] & 0xFFull; yp |= m[w] & 0xFF00000000000000ull;
            zm |= m[w] & 0x0101010101010101ull; zp |= m[w] & 0x8080808080808080ull;
        }
        any[2] = ym; any[3] = yp; any[4] = zm; any[5] = zp;
        for (int f = 0; f < 6; ++f)
            if (any[f] && !g.probe(nkey(L->key, f))) cand.push_back(nkey(L->key, f));
    }
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
    for (uint64_t k : cand) touch_leaf(g, k);
    g.rebuild_order();
    // new masks from the old ones
    std::unordered_map<const Leaf*, std::array<uint64_t, 8>> old;
    old.reserve(g.leaves.size());
    for (const Leaf* L : g.leaves) {
        std::array<uint64_t, 8> a;
        std::memcpy(a.data(), L->mask, 64);
        old[L] = a;
    }
    g.pool.run(g.leaves.size(), [&](size_t a, size_t b) {
        for (size_t i = a; i < b; ++i) {
            Leaf* L = g.leaves[i];
            const uint64_t* own = old.at(L).data();
            const uint64_t* nb[6];
            for (int f = 0; f < 6; ++f) {
                const Leaf* N = g.probe(nkey(L->key, f));
                nb[f] = N ? old.at(N).data() : nullptr;
            }
            for (int x = 0; x < 8; ++x) {
                const uint64_t w = own[x];
                uint64_t d = w | ((w << 1) & 0xFEFEFEFEFEFEFEFEull) | ((w >> 1) & 0x7F7F7F7F7F7F7F7Full) | (w << 8) | (w >> 8);
                d |= x > 0 ? own[x - 1] : (nb[0] ? nb[0][7] : 0);
                d |= x < 7 ? own[x + 1] : (nb[1] ? nb[1][0] : 0);
                if (nb[2]) d |= nb[2][x] >> 56;
                if (nb[3]) d |= nb[3][x] << 56;
                if (nb[4]) d |= (nb[4][x] >> 7) & 0x0101010101010101ull;
                if (nb[5]) d |= (nb[5][x] << 7) & 0x8080808080808080ull;
                L->mask[x] = d;
            }
        }
    });
}

// erodeActiveValues(NN_FACE, IGNORE_TILES), `iter` iterations
void erode(Grid& g, int iter) {
    for (int it = 0; it < iter; ++it) {
        std::unordered_map<const Leaf*, std::array<uint64_t, 8>> old;
        for (const Leaf* L : g.leaves) {
            std::array<uint64_t, 8> a;
            std::memcpy(a.data(), L->mask, 64);
            old[L] = a;
        }
        for (Leaf* L : g.leaves) {
            const uint64_t* own = old.at(L).data();
            uint64_t W[6][8];
            for (int f = 0; f < 6; ++f) {
                const Leaf* N = g.probe(nkey(L->key, f));
                for (int x = 0; x < 8; ++x) W[f][x] = N ? old.at(N)[x] : 0;
            }
            for (int x = 0; x < 8; ++x) {
                const uint64_t w = own[x];
                uint64_t e = w;
                e &= ((w << 1) & 0xFEFEFEFEFEFEFEFEull) | ((W[4][x] >> 7) & 0x0101010101010101ull);
                e &= ((w >> 1) & 0x7F7F7F7F7F7F7F7Full) | ((W[5][x] << 7) & 0x8080808080808080ull);
                e &= (w << 8) | (W[2][x] >> 56);
                e &= (w >> 8) | (W[3][x] << 56);
                e &= x > 0 ? own[x - 1] : W[0][7];
                e &= x < 7 ? own[x + 1] : W[1][0];
                L->mask[x] = e;
            }
        }
    }
}

// Trim (tools/LevelSetTracker.h:473-506)
void trim(Grid& g, int mode) {
    if (mode == GBLS_TRIM_NONE) return;
    const Real gamma = g.gamma;
    if (g.topo && g.topo->replay) {
        // the recorded outcome instead of the thresholds: a voxel the record
        // drops leaves the band at +-gamma by its sign, every other one stays
        static const std::array<uint64_t, 8> none{};
        if (g.topo->pos >= g.topo->masks.size()) {  // more trims than recorded
            g.topo->overrun = true;
            return;
        }
        const auto& rec = g.topo->masks[g.topo->pos++];
        for (Leaf* L : g.leaves) {
            auto it = rec.find(L->key);
            const auto& m = it == rec.end() ? none : it->second;
            for (int n = 0; n < 512; ++n) {
                if (!on(L->mask, n) || ((m[n >> 6] >> (n & 63)) & 1)) continue;
                set_off(L->mask, n);
                L->buf[0][n] = L->buf[0][n] < Real(0.0f) ? -gamma : gamma;
            }
        }
        return;
    }
    g.pool.run(g.leaves.size(), [&](size_t a, size_t b) {
        for (size_t i = a; i < b; ++i) {
            Leaf* L = g.leaves[i];
            for (int n = 0; n < 512; ++n) {
                if (!on(L->mask, n)) continue;
                const Real v = L->buf[0][n];
                if ((mode & 1) && v <= -gamma) { set_off(L->mask, n); L->buf[0][n] = -gamma; }
                else if ((mode & 2) && v >= gamma) { set_off(L->mask, n); L->buf[0][n] = gamma; }
            }
        }
    });
    if (g.topo) {
        std::unordered_map<uint64_t, std::array<uint64_t, 8>> rec;
        for (const Leaf* L : g.leaves) {
            std::array<uint64_t, 8> m;
            std::memcpy(m.data(), L->mask, 64);
            rec[L->key] = m;
        }
        g.topo->masks.push_back(std::move(rec));
    }
}

// pruneLevelSet (tools/Prune.h:266-330, 391-397): bottom-up
void prune_level_set(Grid& g) {
    std::vector<Leaf*> keep;
    for (Leaf* L : g.leaves) {
        bool any = false;
        for (int w = 0; w < 8; ++w) any |= L->mask[w] != 0;
        if (any) { keep.push_back(L); continue; }
        const uint64_t k = L->key;
        auto& ls = g.lower.at(k >> 12);
        const uint32_t n = uint32_t(k & 4095);
        if (L->buf[0][0] < 0) ls[n >> 6] |= uint64_t(1) << (n & 63);
        else ls[n >> 6] &= ~(uint64_t(1) << (n & 63));
        g.index.erase(k);
        delete L;
    }
    g.leaves.swap(keep);
    std::unordered_set<uint64_t> lowerWithLeaves;
    for (Leaf* L : g.leaves) lowerWithLeaves.insert(L->key >> 12);
    for (auto it = g.lower.begin(); it != g.lower.end();) {
        if (lowerWithLeaves.count(it->first)) { ++it; continue; }
        const uint64_t lk = it->first;
        auto& us = g.upper.at(lk >> 15);
        const uint32_t n = uint32_t(lk & 32767);
        if (it->second[0] & 1) us[n >> 6] |= uint64_t(1) << (n & 63);
        else us[n >> 6] &= ~(uint64_t(1) << (n & 63));
        it = g.lower.erase(it);
    }
    std::unordered_set<uint64_t> upperWithLower;
    for (auto& kv : g.lower) upperWithLower.insert(kv.first >> 15);
    for (auto it = g.upper.begin(); it != g.upper.end();) {
        if (upperWithLower.count(it->first)) { ++it; continue; }
        g.root[it->first] = uint8_t(it->second[0] & 1);
        it = g.upper.erase(it);
    }
    for (auto it = g.root.begin(); it != g.root.end();) {  // eraseBackgroundTiles
        if (it->second == 0) it = g.root.erase(it);
        else ++it;
    }
}

// changeLevelSetBackground: every inactive value becomes +-background by sign
void change_background(Grid& g, Real bg) {
    g.gamma = bg;
    g.pool.run(g.leaves.size(), [&](size_t a, size_t b) {
        for (size_t i = a; i < b; ++i) {
            Leaf* L = g.leaves[i];
            for (int n = 0; n < 512; ++n)
                if (!on(L->mask, n)) L->buf[0][n] = L->buf[0][n] < 0 ? -bg : bg;
        }
    });
}

void prune(Grid& g, const Tracker& tr) {
    trim(g, tr.trim);
    prune_level_set(g);
}

void track(Grid& g, const Tracker& tr) {
    dilate1(g);
    normalize(g, tr, nullptr);
    prune(g, tr);
}

void tracker_dilate(Grid& g, const Tracker& tr, int iterations) {
    const Real dx = Real(float(g.voxel_size));
    for (int i = 0; i < iterations; ++i) {
        std::unordered_map<uint64_t, std::array<uint64_t, 8>> before;
        for (const Leaf* L : g.leaves) { std::array<uint64_t, 8> a; std::memcpy(a.data(), L->mask, 64); before[L->key] = a; }
        dilate1(g);
        change_background(g, dx + g.gamma);
        if (tr.norm_count > 0) {
            std::unordered_map<uint64_t, std::vector<uint64_t>> mask;
            for (const Leaf* L : g.leaves) {
                std::vector<uint64_t> m(8);
                auto it = before.find(L->key);
                bool any = false;
                for (int w = 0; w < 8; ++w) {
                    m[w] = L->mask[w] & ~(it == before.end() ? 0 : it->second[w]);
                    any |= m[w] != 0;
                }
                if (any) mask[L->key] = m;
            }
            normalize(g, tr, &mask);
        }
    }
}

void tracker_erode(Grid& g, int iterations) {
    erode(g, iterations);
    prune_level_set(g);
    change_background(g, g.gamma - Real(float(iterations) * float(g.voxel_size)));
}

// ---- LevelSetAdvection (tools/LevelSetAdvect.h:338-572) ---------------------
struct Advector {
    Grid& g;
    const Field& field;
    Tracker tr;
    int temporal = GBLS_TVD_RK3;
    float cfl = 0.0f;
    std::vector<size_t> offsets;
    using Vel = typename VelOf<Real>::type;  // float, or TL for the tangent run
    using Time = Real;
    std::vector<Vel> vel;  // [active][3]

    float sample_field(float t0, float t1) {
        if (g.leaves.empty()) return 0.0f;
        offsets.resize(g.leaves.size() + 1);
        size_t acc = 0;
        for (size_t i = 0; i < g.leaves.size(); ++i) {
            offsets[i] = acc;
            for (int w = 0; w < 8; ++w) acc += size_t(__builtin_popcountll(g.leaves[i]->mask[w]));
        }
        offsets[g.leaves.size()] = acc;
        vel.assign(acc * 3, Vel(0.0f));
        const bool fwd = t0 < t1;
        g.pool.run(g.leaves.size(), [&](size_t a, size_t b) {
            for (size_t i = a; i < b; ++i) {
                const Leaf* L = g.leaves[i];
                int32_t ox, oy, oz;
                origin_of(L->key, ox, oy, oz);
                Vel* v = vel.data() + 3 * offsets[i];
                for (int n = 0; n < 512; ++n) {
                    if (!on(L->mask, n)) continue;
                    float o[3];
                    double od[3][kLanes];
                    field.eval(ox + (n >> 6), oy + ((n >> 3) & 7), oz + (n & 7), t0, o);
                    field.eval_tangent(ox + (n >> 6), oy + ((n >> 3) & 7), oz + (n & 7), od);
                    for (int c = 0; c < 3; ++c) {
                        if (!fwd)
                            for (int q = 0; q < kLanes; ++q) od[c][q] = -od[c][q];
                        v[c] = vel_make(fwd ? o[c] : -o[c], od[c], Vel(0.0f));
                    }
                    v += 3;
                }
            }
        });
        float maxAbsV = 0;
        size_t arg = acc;
        for (size_t i = 0; i < acc; ++i) {
            const Vel* v = vel.data() + 3 * i;
            const float x = vel_value(v[0]), y = vel_value(v[1]), z = vel_value(v[2]);
            const float m = float(fmaxr(Real(maxAbsV), Real(x * x + y * y + z * z)));
            if (m != maxAbsV) arg = i;  // std::max keeps the first of equal maxima
            maxAbsV = m;
        }
        if (!(maxAbsV > 1e-5f) && !(maxAbsV < -1e-5f)) return 0.0f;
        // |v|^2 at the first voxel holding the maximum: its tangent is the
        // time step's dependence on the velocity (tangent runs)
        max_v2 = Time(maxAbsV);
        if (arg < acc) {
            const Vel* v = vel.data() + 3 * arg;
            const Time x = Time(v[0]), y = Time(v[1]), z = Time(v[2]);
            max_v2 = x * x + y * y + z * z;
        }
        return maxAbsV;
    }
    Time max_v2 = Time(0.0f);

    // The substep length at t0 for max |v|^2 = maxAbsV.  cfl == 0: the
    // reference's sampleField (tools/LevelSetAdvect.h:459-466) over [t0, t1].
    // cfl > 0: the reference's advect(tau, tau') driven over greedy intervals
    // tau' = tau + cfl*dx/|v|max (t1 when that reaches it), each interval
    // running the reference's own loop, so a second short substep appears
    // when tau + (tau' - tau) rounds short of tau'.
    // Times: float in the FP32 instance (the reference's), double in the
    // FP64 one, TL in tangent runs, where the substep depends on the
    // velocity through max |v|^2 and on the earlier substeps of its
    // interval through the time reached.
    bool open = false;
    Time end = Time(0.0f);
    static Time abs_t(Time x) { return x < Time(0.0f) ? -x : x; }
    Time substep(Time t0, float t1, Time maxAbsV) {
        const float CFLref = (temporal == GBLS_TVD_RK1 ? 0.3f : temporal == GBLS_TVD_RK2 ? 0.9f : 1.0f) / std::sqrt(3.0f);
        const float dx = float(g.voxel_size);
        const bool fwd = t0 < Time(t1);
        if (!open) {
            end = Time(t1);
            if (cfl > 0.0f) {
                const Time lim = Time(cfl * dx) / sqrt_r(maxAbsV);
                if (lim < abs_t(Time(t1) - t0)) end = fwd ? t0 + lim : t0 - lim;
            }
            if (end - t0 == Time(0.0f)) return Time(0.0f);
            open = true;
        }
        const Time a = abs_t(end - t0), b = Time(CFLref * dx) / sqrt_r(maxAbsV);
        return b < a ? b : a;  // math::Min
    }

    // euler<N,D>(dt, phiBuffer, resultBuffer)
    void euler(Time dt, int phiBuf, int resBuf, Real alpha, bool hasPhi) {
        const double invdx = 1.0 / g.voxel_size;
        const Real beta = Real(1) - alpha;
        g.pool.run(g.leaves.size(), [&](size_t a, size_t b) {
            Tile t;
            for (size_t i = a; i < b; ++i) {
                Leaf* L = g.leaves[i];
                gather(g, L, 0, t);
                const Vel* v = vel.data() + 3 * offsets[i];
                for (int n = 0; n < 512; ++n) {
                    if (!on(L->mask, n)) continue;
                    const int x = n >> 6, y = (n >> 3) & 7, z = n & 7;
                    auto S = [&](int dx_, int dy_, int dz_) { return t.at(x + dx_, y + dy_, z + dz_); };
                    const Real gx = v[0] < 0 ? hj_fd(S(3, 0, 0), S(2, 0, 0), S(1, 0, 0), S(0, 0, 0), S(-1, 0, 0), S(-2, 0, 0))
                                              : hj_bd(S(-3, 0, 0), S(-2, 0, 0), S(-1, 0, 0), S(0, 0, 0), S(1, 0, 0), S(2, 0, 0));
                    const Real gy = v[1] < 0 ? hj_fd(S(0, 3, 0), S(0, 2, 0), S(0, 1, 0), S(0, 0, 0), S(0, -1, 0), S(0, -2, 0))
                                              : hj_bd(S(0, -3, 0), S(0, -2, 0), S(0, -1, 0), S(0, 0, 0), S(0, 1, 0), S(0, 2, 0));
                    const Real gz = v[2] < 0 ? hj_fd(S(0, 0, 3), S(0, 0, 2), S(0, 0, 1), S(0, 0, 0), S(0, 0, -1), S(0, 0, -2))
                                              : hj_bd(S(0, 0, -3), S(0, 0, -2), S(0, 0, -1), S(0, 0, 0), S(0, 0, 1), S(0, 0, 2));
                    // Vec3d -> applyIJT (x 1/dx in double) -> Vec3f
                    const Real g0 = ijt_r(gx, invdx), g1 = ijt_r(gy, invdx), g2 = ijt_r(gz, invdx);
                    const Real av = S(0, 0, 0) - Real(dt) * (Real(v[0]) * g0 + Real(v[1]) * g1 + Real(v[2]) * g2);
                    L->buf[resBuf][n] = hasPhi ? alpha * L->buf[phiBuf][n] + beta * av : av;
                    v += 3;
                }
            }
        });
    }

    uint64_t advect(float t0, float t1, const std::function<bool()>& interrupted, uint64_t* updates) {
        uint64_t count = 0;
        if (t0 - t1 == 0.0f) return 0;
        const bool fwd = t0 < t1;
        open = false;
        Time t = Time(t0);
        while (fwd ? t < Time(t1) : t > Time(t1)) {
            if (interrupted && interrupted()) break;
            copy_aux(g, temporal == GBLS_TVD_RK3 ? 2 : 1);
            const float maxAbsV = sample_field(float(t), t1);
            if (maxAbsV == 0.0f) break;
            const Time dt = substep(t, t1, max_v2);
            if (dt == Time(0.0f)) break;
            if (updates) *updates += offsets.back();
            if (temporal == GBLS_TVD_RK1) {
                euler(dt, 0, 1, Real(0), false); swap_buf(g, 1);
            } else if (temporal == GBLS_TVD_RK2) {
                euler(dt, 0, 1, Real(0), false); swap_buf(g, 1);
                euler(dt, 1, 1, Real(1.0f / 2.0f), true); swap_buf(g, 1);
            } else {
                euler(dt, 0, 1, Real(0), false); swap_buf(g, 1);
                euler(dt, 1, 2, Real(3.0f / 4.0f), true); swap_buf(g, 2);
                euler(dt, 1, 2, Real(1.0f / 3.0f), true); swap_buf(g, 2);
            }
            t += fwd ? dt : -dt;
            if (!(fwd ? t < end : t > end)) open = false;
            ++count;
            track(g, tr);
        }
        return count;
    }
};

// ---- canonical import / export ----------------------------------------------
Grid* import_desc(const gbls_grid_desc* d) {
    Grid* g = new Grid;
    g->gamma = d->background;
    g->voxel_size = d->voxel_size;
    g->map_type = d->map_type;
    for (int i = 0; i < 3; ++i) g->translation[i] = d->translation[i];
    for (int64_t i = 0; i < d->leaf_count; ++i) {
        const int32_t* o = d->leaf_origins + 3 * i;
        Leaf* L = new Leaf;
        L->key = key_of(o[0], o[1], o[2]);
        std::memcpy(L->mask, d->leaf_masks + 8 * i, 64);
        for (int q = 0; q < 512; ++q) L->buf[0][q] = Real(d->leaf_values[512 * i + q]);
        g->leaves.push_back(L);
        g->index[L->key] = L;
    }
    g->rebuild_order();
    for (int64_t i = 0; i < d->lower_count; ++i) {
        const int32_t* o = d->lower_origins + 3 * i;
        const uint64_t lk = key_of(o[0], o[1], o[2]) >> 12;
        std::vector<uint64_t> s(64, 0);
        for (int n = 0; n < 4096; ++n)
            if (d->lower_tiles[i * 4096 + n] < 0) s[n >> 6] |= uint64_t(1) << (n & 63);
        g->lower[lk] = s;
    }
    for (int64_t i = 0; i < d->upper_count; ++i) {
        const int32_t* o = d->upper_origins + 3 * i;
        const uint64_t uk = key_of(o[0], o[1], o[2]) >> 27;
        std::vector<uint64_t> s(512, 0);
        for (int n = 0; n < 32768; ++n)
            if (d->upper_tiles[i * 32768 + n] < 0) s[n >> 6] |= uint64_t(1) << (n & 63);
        g->upper[uk] = s;
    }
    for (int64_t i = 0; i < d->root_tile_count; ++i) {
        const int32_t* o = d->root_tile_origins + 3 * i;
        g->root[key_of(o[0], o[1], o[2]) >> 27] = d->root_tile_values[i] < 0 ? 1 : 0;
    }
    return g;
}

void export_desc(const Grid& g, gbls_grid_desc* d) {
    d->voxel_size = g.voxel_size;
    for (int i = 0; i < 3; ++i) d->translation[i] = g.translation[i];
    d->map_type = g.map_type;
    d->background = float(g.gamma);
    std::unordered_set<uint64_t> leafKeys, lowerKeys;
    for (size_t i = 0; i < g.leaves.size(); ++i) {
        const Leaf* L = g.leaves[i];
        int32_t x, y, z;
        origin_of(L->key, x, y, z);
        d->leaf_origins[3 * i] = x; d->leaf_origins[3 * i + 1] = y; d->leaf_origins[3 * i + 2] = z;
        std::memcpy(d->leaf_masks + 8 * i, L->mask, 64);
        for (int q = 0; q < 512; ++q) d->leaf_values[512 * i + q] = float(L->buf[0][q]);
        leafKeys.insert(L->key);
    }
    size_t i = 0;
    for (auto& kv : g.lower) {
        int32_t x, y, z;
        origin_of(kv.first << 12, x, y, z);
        d->lower_origins[3 * i] = x; d->lower_origins[3 * i + 1] = y; d->lower_origins[3 * i + 2] = z;
        for (int n = 0; n < 4096; ++n) {
            const uint64_t k = (kv.first << 12) | uint64_t(n);
            d->lower_tiles[i * 4096 + n] = leafKeys.count(k) ? 0.0f : float(((kv.second[n >> 6] >> (n & 63)) & 1) ? -g.gamma : g.gamma);
        }
        lowerKeys.insert(kv.first);
        ++i;
    }
    i = 0;
    for (auto& kv : g.upper) {
        int32_t x, y, z;
        origin_of(kv.first << 27, x, y, z);
        d->upper_origins[3 * i] = x; d->upper_origins[3 * i + 1] = y; d->upper_origins[3 * i + 2] = z;
        for (int n = 0; n < 32768; ++n) {
            const uint64_t k = (kv.first << 15) | uint64_t(n);
            d->upper_tiles[i * 32768 + n] = lowerKeys.count(k) ? 0.0f : float(((kv.second[n >> 6] >> (n & 63)) & 1) ? -g.gamma : g.gamma);
        }
        ++i;
    }
    i = 0;
    for (auto& kv : g.root) {
        int32_t x, y, z;
        origin_of(kv.first << 27, x, y, z);
        d->root_tile_origins[3 * i] = x; d->root_tile_origins[3 * i + 1] = y; d->root_tile_origins[3 * i + 2] = z;
        d->root_tile_values[i] = float(kv.second ? -g.gamma : g.gamma);
        ++i;
    }
}


// CPU restatement of OpenVDB's narrow-band level-set advection path — the
// test oracle and CPU baseline of this project (test infrastructure: the
// product never links it).
//
// It follows the reference algorithm operation by operation:
//   tools/LevelSetAdvect.h:338-418   Advect::advect (CFL substep loop)
//   tools/LevelSetAdvect.h:426-464   sampleField (max |v|^2, CFL dt)
//   tools/LevelSetAdvect.h:543-572   euler<N,D> (RK stage)
//   tools/LevelSetTracker.h:302-315  track = dilate, normalize, prune
//   tools/LevelSetTracker.h:279-300  prune = Trim + pruneLevelSet
//   tools/LevelSetTracker.h:317-364  dilate / erode / resize
//   tools/LevelSetTracker.h:528-676  Normalizer (RK loop, eval, masked euler)
//   math/FiniteDifference.h:301-357  WENO5, GodunovsNormSqrd
//   math/FiniteDifference.h:1177-1389 D1<FD_HJWENO5>, D1<BD_HJWENO5>
//   math/Operators.h:195-262,823-846 ISGradientBiased, ISGradientNormSqrd,
//                                    GradientBiased (applyIJT = x 1/dx)
//   tools/Morphology.h:612-812       NN_FACE dilation / erosion semantics
//   tools/Prune.h:266-330            LevelSetPruneOp tile rule
//   tree/InternalNode.h:2848-2888    new children inherit the tile value
// with its own data structures: leaves with dense 512-value buffers in a hash
// map, internal-node tiles as sign bits (every tile of a level set is
// +-background).  Built with -ffp-contract=off and no -march so results are
// bit-identical to the reference on x86-64 and aarch64.
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <string>
#include <thread>
#include <unordered_map>
#include <type_traits>
#include <unordered_set>
#include <vector>

#include "gbls.h"
#include "gbls_fields.h"

namespace {

thread_local std::string g_err;

// ---- keys: integer order = tree order (root lexicographic, then child offsets)
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

// ---- simple thread pool: parallel_for over [0, n) in contiguous chunks
struct Pool {
    int nthreads = 1;
    void run(size_t n, const std::function<void(size_t, size_t)>& body) const {
        if (n == 0) return;
        const size_t nt = std::min<size_t>(size_t(std::max(1, nthreads)), n);
        if (nt == 1) { body(0, n); return; }
        std::vector<std::thread> th;
        for (size_t t = 0; t < nt; ++t)
            th.emplace_back([&, t] { body(n * t / nt, n * (t + 1) / nt); });
        for (auto& x : th) x.join();
    }
};

#include "fixture_port.h"

// The band after every trim of a run (record), imposed on another run of
// the same level set (replay): a finite difference across runs then sees
// no voxel enter or leave the band, only the smooth part of the map.
struct TopoTape {
    bool replay = false;
    bool overrun = false;  // a replay asked for more trims than recorded
    size_t pos = 0;
    std::vector<std::unordered_map<uint64_t, std::array<uint64_t, 8>>> masks;
};

// ---- tangent-linear numbers: the FP64 reference gradient -------------------
// A TL carries the value of the FP32 computation (bit-identical to the
// float instance: every operation rounds its value exactly as a float does)
// and the derivatives of that value along kLanes directions, propagated in
// FP64 through the same branches (upwind sides, Godunov selections,
// trimming, topology).  One forward run gives kLanes directional
// derivatives dL/dphi0 . d or dL/dv . d of the FP32 forward map in FP64,
// without the truncation error or branch switching of a finite difference.
constexpr int kLanes = 8;
struct TL {
    float v = 0.0f;
    double d[kLanes] = {};
    TL() = default;
    TL(float x) : v(x) {}  // constants: zero derivative
    explicit operator float() const { return v; }
    explicit operator double() const { return double(v); }
    TL& operator+=(TL b) {
        v += b.v;
        for (int k = 0; k < kLanes; ++k) d[k] += b.d[k];
        return *this;
    }
};
inline TL operator+(TL a, TL b) {
    TL r(a.v + b.v);
    for (int k = 0; k < kLanes; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
inline TL operator-(TL a, TL b) {
    TL r(a.v - b.v);
    for (int k = 0; k < kLanes; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
inline TL operator-(TL a) {
    TL r(-a.v);
    for (int k = 0; k < kLanes; ++k) r.d[k] = -a.d[k];
    return r;
}
inline TL operator*(TL a, TL b) {
    TL r(a.v * b.v);
    const double av = a.v, bv = b.v;
    for (int k = 0; k < kLanes; ++k) r.d[k] = a.d[k] * bv + av * b.d[k];
    return r;
}
inline TL operator/(TL a, TL b) {
    TL r(a.v / b.v);
    const double q = r.v, bv = b.v;
    for (int k = 0; k < kLanes; ++k) r.d[k] = (a.d[k] - q * b.d[k]) / bv;
    return r;
}
inline bool operator<(TL a, TL b) { return a.v < b.v; }
inline bool operator>(TL a, TL b) { return a.v > b.v; }
inline bool operator<=(TL a, TL b) { return a.v <= b.v; }
inline bool operator>=(TL a, TL b) { return a.v >= b.v; }
inline bool operator==(TL a, TL b) { return a.v == b.v; }
inline bool operator!=(TL a, TL b) { return a.v != b.v; }

inline float sqrt_r(float x) { return std::sqrt(x); }
inline double sqrt_r(double x) { return std::sqrt(x); }
inline TL sqrt_r(TL x) {
    TL r(std::sqrt(x.v));
    if (r.v > 0.0f)
        for (int k = 0; k < kLanes; ++k) r.d[k] = x.d[k] / (2.0 * double(r.v));
    return r;
}
// Vec3d(g) * invdx rounded back (GradientBiased's applyIJT)
inline float ijt_r(float g, double invdx) { return float(double(g) * invdx); }
inline double ijt_r(double g, double invdx) { return double(g) * invdx; }
inline TL ijt_r(TL g, double invdx) {
    TL r(float(double(g.v) * invdx));
    for (int k = 0; k < kLanes; ++k) r.d[k] = g.d[k] * invdx;
    return r;
}

// math::WENO5 (math/FiniteDifference.h:301-321) as the C++ expression with
// ValueType R: for float it mixes float and double exactly as the reference.
template <class R>
inline R weno5_expr(R v1, R v2, R v3, R v4, R v5) {
    const double C = 13.0 / 12.0;
    const double eps = 1.0e-6 * static_cast<double>(0.01f);
    auto p2 = [](auto x) { return x * x; };
    const double A1 = 0.1 / p2(C * p2(v1 - 2 * v2 + v3) + 0.25 * p2(v1 - 4 * v2 + 3.0 * v3) + eps),
                 A2 = 0.6 / p2(C * p2(v2 - 2 * v3 + v4) + 0.25 * p2(v2 - v4) + eps),
                 A3 = 0.3 / p2(C * p2(v3 - 2 * v4 + v5) + 0.25 * p2(3.0 * v3 - 4 * v4 + v5) + eps);
    return static_cast<R>(static_cast<R>(A1 * (2.0 * v1 - 7.0 * v2 + 11.0 * v3) + A2 * (5.0 * v3 - v2 + 2.0 * v4) +
                                         A3 * (2.0 * v3 + 5.0 * v4 - v5)) /
                          (6.0 * (A1 + A2 + A3)));
}
inline float weno5_r(float a, float b, float c, float d, float e) { return weno5_expr<float>(a, b, c, d, e); }
inline double weno5_r(double a, double b, double c, double d, double e) { return weno5_expr<double>(a, b, c, d, e); }
// the value as the float instance, the derivative from the formula's exact
// partial derivatives at the float operands (forward mode in double)
struct Dual {
    double v, d[kLanes];
};
inline Dual dual(double v) {
    Dual r{v, {}};
    return r;
}
inline Dual operator+(const Dual& a, const Dual& b) {
    Dual r{a.v + b.v, {}};
    for (int k = 0; k < kLanes; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
inline Dual operator-(const Dual& a, const Dual& b) {
    Dual r{a.v - b.v, {}};
    for (int k = 0; k < kLanes; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
inline Dual operator*(double c, const Dual& a) {
    Dual r{c * a.v, {}};
    for (int k = 0; k < kLanes; ++k) r.d[k] = c * a.d[k];
    return r;
}
inline Dual operator*(const Dual& a, const Dual& b) {
    Dual r{a.v * b.v, {}};
    for (int k = 0; k < kLanes; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
inline Dual operator/(double c, const Dual& a) {
    Dual r{c / a.v, {}};
    for (int k = 0; k < kLanes; ++k) r.d[k] = -c * a.d[k] / (a.v * a.v);
    return r;
}
inline Dual operator/(const Dual& a, const Dual& b) {
    Dual r{a.v / b.v, {}};
    for (int k = 0; k < kLanes; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
    return r;
}
inline TL weno5_r(TL a, TL b, TL c, TL d, TL e) {
    auto in = [](const TL& x) {
        Dual r{double(x.v), {}};
        for (int k = 0; k < kLanes; ++k) r.d[k] = x.d[k];
        return r;
    };
    const Dual v1 = in(a), v2 = in(b), v3 = in(c), v4 = in(d), v5 = in(e);
    const double C = 13.0 / 12.0, eps = 1.0e-6 * static_cast<double>(0.01f);
    auto sq = [](const Dual& x) { return x * x; };
    const Dual e1 = dual(eps);
    const Dual A1 = 0.1 / sq(C * sq(v1 - 2.0 * v2 + v3) + 0.25 * sq(v1 - 4.0 * v2 + 3.0 * v3) + e1);
    const Dual A2 = 0.6 / sq(C * sq(v2 - 2.0 * v3 + v4) + 0.25 * sq(v2 - v4) + e1);
    const Dual A3 = 0.3 / sq(C * sq(v3 - 2.0 * v4 + v5) + 0.25 * sq(3.0 * v3 - 4.0 * v4 + v5) + e1);
    const Dual num = A1 * (2.0 * v1 - 7.0 * v2 + 11.0 * v3) + A2 * (5.0 * v3 - v2 + 2.0 * v4) +
                     A3 * (2.0 * v3 + 5.0 * v4 - v5);
    const Dual q = num / (6.0 * (A1 + A2 + A3));
    TL r(weno5_expr<float>(a.v, b.v, c.v, d.v, e.v));
    for (int k = 0; k < kLanes; ++k) r.d[k] = q.d[k];
    return r;
}

// Velocities as the advection stores them: float, or TL for the tangent run.
template <class R>
struct VelOf {
    using type = float;
};
template <>
struct VelOf<TL> {
    using type = TL;
};
inline float vel_make(float v, const double*, float) { return v; }
inline TL vel_make(float v, const double* d, TL) {
    TL r(v);
    for (int k = 0; k < kLanes; ++k) r.d[k] = d[k];
    return r;
}
inline float vel_value(float v) { return v; }
inline float vel_value(TL v) { return v.v; }

namespace p32 {
using Real = float;
#include "port_impl.h"
Advector adv_of(Grid&);
}  // namespace p32
namespace p64 {
using Real = double;
#include "port_impl.h"
Advector adv_of(Grid&);
}  // namespace p64
namespace ptl {
using Real = TL;
#include "port_impl.h"
Advector adv_of(Grid&);
}  // namespace ptl

}  // namespace

namespace {

// A grid of either precision behind the C interface.
struct Handle {
    int prec;  // 32, 64, or 1 for the tangent-linear run
    p32::Grid* g32 = nullptr;
    p64::Grid* g64 = nullptr;
    ptl::Grid* gtl = nullptr;
    std::vector<double> vel_tangent;  // tangent run: derivative of the dense velocity
    TopoTape topo;
    ~Handle() {
        delete g32;
        delete g64;
        delete gtl;
    }
};

template <class F32, class F64, class FTL>
auto dispatch(void* hp, F32&& f32, F64&& f64, FTL&& ftl) {
    Handle* h = static_cast<Handle*>(hp);
    return h->prec == 64 ? f64(*h->g64) : h->prec == 1 ? ftl(*h->gtl) : f32(*h->g32);
}


int nthreads_of(int threads) { return threads > 0 ? threads : int(std::max(1u, std::thread::hardware_concurrency())); }

}  // namespace

extern "C" {

const char* oport_last_error() { return g_err.c_str(); }

// math::WENO5<float> (math/FiniteDifference.h:301-321) on n operand
// quintuples v[5*i .. 5*i+4].
void oport_weno5(int64_t n, const float* v, float* out) {
    for (int64_t i = 0; i < n; ++i) out[i] = p32::weno5(v[5 * i], v[5 * i + 1], v[5 * i + 2], v[5 * i + 3], v[5 * i + 4]);
}

// precision 32: bit-identical to the reference; 64: the same scheme in FP64
void* oport_create_prec(const gbls_grid_desc* d, int threads, int precision) {
    Handle* h = new Handle;
    h->prec = precision == 64 ? 64 : precision == 1 ? 1 : 32;
    if (h->prec == 64) {
        h->g64 = p64::import_desc(d);
        h->g64->pool.nthreads = nthreads_of(threads);
    } else if (h->prec == 1) {
        h->gtl = ptl::import_desc(d);
        h->gtl->pool.nthreads = nthreads_of(threads);
    } else {
        h->g32 = p32::import_desc(d);
        h->g32->pool.nthreads = nthreads_of(threads);
    }
    return h;
}
void* oport_create(const gbls_grid_desc* d, int threads) { return oport_create_prec(d, threads, 32); }

// The union of n narrow-band spheres (createLevelSetSphere + csgUnion,
// fixture_port.h) built by the oracle itself.
void* oport_create_spheres(int64_t n, const float* centers, const float* radii, float voxel_size,
                           float half_width, int threads, int precision) {
    fixture::Union u;
    u.build(n, centers, radii, voxel_size, half_width, nthreads_of(threads));
    const gbls_grid_desc d = u.view(voxel_size);
    return oport_create_prec(&d, threads, precision);
}
void oport_free(void* h) { delete static_cast<Handle*>(h); }
void oport_set_threads(void* h, int threads) {
    auto f = [&](auto& g) { g.pool.nthreads = nthreads_of(threads); return 0; };
    dispatch(h, f, f, f);
}

int oport_counts(void* h, gbls_grid_counts* c) {
    auto f = [&](auto& g) {
        c->leaf_count = int64_t(g.leaves.size());
        c->lower_count = int64_t(g.lower.size());
        c->upper_count = int64_t(g.upper.size());
        c->root_tile_count = int64_t(g.root.size());
        c->active_voxel_count = int64_t(g.active_count());
        return 0;
    };
    return dispatch(h, f, f, f);
}

int oport_export(void* h, gbls_grid_desc* d) {
    return dispatch(h, [&](p32::Grid& g) { p32::export_desc(g, d); return 0; },
                    [&](p64::Grid& g) { p64::export_desc(g, d); return 0; },
                    [&](ptl::Grid& g) { ptl::export_desc(g, d); return 0; });
}

// Active values in canonical order, as double.
int oport_active_values(void* h, double* out) {
    auto f = [&](auto& g) {
        size_t k = 0;
        for (const auto* L : g.leaves)
            for (int n = 0; n < 512; ++n)
                if ((L->mask[n >> 6] >> (n & 63)) & 1) out[k++] = double(L->buf[0][n]);
        return 0;
    };
    return dispatch(h, f, f, f);
}

// Replace the active values (canonical order) from doubles.
int oport_set_active_values(void* h, const double* in) {
    auto f = [&](auto& g) {
        size_t k = 0;
        for (auto* L : g.leaves)
            for (int n = 0; n < 512; ++n)
                if ((L->mask[n >> 6] >> (n & 63)) & 1)
                    L->buf[0][n] = std::remove_reference_t<decltype(L->buf[0][0])>(in[k++]);
        return 0;
    };
    return dispatch(h, f, f, f);
}

int oport_tangent_lanes() { return kLanes; }

// mode 0: trims by the thresholds; 1: also records the band after every
// trim (clearing an earlier record); 2: replays the record of `from` (or
// this grid's own when null) from its first trim.
int oport_topology(void* hp, int mode, void* from) {
    Handle* h = static_cast<Handle*>(hp);
    if (mode == 1) {
        h->topo = TopoTape{};
    } else if (mode == 2) {
        if (from) h->topo.masks = static_cast<Handle*>(from)->topo.masks;
        h->topo.replay = true;
        h->topo.pos = 0;
    }
    auto f = [&](auto& g) { g.topo = mode == 0 ? nullptr : &h->topo; return 0; };
    return dispatch(hp, f, f, f);
}
// trims recorded, or (replay) imposed so far; -1 after an overrun
int64_t oport_topology_count(void* hp) {
    const TopoTape& t = static_cast<Handle*>(hp)->topo;
    return t.overrun ? -1 : int64_t(t.replay ? t.pos : t.masks.size());
}

// Tangent run: the derivatives of the active values, in[lane][active]
// (canonical active order).
int oport_set_tangents(void* hp, const double* in) {
    Handle* h = static_cast<Handle*>(hp);
    if (h->prec != 1) { g_err = "not a tangent-linear grid"; return GBLS_ERR_INVALID_ARGUMENT; }
    const size_t na = h->gtl->active_count();
    size_t k = 0;
    for (auto* L : h->gtl->leaves)
        for (int n = 0; n < 512; ++n)
            if ((L->mask[n >> 6] >> (n & 63)) & 1) {
                for (int q = 0; q < kLanes; ++q) L->buf[0][n].d[q] = in[size_t(q) * na + k];
                ++k;
            }
    return 0;
}
int oport_active_tangents(void* hp, double* out) {
    Handle* h = static_cast<Handle*>(hp);
    if (h->prec != 1) { g_err = "not a tangent-linear grid"; return GBLS_ERR_INVALID_ARGUMENT; }
    const size_t na = h->gtl->active_count();
    size_t k = 0;
    for (const auto* L : h->gtl->leaves)
        for (int n = 0; n < 512; ++n)
            if ((L->mask[n >> 6] >> (n & 63)) & 1) {
                for (int q = 0; q < kLanes; ++q) out[size_t(q) * na + k] = L->buf[0][n].d[q];
                ++k;
            }
    return 0;
}
// Tangent run: the derivatives of the dense velocity values,
// dv[lane][nx][ny][nz][3] (n doubles in all; 0 clears them).
int oport_set_velocity_tangent(void* hp, const double* dv, int64_t n) {
    Handle* h = static_cast<Handle*>(hp);
    if (h->prec != 1) { g_err = "not a tangent-linear grid"; return GBLS_ERR_INVALID_ARGUMENT; }
    h->vel_tangent.assign(dv, dv + (n > 0 ? n : 0));
    return 0;
}

// op: 0 track, 1 normalize, 2 prune, 3 dilate(arg), 4 erode(arg), 5 resize(arg)
int oport_tracker_op(void* h, int op, int arg, int spatial, int temporal, int norm_count, int trim_mode, int* result) {
    if (spatial != GBLS_HJWENO5_BIAS) { g_err = "the oracle port implements HJWENO5_BIAS"; return GBLS_ERR_UNSUPPORTED; }
    auto f = [&](auto& g, auto tr) {
        tr.temporal = temporal;
        tr.norm_count = norm_count;
        tr.trim = trim_mode;
        int r = 0;
        using G = std::remove_reference_t<decltype(g)>;
        (void)sizeof(G);
        switch (op) {
        case 0: track(g, tr); break;
        case 1: normalize(g, tr, nullptr); break;
        case 2: prune(g, tr); break;
        case 3: tracker_dilate(g, tr, arg); break;
        case 4: tracker_erode(g, arg); break;
        case 5: {
            const int wOld = int(std::floor(float(g.gamma) / float(g.voxel_size)));
            if (wOld < arg) tracker_dilate(g, tr, arg - wOld);
            else if (wOld > arg) tracker_erode(g, wOld - arg);
            r = wOld != arg;
            break;
        }
        default: g_err = "bad op"; return int(GBLS_ERR_INVALID_ARGUMENT);
        }
        if (result) *result = r;
        return 0;
    };
    return dispatch(h, [&](p32::Grid& g) { return f(g, p32::Tracker{}); },
                    [&](p64::Grid& g) { return f(g, p64::Tracker{}); },
                    [&](ptl::Grid& g) { return f(g, ptl::Tracker{}); });
}

int oport_advect(void* h, const gbls_field_desc* fd, int spatial, int temporal, int tspatial, int ttemporal,
                 int norm_count, float t0, float t1, float cfl, uint64_t* count, uint64_t* updates) {
    if (spatial != GBLS_HJWENO5_BIAS || tspatial != GBLS_HJWENO5_BIAS) {
        g_err = "the oracle port implements HJWENO5_BIAS";
        return GBLS_ERR_UNSUPPORTED;
    }
    auto f = [&](auto& g, auto field) {
        field.d = *fd;
        if (fd->kind == GBLS_FIELD_DENSE)
            field.dense.assign(fd->dense_values,
                               fd->dense_values + size_t(3) * fd->dense_dims[0] * fd->dense_dims[1] * fd->dense_dims[2]);
        field.set_level_set_map(g.map_type, g.voxel_size, g.translation);
        using G = std::remove_reference_t<decltype(g)>;
        using A = decltype(adv_of(g));
        A a{g, field};
        a.tr.temporal = ttemporal;
        a.tr.norm_count = norm_count;
        a.temporal = temporal;
        a.cfl = cfl;
        uint64_t u = 0;
        const uint64_t n = a.advect(t0, t1, nullptr, &u);
        if (count) *count = n;
        if (updates) *updates = u;
        (void)sizeof(G);
        return 0;
    };
    Handle* hh = static_cast<Handle*>(h);
    return dispatch(h, [&](p32::Grid& g) { return f(g, p32::Field{}); },
                    [&](p64::Grid& g) { return f(g, p64::Field{}); },
                    [&](ptl::Grid& g) {
                        ptl::Field field{};
                        field.dense_tangent = hh->vel_tangent;
                        return f(g, field);
                    });
}

}  // extern "C"

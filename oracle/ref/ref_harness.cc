// Test-oracle harness around the UNMODIFIED reference implementation.
//
// This file is compiled (by oracle/ref/build_ref.py) together with the
// reference's own headers and a handful of its .cc files, read in place from
// the reference checkout, into oracle/_ref/libvdbref.so.  It exposes a small
// C interface so the Python tests can (a) build reference level sets
// (tools::createLevelSetSphere, tools::csgUnion), (b) convert between an
// openvdb::FloatGrid and the gbls_grid_desc exchange format, and (c) run the
// reference tools::LevelSetAdvection / tools::LevelSetTracker on them.
// It is test infrastructure only: the product never links it.
#include <openvdb/openvdb.h>
#include <openvdb/tools/Composite.h>
#include <openvdb/tools/LevelSetAdvect.h>
#include <openvdb/tools/LevelSetFilter.h>
#include <openvdb/tools/LevelSetMorph.h>
#include <openvdb/tools/LevelSetSphere.h>
#include <openvdb/tools/LevelSetTracker.h>
#include <openvdb/tools/VelocityFields.h>
#include <openvdb/tools/VolumeAdvect.h>

#include <openvdb/io/GridDescriptor.h>

#include <cstring>
#include <exception>
#include <fstream>
#include <string>
#include <vector>

#include "gbls.h"
#include "gbls_fields.h"

using namespace openvdb;
using FloatTree = openvdb::FloatTree;
using RootT = FloatTree::RootNodeType;
using UpperT = RootT::ChildNodeType;
using LowerT = UpperT::ChildNodeType;
using LeafT = LowerT::ChildNodeType;

namespace {

thread_local std::string gLastError;

int fail(int code, const std::string& msg) {
    gLastError = msg;
    return code;
}

struct RefGrid {
    FloatGrid::Ptr grid;
};

// Velocity functor with the interface tools::LevelSetAdvection expects
// (tools/LevelSetAdvect.h:32-52) evaluating the analytic fields of
// gbls_fields.h at integer coordinates.
struct AnalyticField {
    using ValueType = float;
    using VectorType = math::Vec3<float>;
    gbls_field_desc desc;
    math::Transform::Ptr xform;
    const math::Transform& transform() const { return *xform; }
    VectorType operator()(const Coord& ijk, float t) const {
        float o[3];
        if (desc.kind == GBLS_FIELD_DEFORMATION) {
            gbls_deformation(ijk[0], ijk[1], ijk[2], t, desc.domain, desc.period, desc.scale, o);
        } else {
            gbls_rotation(ijk[0], ijk[1], ijk[2], desc.constant, desc.omega, desc.center, o);
        }
        return VectorType(o[0], o[1], o[2]);
    }
    VectorType operator()(const Vec3d& xyz, float t) const {
        return (*this)(xform->worldToIndexNodeCentered(xyz), t);
    }
};

Vec3fGrid::Ptr makeVelocityGrid(const gbls_field_desc& f, const math::Transform& xform) {
    Vec3fGrid::Ptr vel;
    if (f.kind == GBLS_FIELD_CONSTANT) {
        vel = Vec3fGrid::create(Vec3f(f.constant[0], f.constant[1], f.constant[2]));
    } else {
        vel = Vec3fGrid::create(
            Vec3f(f.dense_background[0], f.dense_background[1], f.dense_background[2]));
        auto acc = vel->getAccessor();
        const int nx = f.dense_dims[0], ny = f.dense_dims[1], nz = f.dense_dims[2];
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j)
                for (int k = 0; k < nz; ++k) {
                    const float* v = f.dense_values + 3 * ((size_t(i) * ny + j) * nz + k);
                    acc.setValue(Coord(f.dense_origin[0] + i, f.dense_origin[1] + j,
                                       f.dense_origin[2] + k),
                                 Vec3f(v[0], v[1], v[2]));
                }
    }
    if (f.kind == GBLS_FIELD_DENSE && f.dense_map_type != 0) {
        // the velocity grid's own transform (1 + GBLS_MAP_*)
        math::Transform::Ptr vx = math::Transform::createLinearTransform(
            f.dense_map_type - 1 == GBLS_MAP_TRANSLATION ? 1.0 : f.dense_voxel_size);
        if (f.dense_map_type - 1 != GBLS_MAP_UNIFORM_SCALE)
            vx->postTranslate(Vec3d(f.dense_translation[0], f.dense_translation[1], f.dense_translation[2]));
        vel->setTransform(vx);
    } else {
        vel->setTransform(xform.copy());
    }
    return vel;
}

template<typename FieldT>
size_t runAdvect(FloatGrid& grid, const FieldT& field, int s, int t, int ts, int tt, int nc,
                 float t0, float t1) {
    tools::LevelSetAdvection<FloatGrid, FieldT> adv(grid, field);
    adv.setSpatialScheme(math::BiasedGradientScheme(s));
    adv.setTemporalScheme(math::TemporalIntegrationScheme(t));
    adv.setTrackerSpatialScheme(math::BiasedGradientScheme(ts));
    adv.setTrackerTemporalScheme(math::TemporalIntegrationScheme(tt));
    adv.setNormCount(nc);
    return adv.advect(t0, t1);
}

// max |v|^2 over the active voxels at time t, as Advect::sampleField computes
// it (tools/LevelSetAdvect.h:441-456): aligned fields at the voxel, others at
// its world position, Vec3f::lengthSqr in float, math::Max over all voxels.
template<typename FieldT>
float maxSpeedSqr(const FloatGrid& grid, const FieldT& field, float t) {
    const bool aligned = field.transform() == grid.transform();
    const math::MapBase::ConstPtr map = grid.transform().baseMap();
    float m = 0.0f;
    for (auto leaf = grid.tree().cbeginLeaf(); leaf; ++leaf) {
        for (auto it = leaf->cbeginValueOn(); it; ++it) {
            const auto v = aligned ? field(it.getCoord(), t) : field(map->applyMap(it.getCoord().asVec3d()), t);
            m = math::Max(m, float(v.lengthSqr()));
        }
    }
    return m;
}

// A CFL number below the reference's fixed one (tools/LevelSetAdvect.h:459-463)
// imposed by the caller: LevelSetAdvection::advect(tau, tau') over greedy
// intervals, tau' = tau + cfl*dx/max|v| with max|v| sampled at tau over the
// current active voxels, the last interval ending at t1.  The reference's own
// loop runs inside each interval; its substep counts are summed.
template<typename FieldT>
size_t runAdvectCfl(FloatGrid& grid, const FieldT& field, int s, int t, int ts, int tt, int nc,
                    float t0, float t1, float cfl) {
    tools::LevelSetAdvection<FloatGrid, FieldT> adv(grid, field);
    adv.setSpatialScheme(math::BiasedGradientScheme(s));
    adv.setTemporalScheme(math::TemporalIntegrationScheme(t));
    adv.setTrackerSpatialScheme(math::BiasedGradientScheme(ts));
    adv.setTrackerTemporalScheme(math::TemporalIntegrationScheme(tt));
    adv.setNormCount(nc);
    size_t count = 0;
    if (math::isZero(t0 - t1)) return 0;
    const bool fwd = t0 < t1;
    const float dx = float(grid.voxelSize()[0]);
    float tau = t0;
    while (fwd ? tau < t1 : tau > t1) {
        if (grid.tree().leafCount() == 0) break;
        const float m = maxSpeedSqr(grid, field, tau);
        if (math::isApproxZero(m, math::Delta<float>::value())) break;
        const float lim = cfl * dx / std::sqrt(m);
        const float span = std::fabs(t1 - tau);
        const float end = (lim < span) ? (fwd ? tau + lim : tau - lim) : t1;
        if (end - tau == 0.0f) break;
        count += adv.advect(tau, end);
        tau = end;
    }
    return count;
}

void configureTracker(tools::LevelSetTracker<FloatGrid>& tr, int ts, int tt, int nc, int trim) {
    tr.setSpatialScheme(math::BiasedGradientScheme(ts));
    tr.setTemporalScheme(math::TemporalIntegrationScheme(tt));
    tr.setNormCount(nc);
    tr.setTrimming(tools::lstrack::TrimMode(trim));
}

}  // namespace

extern "C" {

const char* vdbref_last_error() { return gLastError.c_str(); }

int vdbref_init() { return 0; }

int vdbref_set_threads(int n) {
    tbb::shim::Pool::instance().resize(n);
    return 0;
}

int vdbref_threads() { return tbb::shim::Pool::instance().threads(); }

void vdbref_free(void* g) { delete static_cast<RefGrid*>(g); }

// tools/LevelSetSphere.h:219-230
int vdbref_sphere(float radius, float cx, float cy, float cz, float dx, float hw, void** out) {
    try {
        auto* rg = new RefGrid;
        rg->grid = tools::createLevelSetSphere<FloatGrid>(radius, Vec3f(cx, cy, cz), dx, hw);
        *out = rg;
        return 0;
    } catch (const std::exception& e) {
        return fail(GBLS_ERR_VALUE, e.what());
    }
}

// Sequential csgUnion of spheres (tools/Composite.h:886).
int vdbref_union_spheres(int n, const float* centers, const float* radii, float dx, float hw,
                         void** out) {
    try {
        FloatGrid::Ptr acc;
        for (int i = 0; i < n; ++i) {
            FloatGrid::Ptr s = tools::createLevelSetSphere<FloatGrid>(
                radii[i], Vec3f(centers[3 * i], centers[3 * i + 1], centers[3 * i + 2]), dx, hw);
            if (!acc) acc = s;
            else tools::csgUnion(*acc, *s);
        }
        auto* rg = new RefGrid;
        rg->grid = acc;
        *out = rg;
        return 0;
    } catch (const std::exception& e) {
        return fail(GBLS_ERR_VALUE, e.what());
    }
}

int vdbref_counts(void* g, gbls_grid_counts* c) {
    const FloatTree& tree = static_cast<RefGrid*>(g)->grid->tree();
    const RootT& root = tree.root();
    int64_t nu = 0, nl = 0, nleaf = 0, nt = 0;
    for (auto it = root.cbeginChildOn(); it; ++it) {
        ++nu;
        for (auto lit = it->cbeginChildOn(); lit; ++lit) {
            ++nl;
            for (auto fit = lit->cbeginChildOn(); fit; ++fit) ++nleaf;
        }
    }
    for (auto it = root.cbeginValueAll(); it; ++it) ++nt;
    c->leaf_count = nleaf;
    c->lower_count = nl;
    c->upper_count = nu;
    c->root_tile_count = nt;
    c->active_voxel_count = int64_t(tree.activeVoxelCount());
    return 0;
}

// Canonical export: tree order everywhere, 0.0f at child slots of tile tables.
int vdbref_export(void* g, gbls_grid_desc* d) {
    const FloatGrid& grid = *static_cast<RefGrid*>(g)->grid;
    const FloatTree& tree = grid.tree();
    const RootT& root = tree.root();
    const math::Transform& xf = grid.transform();
    d->voxel_size = grid.voxelSize()[0];
    const Vec3d t = xf.indexToWorld(Vec3d(0, 0, 0));
    d->translation[0] = t[0];
    d->translation[1] = t[1];
    d->translation[2] = t[2];
    d->map_type = xf.mapType() == math::UniformScaleMap::mapType()   ? GBLS_MAP_UNIFORM_SCALE
                  : xf.mapType() == math::TranslationMap::mapType() ? GBLS_MAP_TRANSLATION
                                                                      : GBLS_MAP_UNIFORM_SCALE_TRANSLATE;
    d->background = tree.background();
    int64_t iu = 0, il = 0, ileaf = 0, it_ = 0;
    for (auto uit = root.cbeginChildOn(); uit; ++uit) {
        const UpperT& up = *uit;
        const Coord o = up.origin();
        std::memcpy(d->upper_origins + 3 * iu, o.data(), 12);
        float* ut = d->upper_tiles + size_t(iu) * UpperT::NUM_VALUES;
        for (Index n = 0; n < UpperT::NUM_VALUES; ++n) {
            if (up.getChildMask().isOn(n)) { ut[n] = 0.0f; continue; }
            if (up.getValueMask().isOn(n)) return fail(GBLS_ERR_UNSUPPORTED, "active tile");
            ut[n] = up.getTable()[n].getValue();
        }
        ++iu;
        for (auto lit = up.cbeginChildOn(); lit; ++lit) {
            const LowerT& lo = *lit;
            const Coord lo_o = lo.origin();
            std::memcpy(d->lower_origins + 3 * il, lo_o.data(), 12);
            float* lt = d->lower_tiles + size_t(il) * LowerT::NUM_VALUES;
            for (Index n = 0; n < LowerT::NUM_VALUES; ++n) {
                if (lo.getChildMask().isOn(n)) { lt[n] = 0.0f; continue; }
                if (lo.getValueMask().isOn(n)) return fail(GBLS_ERR_UNSUPPORTED, "active tile");
                lt[n] = lo.getTable()[n].getValue();
            }
            ++il;
            for (auto fit = lo.cbeginChildOn(); fit; ++fit) {
                const LeafT& leaf = *fit;
                const Coord lf_o = leaf.origin();
                std::memcpy(d->leaf_origins + 3 * ileaf, lf_o.data(), 12);
                for (int w = 0; w < 8; ++w)
                    d->leaf_masks[8 * ileaf + w] = leaf.getValueMask().template getWord<uint64_t>(w);
                std::memcpy(d->leaf_values + 512 * size_t(ileaf), leaf.buffer().data(), 2048);
                ++ileaf;
            }
        }
    }
    for (auto vit = root.cbeginValueAll(); vit; ++vit) {
        if (vit.isValueOn()) return fail(GBLS_ERR_UNSUPPORTED, "active root tile");
        const Coord c = vit.getCoord();
        std::memcpy(d->root_tile_origins + 3 * it_, c.data(), 12);
        d->root_tile_values[it_] = *vit;
        ++it_;
    }
    return 0;
}

int vdbref_from_desc(const gbls_grid_desc* d, void** out) {
    try {
        FloatGrid::Ptr grid = FloatGrid::create(d->background);
        math::Transform::Ptr xf = math::Transform::createLinearTransform(d->voxel_size);
        if (d->translation[0] != 0.0 || d->translation[1] != 0.0 || d->translation[2] != 0.0)
            xf->postTranslate(Vec3d(d->translation[0], d->translation[1], d->translation[2]));
        grid->setTransform(xf);
        grid->setGridClass(GRID_LEVEL_SET);
        FloatTree& tree = grid->tree();
        for (int64_t i = 0; i < d->root_tile_count; ++i) {
            const int32_t* o = d->root_tile_origins + 3 * i;
            tree.addTile(3, Coord(o[0], o[1], o[2]), d->root_tile_values[i], false);
        }
        // child slots of every internal node, from the node lists below it
        std::vector<std::vector<char>> upperChild(d->upper_count,
                                                  std::vector<char>(UpperT::NUM_VALUES, 0));
        std::vector<std::vector<char>> lowerChild(d->lower_count,
                                                  std::vector<char>(LowerT::NUM_VALUES, 0));
        auto findUpper = [&](const int32_t* o) -> int64_t {
            for (int64_t u = 0; u < d->upper_count; ++u) {
                const int32_t* uo = d->upper_origins + 3 * u;
                if ((o[0] & ~4095) == uo[0] && (o[1] & ~4095) == uo[1] && (o[2] & ~4095) == uo[2])
                    return u;
            }
            return -1;
        };
        std::vector<int64_t> lowerIndexOfLeaf(d->leaf_count, -1);
        for (int64_t l = 0; l < d->lower_count; ++l) {
            const int32_t* lo = d->lower_origins + 3 * l;
            const int64_t u = findUpper(lo);
            if (u < 0) return fail(GBLS_ERR_INVALID_ARGUMENT, "lower node without upper node");
            const int n = (((lo[0] >> 7) & 31) << 10) | (((lo[1] >> 7) & 31) << 5) | ((lo[2] >> 7) & 31);
            upperChild[u][n] = 1;
        }
        for (int64_t f = 0; f < d->leaf_count; ++f) {
            const int32_t* fo = d->leaf_origins + 3 * f;
            for (int64_t l = 0; l < d->lower_count; ++l) {
                const int32_t* lo = d->lower_origins + 3 * l;
                if ((fo[0] & ~127) == lo[0] && (fo[1] & ~127) == lo[1] && (fo[2] & ~127) == lo[2]) {
                    const int n = (((fo[0] >> 3) & 15) << 8) | (((fo[1] >> 3) & 15) << 4) | ((fo[2] >> 3) & 15);
                    lowerChild[l][n] = 1;
                    lowerIndexOfLeaf[f] = l;
                    break;
                }
            }
            if (lowerIndexOfLeaf[f] < 0) return fail(GBLS_ERR_INVALID_ARGUMENT, "leaf without lower node");
        }
        for (int64_t u = 0; u < d->upper_count; ++u) {
            const int32_t* uo = d->upper_origins + 3 * u;
            const float* ut = d->upper_tiles + size_t(u) * UpperT::NUM_VALUES;
            for (int n = 0; n < int(UpperT::NUM_VALUES); ++n) {
                if (upperChild[u][n]) continue;
                const Coord c(uo[0] + ((n >> 10) & 31) * 128, uo[1] + ((n >> 5) & 31) * 128,
                              uo[2] + (n & 31) * 128);
                tree.addTile(2, c, ut[n], false);
            }
        }
        for (int64_t l = 0; l < d->lower_count; ++l) {
            const int32_t* lo = d->lower_origins + 3 * l;
            const float* lt = d->lower_tiles + size_t(l) * LowerT::NUM_VALUES;
            for (int n = 0; n < int(LowerT::NUM_VALUES); ++n) {
                if (lowerChild[l][n]) continue;
                const Coord c(lo[0] + ((n >> 8) & 15) * 8, lo[1] + ((n >> 4) & 15) * 8,
                              lo[2] + (n & 15) * 8);
                tree.addTile(1, c, lt[n], false);
            }
        }
        for (int64_t f = 0; f < d->leaf_count; ++f) {
            const int32_t* fo = d->leaf_origins + 3 * f;
            LeafT* leaf = tree.touchLeaf(Coord(fo[0], fo[1], fo[2]));
            std::memcpy(leaf->buffer().data(), d->leaf_values + 512 * size_t(f), 2048);
            for (int w = 0; w < 8; ++w)
                leaf->getValueMask().template getWord<uint64_t>(w) = d->leaf_masks[8 * f + w];
        }
        auto* rg = new RefGrid;
        rg->grid = grid;
        *out = rg;
        return 0;
    } catch (const std::exception& e) {
        return fail(GBLS_ERR_VALUE, e.what());
    }
}

// tools::LevelSetAdvection<FloatGrid, FieldT>::advect with the given schemes.
// tools::LevelSetFilter<FloatGrid>: op 0 laplacian, 1 mean(width),
// 2 gaussian(width), 3 offset(value), 4 meanCurvature, 5 fillet,
// 6 median(width), with the given tracker state.
// With `mask` (may be null): the filter's alpha-mask argument, with
// setMaskRange(minMask, maxMask) and invertMask(invert).
int vdbref_filter_masked(void* g, void* mask, int op, int width, float value, int tspatial, int ttemporal,
                         int normCount, int trim, float minMask, float maxMask, int invert) {
    try {
        FloatGrid& grid = *static_cast<RefGrid*>(g)->grid;
        tools::LevelSetFilter<FloatGrid, FloatGrid> f(grid);
        f.setSpatialScheme(math::BiasedGradientScheme(tspatial));
        f.setTemporalScheme(math::TemporalIntegrationScheme(ttemporal));
        f.setNormCount(normCount);
        f.setTrimming(tools::lstrack::TrimMode(trim));
        const FloatGrid* m = mask ? static_cast<RefGrid*>(mask)->grid.get() : nullptr;
        if (m) {
            f.setMaskRange(minMask, maxMask);
            f.invertMask(invert != 0);
        }
        switch (op) {
        case 0: f.laplacian(m); break;
        case 1: f.mean(width, m); break;
        case 2: f.gaussian(width, m); break;
        case 3: f.offset(value, m); break;
        case 4: f.meanCurvature(m); break;
        case 5: f.fillet(m); break;
        case 6: f.median(width, m); break;
        default: return fail(GBLS_ERR_VALUE, "unknown filter");
        }
        return 0;
    } catch (const std::exception& e) {
        return fail(GBLS_ERR_VALUE, e.what());
    }
}

int vdbref_filter(void* g, int op, int width, float value, int tspatial, int ttemporal, int normCount, int trim) {
    return vdbref_filter_masked(g, nullptr, op, width, value, tspatial, ttemporal, normCount, trim, 0.0f, 1.0f, 0);
}

// tools::LevelSetMorphing<FloatGrid>::advect towards `target`, with an
// optional alpha mask (mask may be null).
int vdbref_morph(void* g, void* target, void* mask, int spatial, int temporal, int tspatial, int ttemporal,
                 int normCount, float t0, float t1, float minMask, float maxMask, int invert, uint64_t* count) {
    try {
        FloatGrid& grid = *static_cast<RefGrid*>(g)->grid;
        const FloatGrid& tgt = *static_cast<RefGrid*>(target)->grid;
        tools::LevelSetMorphing<FloatGrid> morph(grid, tgt);
        if (mask) {
            morph.setAlphaMask(*static_cast<RefGrid*>(mask)->grid);
            morph.setMaskRange(minMask, maxMask);
            morph.invertMask(invert != 0);
        }
        morph.setSpatialScheme(math::BiasedGradientScheme(spatial));
        morph.setTemporalScheme(math::TemporalIntegrationScheme(temporal));
        morph.setTrackerSpatialScheme(math::BiasedGradientScheme(tspatial));
        morph.setTrackerTemporalScheme(math::TemporalIntegrationScheme(ttemporal));
        morph.setNormCount(normCount);
        const size_t n = morph.advect(t0, t1);
        if (count) *count = n;
        return 0;
    } catch (const std::exception& e) {
        return fail(GBLS_ERR_VALUE, e.what());
    }
}

// cfl <= 0: the reference's advect(t0, t1); cfl > 0: runAdvectCfl.
int vdbref_advect_cfl(void* g, const gbls_field_desc* f, int spatial, int temporal, int tspatial,
                      int ttemporal, int normCount, float t0, float t1, float cfl, uint64_t* count) {
    try {
        FloatGrid& grid = *static_cast<RefGrid*>(g)->grid;
        size_t n = 0;
        auto run = [&](const auto& field) {
            return cfl > 0.0f
                ? runAdvectCfl(grid, field, spatial, temporal, tspatial, ttemporal, normCount, t0, t1, cfl)
                : runAdvect(grid, field, spatial, temporal, tspatial, ttemporal, normCount, t0, t1);
        };
        if (f->kind == GBLS_FIELD_CONSTANT || f->kind == GBLS_FIELD_DENSE) {
            Vec3fGrid::Ptr vel = makeVelocityGrid(*f, grid.transform());
            tools::DiscreteField<Vec3fGrid> field(*vel);
            n = run(field);
        } else {
            AnalyticField field;
            field.desc = *f;
            field.xform = grid.transform().copy();
            n = run(field);
        }
        if (count) *count = n;
        return 0;
    } catch (const std::exception& e) {
        return fail(GBLS_ERR_VALUE, e.what());
    }
}

// LevelSetAdvection<FloatGrid> with its default field, tools::EnrightField<float>.
int vdbref_advect_enright(void* g, int spatial, int temporal, int tspatial, int ttemporal, int normCount, float t0,
                          float t1, float cfl, uint64_t* count) {
    try {
        FloatGrid& grid = *static_cast<RefGrid*>(g)->grid;
        tools::EnrightField<float> field;
        const size_t n = cfl > 0.0f
            ? runAdvectCfl(grid, field, spatial, temporal, tspatial, ttemporal, normCount, t0, t1, cfl)
            : runAdvect(grid, field, spatial, temporal, tspatial, ttemporal, normCount, t0, t1);
        if (count) *count = n;
        return 0;
    } catch (const std::exception& e) {
        return fail(GBLS_ERR_VALUE, e.what());
    }
}

// tools::VolumeAdvection<Vec3fGrid, false>::advect<FloatGrid, Sampler<1, false>>
// (tools/VolumeAdvect.h:205-222): the grid is replaced by the advected copy.
// The velocity grid comes from the dense descriptor (its own transform, or
// the volume's); max_velocity receives getMaxVelocity().
int vdbref_volume_advect(void* g, const gbls_field_desc* f, int integrator, int limiter, int substeps,
                         double time_step, double* max_velocity) {
    try {
        RefGrid* r = static_cast<RefGrid*>(g);
        Vec3fGrid::Ptr vel = makeVelocityGrid(*f, r->grid->transform());
        tools::VolumeAdvection<Vec3fGrid, false> adv(*vel);
        adv.setIntegrator(tools::Scheme::SemiLagrangian(integrator));
        adv.setLimiter(tools::Scheme::Limiter(limiter));
        adv.setSubSteps(substeps);
        if (max_velocity) *max_velocity = adv.getMaxVelocity();
        r->grid = adv.advect<FloatGrid, tools::Sampler<1, false>>(*r->grid, time_step);
        return 0;
    } catch (const std::exception& e) {
        return fail(GBLS_ERR_VALUE, e.what());
    }
}

int vdbref_advect(void* g, const gbls_field_desc* f, int spatial, int temporal, int tspatial,
                  int ttemporal, int normCount, float t0, float t1, uint64_t* count) {
    return vdbref_advect_cfl(g, f, spatial, temporal, tspatial, ttemporal, normCount, t0, t1, 0.0f, count);
}

// LevelSetTracker::normalize(&mask) with a MaskTree holding the given leaf
// origins and active masks.
int vdbref_normalize_masked(void* g, int64_t n, const int32_t* origins, const uint64_t* masks, int tspatial,
                            int ttemporal, int normCount, int trim) {
    try {
        FloatGrid& grid = *static_cast<RefGrid*>(g)->grid;
        MaskTree mask;
        for (int64_t i = 0; i < n; ++i) {
            auto* leaf = mask.touchLeaf(Coord(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]));
            for (int w = 0; w < 8; ++w) leaf->getValueMask().template getWord<uint64_t>(w) = masks[8 * i + w];
        }
        tools::LevelSetTracker<FloatGrid> tr(grid);
        configureTracker(tr, tspatial, ttemporal, normCount, trim);
        tr.normalize(&mask);
        return 0;
    } catch (const std::exception& e) {
        return fail(GBLS_ERR_VALUE, e.what());
    }
}

// op: 0 track, 1 normalize, 2 prune, 3 dilate(arg), 4 erode(arg), 5 resize(arg)
int vdbref_tracker_op(void* g, int op, int arg, int tspatial, int ttemporal, int normCount,
                      int trim, int* result) {
    try {
        FloatGrid& grid = *static_cast<RefGrid*>(g)->grid;
        tools::LevelSetTracker<FloatGrid> tr(grid);
        configureTracker(tr, tspatial, ttemporal, normCount, trim);
        int r = 0;
        switch (op) {
        case 0: tr.track(); break;
        case 1: tr.normalize(); break;
        case 2: tr.prune(); break;
        case 3: tr.dilate(arg); break;
        case 4: tr.erode(arg); break;
        case 5: r = tr.resize(Index(arg)) ? 1 : 0; break;
        default: return fail(GBLS_ERR_INVALID_ARGUMENT, "bad tracker op");
        }
        if (result) *result = r;
        return 0;
    } catch (const std::exception& e) {
        return fail(GBLS_ERR_RUNTIME, e.what());
    }
}

}  // extern "C"

namespace vdbref_detail {
openvdb::FloatGrid::Ptr grid_of(void* g) { return static_cast<RefGrid*>(g)->grid; }
}

extern "C" {

// ---- .vdb files through the reference's own serialisers ---------------------
// io/Archive.cc needs Boost and is not built, so the file framing around the
// grid record is restated here (header: io/Archive.cc:1010-1080; file
// metadata, grid count and one grid record: io/Archive.cc:1269-1450); every
// byte inside the record comes from the reference: io::GridDescriptor::
// writeHeader/writeStreamPos, MetaMap::writeMeta, math::Transform::write,
// Grid::writeTopology and Grid::writeBuffers, with the stream's compression
// set to COMPRESS_ACTIVE_MASK (a build without Blosc/zlib).  The grid carries
// class, name and the statistics io::Archive adds (file_bbox_min/max,
// file_voxel_count, file_compression), not file_mem_bytes or the
// delayed-load record.  `uuid36` is written verbatim so files compare
// byte for byte.

void registerIoTypes() {
    static bool done = false;
    if (done) return;
    done = true;
    if (!FloatGrid::isRegistered()) FloatGrid::registerGrid();
    if (!math::UniformScaleMap::isRegistered()) math::UniformScaleMap::registerMap();
    if (!math::UniformScaleTranslateMap::isRegistered()) math::UniformScaleTranslateMap::registerMap();
    if (!math::TranslationMap::isRegistered()) math::TranslationMap::registerMap();
    if (!math::ScaleMap::isRegistered()) math::ScaleMap::registerMap();
    if (!math::ScaleTranslateMap::isRegistered()) math::ScaleTranslateMap::registerMap();
    if (!math::AffineMap::isRegistered()) math::AffineMap::registerMap();
    if (!StringMetadata::isRegisteredType()) StringMetadata::registerType();
    if (!Vec3IMetadata::isRegisteredType()) Vec3IMetadata::registerType();
    if (!Int64Metadata::isRegisteredType()) Int64Metadata::registerType();
    if (!BoolMetadata::isRegisteredType()) BoolMetadata::registerType();
}

int vdbref_write_vdb(void* g, const char* name, const char* path, const char* uuid36, int half) {
    try {
        registerIoTypes();
        FloatGrid& src = *static_cast<RefGrid*>(g)->grid;
        GridBase::Ptr copy = src.copyGrid();
        copy->setName(name);
        copy->setGridClass(GRID_LEVEL_SET);
        if (half) copy->setSaveFloatAsHalf(true);
        const uint32_t compression = io::COMPRESS_ACTIVE_MASK;
        const CoordBBox bbox = copy->evalActiveVoxelBoundingBox();
        copy->insertMeta(GridBase::META_FILE_BBOX_MIN, Vec3IMetadata(bbox.min().asVec3i()));
        copy->insertMeta(GridBase::META_FILE_BBOX_MAX, Vec3IMetadata(bbox.max().asVec3i()));
        copy->insertMeta(GridBase::META_FILE_VOXEL_COUNT, Int64Metadata(copy->activeVoxelCount()));
        copy->insertMeta(GridBase::META_FILE_COMPRESSION, StringMetadata(io::compressionToString(compression)));

        std::ofstream os(path, std::ios::binary | std::ios::trunc);
        if (!os) return fail(GBLS_ERR_RUNTIME, "cannot open output file");
        io::setVersion(os, VersionId(OPENVDB_LIBRARY_MAJOR_VERSION, OPENVDB_LIBRARY_MINOR_VERSION),
                       OPENVDB_FILE_VERSION);
        io::setDataCompression(os, compression);
        const int64_t magic = OPENVDB_MAGIC;
        os.write(reinterpret_cast<const char*>(&magic), 8);
        uint32_t v = OPENVDB_FILE_VERSION;
        os.write(reinterpret_cast<const char*>(&v), 4);
        v = OPENVDB_LIBRARY_MAJOR_VERSION;
        os.write(reinterpret_cast<const char*>(&v), 4);
        v = OPENVDB_LIBRARY_MINOR_VERSION;
        os.write(reinterpret_cast<const char*>(&v), 4);
        const char seekable = 1;
        os.write(&seekable, 1);
        os.write(uuid36, 36);
        MetaMap().writeMeta(os);
        const int32_t count = 1;
        os.write(reinterpret_cast<const char*>(&count), 4);

        io::GridDescriptor gd(name, copy->type(), copy->saveFloatAsHalf());
        gd.writeHeader(os);
        const int64_t offsetPos = int64_t(os.tellp());
        gd.writeStreamPos(os);
        gd.setGridPos(os.tellp());
        os.write(reinterpret_cast<const char*>(&compression), 4);
        copy->writeMeta(os);
        copy->writeTransform(os);
        copy->writeTopology(os);
        gd.setBlockPos(os.tellp());
        copy->writeBuffers(os);
        gd.setEndPos(os.tellp());
        os.seekp(offsetPos, std::ios_base::beg);
        gd.writeStreamPos(os);
        gd.seekToEnd(os);
        if (!os) return fail(GBLS_ERR_RUNTIME, "write failed");
        return 0;
    } catch (const std::exception& e) {
        return fail(GBLS_ERR_RUNTIME, e.what());
    }
}

// Reads grid `name` (unique name or grid name) with the reference's
// io::GridDescriptor::read, Grid::readMeta/readTransform/readTopology/
// readBuffers; the header is parsed as io::Archive::readHeader does.
int vdbref_read_vdb(const char* path, const char* name, void** out) {
    try {
        registerIoTypes();
        std::ifstream is(path, std::ios::binary);
        if (!is) return fail(GBLS_ERR_RUNTIME, "cannot open input file");
        int64_t magic = 0;
        uint32_t fileVersion = 0, major = 0, minor = 0;
        char hasOffsets = 0;
        char uuid[36];
        is.read(reinterpret_cast<char*>(&magic), 8);
        is.read(reinterpret_cast<char*>(&fileVersion), 4);
        is.read(reinterpret_cast<char*>(&major), 4);
        is.read(reinterpret_cast<char*>(&minor), 4);
        is.read(&hasOffsets, 1);
        is.read(uuid, 36);
        if (!is || magic != OPENVDB_MAGIC) return fail(GBLS_ERR_RUNTIME, "not a VDB file");
        io::setVersion(is, VersionId(major, minor), fileVersion);
        MetaMap fileMeta;
        fileMeta.readMeta(is);
        int32_t count = 0;
        is.read(reinterpret_cast<char*>(&count), 4);
        for (int32_t i = 0; i < count; ++i) {
            io::GridDescriptor gd;
            GridBase::Ptr grid = gd.read(is);
            if (gd.uniqueName() != name && gd.gridName() != name) {
                if (!hasOffsets) return fail(GBLS_ERR_UNSUPPORTED, "grid skipping needs grid offsets");
                gd.seekToEnd(is);
                continue;
            }
            uint32_t c = 0;
            is.read(reinterpret_cast<char*>(&c), 4);
            io::setDataCompression(is, c);
            grid->readMeta(is);
            grid->readTransform(is);
            grid->readTopology(is);
            grid->readBuffers(is);
            FloatGrid::Ptr fg = GridBase::grid<FloatGrid>(grid);
            if (!fg) return fail(GBLS_ERR_UNSUPPORTED, "not a FloatGrid");
            auto* rg = new RefGrid;
            rg->grid = fg;
            *out = rg;
            return 0;
        }
        return fail(GBLS_ERR_INVALID_ARGUMENT, std::string("no grid named ") + name);
    } catch (const std::exception& e) {
        return fail(GBLS_ERR_RUNTIME, e.what());
    }
}

}  // extern "C"

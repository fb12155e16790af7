// Host side of the C++ drop-in: conversion between an OpenVDB level-set
// grid (Tree4<float,5,4,3>) and the exchange descriptor of the C ABI
// (gbls_grid_desc), status codes rethrown as the exception types OpenVDB's
// LevelSetAdvection / LevelSetTracker throw, and the velocity-field traits.
//
// Header-only; include it from a translation unit that is compiled against
// OpenVDB and link libgbls.so.  Nothing here runs device code: every device
// operation goes through the functions declared in gbls.h.
#pragma once

#include <openvdb/Exceptions.h>
#include <openvdb/Grid.h>
#include <openvdb/math/Transform.h>
#include <openvdb/tools/VelocityFields.h>
#include <openvdb/tree/LeafNode.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "../gbls.h"

namespace openvdb_gb300 {
namespace detail {

// Status -> the exception the reference throws for the same condition
// (tools/LevelSetTracker.h:267-276: RuntimeError for a non-uniform transform
// or a non-level-set; tools/LevelSetAdvect.h:232,251,273: ValueError for an
// unsupported scheme or map).  GBLS_ERR_INTERRUPTED is not an error: the
// reference ends the substep loop and returns the count so far.
inline void check(int rc) {
    if (rc == GBLS_OK || rc == GBLS_ERR_INTERRUPTED) return;
    const std::string msg = gbls_last_error() ? gbls_last_error() : "";
    switch (rc) {
    case GBLS_ERR_VALUE: OPENVDB_THROW(openvdb::ValueError, msg);
    case GBLS_ERR_RUNTIME: OPENVDB_THROW(openvdb::RuntimeError, msg);
    case GBLS_ERR_INVALID_ARGUMENT: OPENVDB_THROW(openvdb::ValueError, msg);
    case GBLS_ERR_DOMAIN: OPENVDB_THROW(openvdb::IndexError, msg);
    case GBLS_ERR_UNSUPPORTED: OPENVDB_THROW(openvdb::NotImplementedError, msg);
    case GBLS_ERR_OUT_OF_MEMORY: throw std::bad_alloc();
    default: OPENVDB_THROW(openvdb::RuntimeError, "gbls status " + std::to_string(rc) + ": " + msg);
    }
}

// Host storage behind one gbls_grid_desc.
struct HostGrid {
    double voxel_size = 1.0;
    double translation[3] = {0.0, 0.0, 0.0};
    int32_t map_type = GBLS_MAP_UNIFORM_SCALE;
    float background = 0.0f;
    std::vector<int32_t> leaf_origins, lower_origins, upper_origins, root_tile_origins;
    std::vector<uint64_t> leaf_masks;
    std::vector<float> leaf_values, lower_tiles, upper_tiles, root_tile_values;

    void resize(const gbls_grid_counts& c) {
        leaf_origins.resize(size_t(c.leaf_count) * 3);
        leaf_masks.resize(size_t(c.leaf_count) * 8);
        leaf_values.resize(size_t(c.leaf_count) * 512);
        lower_origins.resize(size_t(c.lower_count) * 3);
        lower_tiles.resize(size_t(c.lower_count) * 4096);
        upper_origins.resize(size_t(c.upper_count) * 3);
        upper_tiles.resize(size_t(c.upper_count) * 32768);
        root_tile_origins.resize(size_t(c.root_tile_count) * 3);
        root_tile_values.resize(size_t(c.root_tile_count));
    }

    gbls_grid_desc desc() {
        gbls_grid_desc d{};
        d.voxel_size = voxel_size;
        for (int i = 0; i < 3; ++i) d.translation[i] = translation[i];
        d.map_type = map_type;
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
        d.root_tile_count = int64_t(root_tile_origins.size() / 3);
        d.root_tile_origins = root_tile_origins.data();
        d.root_tile_values = root_tile_values.data();
        return d;
    }
};

template <typename GridT>
struct TreeLevels {
    using TreeT = typename GridT::TreeType;
    using RootT = typename TreeT::RootNodeType;
    using UpperT = typename RootT::ChildNodeType;
    using LowerT = typename UpperT::ChildNodeType;
    using LeafT = typename LowerT::ChildNodeType;
    static_assert(std::is_same<typename TreeT::ValueType, float>::value,
                  "the device path holds FP32 level sets (FloatGrid)");
    static_assert(UpperT::NUM_VALUES == 32768 && LowerT::NUM_VALUES == 4096 && LeafT::NUM_VALUES == 512,
                  "the device path uses the Tree4<float,5,4,3> configuration");
};

// Transform -> (voxel size, translation, map type); the tracker's own check
// (uniform scale) is repeated by gbls_create.
inline void exportTransform(const openvdb::math::Transform& xf, HostGrid& h) {
    const openvdb::Vec3d vs = xf.voxelSize();
    h.voxel_size = vs[0];
    if (!(vs[0] == vs[1] && vs[1] == vs[2]) || !xf.isLinear())
        OPENVDB_THROW(openvdb::RuntimeError,
                      "The transform must have uniform scale for the LevelSetTracker to function");
    const openvdb::Vec3d t = xf.indexToWorld(openvdb::Vec3d(0.0, 0.0, 0.0));
    for (int i = 0; i < 3; ++i) h.translation[i] = t[i];
    const openvdb::Name mt = xf.mapType();
    h.map_type = mt == openvdb::math::UniformScaleMap::mapType()   ? GBLS_MAP_UNIFORM_SCALE
                 : mt == openvdb::math::TranslationMap::mapType() ? GBLS_MAP_TRANSLATION
                                                                    : GBLS_MAP_UNIFORM_SCALE_TRANSLATE;
}

// Grid -> exchange format, tree order, 0 at child slots of tile tables.
// Active tiles have no device representation (a level set has none).
template <typename GridT>
HostGrid pack(const GridT& grid) {
    using L = TreeLevels<GridT>;
    const auto& root = grid.tree().root();
    HostGrid h;
    exportTransform(grid.transform(), h);
    h.background = grid.tree().background();
    for (auto uit = root.cbeginChildOn(); uit; ++uit) {
        const typename L::UpperT& up = *uit;
        h.upper_origins.insert(h.upper_origins.end(), up.origin().data(), up.origin().data() + 3);
        const size_t ub = h.upper_tiles.size();
        h.upper_tiles.resize(ub + L::UpperT::NUM_VALUES, 0.0f);
        for (auto t = up.cbeginValueAll(); t; ++t) {
            if (t.isValueOn()) OPENVDB_THROW(openvdb::NotImplementedError, "active tile in a level set");
            h.upper_tiles[ub + t.pos()] = *t;
        }
        for (auto lit = up.cbeginChildOn(); lit; ++lit) {
            const typename L::LowerT& lo = *lit;
            h.lower_origins.insert(h.lower_origins.end(), lo.origin().data(), lo.origin().data() + 3);
            const size_t lb = h.lower_tiles.size();
            h.lower_tiles.resize(lb + L::LowerT::NUM_VALUES, 0.0f);
            for (auto t = lo.cbeginValueAll(); t; ++t) {
                if (t.isValueOn()) OPENVDB_THROW(openvdb::NotImplementedError, "active tile in a level set");
                h.lower_tiles[lb + t.pos()] = *t;
            }
            for (auto fit = lo.cbeginChildOn(); fit; ++fit) {
                const typename L::LeafT& leaf = *fit;
                h.leaf_origins.insert(h.leaf_origins.end(), leaf.origin().data(), leaf.origin().data() + 3);
                for (int w = 0; w < 8; ++w) h.leaf_masks.push_back(leaf.getValueMask().template getWord<uint64_t>(w));
                const float* v = leaf.buffer().data();
                h.leaf_values.insert(h.leaf_values.end(), v, v + 512);
            }
        }
    }
    for (auto t = root.cbeginValueAll(); t; ++t) {
        if (t.isValueOn()) OPENVDB_THROW(openvdb::NotImplementedError, "active root tile in a level set");
        const openvdb::Coord c = t.getCoord();
        h.root_tile_origins.insert(h.root_tile_origins.end(), c.data(), c.data() + 3);
        h.root_tile_values.push_back(*t);
    }
    return h;
}

// Exchange format (tree order, as gbls_download writes it) -> the grid's
// tree, rebuilt in place: the Tree object stays, its nodes are replaced and
// its background takes the downloaded value (dilate/erode change it,
// tools/LevelSetTracker.h changeLevelSetBackground).  One linear walk: the
// lower nodes of an upper node and the leaves of a lower node are
// consecutive in tree order.
template <typename GridT>
void unpack(const HostGrid& h, GridT& grid) {
    using L = TreeLevels<GridT>;
    auto& tree = grid.tree();
    auto& root = tree.root();
    tree.clear();
    root.setBackground(h.background, /*updateChildNodes=*/false);
    const size_t nu = h.upper_origins.size() / 3, nl = h.lower_origins.size() / 3, nf = h.leaf_origins.size() / 3;
    auto coord = [](const std::vector<int32_t>& o, size_t i) { return openvdb::Coord(o[3 * i], o[3 * i + 1], o[3 * i + 2]); };
    size_t li = 0, fi = 0;
    for (size_t u = 0; u < nu; ++u) {
        const openvdb::Coord uo = coord(h.upper_origins, u);
        auto* up = new typename L::UpperT(uo, h.background, false);
        for (openvdb::Index n = 0; n < L::UpperT::NUM_VALUES; ++n)
            up->setValueOnlyUnsafe(n, h.upper_tiles[u * L::UpperT::NUM_VALUES + n]);
        for (; li < nl; ++li) {
            const openvdb::Coord lo = coord(h.lower_origins, li);
            if ((lo & ~(L::UpperT::DIM - 1)) != uo) break;
            auto* low = new typename L::LowerT(lo, h.background, false);
            for (openvdb::Index n = 0; n < L::LowerT::NUM_VALUES; ++n)
                low->setValueOnlyUnsafe(n, h.lower_tiles[li * L::LowerT::NUM_VALUES + n]);
            for (; fi < nf; ++fi) {
                const openvdb::Coord fo = coord(h.leaf_origins, fi);
                if ((fo & ~(L::LowerT::DIM - 1)) != lo) break;
                auto* leaf = new typename L::LeafT(fo, h.background, false);
                std::memcpy(leaf->buffer().data(), h.leaf_values.data() + fi * 512, 512 * sizeof(float));
                for (int w = 0; w < 8; ++w)
                    leaf->getValueMask().template getWord<uint64_t>(w) = h.leaf_masks[fi * 8 + w];
                low->addChild(leaf);
            }
            up->addChild(low);
        }
        root.addChild(up);
    }
    if (li != nl || fi != nf) OPENVDB_THROW(openvdb::ValueError, "exchange lists are not in tree order");
    for (size_t r = 0; r < h.root_tile_values.size(); ++r)
        root.addTile(coord(h.root_tile_origins, r), h.root_tile_values[r], false);
}

// Owner of one device-resident level set (gbls_handle).
class Handle {
public:
    Handle() = default;
    Handle(const Handle&) = delete;
    Handle& operator=(const Handle&) = delete;
    ~Handle() { reset(); }
    void reset() {
        if (mH) gbls_destroy(mH);
        mH = nullptr;
    }
    // Create on first use; later uploads keep the device allocations.
    template <typename GridT>
    void upload(const GridT& grid) {
        HostGrid h = pack(grid);
        gbls_grid_desc d = h.desc();
        if (mH) check(gbls_upload(mH, &d));
        else check(gbls_create(&d, &mH));
    }
    template <typename GridT>
    void download(GridT& grid) const {
        gbls_grid_counts c{};
        check(gbls_get_counts(mH, &c));
        HostGrid h;
        h.resize(c);
        gbls_grid_desc d = h.desc();
        check(gbls_download(mH, &d));
        h.voxel_size = d.voxel_size;
        h.background = d.background;
        unpack(h, grid);
    }
    gbls_handle* get() const { return mH; }

private:
    gbls_handle* mH = nullptr;
};

}  // namespace detail

// ---- velocity fields -------------------------------------------------------

// Analytic fields evaluated on the device (include/gbls_fields.h has their
// definitions).  Each is its own FieldT for LevelSetAdvection.
struct ConstantField {
    using VectorType = openvdb::Vec3f;
    openvdb::Vec3f velocity{0.0f, 0.0f, 0.0f};
};
// LeVeque's deformation on the unit cube mapped to `domain` voxels, scaled by
// cos(pi t / period) and by `scale` voxels per time unit.
struct DeformationField {
    using VectorType = openvdb::Vec3f;
    float domain = 1.0f, period = 1.0f, scale = 1.0f;
};
// Rigid motion: constant + omega x (ijk - center), index space.
struct RotationField {
    using VectorType = openvdb::Vec3f;
    openvdb::Vec3f constant{0.0f, 0.0f, 0.0f}, omega{0.0f, 0.0f, 0.0f}, center{0.0f, 0.0f, 0.0f};
};

// Storage a gbls_field_desc points into, alive for one advect call.
struct FieldStore {
    std::vector<float> values;        // a dense velocity box
    std::shared_ptr<void> context;    // a host sampler's state
};

namespace detail {
// Advect::sample<Aligned> (tools/LevelSetAdvect.h:476-493) over the active
// voxels the library hands to a HOST_SAMPLED field: field(ijk, t) when the
// field's transform equals the level set's, else field(map.applyMap(ijk), t).
template <typename FieldT>
struct HostSampler {
    const FieldT* field;
    openvdb::math::MapBase::ConstPtr map;
    bool aligned;
    static void sample(void* user, int64_t n, const int32_t* ijk, float t, float* velocity) {
        const HostSampler* s = static_cast<const HostSampler*>(user);
        for (int64_t i = 0; i < n; ++i) {
            const openvdb::Coord c(ijk[3 * i], ijk[3 * i + 1], ijk[3 * i + 2]);
            const auto v = s->aligned ? (*s->field)(c, t) : (*s->field)(s->map->applyMap(c.asVec3d()), t);
            velocity[3 * i] = float(v[0]);
            velocity[3 * i + 1] = float(v[1]);
            velocity[3 * i + 2] = float(v[2]);
        }
    }
};
}  // namespace detail

// How a FieldT reaches the device: describe() fills a gbls_field_desc (with
// storage kept alive in `store`) for advecting level set `ls` over [t0, t1].
// The primary template serves every functor with the reference's interface
// (tools/LevelSetAdvect.h:32-52), its default EnrightField included: the
// library samples it on the host once per substep, in the reference's voxel
// order (GBLS_FIELD_HOST_SAMPLED).  The specialisations below give the
// device forms of the fields it can evaluate itself.
template <typename FieldT>
struct FieldTraits {
    template <typename GridT>
    static gbls_field_desc describe(const FieldT& f, const GridT& ls, float, float, FieldStore& store) {
        auto s = std::make_shared<detail::HostSampler<FieldT>>();
        s->field = &f;
        s->map = ls.transform().baseMap();
        s->aligned = f.transform() == ls.transform();
        gbls_field_desc d{};
        d.kind = GBLS_FIELD_HOST_SAMPLED;
        d.host_sample = &detail::HostSampler<FieldT>::sample;
        d.host_user = s.get();
        store.context = s;
        return d;
    }
};

template <>
struct FieldTraits<ConstantField> {
    template <typename GridT>
    static gbls_field_desc describe(const ConstantField& f, const GridT&, float, float, FieldStore&) {
        gbls_field_desc d{};
        d.kind = GBLS_FIELD_CONSTANT;
        for (int i = 0; i < 3; ++i) d.constant[i] = f.velocity[i];
        return d;
    }
};

template <>
struct FieldTraits<DeformationField> {
    template <typename GridT>
    static gbls_field_desc describe(const DeformationField& f, const GridT&, float, float, FieldStore&) {
        gbls_field_desc d{};
        d.kind = GBLS_FIELD_DEFORMATION;
        d.domain = f.domain;
        d.period = f.period;
        d.scale = f.scale;
        return d;
    }
};

template <>
struct FieldTraits<RotationField> {
    template <typename GridT>
    static gbls_field_desc describe(const RotationField& f, const GridT&, float, float, FieldStore&) {
        gbls_field_desc d{};
        d.kind = GBLS_FIELD_ROTATION;
        for (int i = 0; i < 3; ++i) {
            d.constant[i] = f.constant[i];
            d.omega[i] = f.omega[i];
            d.center[i] = f.center[i];
        }
        return d;
    }
};

// Largest dense velocity box the DiscreteField form builds (voxels).
constexpr int64_t kMaxDenseFieldVoxels = int64_t(1) << 28;

// tools::DiscreteField over a Vec3 grid.  Aligned with the level set, the
// index-space lookup of sample<Aligned> (tools/LevelSetAdvect.h:470-478)
// reads field(ijk, t); otherwise every voxel samples the grid trilinearly at
// its world position (sample<false>), which the device reproduces from the
// grid's values and transform.  Either way the device form is a dense box of
// the grid's own values, read exactly through field(Coord, t) in the grid's
// index space, around the band: the level set's active bounding box mapped
// into the grid's index space and widened by the stencil and interpolation
// reach plus the distance the band can travel in [t0, t1] at the largest
// speed inside the box (widened again until that holds).  The grid
// transform must be a uniform scale and/or translation.
template <typename VelGridT, typename SamplerT>
struct FieldTraits<openvdb::tools::DiscreteField<VelGridT, SamplerT>> {
    using FieldT = openvdb::tools::DiscreteField<VelGridT, SamplerT>;
    template <typename GridT>
    static gbls_field_desc describe(const FieldT& f, const GridT& ls, float t0, float t1, FieldStore& fstore) {
        std::vector<float>& store = fstore.values;
        gbls_field_desc d{};
        d.kind = GBLS_FIELD_DENSE;
        openvdb::CoordBBox band;
        if (!ls.tree().evalActiveVoxelBoundingBox(band) || band.empty()) {
            d.kind = GBLS_FIELD_CONSTANT;
            return d;
        }
        const openvdb::math::Transform& vx = f.transform();
        const bool aligned = vx == ls.transform();
        double vox = ls.voxelSize()[0];
        if (!aligned) {
            detail::HostGrid tmp;
            detail::exportTransform(vx, tmp);  // throws unless a uniform linear map
            d.dense_map_type = 1 + tmp.map_type;
            d.dense_voxel_size = tmp.voxel_size;
            for (int i = 0; i < 3; ++i) d.dense_translation[i] = tmp.translation[i];
            vox = tmp.voxel_size;
            // the band's box in the velocity grid's index space
            openvdb::Vec3d lo(std::numeric_limits<double>::max()), hi(-std::numeric_limits<double>::max());
            for (int c = 0; c < 8; ++c) {
                const openvdb::Coord k((c & 1) ? band.max()[0] : band.min()[0], (c & 2) ? band.max()[1] : band.min()[1],
                                       (c & 4) ? band.max()[2] : band.min()[2]);
                const openvdb::Vec3d q = vx.worldToIndex(ls.transform().indexToWorld(k));
                for (int a = 0; a < 3; ++a) {
                    lo[a] = std::min(lo[a], q[a]);
                    hi[a] = std::max(hi[a], q[a]);
                }
            }
            band = openvdb::CoordBBox(openvdb::Coord(int(std::floor(lo[0])), int(std::floor(lo[1])), int(std::floor(lo[2]))),
                                      openvdb::Coord(int(std::ceil(hi[0])), int(std::ceil(hi[1])), int(std::ceil(hi[2]))));
        }
        // distance in grid voxels: the band may travel span * vmax world units
        const double span = std::fabs(double(t1) - double(t0)) / vox;
        const int reach = int(std::ceil(4.0 * ls.voxelSize()[0] / vox)) + 2;
        int margin = reach + 4;
        for (;;) {
            openvdb::CoordBBox box = band;
            box.expand(margin);
            const openvdb::Coord dim = box.dim();
            const int64_t nvox = int64_t(dim[0]) * dim[1] * dim[2];
            if (nvox > kMaxDenseFieldVoxels)
                OPENVDB_THROW(openvdb::NotImplementedError,
                              "DiscreteField around this band exceeds the dense device box limit");
            store.assign(size_t(nvox) * 3, 0.0f);
            double vmax = 0.0;
            size_t k = 0;
            for (int x = box.min()[0]; x <= box.max()[0]; ++x)
                for (int y = box.min()[1]; y <= box.max()[1]; ++y)
                    for (int z = box.min()[2]; z <= box.max()[2]; ++z) {
                        const auto v = f(openvdb::Coord(x, y, z), 0.0f);
                        for (int i = 0; i < 3; ++i) {
                            store[k++] = float(v[i]);
                            vmax = std::max(vmax, std::fabs(double(v[i])));
                        }
                    }
            const int need = int(std::ceil(span * vmax * std::sqrt(3.0))) + reach + 4;
            if (need <= margin) {
                for (int i = 0; i < 3; ++i) {
                    d.dense_origin[i] = box.min()[i];
                    d.dense_dims[i] = dim[i];
                    d.dense_background[i] = store[i];
                }
                d.dense_values = store.data();
                return d;
            }
            margin = need;
        }
    }
};

}  // namespace openvdb_gb300

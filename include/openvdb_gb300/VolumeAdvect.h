// Drop-in for openvdb::tools::VolumeAdvection (tools/VolumeAdvect.h:76-262)
// running on the GPU through the C ABI (gbls.h, gbls_volume_advect).
//
// Same template parameters, scheme and limiter enums
// (openvdb::tools::Scheme), constructor and member functions as the
// reference class.  advect<VolumeGridT, VolumeSamplerT>(grid, dt) packs the
// volume and the velocity grid, advects on the device and returns a new
// grid (a copy of the input's metadata and transform with the advected
// tree), like the reference.  Supported: FloatGrid volumes, a Vec3 velocity
// grid with a uniform-scale / translation transform, collocated velocities
// (StaggeredVelocity = false) and the trilinear sampler (Sampler<1, false>,
// BoxSampler).  Other instantiations and the masked advect() throw
// openvdb::NotImplementedError.
//
//   openvdb_gb300::tools::VolumeAdvection<openvdb::Vec3fGrid> advection(*velocity);
//   advection.setIntegrator(openvdb::tools::Scheme::MAC);
//   openvdb::FloatGrid::Ptr out =
//       advection.advect<openvdb::FloatGrid, openvdb::tools::Sampler<1, false>>(*density, 1.0);
#pragma once

#include <openvdb/tools/Statistics.h>
#include <openvdb/tools/VolumeAdvect.h>

#include <type_traits>

#include "GridExchange.h"

namespace openvdb_gb300 {
namespace detail {

// The velocity grid as a dense box covering every leaf and every tile whose
// value differs from the background (ValueAccessor::getValue at each box
// voxel, background outside); its transform unless it equals the volume's.
template <typename VelGridT, typename VolumeGridT>
gbls_field_desc describeVelocityGrid(const VelGridT& vel, const VolumeGridT& volume, std::vector<float>& store) {
    gbls_field_desc d{};
    const auto bg = vel.background();
    openvdb::CoordBBox box;
    for (auto leaf = vel.tree().cbeginLeaf(); leaf; ++leaf) box.expand(leaf->getNodeBoundingBox());
    for (auto t = vel.tree().cbeginValueAll(); t; ++t) {
        if (t.isVoxelValue() || *t == bg) continue;
        openvdb::CoordBBox tb;
        t.getBoundingBox(tb);
        box.expand(tb);
    }
    for (int i = 0; i < 3; ++i) d.dense_background[i] = float(bg[i]);
    if (box.empty()) {
        d.kind = GBLS_FIELD_CONSTANT;
        for (int i = 0; i < 3; ++i) d.constant[i] = float(bg[i]);
        return d;
    }
    const openvdb::Coord dim = box.dim();
    const int64_t n = int64_t(dim[0]) * dim[1] * dim[2];
    if (n > kMaxDenseFieldVoxels)
        OPENVDB_THROW(openvdb::NotImplementedError, "velocity grid exceeds the dense device box limit");
    d.kind = GBLS_FIELD_DENSE;
    store.assign(size_t(n) * 3, 0.0f);
    auto acc = vel.getConstAccessor();
    size_t k = 0;
    for (int x = box.min()[0]; x <= box.max()[0]; ++x)
        for (int y = box.min()[1]; y <= box.max()[1]; ++y)
            for (int z = box.min()[2]; z <= box.max()[2]; ++z) {
                const auto v = acc.getValue(openvdb::Coord(x, y, z));
                for (int i = 0; i < 3; ++i) store[k++] = float(v[i]);
            }
    for (int i = 0; i < 3; ++i) {
        d.dense_origin[i] = box.min()[i];
        d.dense_dims[i] = dim[i];
    }
    d.dense_values = store.data();
    if (!(vel.transform() == volume.transform())) {
        HostGrid tmp;
        exportTransform(vel.transform(), tmp);  // throws unless a uniform linear map
        d.dense_map_type = 1 + tmp.map_type;
        d.dense_voxel_size = tmp.voxel_size;
        for (int i = 0; i < 3; ++i) d.dense_translation[i] = tmp.translation[i];
    }
    return d;
}

}  // namespace detail

namespace tools {

namespace Scheme = openvdb::tools::Scheme;

template <typename VelocityGridT = openvdb::Vec3fGrid, bool StaggeredVelocity = false,
          typename InterrupterType = openvdb::util::NullInterrupter>
class VolumeAdvection {
public:
    VolumeAdvection(const VelocityGridT& velGrid, InterrupterType* interrupter = nullptr)
        : mVelGrid(velGrid), mInterrupter(interrupter), mIntegrator(Scheme::SEMI), mLimiter(Scheme::CLAMP),
          mGrainSize(128), mSubSteps(1) {
        // getMaxVelocity as the reference computes it (tools/VolumeAdvect.h:92-96)
        openvdb::math::Extrema e = openvdb::tools::extrema(velGrid.cbeginValueAll(), /*threaded=*/true);
        e.add(velGrid.background().length());
        mMaxVelocity = e.max();
    }
    virtual ~VolumeAdvection() = default;
    VolumeAdvection(const VolumeAdvection&) = delete;
    VolumeAdvection& operator=(const VolumeAdvection&) = delete;

    int spatialOrder() const { return (mIntegrator == Scheme::MAC || mIntegrator == Scheme::BFECC) ? 2 : 1; }
    int temporalOrder() const {
        switch (mIntegrator) {
        case Scheme::SEMI: return 1;
        case Scheme::MID: return 2;
        case Scheme::RK3: return 3;
        case Scheme::RK4: return 4;
        case Scheme::BFECC: return 2;
        case Scheme::MAC: return 2;
        }
        return 0;
    }
    void setIntegrator(Scheme::SemiLagrangian integrator) { mIntegrator = integrator; }
    Scheme::SemiLagrangian getIntegrator() const { return mIntegrator; }
    void setLimiter(Scheme::Limiter limiter) { mLimiter = limiter; }
    Scheme::Limiter getLimiter() const { return mLimiter; }
    bool isLimiterOn() const { return this->spatialOrder() > 1 && mLimiter != Scheme::NO_LIMITER; }
    size_t getGrainSize() const { return mGrainSize; }
    void setGrainSize(size_t grainsize) { mGrainSize = grainsize; }
    int getSubSteps() const { return mSubSteps; }
    void setSubSteps(int substeps) { mSubSteps = openvdb::math::Max(1, substeps); }
    double getMaxVelocity() const { return mMaxVelocity; }

    template <typename VolumeGridT>
    int getMaxDistance(const VolumeGridT& inGrid, double dt) const {
        if (!inGrid.hasUniformVoxels()) OPENVDB_THROW(openvdb::RuntimeError, "Volume grid does not have uniform voxels!");
        const double d = mMaxVelocity * openvdb::math::Abs(dt) / inGrid.voxelSize()[0];
        return static_cast<int>(openvdb::math::RoundUp(d));
    }

    // tools/VolumeAdvect.h:205-222
    template <typename VolumeGridT, typename VolumeSamplerT>
    typename VolumeGridT::Ptr advect(const VolumeGridT& inGrid, double timeStep) {
        if (StaggeredVelocity)
            OPENVDB_THROW(openvdb::NotImplementedError, "staggered velocity grids are not supported on the device");
        if (!std::is_same<typename VolumeGridT::ValueType, float>::value)
            OPENVDB_THROW(openvdb::NotImplementedError, "the device advects float volumes");
        if (VolumeSamplerT::order() != 1 || VolumeSamplerT::staggered())
            OPENVDB_THROW(openvdb::NotImplementedError, "the device samples volumes trilinearly (BoxSampler)");
        if (!inGrid.hasUniformVoxels()) OPENVDB_THROW(openvdb::RuntimeError, "Volume grid does not have uniform voxels!");
        detail::HostGrid h = detail::pack(inGrid);
        gbls_grid_desc d = h.desc();
        gbls_handle* handle = nullptr;
        detail::check(gbls_create_volume(&d, &handle));
        struct HandleGuard {
            gbls_handle* h;
            ~HandleGuard() { gbls_destroy(h); }
        } hguard{handle};
        std::vector<float> store;
        const gbls_field_desc fd = detail::describeVelocityGrid(mVelGrid, inGrid, store);
        gbls_field* field = nullptr;
        detail::check(gbls_field_create(&fd, &field));
        struct FieldGuard {
            gbls_field* f;
            ~FieldGuard() { gbls_field_destroy(f); }
        } fguard{field};
        if (mInterrupter) mInterrupter->start("Advecting volume");
        const int rc = gbls_volume_advect(handle, field, int(mIntegrator), int(mLimiter), mSubSteps, timeStep, nullptr);
        if (mInterrupter) mInterrupter->end();
        detail::check(rc);
        gbls_grid_counts c{};
        detail::check(gbls_get_counts(handle, &c));
        detail::HostGrid out;
        out.resize(c);
        gbls_grid_desc od = out.desc();
        detail::check(gbls_download(handle, &od));
        out.voxel_size = od.voxel_size;
        out.background = od.background;
        typename VolumeGridT::Ptr result = inGrid.copyWithNewTree();
        detail::unpack(out, *result);
        return result;
    }

    // tools/VolumeAdvect.h:248-280 (the masked form) is not on the device.
    template <typename VolumeGridT, typename MaskGridT, typename VolumeSamplerT>
    typename VolumeGridT::Ptr advect(const VolumeGridT&, const MaskGridT&, double) {
        OPENVDB_THROW(openvdb::NotImplementedError, "masked volume advection is not on the device");
    }

private:
    const VelocityGridT& mVelGrid;
    double mMaxVelocity;
    InterrupterType* mInterrupter;
    Scheme::SemiLagrangian mIntegrator;
    Scheme::Limiter mLimiter;
    size_t mGrainSize;
    int mSubSteps;
};

}  // namespace tools
}  // namespace openvdb_gb300

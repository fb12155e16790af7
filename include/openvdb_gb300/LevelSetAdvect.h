// Drop-in for openvdb::tools::LevelSetAdvection (tools/LevelSetAdvect.h:71-213)
// running on the GPU through the C ABI (gbls.h).
//
// Same template parameters, types, constructor and member functions as the
// reference class.  advect(t0, t1) uploads the grid and the velocity field,
// runs the whole CFL substep loop (RK stages + track() per substep) on the
// device and writes the result back into the same tree; it returns the
// number of CFL substeps, like the reference.  FieldT reaches the device
// through openvdb_gb300::FieldTraits (a tools::DiscreteField, aligned or
// with its own transform, or the analytic ConstantField / DeformationField /
// RotationField).  The device level set is kept between advect() calls.
//
//   openvdb::tools::DiscreteField<openvdb::Vec3SGrid> field(*velocity);
//   openvdb_gb300::tools::LevelSetAdvection<openvdb::FloatGrid,
//       openvdb::tools::DiscreteField<openvdb::Vec3SGrid>> advection(grid, field);
//   advection.setTemporalScheme(openvdb::math::TVD_RK3);
//   advection.setNormCount(1);
//   size_t substeps = advection.advect(0.0f, 1.0f);
//
// Difference: setCFL() is an addition (0, the default, keeps the reference's
// CFL number of the temporal scheme).
#pragma once

#include <openvdb/tools/LevelSetAdvect.h>

#include "LevelSetTracker.h"

namespace openvdb_gb300 {
namespace tools {

template <typename GridT, typename FieldT = openvdb::tools::EnrightField<typename GridT::ValueType>,
          typename InterruptT = openvdb::util::NullInterrupter>
class LevelSetAdvection {
public:
    using GridType = GridT;
    using TrackerT = LevelSetTracker<GridT, InterruptT>;
    using LeafRange = typename TrackerT::LeafRange;
    using LeafType = typename TrackerT::LeafType;
    using BufferType = typename TrackerT::BufferType;
    using ValueType = typename TrackerT::ValueType;
    using VectorType = typename FieldT::VectorType;

    // The field is copied, as in the reference (tools/LevelSetAdvect.h:209).
    LevelSetAdvection(GridT& grid, const FieldT& field, InterruptT* interrupt = nullptr)
        : mTracker(grid, interrupt), mField(field), mSpatialScheme(openvdb::math::HJWENO5_BIAS),
          mTemporalScheme(openvdb::math::TVD_RK2) {}
    virtual ~LevelSetAdvection() = default;
    LevelSetAdvection(const LevelSetAdvection&) = delete;
    LevelSetAdvection& operator=(const LevelSetAdvection&) = delete;

    openvdb::math::BiasedGradientScheme getSpatialScheme() const { return mSpatialScheme; }
    void setSpatialScheme(openvdb::math::BiasedGradientScheme scheme) { mSpatialScheme = scheme; }
    openvdb::math::TemporalIntegrationScheme getTemporalScheme() const { return mTemporalScheme; }
    void setTemporalScheme(openvdb::math::TemporalIntegrationScheme scheme) { mTemporalScheme = scheme; }
    openvdb::math::BiasedGradientScheme getTrackerSpatialScheme() const { return mTracker.getSpatialScheme(); }
    void setTrackerSpatialScheme(openvdb::math::BiasedGradientScheme scheme) { mTracker.setSpatialScheme(scheme); }
    openvdb::math::TemporalIntegrationScheme getTrackerTemporalScheme() const { return mTracker.getTemporalScheme(); }
    void setTrackerTemporalScheme(openvdb::math::TemporalIntegrationScheme scheme) {
        mTracker.setTemporalScheme(scheme);
    }
    int getNormCount() const { return mTracker.getNormCount(); }
    void setNormCount(int n) { mTracker.setNormCount(n); }
    int getGrainSize() const { return mTracker.getGrainSize(); }
    void setGrainSize(int grainsize) { mTracker.setGrainSize(grainsize); }

    // CFL number of the substep loop; 0 selects the reference's value
    // ({0.3, 0.9, 1.0}/sqrt(3) for TVD_RK1/2/3).
    void setCFL(float cfl) { mCfl = cfl; }
    float getCFL() const { return mCfl; }

    // tools/LevelSetAdvect.h:216-289 + Advect::advect :338-418.
    size_t advect(ValueType time0, ValueType time1) {
        FieldStore store;
        const gbls_field_desc fd =
            FieldTraits<FieldT>::describe(mField, mTracker.grid(), float(time0), float(time1), store);
        gbls_field* field = nullptr;
        detail::check(gbls_field_create(&fd, &field));
        struct FieldGuard {
            gbls_field* f;
            ~FieldGuard() { gbls_field_destroy(f); }
        } guard{field};
        detail::Handle& h = mTracker.device();
        h.upload(mTracker.grid());
        mTracker.configure(h.get());
        uint64_t count = 0;
        detail::check(gbls_advect(h.get(), field, int(mSpatialScheme), int(mTemporalScheme), float(time0),
                                  float(time1), mCfl, &count));
        h.download(mTracker.mutableGrid());
        mTracker.rebuildLeafs();
        return size_t(count);
    }

private:
    TrackerT mTracker;
    const FieldT mField;
    openvdb::math::BiasedGradientScheme mSpatialScheme;
    openvdb::math::TemporalIntegrationScheme mTemporalScheme;
    float mCfl = 0.0f;
};

}  // namespace tools
}  // namespace openvdb_gb300

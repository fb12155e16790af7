// Drop-in for openvdb::tools::LevelSetMorphing (tools/LevelSetMorph.h:47-141)
// running on the GPU through the C ABI (gbls.h).
//
// Same template parameters, types, constructor and member functions as the
// reference class.  advect(t0, t1) uploads the source, the target and the
// alpha mask (level sets with the source's transform), runs the CFL loop on
// the device (speed sampling, RK stages, tracker pass per substep) and writes
// the result back into the source grid's tree; it returns the number of CFL
// substeps.  Difference: a target or mask whose transform differs from the
// source's (trilinear sampling) throws NotImplementedError.
//
//   openvdb_gb300::tools::LevelSetMorphing<openvdb::FloatGrid> morph(*source, *target);
//   morph.setTemporalScheme(openvdb::math::TVD_RK3);
//   size_t substeps = morph.advect(0.0f, 1.0f);
#pragma once

#include <openvdb/tools/LevelSetMorph.h>

#include "LevelSetTracker.h"

namespace openvdb_gb300 {
namespace tools {

template <typename GridT, typename InterruptT = openvdb::util::NullInterrupter>
class LevelSetMorphing {
public:
    using GridType = GridT;
    using TreeType = typename GridT::TreeType;
    using TrackerT = LevelSetTracker<GridT, InterruptT>;
    using LeafRange = typename TrackerT::LeafRange;
    using LeafType = typename TrackerT::LeafType;
    using BufferType = typename TrackerT::BufferType;
    using ValueType = typename TrackerT::ValueType;

    LevelSetMorphing(GridT& sourceGrid, const GridT& targetGrid, InterruptT* interrupt = nullptr)
        : mTracker(sourceGrid, interrupt), mTarget(&targetGrid), mMask(nullptr),
          mSpatialScheme(openvdb::math::HJWENO5_BIAS), mTemporalScheme(openvdb::math::TVD_RK2) {}
    virtual ~LevelSetMorphing() = default;
    LevelSetMorphing(const LevelSetMorphing&) = delete;
    LevelSetMorphing& operator=(const LevelSetMorphing&) = delete;

    void setTarget(const GridT& targetGrid) { mTarget = &targetGrid; }
    void setAlphaMask(const GridT& maskGrid) { mMask = &maskGrid; }
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
    ValueType minMask() const { return mMinMask; }
    ValueType maxMask() const { return mDeltaMask + mMinMask; }
    void setMaskRange(ValueType min, ValueType max) {
        if (!(min < max)) OPENVDB_THROW(openvdb::ValueError, "Invalid mask range (expects min < max)");
        mMinMask = min;
        mMaxMask = max;
        mDeltaMask = max - min;
    }
    bool isMaskInverted() const { return mInvertMask; }
    void invertMask(bool invert = true) { mInvertMask = invert; }

    // tools/LevelSetMorph.h:243-262 + Morph::advect :479-510.
    size_t advect(ValueType time0, ValueType time1) {
        detail::Handle& h = mTracker.device();
        h.upload(mTracker.grid());
        mTargetDevice.upload(*mTarget);
        if (mMask) mMaskDevice.upload(*mMask);
        mTracker.configure(h.get());
        uint64_t count = 0;
        detail::check(gbls_morph(h.get(), mTargetDevice.get(), mMask ? mMaskDevice.get() : nullptr, int(mSpatialScheme),
                                 int(mTemporalScheme), float(time0), float(time1), float(mMinMask),
                                 float(mMaxMask), mInvertMask ? 1 : 0, &count));
        h.download(mTracker.mutableGrid());
        mTracker.rebuildLeafs();
        return size_t(count);
    }

private:
    TrackerT mTracker;
    const GridT *mTarget, *mMask;
    openvdb::math::BiasedGradientScheme mSpatialScheme;
    openvdb::math::TemporalIntegrationScheme mTemporalScheme;
    // the range as given (gbls_morph forms max - min as setMaskRange does)
    ValueType mMinMask = 0, mMaxMask = 1, mDeltaMask = 1;
    bool mInvertMask = false;
    detail::Handle mTargetDevice, mMaskDevice;
};

}  // namespace tools
}  // namespace openvdb_gb300

// Drop-in for openvdb::tools::LevelSetTracker (tools/LevelSetTracker.h:56-256)
// running on the GPU through the C ABI (gbls.h).
//
// Same template parameters, types, constructor and member functions as the
// reference class; each operation uploads the grid, runs on the device and
// writes the result back into the same tree (the grid is borrowed by
// reference and mutated in place, as in the reference).  leafs() is a
// LeafManager over the host tree, rebuilt after every operation.
//
//   openvdb_gb300::tools::LevelSetTracker<openvdb::FloatGrid> tracker(grid);
//   tracker.setNormCount(1);
//   tracker.track();
#pragma once

#include <vector>

#include <openvdb/tools/LevelSetTracker.h>
#include <openvdb/util/NullInterrupter.h>

#include <memory>

#include "GridExchange.h"

namespace openvdb_gb300 {
namespace detail {

// gbls_interrupter hooks forwarding to an OpenVDB interrupter
// (util/NullInterrupter.h: start / end / wasInterrupted).
template <typename InterruptT>
struct InterruptBridge {
    static void start(void* u, const char* name) { static_cast<InterruptT*>(u)->start(name); }
    static void end(void* u) { static_cast<InterruptT*>(u)->end(); }
    static int was(void* u, int percent) { return openvdb::util::wasInterrupted(static_cast<InterruptT*>(u), percent) ? 1 : 0; }
    static gbls_interrupter make(InterruptT* i) {
        gbls_interrupter g{};
        if (i) {
            g.start = &start;
            g.end = &end;
            g.was_interrupted = &was;
            g.user = i;
        }
        return g;
    }
};

}  // namespace detail

namespace tools {

template <typename GridT, typename InterruptT = openvdb::util::NullInterrupter>
class LevelSetTracker {
public:
    using Reference = openvdb::tools::LevelSetTracker<GridT, InterruptT>;
    using TrimMode = openvdb::tools::lstrack::TrimMode;
    using GridType = GridT;
    using TreeType = typename GridT::TreeType;
    using LeafType = typename TreeType::LeafNodeType;
    using ValueType = typename TreeType::ValueType;
    using LeafManagerType = typename openvdb::tree::LeafManager<TreeType>;
    using LeafRange = typename LeafManagerType::LeafRange;
    using BufferType = typename LeafManagerType::BufferType;
    using MaskTreeType = typename TreeType::template ValueConverter<openvdb::ValueMask>::Type;
    using State = typename Reference::State;

    // tools/LevelSetTracker.h:262-277: the same checks, the same exceptions.
    LevelSetTracker(GridT& grid, InterruptT* interrupt = nullptr)
        : mGrid(&grid), mInterrupter(interrupt), mDx(static_cast<ValueType>(grid.voxelSize()[0])) {
        if (!grid.hasUniformVoxels())
            OPENVDB_THROW(openvdb::RuntimeError,
                          "The transform must have uniform scale for the LevelSetTracker to function");
        if (grid.getGridClass() != openvdb::GRID_LEVEL_SET)
            OPENVDB_THROW(openvdb::RuntimeError,
                          "LevelSetTracker expected a level set, got a grid of class \"" +
                              grid.gridClassToString(grid.getGridClass()) + "\" [hint: Grid::setGridClass(openvdb::GRID_LEVEL_SET)]");
        mLeafs.reset(new LeafManagerType(grid.tree()));
    }
    virtual ~LevelSetTracker() = default;
    LevelSetTracker(const LevelSetTracker&) = delete;
    LevelSetTracker& operator=(const LevelSetTracker&) = delete;

    // The masked form renormalises only the active voxels of the mask tree's
    // leaves that share an origin with a leaf of the level set
    // (gbls_normalize_masked); MaskType is a tree type.  A mask covering a
    // voxel that is inactive in the level set throws NotImplementedError.
    template <typename MaskType>
    void normalize(const MaskType* mask) {
        if (!mask) {
            run([](gbls_handle* h) { return gbls_normalize(h); });
            return;
        }
        std::vector<int32_t> origins;
        std::vector<uint64_t> words;
        for (auto leaf = mask->cbeginLeaf(); leaf; ++leaf) {
            const openvdb::Coord o = leaf->origin();
            origins.insert(origins.end(), {o.x(), o.y(), o.z()});
            for (int w = 0; w < 8; ++w) words.push_back(leaf->getValueMask().template getWord<uint64_t>(w));
        }
        const int64_t n = int64_t(origins.size() / 3);
        run([&](gbls_handle* h) { return gbls_normalize_masked(h, n, origins.data(), words.data()); });
    }
    void normalize() { this->normalize<MaskTreeType>(nullptr); }
    void track() { run([](gbls_handle* h) { return gbls_track(h); }); }
    void prune() { run([](gbls_handle* h) { return gbls_prune(h); }); }
    void dilate(int iterations = 1) { run([=](gbls_handle* h) { return gbls_dilate(h, iterations); }); }
    void erode(int iterations = 1) { run([=](gbls_handle* h) { return gbls_erode(h, iterations); }); }
    bool resize(openvdb::Index halfWidth = static_cast<openvdb::Index>(openvdb::LEVEL_SET_HALF_WIDTH)) {
        int changed = 0;
        run([&](gbls_handle* h) { return gbls_resize(h, uint32_t(halfWidth), &changed); });
        return changed != 0;
    }

    ValueType getHalfWidth() const { return mGrid->background() / mDx; }
    State getState() const { return mState; }
    void setState(const State& s) { mState = s; }
    openvdb::math::BiasedGradientScheme getSpatialScheme() const { return mState.spatialScheme; }
    void setSpatialScheme(openvdb::math::BiasedGradientScheme s) { mState.spatialScheme = s; }
    openvdb::math::TemporalIntegrationScheme getTemporalScheme() const { return mState.temporalScheme; }
    void setTemporalScheme(openvdb::math::TemporalIntegrationScheme s) { mState.temporalScheme = s; }
    int getNormCount() const { return mState.normCount; }
    void setNormCount(int n) { mState.normCount = n; }
    int getGrainSize() const { return mState.grainSize; }
    void setGrainSize(int grainsize) { mState.grainSize = grainsize; }
    TrimMode trimming() const { return mTrimMode; }
    void setTrimming(TrimMode mode) { mTrimMode = mode; }
    ValueType voxelSize() const { return mDx; }

    void startInterrupter(const char* msg) {
        if (mInterrupter) mInterrupter->start(msg);
    }
    void endInterrupter() {
        if (mInterrupter) mInterrupter->end();
    }
    bool checkInterrupter() { return !openvdb::util::wasInterrupted(mInterrupter); }

    const GridType& grid() const { return *mGrid; }
    LeafManagerType& leafs() { return *mLeafs; }
    const LeafManagerType& leafs() const { return *mLeafs; }

    // Device state of the tracker settings (gbls_set_tracker_state /
    // gbls_set_trimming / gbls_set_interrupter) on a handle.
    void configure(gbls_handle* h) const {
        detail::check(gbls_set_tracker_state(h, int(mState.spatialScheme), int(mState.temporalScheme),
                                             mState.normCount, mState.grainSize));
        detail::check(gbls_set_trimming(h, int(mTrimMode)));
        const gbls_interrupter in = detail::InterruptBridge<InterruptT>::make(mInterrupter);
        detail::check(gbls_set_interrupter(h, mInterrupter ? &in : nullptr));
    }
    GridType& mutableGrid() { return *mGrid; }
    void rebuildLeafs() { mLeafs->rebuildLeafArray(); }

protected:
    // Upload, apply `op` to the device level set, download into the grid.
    template <typename Op>
    void run(Op op) {
        mDevice.upload(*mGrid);
        configure(mDevice.get());
        const int rc = op(mDevice.get());
        detail::check(rc);
        mDevice.download(*mGrid);
        rebuildLeafs();
    }

public:
    // The device level set of this tracker, kept between calls so that
    // repeated operations re-use its allocations (gbls_upload).
    detail::Handle& device() { return mDevice; }

private:
    detail::Handle mDevice;
    GridType* mGrid;
    std::unique_ptr<LeafManagerType> mLeafs;
    InterruptT* mInterrupter;
    const ValueType mDx;
    State mState;
    TrimMode mTrimMode = TrimMode::kAll;
};

}  // namespace tools
}  // namespace openvdb_gb300

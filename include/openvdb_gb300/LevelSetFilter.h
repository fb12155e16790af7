// Drop-in for openvdb::tools::LevelSetFilter (tools/LevelSetFilter.h:30-160)
// running on the GPU through the C ABI (gbls.h).
//
// Same template parameters and member functions as the reference class, a
// LevelSetTracker (the drop-in one) with filters; every filter uploads the
// grid, runs the filter and the tracker pass on the device and writes the
// result back into the same tree.  Every filter has a device form
// (mean, gaussian and median for half widths 1..3), with or without an alpha
// mask.  The mask is uploaded as a device level set: a mask grid that is not
// a narrow-band level set (positive background, inactive values
// +-background) or whose transform differs from the filtered grid's has no
// device form and throws (RuntimeError / NotImplementedError).
//
//   openvdb_gb300::tools::LevelSetFilter<openvdb::FloatGrid> filter(*grid);
//   filter.gaussian(1);
//   filter.offset(-0.5f);
#pragma once

#include <openvdb/tools/LevelSetFilter.h>

#include "LevelSetTracker.h"

namespace openvdb_gb300 {
namespace tools {

template <typename GridT, typename MaskT = typename GridT::template ValueConverter<float>::Type,
          typename InterruptT = openvdb::util::NullInterrupter>
class LevelSetFilter : public LevelSetTracker<GridT, InterruptT> {
public:
    using BaseType = LevelSetTracker<GridT, InterruptT>;
    using GridType = GridT;
    using MaskType = MaskT;
    using TreeType = typename GridType::TreeType;
    using ValueType = typename TreeType::ValueType;
    using AlphaType = typename MaskType::ValueType;
    static_assert(std::is_floating_point<AlphaType>::value,
                  "LevelSetFilter requires a mask grid with floating-point values");

    LevelSetFilter(GridType& grid, InterruptT* interrupt = nullptr)
        : BaseType(grid, interrupt), mMinMask(0), mMaxMask(1), mInvertMask(false) {}
    ~LevelSetFilter() override {}

    AlphaType minMask() const { return mMinMask; }
    AlphaType maxMask() const { return mMaxMask; }
    void setMaskRange(AlphaType min, AlphaType max) {
        if (!(min < max)) OPENVDB_THROW(openvdb::ValueError, "Invalid mask range (expects min < max)");
        mMinMask = min;
        mMaxMask = max;
    }
    bool isMaskInverted() const { return mInvertMask; }
    void invertMask(bool invert = true) { mInvertMask = invert; }

    void meanCurvature(const MaskType* mask = nullptr) { apply(GBLS_FILTER_MEAN_CURVATURE, 1, 0.0f, mask); }
    void fillet(const MaskType* mask = nullptr) { apply(GBLS_FILTER_FILLET, 1, 0.0f, mask); }
    void laplacian(const MaskType* mask = nullptr) { apply(GBLS_FILTER_LAPLACIAN, 1, 0.0f, mask); }
    void gaussian(int width = 1, const MaskType* mask = nullptr) { apply(GBLS_FILTER_GAUSSIAN, width, 0.0f, mask); }
    void offset(ValueType offset, const MaskType* mask = nullptr) {
        apply(GBLS_FILTER_OFFSET, 1, float(offset), mask);
    }
    void median(int width = 1, const MaskType* mask = nullptr) { apply(GBLS_FILTER_MEDIAN, width, 0.0f, mask); }
    void mean(int width = 1, const MaskType* mask = nullptr) { apply(GBLS_FILTER_MEAN, width, 0.0f, mask); }

private:
    void apply(int filter, int width, float value, const MaskType* mask) {
        if (!mask) {
            this->run([=](gbls_handle* h) { return gbls_filter(h, filter, width, value); });
            return;
        }
        mMaskDevice.upload(*mask);
        gbls_handle* m = mMaskDevice.get();
        const float lo = float(mMinMask), hi = float(mMaxMask);
        const int inv = mInvertMask ? 1 : 0;
        this->run([=](gbls_handle* h) { return gbls_filter_masked(h, filter, width, value, m, lo, hi, inv); });
    }

    AlphaType mMinMask, mMaxMask;
    bool mInvertMask;
    detail::Handle mMaskDevice;  // the alpha mask as a device level set
};

}  // namespace tools
}  // namespace openvdb_gb300

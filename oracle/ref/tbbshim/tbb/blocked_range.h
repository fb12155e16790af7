// Project-written TBB-API shim (test oracle only): tbb::blocked_range.
#ifndef GBLS_TBBSHIM_BLOCKED_RANGE_H
#define GBLS_TBBSHIM_BLOCKED_RANGE_H
#include "detail/shim_core.h"
namespace tbb {
template<typename Value>
class blocked_range {
public:
    using const_iterator = Value;
    using size_type = std::size_t;
    blocked_range() : mBegin(), mEnd(), mGrain(1) {}
    blocked_range(Value b, Value e, size_type grain = 1) : mBegin(b), mEnd(e), mGrain(grain) {}
    blocked_range(blocked_range& r, split) : mBegin(), mEnd(r.mEnd), mGrain(r.mGrain) {
        Value middle = r.mBegin + (r.mEnd - r.mBegin) / 2u;
        r.mEnd = middle;
        mBegin = middle;
    }
    const_iterator begin() const { return mBegin; }
    const_iterator end() const { return mEnd; }
    size_type size() const { return size_type(mEnd - mBegin); }
    size_type grainsize() const { return mGrain; }
    bool empty() const { return !(mBegin < mEnd); }
    bool is_divisible() const { return mGrain < size(); }
private:
    Value mBegin, mEnd;
    size_type mGrain;
};
} // namespace tbb
#endif

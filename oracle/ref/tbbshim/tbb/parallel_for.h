// Project-written TBB-API shim (test oracle only): tbb::parallel_for.
// Each piece runs on its own copy of the body, as TBB does.
#ifndef GBLS_TBBSHIM_PARALLEL_FOR_H
#define GBLS_TBBSHIM_PARALLEL_FOR_H
#include "detail/shim_core.h"
#include "blocked_range.h"
#include "partitioner.h"
#include <type_traits>
namespace tbb {
template<typename Range, typename Body>
void parallel_for(const Range& range, const Body& body) {
    if (range.empty()) return;
    std::deque<Range> parts = shim::splitRange(range, shim::targetPieces());
    shim::Pool::instance().run(parts.size(), [&](size_t i) {
        Body local(body);
        local(parts[i]);
    });
}
template<typename Range, typename Body, typename Partitioner>
void parallel_for(const Range& range, const Body& body, Partitioner&) { parallel_for(range, body); }
template<typename Range, typename Body, typename Partitioner>
void parallel_for(const Range& range, const Body& body, const Partitioner&) { parallel_for(range, body); }

template<typename Index, typename Func,
         typename = typename std::enable_if<std::is_integral<Index>::value>::type>
void parallel_for(Index first, Index last, const Func& f) {
    if (!(first < last)) return;
    parallel_for(blocked_range<Index>(first, last), [&f](const blocked_range<Index>& r) {
        for (Index i = r.begin(); i != r.end(); ++i) f(i);
    });
}
template<typename Index, typename Func,
         typename = typename std::enable_if<std::is_integral<Index>::value>::type>
void parallel_for(Index first, Index last, Index step, const Func& f) {
    if (!(first < last) || step <= 0) return;
    const Index n = (last - first + step - 1) / step;
    parallel_for(Index(0), n, [&](Index k) { f(first + k * step); });
}
} // namespace tbb
#endif

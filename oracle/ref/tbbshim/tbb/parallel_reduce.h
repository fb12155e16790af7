// Project-written TBB-API shim (test oracle only): tbb::parallel_reduce.
// Split bodies are constructed up front on the calling thread and joined
// left to right after all pieces finish, so the reduction order is fixed.
#ifndef GBLS_TBBSHIM_PARALLEL_REDUCE_H
#define GBLS_TBBSHIM_PARALLEL_REDUCE_H
#include "detail/shim_core.h"
#include "blocked_range.h"
#include "partitioner.h"
#include <memory>
namespace tbb {
template<typename Range, typename Body>
void parallel_reduce(const Range& range, Body& body) {
    if (range.empty()) return;
    std::deque<Range> parts = shim::splitRange(range, shim::targetPieces());
    std::vector<std::unique_ptr<Body>> bodies(parts.size());
    for (size_t i = 1; i < parts.size(); ++i) bodies[i].reset(new Body(body, split()));
    shim::Pool::instance().run(parts.size(), [&](size_t i) {
        if (i == 0) body(parts[0]);
        else (*bodies[i])(parts[i]);
    });
    for (size_t i = 1; i < parts.size(); ++i) body.join(*bodies[i]);
}
template<typename Range, typename Body, typename Partitioner>
void parallel_reduce(const Range& range, Body& body, Partitioner&) { parallel_reduce(range, body); }
template<typename Range, typename Body, typename Partitioner>
void parallel_reduce(const Range& range, Body& body, const Partitioner&) { parallel_reduce(range, body); }

template<typename Range, typename Value, typename RealBody, typename Reduction>
Value parallel_reduce(const Range& range, const Value& identity,
                      const RealBody& realBody, const Reduction& reduction) {
    if (range.empty()) return identity;
    std::deque<Range> parts = shim::splitRange(range, shim::targetPieces());
    std::vector<Value> partial(parts.size(), identity);
    shim::Pool::instance().run(parts.size(), [&](size_t i) {
        partial[i] = realBody(parts[i], identity);
    });
    Value result = partial[0];
    for (size_t i = 1; i < parts.size(); ++i) result = reduction(result, partial[i]);
    return result;
}
template<typename Range, typename Value, typename RealBody, typename Reduction, typename P>
Value parallel_reduce(const Range& range, const Value& identity, const RealBody& realBody,
                      const Reduction& reduction, const P&) {
    return parallel_reduce(range, identity, realBody, reduction);
}
} // namespace tbb
#endif

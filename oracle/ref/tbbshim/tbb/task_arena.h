// Project-written TBB-API shim (test oracle only): task_arena queries.
#ifndef GBLS_TBBSHIM_TASK_ARENA_H
#define GBLS_TBBSHIM_TASK_ARENA_H
#include "detail/shim_core.h"
namespace tbb {
namespace this_task_arena {
inline int max_concurrency() { return shim::Pool::instance().threads(); }
inline int current_thread_index() { return 0; }
}
class task_arena {
public:
    static const int automatic = -1;
    explicit task_arena(int = automatic, unsigned = 1) {}
    template<typename F> auto execute(const F& f) -> decltype(f()) { return f(); }
    int max_concurrency() const { return shim::Pool::instance().threads(); }
};
} // namespace tbb
#endif

// Project-written TBB-API shim (test oracle only): tbb::task_group (runs
// each task on the calling thread when it is submitted).
#ifndef GBLS_TBBSHIM_TASK_GROUP_H
#define GBLS_TBBSHIM_TASK_GROUP_H
#include "detail/shim_core.h"
#include "task.h"
namespace tbb {
enum task_group_status { not_complete, complete, canceled };
class task_group {
public:
    template<typename F> void run(const F& f) { f(); }
    template<typename F> task_group_status run_and_wait(const F& f) { f(); return complete; }
    task_group_status wait() { return complete; }
    void cancel() {}
};
} // namespace tbb
#endif

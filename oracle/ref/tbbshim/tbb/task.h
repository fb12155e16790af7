// Project-written TBB-API shim (test oracle only): tbb::task::current_context.
// There is no task-group cancellation: current_context() returns nullptr.
#ifndef GBLS_TBBSHIM_TASK_H
#define GBLS_TBBSHIM_TASK_H
#include "detail/shim_core.h"
namespace tbb {
class task_group_context {
public:
    bool cancel_group_execution() { return false; }
    bool is_group_execution_cancelled() const { return false; }
};
namespace task {
inline task_group_context* current_context() { return nullptr; }
}
} // namespace tbb
#endif

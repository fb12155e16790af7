// Project-written TBB-API shim (test oracle only): partitioner tags.
#ifndef GBLS_TBBSHIM_PARTITIONER_H
#define GBLS_TBBSHIM_PARTITIONER_H
namespace tbb {
class auto_partitioner {};
class simple_partitioner {};
class static_partitioner {};
class affinity_partitioner {};
} // namespace tbb
#endif

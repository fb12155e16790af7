// Project-written TBB-API shim (test oracle only): tbb::parallel_sort.
#ifndef GBLS_TBBSHIM_PARALLEL_SORT_H
#define GBLS_TBBSHIM_PARALLEL_SORT_H
#include <algorithm>
namespace tbb {
template<typename It> void parallel_sort(It b, It e) { std::sort(b, e); }
template<typename It, typename Cmp> void parallel_sort(It b, It e, const Cmp& c) { std::sort(b, e, c); }
template<typename Seq> void parallel_sort(Seq& s) { std::sort(s.begin(), s.end()); }
} // namespace tbb
#endif

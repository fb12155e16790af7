// Project-written TBB-API shim (test oracle only): tbb::concurrent_vector.
#ifndef GBLS_TBBSHIM_CV_H
#define GBLS_TBBSHIM_CV_H
#include <deque>
#include <mutex>
namespace tbb {
template<typename T>
class concurrent_vector {
public:
    using iterator = typename std::deque<T>::iterator;
    void push_back(const T& v) { std::lock_guard<std::mutex> lk(mMutex); mItems.push_back(v); }
    size_t size() const { return mItems.size(); }
    bool empty() const { return mItems.empty(); }
    T& operator[](size_t i) { return mItems[i]; }
    const T& operator[](size_t i) const { return mItems[i]; }
    iterator begin() { return mItems.begin(); }
    iterator end() { return mItems.end(); }
    void clear() { mItems.clear(); }
private:
    std::deque<T> mItems;
    std::mutex mMutex;
};
} // namespace tbb
#endif

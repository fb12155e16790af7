// Project-written TBB-API shim (test oracle only): tbb::enumerable_thread_specific.
// Instances live in a std::deque (stable references, random-access iterators)
// and are looked up by std::thread::id.
#ifndef GBLS_TBBSHIM_ETS_H
#define GBLS_TBBSHIM_ETS_H
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <type_traits>
namespace tbb {
template<typename T>
class enumerable_thread_specific {
public:
    using value_type = T;
    using reference = T&;
    using iterator = typename std::deque<T>::iterator;
    using const_iterator = typename std::deque<T>::const_iterator;
    enumerable_thread_specific() : mHasExemplar(false) {}
    explicit enumerable_thread_specific(const T& exemplar) : mHasExemplar(true), mExemplar(new T(exemplar)) {}
    ~enumerable_thread_specific() { delete mExemplar; }
    T& local() { bool e; return local(e); }
    T& local(bool& exists) {
        std::lock_guard<std::mutex> lk(mMutex);
        const auto id = std::this_thread::get_id();
        auto it = mIndex.find(id);
        if (it != mIndex.end()) { exists = true; return mItems[it->second]; }
        exists = false;
        if constexpr (std::is_copy_constructible<T>::value) {
            if (mHasExemplar) mItems.emplace_back(*mExemplar);
            else mItems.emplace_back();
        } else {
            mItems.emplace_back();
        }
        mIndex[id] = mItems.size() - 1;
        return mItems.back();
    }
    iterator begin() { return mItems.begin(); }
    iterator end() { return mItems.end(); }
    const_iterator begin() const { return mItems.begin(); }
    const_iterator end() const { return mItems.end(); }
    size_t size() const { return mItems.size(); }
    bool empty() const { return mItems.empty(); }
    void clear() { mItems.clear(); mIndex.clear(); }
    template<typename F> void combine_each(F f) { for (auto& v : mItems) f(v); }
    template<typename F> T combine(F f) {
        if (mItems.empty()) return T();
        T r = mItems[0];
        for (size_t i = 1; i < mItems.size(); ++i) r = f(r, mItems[i]);
        return r;
    }
private:
    enumerable_thread_specific(const enumerable_thread_specific&) = delete;
    bool mHasExemplar;
    T* mExemplar = nullptr;
    std::deque<T> mItems;
    std::map<std::thread::id, size_t> mIndex;
    std::mutex mMutex;
};
} // namespace tbb
#endif

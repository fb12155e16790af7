// Project-written TBB-API shim (test oracle only): tbb::concurrent_hash_map
// as a mutex-guarded std::map (OpenVDB only uses it as an accessor registry).
#ifndef GBLS_TBBSHIM_CHM_H
#define GBLS_TBBSHIM_CHM_H
#include <map>
#include <mutex>
namespace tbb {
template<typename K, typename V, typename HashCompare = void>
class concurrent_hash_map {
    using Map = std::map<K, V>;
public:
    using value_type = typename Map::value_type;
    using iterator = typename Map::iterator;
    using const_iterator = typename Map::const_iterator;
    class accessor {
    public:
        accessor() : mItem(nullptr) {}
        value_type* operator->() const { return mItem; }
        value_type& operator*() const { return *mItem; }
        bool empty() const { return mItem == nullptr; }
        void release() { mItem = nullptr; }
        value_type* mItem;
    };
    class const_accessor {
    public:
        const_accessor() : mItem(nullptr) {}
        const value_type* operator->() const { return mItem; }
        const value_type& operator*() const { return *mItem; }
        bool empty() const { return mItem == nullptr; }
        void release() { mItem = nullptr; }
        const value_type* mItem;
    };
    concurrent_hash_map() {}
    concurrent_hash_map(const concurrent_hash_map& o) : mMap(o.mMap) {}
    concurrent_hash_map& operator=(const concurrent_hash_map& o) { mMap = o.mMap; return *this; }
    bool insert(accessor& a, const K& k) {
        std::lock_guard<std::mutex> lk(mMutex);
        auto r = mMap.emplace(k, V());
        a.mItem = &*r.first;
        return r.second;
    }
    bool insert(const_accessor& a, const K& k) {
        std::lock_guard<std::mutex> lk(mMutex);
        auto r = mMap.emplace(k, V());
        a.mItem = &*r.first;
        return r.second;
    }
    bool insert(const value_type& v) {
        std::lock_guard<std::mutex> lk(mMutex);
        return mMap.insert(v).second;
    }
    bool find(accessor& a, const K& k) {
        std::lock_guard<std::mutex> lk(mMutex);
        auto it = mMap.find(k);
        if (it == mMap.end()) return false;
        a.mItem = &*it;
        return true;
    }
    bool find(const_accessor& a, const K& k) const {
        std::lock_guard<std::mutex> lk(mMutex);
        auto it = mMap.find(k);
        if (it == mMap.end()) return false;
        a.mItem = &*it;
        return true;
    }
    bool erase(const K& k) {
        std::lock_guard<std::mutex> lk(mMutex);
        return mMap.erase(k) > 0;
    }
    void clear() { std::lock_guard<std::mutex> lk(mMutex); mMap.clear(); }
    size_t size() const { return mMap.size(); }
    bool empty() const { return mMap.empty(); }
    iterator begin() { return mMap.begin(); }
    iterator end() { return mMap.end(); }
    const_iterator begin() const { return mMap.begin(); }
    const_iterator end() const { return mMap.end(); }
private:
    Map mMap;
    mutable std::mutex mMutex;
};
} // namespace tbb
#endif

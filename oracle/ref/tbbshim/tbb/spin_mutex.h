// Project-written TBB-API shim (test oracle only): tbb::spin_mutex.
#ifndef GBLS_TBBSHIM_SPIN_MUTEX_H
#define GBLS_TBBSHIM_SPIN_MUTEX_H
#include <mutex>
namespace tbb {
class spin_mutex {
public:
    void lock() { mMutex.lock(); }
    void unlock() { mMutex.unlock(); }
    bool try_lock() { return mMutex.try_lock(); }
    class scoped_lock {
    public:
        scoped_lock() : mMutex(nullptr) {}
        explicit scoped_lock(spin_mutex& m) : mMutex(&m) { m.lock(); }
        ~scoped_lock() { if (mMutex) mMutex->unlock(); }
        void acquire(spin_mutex& m) { mMutex = &m; m.lock(); }
        bool try_acquire(spin_mutex& m) { if (m.try_lock()) { mMutex = &m; return true; } return false; }
        void release() { if (mMutex) { mMutex->unlock(); mMutex = nullptr; } }
    private:
        spin_mutex* mMutex;
    };
private:
    std::mutex mMutex;
};
} // namespace tbb
#endif

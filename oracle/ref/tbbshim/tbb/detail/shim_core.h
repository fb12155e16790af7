// Project-written stand-in for the subset of the oneTBB API that OpenVDB's
// level-set advection path includes (parallel_for, parallel_reduce,
// blocked_range, enumerable_thread_specific, spin_mutex, task_group,
// task_arena, concurrent_hash_map, parallel_sort).  It exists only so the
// reference headers can be compiled into the test oracle in an image that has
// no TBB.  It is test infrastructure: nothing in the product links it.
//
// Execution model: one process-wide pool of std::threads.  A top-level
// parallel_for / parallel_reduce pre-splits its range breadth-first into
// about 8 pieces per thread (never past is_divisible()), and the pool threads
// plus the caller pull pieces from an atomic counter.  Calls made from inside
// a running piece (nested parallelism) run serially on the calling thread,
// which is always a legal TBB schedule.  Every body on the OpenVDB path is
// partition-independent, so results do not depend on the thread count.
#ifndef GBLS_TBBSHIM_CORE_H
#define GBLS_TBBSHIM_CORE_H

#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <cstdlib>
#include <deque>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#define TBB_INTERFACE_VERSION 12140
#define TBB_VERSION_MAJOR 2021
#define TBB_VERSION_MINOR 14
#define TBB_VERSION_STRING "2021.14-shim"

namespace tbb {

struct split {};

namespace shim {

class Pool {
public:
    static Pool& instance() {
        static Pool pool;
        return pool;
    }

    int threads() const { return mThreads; }

    // Set the worker count (1 = serial).  Must not be called while a job runs.
    void resize(int n) {
        std::lock_guard<std::mutex> jobLock(mJobMutex);
        stopWorkers();
        mThreads = n < 1 ? 1 : n;
        startWorkers();
    }

    static bool& inWorker() {
        thread_local bool flag = false;
        return flag;
    }

    // Run fn(i) for i in [0, n) on the pool; the caller participates.
    void run(size_t n, const std::function<void(size_t)>& fn) {
        if (n == 0) return;
        if (inWorker() || mThreads <= 1 || n == 1) {
            const bool saved = inWorker();
            inWorker() = true;
            for (size_t i = 0; i < n; ++i) fn(i);
            inWorker() = saved;
            return;
        }
        std::lock_guard<std::mutex> jobLock(mJobMutex);
        {
            std::lock_guard<std::mutex> lk(mMutex);
            mFn = &fn;
            mCount = n;
            mNext.store(0);
            mPending = mThreads - 1;
            ++mGeneration;
        }
        mCv.notify_all();
        inWorker() = true;
        drain();
        inWorker() = false;
        std::unique_lock<std::mutex> lk(mMutex);
        mDoneCv.wait(lk, [this] { return mPending == 0; });
        mFn = nullptr;
    }

private:
    Pool() {
        int n = 0;
        if (const char* s = std::getenv("TBBSHIM_THREADS")) n = std::atoi(s);
        if (n <= 0) n = int(std::thread::hardware_concurrency());
        mThreads = n < 1 ? 1 : n;
        startWorkers();
    }
    ~Pool() { stopWorkers(); }

    void drain() {
        for (;;) {
            const size_t i = mNext.fetch_add(1);
            if (i >= mCount) break;
            (*mFn)(i);
        }
    }

    void startWorkers() {
        mStop = false;
        for (int t = 1; t < mThreads; ++t) {
            mWorkers.emplace_back([this] {
                inWorker() = true;
                uint64_t seen = 0;
                for (;;) {
                    {
                        std::unique_lock<std::mutex> lk(mMutex);
                        mCv.wait(lk, [&] { return mStop || mGeneration != seen; });
                        if (mStop) return;
                        seen = mGeneration;
                    }
                    drain();
                    {
                        std::lock_guard<std::mutex> lk(mMutex);
                        if (--mPending == 0) mDoneCv.notify_all();
                    }
                }
            });
        }
    }

    void stopWorkers() {
        {
            std::lock_guard<std::mutex> lk(mMutex);
            mStop = true;
        }
        mCv.notify_all();
        for (auto& w : mWorkers) w.join();
        mWorkers.clear();
    }

    int mThreads = 1;
    std::vector<std::thread> mWorkers;
    std::mutex mJobMutex, mMutex;
    std::condition_variable mCv, mDoneCv;
    const std::function<void(size_t)>* mFn = nullptr;
    size_t mCount = 0;
    std::atomic<size_t> mNext{0};
    int mPending = 0;
    uint64_t mGeneration = 0;
    bool mStop = false;
};

// Breadth-first split of a range into at most `target` pieces.
template<typename Range>
std::deque<Range> splitRange(const Range& range, size_t target) {
    std::deque<Range> parts;
    parts.push_back(range);
    for (;;) {
        std::deque<Range> next;
        bool any = false;
        for (size_t i = 0; i < parts.size(); ++i) {
            Range r(parts[i]);
            if (r.is_divisible() && next.size() + (parts.size() - i) < target) {
                Range right(r, tbb::split());
                next.push_back(r);
                next.push_back(right);
                any = true;
            } else {
                next.push_back(r);
            }
        }
        parts.swap(next);
        if (!any || parts.size() >= target) break;
    }
    return parts;
}

inline size_t targetPieces() { return size_t(Pool::instance().threads()) * 8; }

} // namespace shim
} // namespace tbb

#endif

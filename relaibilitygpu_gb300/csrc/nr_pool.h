// nr_pool.h -- the host worker pool of a context (host C++ only).
#pragma once

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

// Worker threads kept by a context for the host side of batch calls (table
// building and validation), so a call does not pay for thread creation.  A
// batch call runs several short jobs back to back, and batch calls often follow
// one another: between jobs the workers (and the caller waiting for a job's
// end) poll, yielding the core, for up to kSpin before they block, so a job
// rarely waits for threads to be woken from sleep.
#ifndef NR_POOL_MAX
#define NR_POOL_MAX 32          // host threads of a batch call at most (the caller's included)
#endif
#ifndef NR_POOL_SPIN_US
#define NR_POOL_SPIN_US 2000    // idle workers poll this long before they sleep
#endif
class NrPool {
public:
    explicit NrPool(int workers)
    {
        for (int i = 0; i < workers; ++i) th_.emplace_back([this, i] { loop(i); });
    }
    ~NrPool()
    {
        {
            std::lock_guard<std::mutex> l(mu_);
            quit_ = true;
            // a new job number with no helper slot: spinning workers stop and see quit_
            const unsigned long long job = (state_.load(std::memory_order_relaxed) >> 32) + 1;
            state_.store(job << 32, std::memory_order_release);
        }
        cv_.notify_all();
        for (auto &t : th_) t.join();
    }
    int size() const { return (int)th_.size() + 1; }
    // run fn(i) for i in [0, n) on the calling thread and `helpers` workers; the
    // threads take `grain` consecutive indices at a time
    void run(int n, int helpers, int grain, const std::function<void(int)> &fn)
    {
        helpers = std::max(0, std::min(helpers, (int)th_.size()));
        if (helpers == 0) {
            for (int i = 0; i < n; ++i) fn(i);
            return;
        }
        {
            // publish the job: its fields, then a new job number with no helper slot claimed
            std::lock_guard<std::mutex> l(mu_);
            fn_.store(&fn, std::memory_order_relaxed);
            n_.store(n, std::memory_order_relaxed);
            grain_.store(std::max(1, grain), std::memory_order_relaxed);
            next_.store(0, std::memory_order_relaxed);
            busy_.store(helpers, std::memory_order_relaxed);
            const unsigned long long job = (state_.load(std::memory_order_relaxed) >> 32) + 1;
            state_.store((job << 32) | ((unsigned long long)helpers << 16), std::memory_order_release);
        }
        cv_.notify_all();
        work();
        for (int it = 0; it < kBusyPolls && busy_.load(std::memory_order_acquire) != 0; ++it) {}
        const auto t0 = std::chrono::steady_clock::now();
        while (busy_.load(std::memory_order_acquire) != 0) {
            if (std::chrono::steady_clock::now() - t0 > kSpin) {
                std::unique_lock<std::mutex> l(mu_);
                done_.wait(l, [this] { return busy_.load(std::memory_order_acquire) == 0; });
                break;
            }
            std::this_thread::yield();
        }
        fn_.store(nullptr, std::memory_order_relaxed);
    }

private:
    static constexpr std::chrono::microseconds kSpin{NR_POOL_SPIN_US};
    static constexpr int kBusyPolls = 20000;    // loads of the job word before yielding (tens of us)
    void work()
    {
        const int n = n_.load(std::memory_order_relaxed), grain = grain_.load(std::memory_order_relaxed);
        const std::function<void(int)> &fn = *fn_.load(std::memory_order_relaxed);
        for (;;) {
            const int b = next_.fetch_add(grain);
            if (b >= n) break;
            const int e = std::min(n, b + grain);
            for (int i = b; i < e; ++i) fn(i);
        }
    }
    // A worker joins a job by claiming one of its helper slots with a compare-and-swap
    // on state_ (job number << 32 | helper slots << 16 | slots claimed): no lock on the
    // way in.  The slot count travels in the same word as the claims, so a worker that
    // read an old job's word can only see it full (a job ends only after all its slots
    // were claimed and their helpers finished) and can never claim into a job whose
    // fields are being rewritten.  The mutex is taken only to sleep.
    void loop(int)
    {
        unsigned long long seen = 0;           // last job this worker has dealt with
        for (;;) {
            unsigned long long s = state_.load(std::memory_order_acquire);
            if ((s >> 32) == seen) {
                const auto t0 = std::chrono::steady_clock::now();
                // poll the word itself for a few tens of microseconds (a new job is seen within
                // a cache-line transfer), then yield the core between polls, then sleep
                for (int it = 0; it < kBusyPolls && ((s = state_.load(std::memory_order_acquire)) >> 32) == seen; ++it) {}
                while (((s = state_.load(std::memory_order_acquire)) >> 32) == seen &&
                       std::chrono::steady_clock::now() - t0 < kSpin)
                    std::this_thread::yield();
                if ((s >> 32) == seen) {
                    std::unique_lock<std::mutex> l(mu_);
                    cv_.wait(l, [&] { return quit_ || (state_.load(std::memory_order_relaxed) >> 32) != seen; });
                    if (quit_) return;
                    continue;
                }
            }
            if (quit_.load(std::memory_order_acquire)) return;
            bool joined = false;
            while ((s >> 32) != seen) {
                if ((s & 0xffffull) >= ((s >> 16) & 0xffffull)) {   // every slot of this job taken
                    seen = s >> 32;
                    break;
                }
                if (state_.compare_exchange_weak(s, s + 1, std::memory_order_acq_rel, std::memory_order_acquire)) {
                    seen = s >> 32;
                    joined = true;
                    break;
                }
            }
            if (!joined) continue;
            work();
            if (busy_.fetch_sub(1, std::memory_order_acq_rel) == 1) {
                std::lock_guard<std::mutex> l(mu_);
                done_.notify_one();
            }
        }
    }
    std::vector<std::thread> th_;
    std::mutex mu_;
    std::condition_variable cv_, done_;
    // the job: written by the caller before it publishes a job number in state_; a worker
    // reads them after its claim on state_ (an acquire) succeeded
    std::atomic<const std::function<void(int)> *> fn_{nullptr};
    std::atomic<int> n_{0}, grain_{1};
    std::atomic<int> next_{0}, busy_{0};
    std::atomic<unsigned long long> state_{0};   // job number << 32 | helper slots << 16 | claimed
    std::atomic<bool> quit_{false};
};

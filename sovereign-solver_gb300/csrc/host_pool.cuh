// host_pool.cuh — host worker threads for the set-up's data-parallel loops.
//
// sps_create runs about ten loops over the rows, columns or nonzeros of the LP
// on host threads (validation scans, plan histograms and placement, prefix
// sums, the inverse orders, the ordering of long columns).  Creating and
// joining up to 16 threads per loop cost a few hundred microseconds each time;
// the pool's threads are created once per process, on first use, and a loop
// costs one wake-up.  One loop runs on the pool at a time: a caller that finds
// it busy (another thread's sps_create, or a loop started from inside a pool
// task) or that runs in a child process forked after the pool started gets
// threads of its own for that loop, as before.  Every loop's chunks and their
// order of results are fixed by the caller, so results do not depend on which
// thread ran a chunk.
#pragma once

#include <unistd.h>

#include <algorithm>
#include <condition_variable>
#include <cstdint>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace sps {

class HostPool {
public:
    static constexpr int kMaxThreads = 16;   // threads of one loop, the caller's included

    // f(t) for every t in [0, nt), f(0) on the calling thread; returns when all have run.
    template <class F>
    static void run(int nt, F&& f) {
        if (nt <= 1) {
            if (nt == 1) f(0);
            return;
        }
        HostPool& p = instance();
        std::unique_lock<std::mutex> own(p.call_mu_, std::try_to_lock);
        if (!own.owns_lock() || getpid() != p.pid_ || nt - 1 > p.workers_) {
            std::vector<std::thread> threads;
            for (int t = 1; t < nt; ++t) threads.emplace_back([&f, t] { f(t); });
            f(0);
            for (auto& th : threads) th.join();
            return;
        }
        std::function<void(int)> job = [&f](int t) { f(t); };
        {
            std::lock_guard<std::mutex> lk(p.mu_);
            p.job_ = &job;
            p.nt_ = nt;
            p.next_ = 1;
            p.left_ = nt - 1;
            ++p.gen_;
        }
        p.wake_.notify_all();
        f(0);
        std::unique_lock<std::mutex> lk(p.mu_);
        p.done_.wait(lk, [&] { return p.left_ == 0; });
        p.job_ = nullptr;
    }

private:
    // never destroyed: its threads wait for work until the process exits
    static HostPool& instance() {
        static HostPool* p = new HostPool();
        return *p;
    }
    HostPool() : pid_(getpid()) {
        const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
        workers_ = std::min(kMaxThreads, hw) - 1;
        for (int i = 0; i < workers_; ++i) std::thread([this] { serve(); }).detach();
    }
    void serve() {
        uint64_t seen = 0;
        std::unique_lock<std::mutex> lk(mu_);
        for (;;) {
            wake_.wait(lk, [&] { return gen_ != seen; });
            seen = gen_;
            while (job_ && next_ < nt_) {
                const int t = next_++;
                std::function<void(int)>* job = job_;
                lk.unlock();
                (*job)(t);
                lk.lock();
                if (--left_ == 0) done_.notify_one();
            }
        }
    }

    const pid_t pid_;
    int workers_ = 0;
    std::mutex call_mu_;                 // held by the caller of the loop on the pool
    std::mutex mu_;
    std::condition_variable wake_, done_;
    std::function<void(int)>* job_ = nullptr;
    int nt_ = 0, next_ = 0, left_ = 0;
    uint64_t gen_ = 0;
};

}  // namespace sps

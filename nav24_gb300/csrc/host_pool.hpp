// host_pool.hpp - host worker threads owned by one context.
//
// The host side of a batched solve (validation and graph build of every window, staging of the
// concatenated arrays, scattering of the results) is split over the host's cores.  Creating the
// threads on every call costs tens of microseconds per thread and adds jitter to the end-to-end
// time, so each context keeps its workers: they are started by the first call that needs them
// and joined when the context is destroyed.  There is no process-wide state.
#pragma once

#include <algorithm>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace navba {

class HostPool {
public:
    HostPool() = default;
    HostPool(const HostPool&) = delete;
    HostPool& operator=(const HostPool&) = delete;
    ~HostPool() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        wake_.notify_all();
        for (auto& t : th_) t.join();
    }

    // Number of tasks worth splitting n items into: one per core, at least min_items items each.
    static int tasks_for(int n, int min_items) {
        const int hw = std::max(1, (int)std::thread::hardware_concurrency());
        return std::max(1, std::min(hw, n / std::max(1, min_items)));
    }

    // fn(t) for every t in [0, ntask), on the calling thread and the workers; returns when all
    // have returned.  Which thread runs a task does not change what the task computes.
    void run(int ntask, const std::function<void(int)>& fn) {
        if (ntask <= 1) {
            if (ntask == 1) fn(0);
            return;
        }
        std::unique_lock<std::mutex> lk(mu_);
        while ((int)th_.size() < ntask - 1) th_.emplace_back([this] { work(); });
        job_ = &fn;
        ntask_ = ntask;
        next_ = 0;
        pending_ = ntask;
        lk.unlock();
        wake_.notify_all();
        drain();
        lk.lock();
        done_.wait(lk, [this] { return pending_ == 0; });
        job_ = nullptr;
    }

private:
    // take and run tasks of the current job until none is left
    void drain() {
        for (;;) {
            int t;
            const std::function<void(int)>* fn;
            {
                std::lock_guard<std::mutex> lk(mu_);
                if (!job_ || next_ >= ntask_) return;
                t = next_++;
                fn = job_;
            }
            (*fn)(t);
            std::lock_guard<std::mutex> lk(mu_);
            if (--pending_ == 0) done_.notify_all();
        }
    }

    void work() {
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu_);
                wake_.wait(lk, [this] { return stop_ || (job_ && next_ < ntask_); });
                if (stop_) return;
            }
            drain();
        }
    }

    std::vector<std::thread> th_;
    std::mutex mu_;
    std::condition_variable wake_, done_;
    const std::function<void(int)>* job_ = nullptr;
    int ntask_ = 0, next_ = 0, pending_ = 0;
    bool stop_ = false;
};

}  // namespace navba

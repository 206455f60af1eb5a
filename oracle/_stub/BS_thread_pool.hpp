// Minimal stand-in for the BS::thread_pool v5.1.0 interface that the reference solver's job
// pool uses (src/avbd/job_pool.hpp:17,156-174): a default constructor, detach_task() and
// get_thread_count(). Scheduling only; it performs no arithmetic, so solver results do not
// depend on it. Test infrastructure for the compiled reference under oracle/_ref.
#pragma once

#include <condition_variable>
#include <cstddef>
#include <deque>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace BS {

template <typename = void>
class thread_pool {
public:
    thread_pool() {
        unsigned n = std::thread::hardware_concurrency();
        if (n == 0)
            n = 1;
        for (unsigned i = 0; i < n; ++i)
            workers_.emplace_back([this] { run(); });
    }
    ~thread_pool() {
        {
            std::lock_guard<std::mutex> lock(mutex_);
            stop_ = true;
        }
        cv_.notify_all();
        for (std::thread &t : workers_)
            t.join();
    }
    thread_pool(const thread_pool &) = delete;
    thread_pool &operator=(const thread_pool &) = delete;

    template <typename F>
    void detach_task(F &&task) {
        {
            std::lock_guard<std::mutex> lock(mutex_);
            tasks_.emplace_back(std::forward<F>(task));
        }
        cv_.notify_one();
    }

    std::size_t get_thread_count() const { return workers_.size(); }

private:
    void run() {
        for (;;) {
            std::function<void()> task;
            {
                std::unique_lock<std::mutex> lock(mutex_);
                cv_.wait(lock, [this] { return stop_ || !tasks_.empty(); });
                if (stop_ && tasks_.empty())
                    return;
                task = std::move(tasks_.front());
                tasks_.pop_front();
            }
            task();
        }
    }

    std::vector<std::thread> workers_;
    std::deque<std::function<void()>> tasks_;
    std::mutex mutex_;
    std::condition_variable cv_;
    bool stop_ = false;
};

} // namespace BS

/*
 * Host worker pool that calls the data sources' getData for a frame's
 * missing bricks in parallel, each into its own pinned staging buffer. The
 * reference fetches on one upload thread
 * (livre/lib/pipeline/RenderPipeline.cpp:42, DataUploadFilter.cpp:45-72);
 * here a volume whose getData is re-entrant opts in to several fetchers
 * (lv_volume_set_fetch_threads), and the copies of one group of bricks to
 * the device overlap the fetch of the next.
 *
 * parallel_for runs body(i) for every i in [0, n) on the calling thread plus
 * up to width - 1 workers and returns when all calls have returned. One job
 * runs at a time; a second caller waits for the first.
 */
#ifndef LIVRE_GB300_HOST_POOL_H
#define LIVRE_GB300_HOST_POOL_H

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace lv
{
class HostPool
{
public:
    explicit HostPool(uint32_t workers)
    {
        for (uint32_t i = 0; i < workers; ++i)
            threads_.emplace_back([this] { work(); });
    }
    ~HostPool()
    {
        {
            std::lock_guard<std::mutex> lock(m_);
            stop_ = true;
        }
        wake_.notify_all();
        for (std::thread& t : threads_)
            t.join();
    }
    HostPool(const HostPool&) = delete;
    HostPool& operator=(const HostPool&) = delete;

    uint32_t workers() const { return uint32_t(threads_.size()); }

    void parallel_for(uint32_t n, uint32_t width, const std::function<void(uint32_t)>& body)
    {
        if (n == 0)
            return;
        std::lock_guard<std::mutex> job(job_);
        const uint32_t helpers =
            std::min<uint32_t>(width > 0 ? width - 1 : 0, std::min<uint32_t>(workers(), n - 1));
        if (helpers == 0)
        {
            for (uint32_t i = 0; i < n; ++i)
                body(i);
            return;
        }
        {
            std::lock_guard<std::mutex> lock(m_);
            body_ = &body;
            n_ = n;
            next_.store(0, std::memory_order_relaxed);
            wanted_ = helpers;
        }
        wake_.notify_all();
        drain();
        std::unique_lock<std::mutex> lock(m_);
        wanted_ = 0; /* helpers that have not started yet are not needed */
        done_.wait(lock, [this] { return running_ == 0; });
        body_ = nullptr;
    }

private:
    void drain()
    {
        for (uint32_t i = next_.fetch_add(1, std::memory_order_relaxed); i < n_;
             i = next_.fetch_add(1, std::memory_order_relaxed))
            (*body_)(i);
    }

    void work()
    {
        std::unique_lock<std::mutex> lock(m_);
        for (;;)
        {
            wake_.wait(lock, [this] { return stop_ || wanted_ > 0; });
            if (stop_)
                return;
            --wanted_;
            ++running_;
            lock.unlock();
            drain();
            lock.lock();
            if (--running_ == 0)
                done_.notify_all();
        }
    }

    std::vector<std::thread> threads_;
    std::mutex job_; /* one parallel_for at a time */
    std::mutex m_;
    std::condition_variable wake_, done_;
    const std::function<void(uint32_t)>* body_ = nullptr;
    uint32_t n_ = 0;
    std::atomic<uint32_t> next_{0};
    uint32_t wanted_ = 0, running_ = 0;
    bool stop_ = false;
};
} // namespace lv

#endif

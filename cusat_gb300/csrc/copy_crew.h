// Host-side helper of the receive chain: one large copy split across helper
// threads.  Header-only (standard library only) so that it can be checked on
// its own (tests/copy_crew_check.cc).
#pragma once

#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <vector>

namespace cusat_internal {

// Splits a frame's copy into the pinned ring across helper threads (opt-in:
// one Grace core copies about 18 GB/s, so a 172.8 KB frame costs ~8-9 us on
// the submitting thread alone).  Helpers spin while copies keep coming and
// sleep on a condition variable after a quiet interval.
class CopyCrew {
  public:
    explicit CopyCrew(int helpers) : helpers_(helpers)
    {
        for (int i = 0; i < helpers_; i++)
            th_.emplace_back([this, i] { run(i + 1); });
    }
    ~CopyCrew()
    {
        {
            std::lock_guard<std::mutex> lk(m_);
            stop_.store(true);
        }
        cv_.notify_all();
        for (auto& t : th_)
            t.join();
    }
    void copy(void* dst, const void* src, size_t bytes)
    {
        if (helpers_ == 0 || bytes < kMinSplit) {
            memcpy(dst, src, bytes);
            return;
        }
        dst_ = static_cast<uint8_t*>(dst);
        src_ = static_cast<const uint8_t*>(src);
        bytes_ = bytes;
        pending_.store(helpers_, std::memory_order_relaxed);
        gen_.fetch_add(1, std::memory_order_release);
        {
            std::lock_guard<std::mutex> lk(m_);  // a helper between its check and its wait sees the job
        }
        cv_.notify_all();
        part(0);
        while (pending_.load(std::memory_order_acquire) > 0) {
        }
    }

  private:
    static constexpr size_t kMinSplit = 32 << 10;  // smaller copies stay on the calling thread
    void part(int id)
    {
        const int parts = helpers_ + 1;
        const size_t chunk = ((bytes_ + parts - 1) / parts + 63) & ~(size_t)63;
        const size_t b0 = std::min(bytes_, chunk * (size_t)id), b1 = std::min(bytes_, b0 + chunk);
        if (b1 > b0)
            memcpy(dst_ + b0, src_ + b0, b1 - b0);
    }
    void run(int id)
    {
        uint64_t seen = 0;  // the generation at construction: a job published before this thread runs is still new
        for (;;) {
            auto last = std::chrono::steady_clock::now();
            while (gen_.load(std::memory_order_acquire) == seen && !stop_.load()) {
                if (std::chrono::steady_clock::now() - last > std::chrono::microseconds(500)) {
                    std::unique_lock<std::mutex> lk(m_);
                    cv_.wait_for(lk, std::chrono::milliseconds(5),
                                 [&] { return gen_.load(std::memory_order_acquire) != seen || stop_.load(); });
                    last = std::chrono::steady_clock::now();
                }
            }
            if (stop_.load())
                return;
            seen = gen_.load(std::memory_order_acquire);
            part(id);
            pending_.fetch_sub(1, std::memory_order_release);
        }
    }
    const int helpers_;
    std::vector<std::thread> th_;
    std::atomic<uint64_t> gen_{0};
    std::atomic<int> pending_{0};
    std::atomic<bool> stop_{false};
    std::mutex m_;
    std::condition_variable cv_;
    uint8_t* dst_ = nullptr;
    const uint8_t* src_ = nullptr;
    size_t bytes_ = 0;
};

}  // namespace cusat_internal

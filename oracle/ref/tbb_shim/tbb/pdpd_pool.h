// A stand-in for the parts of oneTBB that the reference's TBB engines use, so that those
// engines compile unchanged where oneTBB is not installed (baseline infrastructure only: the
// timed CPU baseline and nothing else).  This file is the scheduler: one persistent pool of
// worker threads; a parallel loop cuts its range into chunks up front and the workers (and
// the calling thread) take chunks from the loop's atomic counter.  Workers spin briefly
// between loops before they sleep, as TBB's workers do, so the many short loops of one DPD
// step do not each pay a sleep and a wake-up.
//
// Thread count: PDPD_NUM_THREADS if set, else std::thread::hardware_concurrency(); a
// tbb::global_control of max_allowed_parallelism lowers it while it lives.
#pragma once

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace pdpd_tbb_shim {

class Pool {
public:
    static Pool &instance()
    {
        static Pool p;
        return p;
    }

    unsigned max_threads() const { return (unsigned)workers_.size() + 1; }
    unsigned threads() const
    {
        const unsigned l = limit_.load();
        return (l && l < max_threads()) ? l : max_threads();
    }
    void set_limit(unsigned n) { limit_.store(n); }

    // Runs body(c) for every chunk c in [0, n_chunks) on up to threads() threads and returns
    // when all are done.  A loop started from inside a chunk runs serially on its thread.
    void run(size_t n_chunks, const std::function<void(size_t)> &body)
    {
        if (n_chunks == 0) return;
        const unsigned nt = threads();
        if (n_chunks == 1 || nt <= 1 || in_loop_) {
            for (size_t c = 0; c < n_chunks; c++) body(c);
            return;
        }
        std::lock_guard<std::mutex> one_loop_at_a_time(run_mutex_);
        Loop L;
        L.body = &body;
        L.n = n_chunks;
        L.seats = nt - 1;
        {
            std::lock_guard<std::mutex> lk(m_);
            current_ = &L;
            generation_.fetch_add(1, std::memory_order_release);
        }
        cv_.notify_all();
        in_loop_ = true;
        L.work();
        in_loop_ = false;
        while (L.done.load(std::memory_order_acquire) < n_chunks) std::this_thread::yield();
        {
            std::lock_guard<std::mutex> lk(m_);
            current_ = nullptr;
        }
        // Workers that joined hold a reference until they leave the loop.
        while (L.refs.load(std::memory_order_acquire) != 0) std::this_thread::yield();
    }

private:
    struct Loop {
        const std::function<void(size_t)> *body = nullptr;
        size_t n = 0;
        unsigned seats = 0;  // how many workers may join (the thread limit)
        std::atomic<size_t> next{0}, done{0};
        std::atomic<unsigned> refs{0};
        void work()
        {
            for (;;) {
                const size_t c = next.fetch_add(1, std::memory_order_relaxed);
                if (c >= n) return;
                (*body)(c);
                done.fetch_add(1, std::memory_order_release);
            }
        }
    };

    Pool()
    {
        unsigned n = std::thread::hardware_concurrency();
        if (const char *e = std::getenv("PDPD_NUM_THREADS")) {
            const int k = std::atoi(e);
            if (k > 0) n = (unsigned)k;
        }
        if (n < 1) n = 1;
        for (unsigned i = 1; i < n; i++) workers_.emplace_back([this] { worker(); });
    }
    ~Pool()
    {
        {
            std::lock_guard<std::mutex> lk(m_);
            stop_ = true;
            generation_.fetch_add(1);
        }
        cv_.notify_all();
        for (auto &t : workers_) t.join();
    }

    void worker()
    {
        in_loop_ = true;  // loops started from a chunk run serially
        unsigned seen = 0;
        for (;;) {
            const auto t0 = std::chrono::steady_clock::now();
            while (generation_.load(std::memory_order_acquire) == seen) {
                if (std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(300)) {
                    std::unique_lock<std::mutex> lk(m_);
                    cv_.wait(lk, [&] { return generation_.load() != seen; });
                }
            }
            Loop *L = nullptr;
            {
                std::lock_guard<std::mutex> lk(m_);
                seen = generation_.load();
                if (stop_) return;
                if (current_ && current_->refs.load() < current_->seats) {
                    L = current_;
                    L->refs.fetch_add(1);
                }
            }
            if (L) {
                L->work();
                L->refs.fetch_sub(1, std::memory_order_release);
            }
        }
    }

    std::vector<std::thread> workers_;
    std::mutex m_, run_mutex_;
    std::condition_variable cv_;
    std::atomic<unsigned> generation_{0};
    std::atomic<unsigned> limit_{0};
    Loop *current_ = nullptr;
    bool stop_ = false;
    static thread_local bool in_loop_;
};

inline thread_local bool Pool::in_loop_ = false;

}  // namespace pdpd_tbb_shim

// par.hpp -- host-thread helpers of the planning code (neighbour search,
// patch tables, full-tree planning). The work items are independent per
// block and write disjoint ranges. A persistent pool of worker threads runs
// them: a planning pass makes dozens of parallel calls, and starting threads
// per call costs more than the small ones take.
#pragma once
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace wg {

inline int host_threads() {
    const unsigned h = std::thread::hardware_concurrency();
    return h ? (int)std::min(h, 32u) : 4;
}

// Fork-join pool: run(n, f) calls f(0..n-1) on the workers and the caller
// and returns when all calls are done. One job at a time (callers from
// several threads take turns); a call from inside a job runs inline. The
// job's state lives on the caller's stack: a worker joins it under the lock
// while it is posted, and the caller returns only after every joined worker
// has left. The pool is rebuilt in a forked child (threads do not survive
// fork).
class Pool {
public:
    static Pool &get() {
        static std::mutex m;
        static Pool *p = nullptr;
        std::lock_guard<std::mutex> lk(m);
        if (!p || p->pid_ != getpid()) p = new Pool(host_threads() - 1);   // a parent's pool is left as is
        return *p;
    }
    void run(int n, const std::function<void(int)> &f) {
        if (n <= 0) return;
        if (in_job() || workers_.empty() || n == 1) {
            for (int i = 0; i < n; i++) f(i);
            return;
        }
        std::lock_guard<std::mutex> one(job_mutex_);
        Job job;
        job.f = &f;
        job.n = n;
        job.left.store(n);
        {
            std::lock_guard<std::mutex> lk(m_);
            cur_ = &job;
            gen_++;
        }
        cv_.notify_all();
        work(job);
        std::unique_lock<std::mutex> lk(m_);
        cur_ = nullptr;   // no worker joins any more
        done_.wait(lk, [&] { return job.left.load() == 0 && job.active == 0; });
    }

private:
    struct Job {
        const std::function<void(int)> *f = nullptr;
        int n = 0;
        std::atomic<int> next{0}, left{0};
        int active = 0;   // workers inside the job (guarded by m_)
    };
    explicit Pool(int nworkers) : pid_(getpid()) {
        for (int i = 0; i < nworkers; i++) workers_.emplace_back([this] { loop(); });
        for (auto &t : workers_) t.detach();
    }
    static bool &in_job() {
        static thread_local bool flag = false;
        return flag;
    }
    void work(Job &j) {
        const bool outer = in_job();
        in_job() = true;
        for (;;) {
            const int i = j.next.fetch_add(1);
            if (i >= j.n) break;
            (*j.f)(i);
            if (j.left.fetch_sub(1) == 1) {
                std::lock_guard<std::mutex> lk(m_);
                done_.notify_all();
            }
        }
        in_job() = outer;
    }
    void loop() {
        unsigned long long seen = 0;
        for (;;) {
            Job *j;
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
                j = cur_;
                if (!j) continue;
                j->active++;
            }
            work(*j);
            {
                std::lock_guard<std::mutex> lk(m_);
                j->active--;
            }
            done_.notify_all();
        }
    }
    pid_t pid_;
    std::vector<std::thread> workers_;
    std::mutex m_, job_mutex_;
    std::condition_variable cv_, done_;
    Job *cur_ = nullptr;
    unsigned long long gen_ = 0;
};

// f(chunk, lo, hi) on contiguous chunks of [0, n); below min_n items one
// call on the calling thread
template <class F>
void par_chunks(int n, int nchunk, F f, int min_n = 8192) {
    if (nchunk <= 1 || n < min_n) {
        f(0, 0, n);
        return;
    }
    Pool::get().run(nchunk, [&](int c) {
        const int lo = (int)((long long)n * c / nchunk), hi = (int)((long long)n * (c + 1) / nchunk);
        f(c, lo, hi);
    });
}

// f(task) for task = 0..ntask-1
template <class F>
void par_tasks(int ntask, F f) {
    Pool::get().run(ntask, [&](int t) { f(t); });
}

}  // namespace wg

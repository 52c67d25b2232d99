// Host check of the planning thread pool (wabbit_gb300/csrc/par.hpp): every
// index of every job runs exactly once, nested calls run inline, callers on
// several threads take turns, and a forked child gets a working pool.
#include "par.hpp"

#include <sys/wait.h>
#include <unistd.h>

#include <atomic>
#include <cstdio>
#include <thread>
#include <vector>

static int check_jobs(int njobs, int seed) {
    int fail = 0;
    for (int j = 0; j < njobs; j++) {
        const int n = 1 + (j * 7919 + seed) % 97;
        std::vector<std::atomic<int>> hits(n);
        for (auto &h : hits) h.store(0);
        wg::par_tasks(n, [&](int i) { hits[i].fetch_add(1); });
        for (int i = 0; i < n; i++) fail += hits[i].load() != 1;
    }
    return fail;
}

int main() {
    int fail = 0;
    // many small jobs in a row (workers joining late must not touch the next job)
    fail += check_jobs(5000, 1);
    // chunks cover [0, n) exactly once
    {
        const int n = 100000;
        std::vector<std::atomic<int>> hits(n);
        for (auto &h : hits) h.store(0);
        wg::par_chunks(n, wg::host_threads(), [&](int, int lo, int hi) {
            for (int i = lo; i < hi; i++) hits[i].fetch_add(1);
        }, 1);
        for (int i = 0; i < n; i++) fail += hits[i].load() != 1;
    }
    // a parallel call inside a job runs inline
    {
        std::atomic<int> inner{0};
        wg::par_tasks(8, [&](int) { wg::par_tasks(8, [&](int) { inner.fetch_add(1); }); });
        fail += inner.load() != 64;
    }
    // callers on several threads take turns
    {
        std::atomic<int> bad{0};
        std::vector<std::thread> th;
        for (int t = 0; t < 4; t++) th.emplace_back([&, t] { bad += check_jobs(500, 10 + t); });
        for (auto &x : th) x.join();
        fail += bad.load();
    }
    // a forked child builds its own pool
    {
        const pid_t pid = fork();
        if (pid == 0) _exit(check_jobs(200, 99) == 0 ? 0 : 1);
        int status = 0;
        waitpid(pid, &status, 0);
        fail += !(WIFEXITED(status) && WEXITSTATUS(status) == 0);
    }
    std::printf("pool failures %d\n", fail);
    return fail ? 1 : 0;
}

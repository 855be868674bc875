// Test helper (host code only): exercises sps::HostPool
// (sovereign-solver_gb300/csrc/host_pool.cuh) for tests/test_host_pool.py.
// Every check prints one line; the exit status is 0 when all hold.
//   loops     many loops in a row: every chunk of every loop runs exactly once
//   callers   four threads start loops at once (the pool takes one, the others
//             fall back to threads of their own)
//   nested    a loop started from inside a pool task (falls back)
//   fork      a child process forked after the pool started runs loops (falls back)
#include "host_pool.cuh"

#include <sys/wait.h>

#include <atomic>
#include <cstdio>
#include <vector>

using sps::HostPool;

static bool one_loop(int nt, int items) {
    std::vector<std::atomic<int>> hits(items);
    for (auto& h : hits) h = 0;
    HostPool::run(nt, [&](int t) {
        for (int i = items * t / nt; i < items * (t + 1) / nt; ++i) hits[i]++;
    });
    for (auto& h : hits)
        if (h != 1) return false;
    return true;
}

int main() {
    bool ok = true, r = true;
    for (int k = 0; k < 2000 && r; ++k) r = one_loop(1 + k % 16, 1000 + k);
    std::printf("loops %s\n", r ? "ok" : "FAIL");
    ok &= r;

    std::atomic<bool> all{true};
    std::vector<std::thread> callers;
    for (int c = 0; c < 4; ++c)
        callers.emplace_back([&, c] {
            for (int k = 0; k < 300; ++k)
                if (!one_loop(2 + (k + c) % 15, 5000)) all = false;
        });
    for (auto& t : callers) t.join();
    std::printf("callers %s\n", all ? "ok" : "FAIL");
    ok &= all.load();

    std::atomic<int> inner{0};
    HostPool::run(8, [&](int) {
        HostPool::run(4, [&](int) { inner++; });
    });
    std::printf("nested %s\n", inner == 32 ? "ok" : "FAIL");
    ok &= inner == 32;

    const pid_t pid = fork();
    if (pid == 0) {
        bool c = true;
        for (int k = 0; k < 50 && c; ++k) c = one_loop(8, 4096);
        _exit(c ? 0 : 1);
    }
    int status = 1;
    const bool forked = pid > 0 && waitpid(pid, &status, 0) == pid && WIFEXITED(status) && WEXITSTATUS(status) == 0;
    std::printf("fork %s\n", forked ? "ok" : "FAIL");
    ok &= forked;
    return ok ? 0 : 1;
}

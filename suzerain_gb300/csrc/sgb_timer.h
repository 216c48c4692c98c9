// Per-phase CUDA-event timing on the launching stream and a launch counter,
// used by the benchmark to attribute time to kernels without a profiler.
#pragma once
#include <cuda_runtime.h>
#include <atomic>
#include <map>
#include <string>
#include <vector>

namespace sgb {

// Every kernel launch of the library increments this counter.
extern std::atomic<long long> g_launches;
inline void count_launch(long long k = 1) { g_launches.fetch_add(k, std::memory_order_relaxed); }

struct PhaseTimer {
    bool on = false;
    struct Rec { std::string name; cudaEvent_t a, b; };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    std::map<std::string, std::pair<double, long long>> acc;   // ms, calls
    std::string open_name;
    cudaEvent_t open_ev = nullptr;

    cudaEvent_t ev()
    {
        if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
    void begin(const char *name, cudaStream_t st)
    {
        if (!on) return;
        open_name = name;
        open_ev = ev();
        cudaEventRecord(open_ev, st);
    }
    void end(cudaStream_t st)
    {
        if (!on || !open_ev) return;
        cudaEvent_t b = ev();
        cudaEventRecord(b, st);
        recs.push_back({open_name, open_ev, b});
        open_ev = nullptr;
    }
    void collect()
    {
        for (auto &r : recs) {
            cudaEventSynchronize(r.b);
            float ms = 0;
            cudaEventElapsedTime(&ms, r.a, r.b);
            auto &x = acc[r.name];
            x.first += ms;
            x.second += 1;
            pool.push_back(r.a);
            pool.push_back(r.b);
        }
        recs.clear();
    }
    ~PhaseTimer()
    {
        for (auto &r : recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
        for (auto e : pool) cudaEventDestroy(e);
    }
};

}  // namespace sgb

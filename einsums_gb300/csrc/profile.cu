// Kernel launch accounting and event-based per-kernel timing.
#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace eg {
namespace {
std::atomic<uint64_t> g_launches{0};
thread_local bool g_capture = false; // launches being captured into a graph are counted at replay
std::atomic<int> g_enabled{0};
struct Rec {
    const char *name;
    cudaEvent_t e0, e1;
};
std::mutex &g_mu = *new std::mutex;
std::vector<Rec> &g_pending = *new std::vector<Rec>;
std::vector<cudaEvent_t> &g_pool = *new std::vector<cudaEvent_t>;
auto &g_totals = *new std::map<std::string, std::pair<uint64_t, double>>;

cudaEvent_t get_event() {
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

eg_status drain() {
    for (const Rec &r : g_pending) {
        cudaError_t err = cudaEventSynchronize(r.e1);
        if (err != cudaSuccess) return cuda_fail(err, "cudaEventSynchronize");
        float ms = 0.f;
        err = cudaEventElapsedTime(&ms, r.e0, r.e1);
        if (err != cudaSuccess) return cuda_fail(err, "cudaEventElapsedTime");
        auto &t = g_totals[r.name];
        t.first += 1;
        t.second += ms;
        g_pool.push_back(r.e0);
        g_pool.push_back(r.e1);
    }
    g_pending.clear();
    return EG_SUCCESS;
}
} // namespace

void set_capture_mode(bool on) { g_capture = on; }
void count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

LaunchScope::LaunchScope(const char *name, cudaStream_t s) : name_(name), s_(s) {
    if (g_capture) return;
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (g_enabled.load(std::memory_order_relaxed)) {
        std::lock_guard<std::mutex> lk(g_mu);
        e0_ = get_event();
        e1_ = get_event();
        cudaEventRecord(e0_, s_);
    }
}

LaunchScope::~LaunchScope() {
    if (e0_) {
        cudaEventRecord(e1_, s_);
        std::lock_guard<std::mutex> lk(g_mu);
        g_pending.push_back(Rec{name_, e0_, e1_});
        if (g_pending.size() > 4096) drain();
    }
}

} // namespace eg

extern "C" {
eg_status eg_kernel_launches(uint64_t *count) {
    if (!count) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "count is NULL");
    *count = eg::g_launches.load();
    return EG_SUCCESS;
}

eg_status eg_profile_enable(int32_t on) {
    eg::g_enabled.store(on ? 1 : 0);
    return EG_SUCCESS;
}

eg_status eg_profile_reset(void) {
    std::lock_guard<std::mutex> lk(eg::g_mu);
    eg_status st = eg::drain();
    eg::g_totals.clear();
    return st;
}

eg_status eg_profile_summary(char *buf, size_t cap) {
    if (!buf || cap == 0) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "buffer is NULL");
    std::lock_guard<std::mutex> lk(eg::g_mu);
    eg_status st = eg::drain();
    if (st != EG_SUCCESS) return st;
    std::string out;
    for (auto &kv : eg::g_totals)
        out += kv.first + "," + std::to_string(kv.second.first) + "," + std::to_string(kv.second.second) + "\n";
    size_t n = out.size() < cap - 1 ? out.size() : cap - 1;
    memcpy(buf, out.data(), n);
    buf[n] = 0;
    return EG_SUCCESS;
}
}

// gvr_profile.cu -- per-kernel timing with CUDA events on the launching
// stream (enabled on demand) and a count of every kernel the library launches.
#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "gvr_profile.h"

namespace gvr {
namespace {

struct Pending {
    const char *name;
    cudaEvent_t a, b;
};

struct Tally {
    long long launches = 0;
    double ms = 0.0;
};

std::mutex g_mu;
bool g_enabled = false;
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_pool;
std::map<std::string, Tally> g_tally;
std::atomic<long long> g_launches{0};

cudaEvent_t take_event() {
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void drain_locked() {
    for (auto &p : g_pending) {
        float ms = 0.0f;
        if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            Tally &t = g_tally[p.name];
            t.launches += 1;
            t.ms += ms;
        }
        g_pool.push_back(p.a);
        g_pool.push_back(p.b);
    }
    g_pending.clear();
}

}  // namespace

KernelScope::KernelScope(cudaStream_t st, const char *name) : st_(st), name_(name) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_enabled) return;
    // no timing inside a stream capture: the launch becomes a graph node
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st_, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) return;
    a_ = take_event();
    b_ = take_event();
    if (a_ && b_) cudaEventRecord(a_, st_);
}

KernelScope::~KernelScope() {
    if (!a_ || !b_) return;
    cudaEventRecord(b_, st_);
    std::lock_guard<std::mutex> lk(g_mu);
    g_pending.push_back(Pending{name_, a_, b_});
}

}  // namespace gvr

extern "C" {

int gvr_profile_enable(int enable) {
    std::lock_guard<std::mutex> lk(gvr::g_mu);
    int prev = gvr::g_enabled ? 1 : 0;
    gvr::drain_locked();
    gvr::g_tally.clear();
    gvr::g_enabled = enable != 0;
    return prev;
}

int gvr_profile_read(GvrKernelTime *out, int capacity) {
    std::lock_guard<std::mutex> lk(gvr::g_mu);
    gvr::drain_locked();
    int n = 0;
    for (auto &kv : gvr::g_tally) {
        if (out && n < capacity) {
            std::memset(&out[n], 0, sizeof(GvrKernelTime));
            std::strncpy(out[n].name, kv.first.c_str(), sizeof(out[n].name) - 1);
            out[n].launches = kv.second.launches;
            out[n].total_ms = kv.second.ms;
        }
        ++n;
    }
    return n;
}

long long gvr_launch_count(void) { return gvr::g_launches.load(); }

}  // extern "C"

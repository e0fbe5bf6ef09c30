// gvr_profile.cu -- per-kernel timing with CUDA events on the launching
// stream (enabled on demand) and a count of every kernel the library launches.
#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <cstdint>

#include "gvr.h"
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

// Every thread walks a linear congruential sequence of sector indices; the
// sector's first float (or float4) takes the addition.  Indices stay below
// `sectors`, so every access lies in the buffer.
__global__ void __launch_bounds__(256) k_probe_reductions(float *__restrict__ buf, unsigned sectors, int vector4,
                                                          int rounds) {
    unsigned h = (blockIdx.x * 256u + threadIdx.x) * 2654435761u + 12345u;
    for (int r = 0; r < rounds; ++r) {
        h = h * 1664525u + 1013904223u;
        const size_t s = (size_t)(h % sectors) * 8;
        if (vector4) atomicAdd(reinterpret_cast<float4 *>(buf + s), make_float4(1.0f, 1.0f, 1.0f, 1.0f));
        else atomicAdd(buf + s, 1.0f);
    }
}

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

int gvr_probe_reductions(float *buf, long long words, int vector4, int rounds, int grid, void *stream) {
    if (!buf || words < 8 || words % 8 != 0 || words / 8 > 0xffffffffll || rounds < 1 || grid < 1 ||
        (reinterpret_cast<uintptr_t>(buf) & 31) != 0)
        return GVR_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    GVR_LAUNCH(st, "k_probe_reductions",
               gvr::k_probe_reductions<<<grid, 256, 0, st>>>(buf, (unsigned)(words / 8), vector4, rounds));
    return cudaGetLastError() == cudaSuccess ? GVR_OK : GVR_ERR_CUDA;
}

}  // extern "C"

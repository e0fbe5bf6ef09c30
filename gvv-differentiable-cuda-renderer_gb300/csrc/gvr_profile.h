// gvr_profile.h -- scope object wrapped around every kernel launch.
#pragma once

#include <cuda_runtime.h>

#include <utility>

#include "gvr.h"

namespace gvr {

// Counts the launch; when profiling is on, records an event pair around it
// on `st` (read back by gvr_profile_read).
class KernelScope {
   public:
    KernelScope(cudaStream_t st, const char *name);
    ~KernelScope();
    KernelScope(const KernelScope &) = delete;
    KernelScope &operator=(const KernelScope &) = delete;

   private:
    cudaStream_t st_;
    const char *name_;
    cudaEvent_t a_ = nullptr, b_ = nullptr;
};

}  // namespace gvr

// Launches kernel<<<grid, block, smem, st>>>(args...) as a programmatic
// dependent launch: the grid may be launched while the previous kernel on
// `st` runs its last wave (the kernels of a call let their dependents launch
// as they start), and each such kernel begins with pdl_enter(), which waits
// until the previous kernel has completed and its writes are visible.  This
// takes the launch latency and the ramp-up of each grid off the critical
// path between the dependent kernels of a call.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

#define GVR_LAUNCH(st, name, ...)              \
    do {                                       \
        ::gvr::KernelScope _gvr_scope(st, name); \
        __VA_ARGS__;                           \
    } while (0)

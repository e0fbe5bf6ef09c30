// gvr_profile.h -- scope object wrapped around every kernel launch.
#pragma once

#include <cuda_runtime.h>

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

#define GVR_LAUNCH(st, name, ...)              \
    do {                                       \
        ::gvr::KernelScope _gvr_scope(st, name); \
        __VA_ARGS__;                           \
    } while (0)

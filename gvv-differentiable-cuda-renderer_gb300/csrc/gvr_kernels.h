// gvr_kernels.h -- host-side launchers shared by the C-ABI layer.
#pragma once

#include "gvr_internal.cuh"

namespace gvr {

// Stages of the batched forward; each has its own index space per job.
enum BatchStage { kStageViews = 0, kStageFaces, kStageVertices, kStageBinCount, kStageBinFill, kNumStages };
constexpr int kBatchBlock = 256;  // threads per block of the batched stage kernels

// Device tables of one batched forward (all pointers device memory).
struct BatchLaunch {
    const FwdJob *jobs;                 // [nJobs]
    const int *blockStart[kNumStages];  // [nJobs + 1] first block of each job per stage
    int blocks[kNumStages];             // total blocks per stage
    const int *itemStart;               // [nJobs + 1] first raster item (view tile) of each job
    int *counter;                       // persistent raster work counter (cleared per launch)
    int nJobs;
    int rasterGrid;                     // resident blocks of the persistent raster
    void *zeroBase;                     // every job's per-call counters, contiguous, and the work counter
    size_t zeroBytes;
};

cudaError_t launch_cameras(const float *extr, const float *intr, Camera *cams, int count, cudaStream_t st);
cudaError_t launch_face_geo(const float *verts, const Topology &topo, FaceGeo *geo, float4 *fnormal, int B,
                            cudaStream_t st, float4 *bwdRec = nullptr);
cudaError_t launch_forward(const FwdJob &J, cudaStream_t st);
cudaError_t launch_forward_normal_map(const FwdJob &J, int *uvOwner, float *normal_map, cudaStream_t st);
cudaError_t launch_forward_batched(const BatchLaunch &L, cudaStream_t st);
cudaError_t launch_normal_map(const Topology &topo, const FrameDims &dims, int *owner, const float *vnormal,
                              float *normal_map, int32_t *face, float *bary, float *render, cudaStream_t st);
cudaError_t launch_backward(const Topology &topo, const FrameDims &dims, const BwdScratch &ws, const GvrBackwardArgs &a,
                            int imageFilter, cudaStream_t st);
cudaError_t launch_raster(const FwdJob &J, cudaStream_t st);
cudaError_t launch_raster_persistent(const FwdJob *jobs, const int *itemStart, int nJobs, int *counter, int grid,
                                     cudaStream_t st);
int raster_persistent_blocks_per_sm();
cudaError_t launch_debug_rays(const Camera *cams, float *out, int BC, int W, int H, cudaStream_t st);

}  // namespace gvr

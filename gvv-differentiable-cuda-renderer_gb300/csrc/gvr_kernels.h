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

// Stages of the batched backward, each with its own index space per job.
enum BwdBatchStage { kBStageViews = 0, kBStageFaces, kBStageVertices, kBStageSH, kNumBwdStages };

// A device region cleared by the batched backward (a gradient output or a
// per-face accumulator), in floats.
struct ZeroRegion {
    float *ptr;
    long long count;
};
constexpr int kZeroPerBlock = 4096;  // floats one block of the zeroing kernel clears

// Variant of the backward pixel kernel: albedo class x shaded x target
// gradient x albedo-through-barycentrics (see backward_variant).
constexpr int kNumBwdVariants = 32;

// Device tables of one batched backward (all pointers device memory).
struct BwdBatchLaunch {
    const BwdJob *jobs;                     // [nJobs]
    const int *blockStart[kNumBwdStages];   // [nJobs + 1] first block of each job per stage
    int blocks[kNumBwdStages];
    const ZeroRegion *zeros;                // [nZero]
    const int *zeroStart;                   // [nZero + 1] first block of each region
    int nZero, zeroBlocks;
    // the pixel kernel, one launch per variant present: jobs of the variant
    // and their first tile blocks
    int nGroups;
    int groupVariant[kNumBwdVariants];
    const int *groupJobs[kNumBwdVariants];  // [groupCount[g]] job indices
    const int *groupStart[kNumBwdVariants]; // [groupCount[g] + 1]
    int groupCount[kNumBwdVariants];
    int groupBlocks[kNumBwdVariants];
    int nJobs;
};

// The pixel-kernel variant of a backward call, or -1 for the zero-gradient modes.
int backward_variant(int albedo, int shading, bool target, bool albpos);

// One call's set-up in one launch (k_setup): face pass, camera records and
// a region cleared to zero.
struct SetupArgs {
    const float *verts;       // [B,N,3]
    const int32_t *faces;     // [F*3]
    const float *uvs;         // [F*6] (the backward's face records) or null
    int N, F, B;
    FaceGeo *geo;             // [B*F]
    float4 *fnormal;          // [B*F] or null
    float4 *faceC;            // [B*F] centroid and smallest altitude (the forward's skip tests), or null
    float4 *rec;              // [B*F*kBwdFaceRows] backward face records, or null
    float4 *faceAcc;          // [B*F*kFaceAccFloats/4] cleared, or null
    const float *extr, *intr; // [views,12], [views,9]
    Camera *cams;             // [views]
    int views;
    void *zero;               // region cleared (zeroWords 4-byte words), or null
    long long zeroWords;
    int zeroVec;              // set by the launcher: the region is 16-byte aligned
};
cudaError_t launch_setup(SetupArgs a, cudaStream_t st);
cudaError_t launch_cameras(const float *extr, const float *intr, Camera *cams, int count, cudaStream_t st);
cudaError_t launch_face_geo(const float *verts, const Topology &topo, FaceGeo *geo, float4 *fnormal, int B,
                            cudaStream_t st, float4 *bwdRec = nullptr);
cudaError_t launch_forward(const FwdJob &J, cudaStream_t st);
cudaError_t launch_forward_normal_map(const FwdJob &J, int *uvOwner, float *normal_map, cudaStream_t st);
cudaError_t launch_forward_batched(const BatchLaunch &L, cudaStream_t st, bool raster = true);
cudaError_t launch_normal_map(const Topology &topo, const FrameDims &dims, int *owner, const float *vnormal,
                              float *normal_map, int32_t *face, float *bary, float *render, cudaStream_t st);
cudaError_t launch_backward(const Topology &topo, const FrameDims &dims, const BwdScratch &ws, const GvrBackwardArgs &a,
                            int imageFilter, cudaStream_t st);
cudaError_t launch_backward_batched(const BwdBatchLaunch &L, cudaStream_t st);
cudaError_t launch_bwd_geo_batched(const BwdBatchLaunch &L, cudaStream_t st);
cudaError_t launch_raster(const FwdJob &J, cudaStream_t st);
cudaError_t launch_raster_persistent(const FwdJob *jobs, const int *itemStart, int nJobs, int *counter, int grid,
                                     cudaStream_t st);
int raster_persistent_blocks_per_sm();
cudaError_t launch_debug_rays(const Camera *cams, float *out, int BC, int W, int H, cudaStream_t st);

}  // namespace gvr

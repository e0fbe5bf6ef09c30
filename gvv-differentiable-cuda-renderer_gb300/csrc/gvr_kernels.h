// gvr_kernels.h -- host-side launchers shared by the C-ABI layer.
#pragma once

#include "gvr_internal.cuh"

namespace gvr {

cudaError_t launch_cameras(const float *extr, const float *intr, Camera *cams, int count, cudaStream_t st);
cudaError_t launch_face_geo(const float *verts, const Topology &topo, FaceGeo *geo, float4 *fnormal, int B,
                            cudaStream_t st);
cudaError_t launch_forward(const Topology &topo, const FrameDims &dims, const FwdScratch &ws, const float *verts,
                           const float *colors, const float *texture, const float *sh, const float *extr,
                           const float *intr, float *bary, int32_t *face, float *render, float *vnormal,
                           float4 *proj, cudaStream_t st);
cudaError_t launch_backward(const Topology &topo, const FrameDims &dims, const BwdScratch &ws, const GvrBackwardArgs &a,
                            int imageFilter, cudaStream_t st);
cudaError_t launch_raster(const Topology &topo, const FrameDims &dims, const FwdScratch &ws, const RasterIO &io,
                          cudaStream_t st);
cudaError_t launch_debug_rays(const Camera *cams, float *out, int BC, int W, int H, cudaStream_t st);

}  // namespace gvr

// gvr_image.cu -- image-space helpers of the reference renderer
// (cpp/src/Renderer/gradientImage.cu:8-67): a 3x3 Sobel gradient scaled by
// 1/8 and a 3x3 binomial blur over float RGB images [B, H, W, 3].
//
// Same stencils, borders and FP32 operation order as the reference (every
// operation rounded on its own, as the reference built with -fmad=false):
//   gradient: zero where x < 1, y < 1, x >= W - 2 or y >= H - 2;
//   blur:     pixels with x < 1, y < 1, x > W - 2 or y > H - 2 are not written.
// One thread per pixel, 16 x 16 blocks; unlike the reference launch, pixels
// outside the image are never written.
#include "gvr_internal.cuh"
#include "gvr_profile.h"

namespace gvr {
namespace {

__device__ __forceinline__ V3 ld(const float *img, int W, int x, int y) {
    const float *p = img + 3 * ((size_t)y * W + x);
    return v3(p[0], p[1], p[2]);
}
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return v3(xs(a.x, b.x), xs(a.y, b.y), xs(a.z, b.z)); }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return v3(xa(a.x, b.x), xa(a.y, b.y), xa(a.z, b.z)); }
__device__ __forceinline__ V3 scl(float s, V3 a) { return v3(xm(s, a.x), xm(s, a.y), xm(s, a.z)); }
__device__ __forceinline__ void st(float *img, int W, int x, int y, V3 v) {
    float *p = img + 3 * ((size_t)y * W + x);
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}

__global__ void k_image_gradient(const float *__restrict__ in, float *__restrict__ gx, float *__restrict__ gy, int W,
                                 int H) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const size_t img = (size_t)blockIdx.z * W * H * 3;
    const float *I = in + img;
    if (x < 1 || y < 1 || x >= W - 2 || y >= H - 2) {
        st(gx + img, W, x, y, v3(0.0f, 0.0f, 0.0f));
        st(gy + img, W, x, y, v3(0.0f, 0.0f, 0.0f));
        return;
    }
    const V3 i00 = ld(I, W, x - 1, y - 1), i01 = ld(I, W, x, y - 1), i02 = ld(I, W, x + 1, y - 1);
    const V3 i10 = ld(I, W, x - 1, y), i12 = ld(I, W, x + 1, y);
    const V3 i20 = ld(I, W, x - 1, y + 1), i21 = ld(I, W, x, y + 1), i22 = ld(I, W, x + 1, y + 1);
    st(gx + img, W, x, y, scl(0.125f, add(add(sub(i02, i00), scl(2.0f, sub(i12, i10))), sub(i22, i20))));
    st(gy + img, W, x, y, scl(0.125f, add(add(sub(i20, i00), scl(2.0f, sub(i21, i01))), sub(i22, i02))));
}

__global__ void k_image_gaussian3x3(const float *__restrict__ in, float *__restrict__ out, int W, int H) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H || x < 1 || y < 1 || x > W - 2 || y > H - 2) return;
    const size_t img = (size_t)blockIdx.z * W * H * 3;
    const float *I = in + img;
    const V3 corners = add(add(add(ld(I, W, x - 1, y - 1), ld(I, W, x + 1, y - 1)), ld(I, W, x - 1, y + 1)),
                           ld(I, W, x + 1, y + 1));
    const V3 edges = add(add(add(ld(I, W, x, y - 1), ld(I, W, x - 1, y)), ld(I, W, x + 1, y)), ld(I, W, x, y + 1));
    st(out + img, W, x, y, add(add(scl(0.0625f, corners), scl(0.125f, edges)), scl(0.25f, ld(I, W, x, y))));
}

dim3 grid_of(int W, int H, int B) { return dim3((W + 15) / 16, (H + 15) / 16, B); }

}  // namespace
}  // namespace gvr

extern "C" {

int gvr_image_gradient(const float *image, float *grad_x, float *grad_y, int32_t batch, int32_t width,
                       int32_t height, void *stream) {
    if (!image || !grad_x || !grad_y || batch < 1 || batch > 65535 || width < 1 || height < 1)
        return GVR_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    GVR_LAUNCH(st, "k_image_gradient",
               (gvr::k_image_gradient<<<gvr::grid_of(width, height, batch), dim3(16, 16), 0, st>>>(image, grad_x, grad_y,
                                                                                                  width, height)));
    return cudaGetLastError() == cudaSuccess ? GVR_OK : GVR_ERR_CUDA;
}

int gvr_image_gaussian3x3(const float *image, float *out, int32_t batch, int32_t width, int32_t height, void *stream) {
    if (!image || !out || batch < 1 || batch > 65535 || width < 1 || height < 1) return GVR_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    GVR_LAUNCH(st, "k_image_gaussian3x3",
               (gvr::k_image_gaussian3x3<<<gvr::grid_of(width, height, batch), dim3(16, 16), 0, st>>>(image, out,
                                                                                                     width, height)));
    return cudaGetLastError() == cudaSuccess ? GVR_OK : GVR_ERR_CUDA;
}

}  // extern "C"

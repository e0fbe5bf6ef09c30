// gvr_normal_map.cu -- texture-space normal map (compute_normal_map).
//
// The reference rasterises the UV layout once on the host
// (CUDABasedRasterization.cpp:241-294: for every face, every texel of its
// UV box widened by 2 texels, the ray/triangle test of
// rayTriangleIntersectHost, :158-236, with the ray (x+.5, y+.5, 1) -> -z)
// and then interpolates the vertex normals per texel on the device
// (renderNormalMapDevice, CUDABasedRasterization.cu:415-445).  The frame
// buffers keep their cleared state (initializeDevice, :73-91): with the
// normal map on, the depth and shading passes do not run.
//
// Here both steps run on the GPU in every call: one thread per face marks
// the texels its UV triangle covers with atomicMax (the largest face id
// wins where UV triangles overlap, which is what the reference's serial
// face loop leaves), then one thread per (batch element, texel) recomputes
// the owner's barycentrics with the same FP32 operations and writes the
// normal.  Every operation is IEEE round-to-nearest without contraction, so
// the result equals the reference built with -fmad=false bit for bit.
#include "gvr_internal.cuh"
#include "gvr_kernels.h"
#include "gvr_profile.h"

namespace gvr {
namespace {

__host__ __device__ inline unsigned blocks_of(size_t n, int b) { return (unsigned)((n + b - 1) / b); }

// Texel-space corners of face f: (Wt * u, Ht * (1 - v), 0), the reference's texCoord0..2.
__device__ __forceinline__ void uv_corners(const float *uv6, int Wt, int Ht, V3 &t0, V3 &t1, V3 &t2) {
    const float w = (float)Wt, h = (float)Ht;
    t0 = v3(xm(w, uv6[0]), xm(h, xs(1.0f, uv6[1])), 0.0f);
    t1 = v3(xm(w, uv6[2]), xm(h, xs(1.0f, uv6[3])), 0.0f);
    t2 = v3(xm(w, uv6[4]), xm(h, xs(1.0f, uv6[5])), 0.0f);
}

// rayTriangleIntersectHost's per-face terms: corners scaled by 1/1000, the
// cross product N, dot(v0, N) and dot(N, N) -- the same values the
// reference computes inside its per-texel call.
__device__ __forceinline__ FaceSetup uv_face_setup(V3 t0, V3 t1, V3 t2) {
    FaceSetup s;
    s.v0 = v3(xd(t0.x, 1000.0f), xd(t0.y, 1000.0f), xd(t0.z, 1000.0f));
    s.v1 = v3(xd(t1.x, 1000.0f), xd(t1.y, 1000.0f), xd(t1.z, 1000.0f));
    s.v2 = v3(xd(t2.x, 1000.0f), xd(t2.y, 1000.0f), xd(t2.z, 1000.0f));
    s.n = xcross(xsub(s.v1, s.v0), xsub(s.v2, s.v0));
    s.v0dn = xdot(s.v0, s.n);
    s.denom = xdot(s.n, s.n);
    return s;
}

// The texel's hit test; abc = (a, b, 1 - a - b) or (-1, -1, -1).
__device__ __forceinline__ V3 uv_hit(const FaceSetup &s, int x, int y) {
    const V3 o = v3(xd((float)x + 0.5f, 1000.0f), xd((float)y + 0.5f, 1000.0f), xd(1.0f, 1000.0f));
    return barycentric(s, o, xdot(o, s.n), v3(0.0f, 0.0f, -1.0f));
}

__device__ __forceinline__ bool hit_ok(V3 abc) { return abc.x != -1.0f && abc.y != -1.0f && abc.z != -1.0f; }

__global__ void k_uv_owner(const Topology topo, int Ht, int Wt, int *__restrict__ owner) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= topo.F) return;
    V3 t0, t1, t2;
    uv_corners(topo.uvs + 6 * (size_t)f, Wt, Ht, t0, t1, t2);
    // the reference's box: int(fmax(min - 2, 0)) .. int(fmin(max + 2, size)), upper bound exclusive
    const int x0 = __float2int_rz(fmaxf(xs(fminf(t0.x, fminf(t1.x, t2.x)), 2.0f), 0.0f));
    const int x1 = __float2int_rz(fminf(xa(fmaxf(t0.x, fmaxf(t1.x, t2.x)), 2.0f), (float)Wt));
    const int y0 = __float2int_rz(fmaxf(xs(fminf(t0.y, fminf(t1.y, t2.y)), 2.0f), 0.0f));
    const int y1 = __float2int_rz(fminf(xa(fmaxf(t0.y, fmaxf(t1.y, t2.y)), 2.0f), (float)Ht));
    const FaceSetup s = uv_face_setup(t0, t1, t2);
    for (int y = y0; y < y1; ++y)
        for (int x = x0; x < x1; ++x)
            if (hit_ok(uv_hit(s, x, y))) atomicMax(owner + (size_t)y * Wt + x, f);
}

// One thread per (batch element, texel).  vnormal is [B, C, N, 3]; the
// reference reads the first view's block (all views hold the same normals).
__global__ void k_normal_map(const Topology topo, const int *__restrict__ owner, const float *__restrict__ vnormal,
                             int B, int C, int Ht, int Wt, float *__restrict__ out) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t texels = (size_t)Ht * Wt;
    if (i >= (size_t)B * texels) return;
    const int b = (int)(i / texels);
    const int texel = (int)(i - (size_t)b * texels);
    const int o = owner[texel];
    // an uncovered texel holds (face 0, 0, 0, 0) in the reference
    const int f = o >= 0 ? o : 0;
    V3 abc = v3(0.0f, 0.0f, 0.0f);
    if (o >= 0) {
        V3 t0, t1, t2;
        uv_corners(topo.uvs + 6 * (size_t)f, Wt, Ht, t0, t1, t2);
        abc = uv_hit(uv_face_setup(t0, t1, t2), texel % Wt, texel / Wt);
    }
    const float *VN = vnormal + (size_t)b * C * topo.N * 3;
    const int i0 = topo.faces[3 * f], i1 = topo.faces[3 * f + 1], i2 = topo.faces[3 * f + 2];
    V3 n = pixel_normal_un(ld3(VN + 3 * i0), ld3(VN + 3 * i1), ld3(VN + 3 * i2), abc);
    const float len = __fsqrt_rn(xdot(n, n));
    if (len != 0.0f) n = v3(xd(n.x, len), xd(n.y, len), xd(n.z, len));
    float *q = out + 3 * i;
    q[0] = xd(xa(n.x, 1.0f), 2.0f);
    q[1] = xd(xa(n.y, 1.0f), 2.0f);
    q[2] = xd(xa(n.z, 1.0f), 2.0f);
}

// The cleared frame of initializeDevice: face -1, barycentrics 0, green.
__global__ void k_background(int32_t *__restrict__ face, float2 *__restrict__ bary, float *__restrict__ render,
                             size_t pixels) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= pixels) return;
    face[p] = -1;
    bary[p] = make_float2(0.0f, 0.0f);
    render[3 * p + 0] = 0.0f;
    render[3 * p + 1] = 1.0f;
    render[3 * p + 2] = 0.0f;
}

}  // namespace

cudaError_t launch_normal_map(const Topology &topo, const FrameDims &dims, int *owner, const float *vnormal,
                              float *normal_map, int32_t *face, float *bary, float *render, cudaStream_t st) {
    const size_t texels = (size_t)dims.Ht * dims.Wt;
    const size_t pixels = (size_t)dims.B * dims.C * dims.W * dims.H;
    GVR_LAUNCH(st, "k_background",
               k_background<<<blocks_of(pixels, 256), 256, 0, st>>>(face, reinterpret_cast<float2 *>(bary), render,
                                                                     pixels));
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    if ((err = cudaMemsetAsync(owner, 0xff, texels * sizeof(int), st)) != cudaSuccess) return err;
    GVR_LAUNCH(st, "k_uv_owner", k_uv_owner<<<blocks_of(topo.F, 128), 128, 0, st>>>(topo, dims.Ht, dims.Wt, owner));
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    GVR_LAUNCH(st, "k_normal_map",
               k_normal_map<<<blocks_of((size_t)dims.B * texels, 256), 256, 0, st>>>(topo, owner, vnormal, dims.B,
                                                                                     dims.C, dims.Ht, dims.Wt,
                                                                                     normal_map));
    return cudaGetLastError();
}

}  // namespace gvr

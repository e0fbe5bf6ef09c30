// refcore.cu -- runs the reference's own CUDA kernels (compiled from its
// sources into oracle/_ref/*.fatbin) on the GPU.  Test infrastructure only:
// it is the checker that pins the oracle and the new kernels to the
// reference implementation itself; the product never loads it.
//
// The harness replicates what the reference host code does around its
// kernels: the renderer constructors' allocations and vertex->face lists
// (cpp/src/Renderer/CUDABasedRasterization.cpp:11-154,
// CUDABasedRasterizationGrad.cpp:7-120), the launch sequences of
// renderBuffersGPU (CUDABasedRasterization.cu:449-473) and
// renderBuffersGradGPU (CUDABasedRasterizationGrad.cu:624-635), one batch
// element per call as CudaRenderer::Compute does.  The kernels take the
// parameter structs CUDABasedRasterizationInput / ...GradInput by value;
// RefFwdInput / RefBwdInput below restate their field order and types, and
// refcore_layout() exposes the offsets so the build can compare them with
// the offsets compiled from the reference header.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct RefFwdInput {
    int numberOfCameras, w, h, F, N;
    int3 *d_facesVertex;
    int *d_vertexFaces;
    int2 *d_vertexFacesId;
    float *d_textureCoordinates;
    float4 *d_textureMapIds;
    bool computeNormal;
    int4 *d_BBoxes;
    float3 *d_projectedVertices;
    float3 *d_faceNormal;
    int albedoMode, shadingMode;
    float4 *d_inverseExtrinsics, *d_inverseProjection;
    float3 *d_vertices, *d_vertexColor;
    int texWidth, texHeight;
    const float *d_textureMap, *d_shCoeff;
    float4 *d_cameraExtrinsics;
    float3 *d_cameraIntrinsics;
    int *d_faceIDBuffer, *d_depthBuffer;
    float *d_barycentricCoordinatesBuffer, *d_renderBuffer;
    float3 *d_vertexNormal, *d_normalMap;
};

struct RefBwdInput {
    int numberOfCameras, w, h, F, N;
    int3 *d_facesVertex;
    float *d_textureCoordinates;
    int *d_vertexFaces;
    int2 *d_vertexFacesId;
    int albedoMode, shadingMode;
    float4 *d_inverseExtrinsics, *d_inverseProjection;
    int imageFilterSize, textureFilterSize;
    float3 *d_renderBufferGrad, *d_targetBufferGrad;
    float3 *d_vertices, *d_vertexColor;
    const float *d_textureMap, *d_shCoeff;
    float3 *d_vertexNormal;
    float2 *d_barycentricCoordinatesBuffer;
    int *d_faceIDBuffer;
    const float *d_targetImage;
    int texWidth, texHeight;
    float4 *d_cameraExtrinsics;
    float3 *d_cameraIntrinsics;
    float3 *d_vertexPosGrad, *d_vertexColorGrad, *d_textureGrad;
    float *d_shCoeffGrad;
};

thread_local std::string g_err;

int fail(const std::string &m) {
    g_err = m;
    return -1;
}

#ifndef REFCORE_LAYOUT_ONLY
bool cu_ok(CUresult r, const char *what) {
    if (r == CUDA_SUCCESS) return true;
    const char *s = nullptr;
    cuGetErrorString(r, &s);
    g_err = std::string(what) + ": " + (s ? s : "?");
    return false;
}
#endif

bool rt_ok(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

// Itanium-mangled name of `void name(T)` for a struct T passed by value.
std::string mangled(const char *name, const char *type) {
    return "_Z" + std::to_string(std::strlen(name)) + name + std::to_string(std::strlen(type)) + type;
}

// getVertexFaces (CUDABasedRasterization.cpp:125-154): for each vertex the
// faces containing it in ascending order; (start, count) only for vertices
// that have faces, as the reference does.
void vertex_faces(int N, const int32_t *faces, int F, std::vector<int> &vf, std::vector<int> &vfid) {
    std::vector<std::vector<int>> per(N);
    for (int f = 0; f < F; ++f) {
        const int a = faces[3 * f], b = faces[3 * f + 1], c = faces[3 * f + 2];
        per[a].push_back(f);
        if (b != a) per[b].push_back(f);
        if (c != a && c != b) per[c].push_back(f);
    }
    for (int v = 0; v < N; ++v) {
        if (per[v].empty()) continue;
        vfid.push_back((int)vf.size());
        vfid.push_back((int)per[v].size());
        vf.insert(vf.end(), per[v].begin(), per[v].end());
    }
}

struct DeviceBuf {
    std::vector<void *> ptrs;
    ~DeviceBuf() {
        for (void *p : ptrs) cudaFree(p);
    }
    template <typename T>
    T *alloc(size_t bytes) {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
        cudaMemset(p, 0, bytes ? bytes : 16);
        ptrs.push_back(p);
        return static_cast<T *>(p);
    }
    template <typename T>
    T *upload(const void *src, size_t bytes) {
        T *d = alloc<T>(bytes);
        if (d && bytes) cudaMemcpy(d, src, bytes, cudaMemcpyHostToDevice);
        return d;
    }
};

}  // namespace

#ifndef REFCORE_LAYOUT_ONLY  // the layout-only build needs no CUDA driver
struct RefcoreHandle {
    CUmodule fwd = nullptr, bwd = nullptr;
};

extern "C" {

const char *refcore_error(void) { return g_err.c_str(); }

int refcore_open(const char *fwd_fatbin, const char *bwd_fatbin, RefcoreHandle **out) {
    *out = nullptr;
    if (!rt_ok(cudaFree(nullptr), "cuda init")) return -1;  // makes the primary context current
    RefcoreHandle *h = new RefcoreHandle();
    if (!cu_ok(cuModuleLoad(&h->fwd, fwd_fatbin), "load forward fatbin") ||
        !cu_ok(cuModuleLoad(&h->bwd, bwd_fatbin), "load backward fatbin")) {
        if (h->fwd) cuModuleUnload(h->fwd);
        delete h;
        return -1;
    }
    *out = h;
    return 0;
}

void refcore_close(RefcoreHandle *h) {
    if (!h) return;
    if (h->fwd) cuModuleUnload(h->fwd);
    if (h->bwd) cuModuleUnload(h->bwd);
    delete h;
}

static int launch(CUmodule mod, const char *name, const char *type, unsigned grid, unsigned block, void *param) {
    CUfunction fn;
    const std::string m = mangled(name, type);
    if (!cu_ok(cuModuleGetFunction(&fn, mod, m.c_str()), m.c_str())) return -1;
    void *args[] = {param};
    if (!cu_ok(cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, 0, nullptr, args, nullptr), name)) return -1;
    return 0;
}

static unsigned blocks(long long n) { return (unsigned)((n + 255) / 256); }

// One batch element of CudaRendererGpu (device pointers; faces/uvs on the host).
int refcore_forward(RefcoreHandle *h, const int32_t *faces, const float *uvs, int N, int F, int C, int W, int H,
                    int albedo, int shading, int Ht, int Wt, const float *verts, const float *colors,
                    const float *texture, const float *sh, const float *extr, const float *intr, int32_t *face,
                    float *bary, float *render, float *vnormal, float *ms_out) {
    if (!h) return fail("null handle");
    DeviceBuf buf;
    std::vector<int> vf, vfid;
    vertex_faces(N, faces, F, vf, vfid);
    RefFwdInput in;
    std::memset(&in, 0, sizeof(in));
    in.numberOfCameras = C;
    in.w = W;
    in.h = H;
    in.F = F;
    in.N = N;
    in.d_facesVertex = buf.upload<int3>(faces, sizeof(int) * 3 * (size_t)F);
    in.d_vertexFaces = buf.upload<int>(vf.data(), sizeof(int) * vf.size());
    in.d_vertexFacesId = buf.upload<int2>(vfid.data(), sizeof(int) * vfid.size());
    in.d_textureCoordinates = buf.upload<float>(uvs, sizeof(float) * 6 * (size_t)F);
    in.computeNormal = false;
    in.d_BBoxes = buf.alloc<int4>(sizeof(int4) * (size_t)F * C);
    in.d_projectedVertices = buf.alloc<float3>(sizeof(float3) * (size_t)N * C);
    in.d_faceNormal = buf.alloc<float3>(sizeof(float3) * (size_t)F * C);
    in.albedoMode = albedo;
    in.shadingMode = shading;
    in.d_inverseExtrinsics = buf.alloc<float4>(sizeof(float4) * 4 * (size_t)C);
    in.d_inverseProjection = buf.alloc<float4>(sizeof(float4) * 4 * (size_t)C);
    in.d_vertices = (float3 *)verts;
    in.d_vertexColor = (float3 *)colors;
    in.texWidth = Wt;
    in.texHeight = Ht;
    in.d_textureMap = texture;
    in.d_shCoeff = sh;
    in.d_cameraExtrinsics = (float4 *)extr;
    in.d_cameraIntrinsics = (float3 *)intr;
    in.d_faceIDBuffer = face;
    in.d_depthBuffer = buf.alloc<int>(sizeof(int) * (size_t)C * H * W);
    in.d_barycentricCoordinatesBuffer = bary;
    in.d_renderBuffer = render;
    in.d_vertexNormal = (float3 *)vnormal;
    in.d_normalMap = nullptr;
    if (!in.d_facesVertex || !in.d_depthBuffer) return fail("allocation failed");
    if (!rt_ok(cudaDeviceSynchronize(), "setup")) return -1;
    const char *T = "CUDABasedRasterizationInput";
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, nullptr);
    const long long CF = (long long)C * F, CN = (long long)C * N, CP = (long long)C * W * H;
    int rc = launch(h->fwd, "initializeCamerasDevice", T, 1, 1, &in);
    if (!rc) rc = launch(h->fwd, "initializeDevice", T, blocks(CP), 256, &in);
    if (!rc) rc = launch(h->fwd, "projectVerticesDevice", T, blocks(CN), 256, &in);
    if (!rc) rc = launch(h->fwd, "projectFacesDevice", T, blocks(CF), 256, &in);
    if (!rc) rc = launch(h->fwd, "renderFaceNormalDevice", T, blocks(CF), 256, &in);
    if (!rc) rc = launch(h->fwd, "renderVertexNormalDevice", T, blocks(CN), 256, &in);
    if (!rc) rc = launch(h->fwd, "renderDepthBufferDevice", T, blocks(CF), 256, &in);
    if (!rc) rc = launch(h->fwd, "renderBuffersDevice", T, blocks(CF), 256, &in);
    cudaEventRecord(e1, nullptr);
    if (!rc && !rt_ok(cudaDeviceSynchronize(), "forward kernels")) rc = -1;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms_out) *ms_out = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

// One batch element of CudaRendererGradGpu.
int refcore_backward(RefcoreHandle *h, const int32_t *faces, const float *uvs, int N, int F, int C, int W, int H,
                     int albedo, int shading, int imageFilter, int textureFilter, int Ht, int Wt,
                     const float *grad_render, const float *grad_target, const float *verts, const float *colors,
                     const float *texture, const float *sh, const float *vnormal, const float *bary,
                     const int32_t *face, const float *target, const float *extr, const float *intr, float *gpos,
                     float *gcol, float *gtex, float *gsh, float *ms_out) {
    if (!h) return fail("null handle");
    DeviceBuf buf;
    std::vector<int> vf, vfid;
    vertex_faces(N, faces, F, vf, vfid);
    RefBwdInput in;
    std::memset(&in, 0, sizeof(in));
    in.numberOfCameras = C;
    in.w = W;
    in.h = H;
    in.F = F;
    in.N = N;
    in.d_facesVertex = buf.upload<int3>(faces, sizeof(int) * 3 * (size_t)F);
    in.d_textureCoordinates = buf.upload<float>(uvs, sizeof(float) * 6 * (size_t)F);
    in.d_vertexFaces = buf.upload<int>(vf.data(), sizeof(int) * vf.size());
    in.d_vertexFacesId = buf.upload<int2>(vfid.data(), sizeof(int) * vfid.size());
    in.albedoMode = albedo;
    in.shadingMode = shading;
    in.d_inverseExtrinsics = buf.alloc<float4>(sizeof(float4) * 4 * (size_t)C);
    in.d_inverseProjection = buf.alloc<float4>(sizeof(float4) * 4 * (size_t)C);
    in.imageFilterSize = imageFilter;
    in.textureFilterSize = textureFilter;
    in.d_renderBufferGrad = (float3 *)grad_render;
    in.d_targetBufferGrad = (float3 *)grad_target;
    in.d_vertices = (float3 *)verts;
    in.d_vertexColor = (float3 *)colors;
    in.d_textureMap = texture;
    in.d_shCoeff = sh;
    in.d_vertexNormal = (float3 *)vnormal;
    in.d_barycentricCoordinatesBuffer = (float2 *)bary;
    in.d_faceIDBuffer = (int *)face;
    in.d_targetImage = target;
    in.texWidth = Wt;
    in.texHeight = Ht;
    in.d_cameraExtrinsics = (float4 *)extr;
    in.d_cameraIntrinsics = (float3 *)intr;
    in.d_vertexPosGrad = (float3 *)gpos;
    in.d_vertexColorGrad = (float3 *)gcol;
    in.d_textureGrad = (float3 *)gtex;
    in.d_shCoeffGrad = gsh;
    if (!in.d_facesVertex) return fail("allocation failed");
    if (!rt_ok(cudaDeviceSynchronize(), "setup")) return -1;
    const char *T = "CUDABasedRasterizationGradInput";
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, nullptr);
    int rc = launch(h->bwd, "initializeCamerasGradDevice", T, 1, 1, &in);
    if (!rc) rc = launch(h->bwd, "initBuffersGradDevice2", T, blocks((long long)C * 27), 256, &in);
    if (!rc) rc = launch(h->bwd, "initBuffersGradDevice1", T, blocks((long long)Ht * Wt), 256, &in);
    if (!rc) rc = launch(h->bwd, "initBuffersGradDevice0", T, blocks(N), 256, &in);
    if (!rc) rc = launch(h->bwd, "renderBuffersGradDevice", T, blocks((long long)C * W * H), 256, &in);
    cudaEventRecord(e1, nullptr);
    if (!rc && !rt_ok(cudaDeviceSynchronize(), "backward kernels")) rc = -1;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms_out) *ms_out = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

// renderNormalMapDevice (CUDABasedRasterization.cu:415-445) on a texture
// face map given as the reference's float4 (face, a, b, c) per texel (host)
// and one view's vertex normals (device [N,3]); out is device [Ht,Wt,3].
int refcore_normal_map(RefcoreHandle *h, const int32_t *faces, int F, int N, int Ht, int Wt,
                       const float *texture_map_ids, const float *vnormal, float *out) {
    if (!h) return fail("null handle");
    DeviceBuf buf;
    RefFwdInput in;
    std::memset(&in, 0, sizeof(in));
    in.numberOfCameras = 1;
    in.F = F;
    in.N = N;
    in.d_facesVertex = buf.upload<int3>(faces, sizeof(int) * 3 * (size_t)F);
    in.d_textureMapIds = buf.upload<float4>(texture_map_ids, sizeof(float4) * (size_t)Ht * Wt);
    in.computeNormal = true;
    in.texWidth = Wt;
    in.texHeight = Ht;
    in.d_vertexNormal = (float3 *)vnormal;
    in.d_normalMap = (float3 *)out;
    if (!in.d_facesVertex || !in.d_textureMapIds) return fail("allocation failed");
    if (!rt_ok(cudaDeviceSynchronize(), "setup")) return -1;
    int rc = launch(h->fwd, "renderNormalMapDevice", "CUDABasedRasterizationInput", blocks((long long)Ht * Wt), 256,
                    &in);
    if (!rc && !rt_ok(cudaDeviceSynchronize(), "normal map kernel")) rc = -1;
    return rc;
}

}  // extern "C"
#endif

extern "C" {

// Offsets of the replicated parameter structs (which: 0 forward, 1 backward).
int refcore_layout(int which, const char **names, long long *offsets, int cap) {
#define R(S, m)                                   \
    do {                                          \
        if (n < cap) {                            \
            names[n] = #m;                        \
            offsets[n] = (long long)offsetof(S, m); \
        }                                         \
        ++n;                                      \
    } while (0)
    int n = 0;
    if (which == 0) {
        using S = RefFwdInput;
        R(S, numberOfCameras); R(S, w); R(S, h); R(S, F); R(S, N); R(S, d_facesVertex); R(S, d_vertexFaces);
        R(S, d_vertexFacesId); R(S, d_textureCoordinates); R(S, d_textureMapIds); R(S, computeNormal); R(S, d_BBoxes);
        R(S, d_projectedVertices); R(S, d_faceNormal); R(S, albedoMode); R(S, shadingMode); R(S, d_inverseExtrinsics);
        R(S, d_inverseProjection); R(S, d_vertices); R(S, d_vertexColor); R(S, texWidth); R(S, texHeight);
        R(S, d_textureMap); R(S, d_shCoeff); R(S, d_cameraExtrinsics); R(S, d_cameraIntrinsics); R(S, d_faceIDBuffer);
        R(S, d_depthBuffer); R(S, d_barycentricCoordinatesBuffer); R(S, d_renderBuffer); R(S, d_vertexNormal);
        R(S, d_normalMap);
        if (n < cap) { names[n] = "sizeof"; offsets[n] = (long long)sizeof(S); }
        ++n;
    } else {
        using S = RefBwdInput;
        R(S, numberOfCameras); R(S, w); R(S, h); R(S, F); R(S, N); R(S, d_facesVertex); R(S, d_textureCoordinates);
        R(S, d_vertexFaces); R(S, d_vertexFacesId); R(S, albedoMode); R(S, shadingMode); R(S, d_inverseExtrinsics);
        R(S, d_inverseProjection); R(S, imageFilterSize); R(S, textureFilterSize); R(S, d_renderBufferGrad);
        R(S, d_targetBufferGrad); R(S, d_vertices); R(S, d_vertexColor); R(S, d_textureMap); R(S, d_shCoeff);
        R(S, d_vertexNormal); R(S, d_barycentricCoordinatesBuffer); R(S, d_faceIDBuffer); R(S, d_targetImage);
        R(S, texWidth); R(S, texHeight); R(S, d_cameraExtrinsics); R(S, d_cameraIntrinsics); R(S, d_vertexPosGrad);
        R(S, d_vertexColorGrad); R(S, d_textureGrad); R(S, d_shCoeffGrad);
        if (n < cap) { names[n] = "sizeof"; offsets[n] = (long long)sizeof(S); }
        ++n;
    }
#undef R
    return n;
}

}  // extern "C"

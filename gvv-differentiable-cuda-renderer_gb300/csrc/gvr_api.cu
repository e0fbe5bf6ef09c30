// gvr_api.cu -- the C ABI (include/gvr.h): validation, topology upload,
// workspace layout and dispatch.  Errors are returned, never fatal.
#include <climits>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gvr_kernels.h"

struct GvrHandle {
    int device;
    GvrAttrs attrs;   // shading forced to shadeless for foregroundMask
    int N, F, nnz;
    int tilesX, tilesY;
    int32_t *d_faces;
    float *d_uvs;
    int32_t *d_vstart;
    int32_t *d_vfaces;

    gvr::Topology topo() const { return gvr::Topology{d_faces, d_uvs, d_vstart, d_vfaces, N, F}; }
};

namespace {

thread_local std::string g_error;

int fail(int code, const std::string &msg) {
    g_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    return fail(e == cudaErrorMemoryAllocation ? GVR_ERR_OUT_OF_MEMORY : GVR_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

// Restores the caller's current device on scope exit.
struct DeviceGuard {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceGuard(int dev) {
        err = cudaGetDevice(&prev);
        if (err == cudaSuccess && prev != dev) err = cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

// Carves aligned sub-buffers out of one workspace; with base == nullptr it only measures.
struct Carver {
    char *base;
    size_t off = 0;
    explicit Carver(void *b) : base(static_cast<char *>(b)) {}
    template <typename T>
    T *take(size_t count) {
        off = (off + 255) & ~size_t(255);
        T *p = base ? reinterpret_cast<T *>(base + off) : nullptr;
        off += count * sizeof(T);
        return p;
    }
};

struct FwdLayout {
    gvr::FwdScratch s;
    float4 *proj;
    size_t bytes;
};

FwdLayout fwd_layout(const GvrHandle *h, int B, void *base) {
    const size_t BC = (size_t)B * h->attrs.num_cameras, T = (size_t)h->tilesX * h->tilesY;
    Carver c(base);
    FwdLayout L{};
    L.s.cams = c.take<gvr::Camera>(BC);
    L.s.geo = c.take<gvr::FaceGeo>((size_t)B * h->F);
    L.s.fnormal = c.take<float4>((size_t)B * h->F);
    L.proj = c.take<float4>(BC * h->N);
    L.s.vface = c.take<gvr::ViewFace>(BC * h->F);
    L.s.tileStart = c.take<int>(BC * T + 1);
    L.s.bins = c.take<int>((size_t)gvr::kBigTiles * BC * h->F);
    L.s.bigList = c.take<int>(BC * h->F);
    // per-call zeroed counters, contiguous
    L.s.tileCount = c.take<int>(BC * T);
    size_t z0 = c.off - BC * T * sizeof(int);
    L.s.tileCursor = c.take<int>(BC * T);
    L.s.bigCount = c.take<int>(BC);
    L.s.zeroBase = base ? c.base + z0 : nullptr;
    L.s.zeroBytes = c.off - z0;
    L.bytes = c.off + 256;
    return L;
}

struct BwdLayout {
    gvr::BwdScratch s;
    size_t bytes;
};

BwdLayout bwd_layout(const GvrHandle *h, int B, void *base) {
    const size_t BC = (size_t)B * h->attrs.num_cameras, T = (size_t)h->tilesX * h->tilesY;
    Carver c(base);
    BwdLayout L{};
    L.s.cams = c.take<gvr::Camera>(BC);
    L.s.geo = c.take<gvr::FaceGeo>((size_t)B * h->F);
    L.s.faceAcc = c.take<float4>((size_t)B * h->F * (gvr::kFaceAccFloats / 4));
    L.s.gN = c.take<float4>((size_t)B * h->N);
    L.s.shPartial = c.take<float>(BC * T * 27);
    L.bytes = c.off + 256;
    return L;
}

// Scratch for one call: the caller's workspace or stream-ordered memory.
struct CallScratch {
    void *ptr = nullptr;
    bool owned = false;
    cudaStream_t st = nullptr;
    int acquire(void *ws, size_t wsBytes, size_t need, cudaStream_t stream) {
        st = stream;
        if (ws) {
            if (wsBytes < need)
                return fail(GVR_ERR_WORKSPACE, "workspace of " + std::to_string(wsBytes) + " bytes < required " +
                                                   std::to_string(need));
            if (reinterpret_cast<uintptr_t>(ws) % 256)
                return fail(GVR_ERR_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
            ptr = ws;
            return GVR_OK;
        }
        cudaError_t e = cudaMallocAsync(&ptr, need, stream);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync(workspace)");
        owned = true;
        return GVR_OK;
    }
    ~CallScratch() {
        if (owned && ptr) cudaFreeAsync(ptr, st);
    }
};

bool batch_fits(const GvrHandle *h, int B) {
    const long long BC = (long long)B * h->attrs.num_cameras;
    const long long T = (long long)h->tilesX * h->tilesY;
    return B >= 1 && BC * h->F * gvr::kBigTiles < INT_MAX && BC * T * 27 < INT_MAX && (long long)B * h->N < INT_MAX &&
           BC * T < INT_MAX;
}

}  // namespace

extern "C" {

const char *gvr_last_error(void) { return g_error.c_str(); }

int gvr_abi_version(void) { return GVR_ABI_VERSION; }

int gvr_create(const GvrTopology *topo, const GvrAttrs *attrs, GvrHandle **out) {
    if (!out) return fail(GVR_ERR_INVALID_ARGUMENT, "out_handle is NULL");
    *out = nullptr;
    if (!topo || !attrs) return fail(GVR_ERR_INVALID_ARGUMENT, "topology/attrs is NULL");
    const int N = topo->num_vertices, F = topo->num_faces;
    // CudaRenderer.cpp:37-80 attr checks
    if (N <= 0) return fail(GVR_ERR_INVALID_ARGUMENT, "number_of_vertices not set!");
    if (F <= 0 || !topo->faces) return fail(GVR_ERR_INVALID_ARGUMENT, "No triangular faces!");
    if (attrs->num_cameras <= 0) return fail(GVR_ERR_INVALID_ARGUMENT, "number_of_cameras not set!");
    if (attrs->render_resolution_u <= 0) return fail(GVR_ERR_INVALID_ARGUMENT, "render_resolution_u not set!");
    if (attrs->render_resolution_v <= 0) return fail(GVR_ERR_INVALID_ARGUMENT, "render_resolution_v not set!");
    if (attrs->render_resolution_u > 32768 || attrs->render_resolution_v > 32768)
        return fail(GVR_ERR_INVALID_ARGUMENT, "render resolution above 32768");
    if (attrs->albedo_mode < GVR_ALBEDO_VERTEX_COLOR || attrs->albedo_mode > GVR_ALBEDO_FOREGROUND_MASK)
        return fail(GVR_ERR_INVALID_ARGUMENT, "INVALID ALBEDO MODE");
    if (attrs->shading_mode != GVR_SHADING_SHADED && attrs->shading_mode != GVR_SHADING_SHADELESS)
        return fail(GVR_ERR_INVALID_ARGUMENT, "INVALID SHADING MODE");
    // CudaRendererGrad.cpp:84-98
    if (attrs->image_filter_size <= 0) return fail(GVR_ERR_INVALID_ARGUMENT, "INVALID IMAGE FILTER SIZE");
    if (attrs->texture_filter_size <= 0) return fail(GVR_ERR_INVALID_ARGUMENT, "INVALID TEXTURE FILTER SIZE");
    if (attrs->compute_normal_map) return fail(GVR_ERR_UNSUPPORTED, "compute_normal_map is not supported by this build");
    for (int i = 0; i < 3 * F; ++i)
        if (topo->faces[i] < 0 || topo->faces[i] >= N)
            return fail(GVR_ERR_INVALID_ARGUMENT, "face " + std::to_string(i / 3) + " references vertex " +
                                                      std::to_string(topo->faces[i]) + " outside [0, N)");

    // vertex -> face adjacency, ascending face id, each face once per distinct vertex
    std::vector<int32_t> start(N + 1, 0), fill(N, 0);
    for (int f = 0; f < F; ++f) {
        const int a = topo->faces[3 * f], b = topo->faces[3 * f + 1], c = topo->faces[3 * f + 2];
        start[a + 1]++;
        if (b != a) start[b + 1]++;
        if (c != a && c != b) start[c + 1]++;
    }
    for (int v = 0; v < N; ++v) start[v + 1] += start[v];
    const int nnz = start[N];
    std::vector<int32_t> adj(nnz > 0 ? nnz : 1);
    for (int f = 0; f < F; ++f) {
        const int a = topo->faces[3 * f], b = topo->faces[3 * f + 1], c = topo->faces[3 * f + 2];
        adj[start[a] + fill[a]++] = f;
        if (b != a) adj[start[b] + fill[b]++] = f;
        if (c != a && c != b) adj[start[c] + fill[c]++] = f;
    }

    GvrHandle *h = new GvrHandle();
    std::memset(h, 0, sizeof(*h));
    cudaError_t e = cudaGetDevice(&h->device);
    if (e != cudaSuccess) {
        delete h;
        return cuda_fail(e, "cudaGetDevice");
    }
    h->attrs = *attrs;
    if (h->attrs.albedo_mode == GVR_ALBEDO_FOREGROUND_MASK) h->attrs.shading_mode = GVR_SHADING_SHADELESS;
    h->N = N;
    h->F = F;
    h->nnz = nnz;
    h->tilesX = (attrs->render_resolution_u + gvr::kTile - 1) / gvr::kTile;
    h->tilesY = (attrs->render_resolution_v + gvr::kTile - 1) / gvr::kTile;
    std::vector<float> uvs((size_t)F * 6, 0.0f);
    if (topo->texture_coordinates) std::memcpy(uvs.data(), topo->texture_coordinates, uvs.size() * sizeof(float));
    struct Up { void **dst; const void *src; size_t bytes; } ups[] = {
        {(void **)&h->d_faces, topo->faces, (size_t)F * 3 * sizeof(int32_t)},
        {(void **)&h->d_uvs, uvs.data(), uvs.size() * sizeof(float)},
        {(void **)&h->d_vstart, start.data(), start.size() * sizeof(int32_t)},
        {(void **)&h->d_vfaces, adj.data(), adj.size() * sizeof(int32_t)},
    };
    for (auto &u : ups) {
        if ((e = cudaMalloc(u.dst, u.bytes)) != cudaSuccess || (e = cudaMemcpy(*u.dst, u.src, u.bytes, cudaMemcpyHostToDevice)) != cudaSuccess) {
            gvr_destroy(h);
            return cuda_fail(e, "gvr_create upload");
        }
    }
    *out = h;
    return GVR_OK;
}

void gvr_destroy(GvrHandle *h) {
    if (!h) return;
    DeviceGuard g(h->device);
    cudaFree(h->d_faces);
    cudaFree(h->d_uvs);
    cudaFree(h->d_vstart);
    cudaFree(h->d_vfaces);
    delete h;
}

size_t gvr_forward_workspace_size(const GvrHandle *h, int32_t batch, int32_t, int32_t) {
    if (!h || batch < 1) return 0;
    return fwd_layout(h, batch, nullptr).bytes;
}

size_t gvr_backward_workspace_size(const GvrHandle *h, int32_t batch, int32_t, int32_t) {
    if (!h || batch < 1) return 0;
    return bwd_layout(h, batch, nullptr).bytes;
}

static gvr::FrameDims dims_of(const GvrHandle *h, int B, int Ht, int Wt) {
    gvr::FrameDims d;
    d.B = B;
    d.C = h->attrs.num_cameras;
    d.W = h->attrs.render_resolution_u;
    d.H = h->attrs.render_resolution_v;
    d.tilesX = h->tilesX;
    d.tilesY = h->tilesY;
    d.Ht = Ht;
    d.Wt = Wt;
    d.albedo = h->attrs.albedo_mode;
    d.shading = h->attrs.shading_mode;
    return d;
}

int gvr_forward(GvrHandle *h, const GvrForwardArgs *a, void *stream) {
    if (!h || !a) return fail(GVR_ERR_INVALID_ARGUMENT, "handle/args is NULL");
    const int B = a->batch;
    if (!batch_fits(h, B)) return fail(GVR_ERR_INVALID_ARGUMENT, "batch must be >= 1 and the call within int32 index range");
    const int mode = h->attrs.albedo_mode;
    const bool textured = mode == GVR_ALBEDO_TEXTURED;
    if (textured && (a->texture_height < 1 || a->texture_width < 1 || !a->texture))
        return fail(GVR_ERR_INVALID_ARGUMENT, "textured mode needs a texture of at least 1x1");
    if (!a->vertex_pos || !a->extrinsics || !a->intrinsics || !a->sh_coeff)
        return fail(GVR_ERR_INVALID_ARGUMENT, "vertex_pos, sh_coeff, extrinsics and intrinsics are required");
    if (mode == GVR_ALBEDO_VERTEX_COLOR && !a->vertex_color)
        return fail(GVR_ERR_INVALID_ARGUMENT, "vertexColor mode needs vertex_color");
    if (!a->barycentric || !a->face || !a->render || !a->vertex_normal)
        return fail(GVR_ERR_INVALID_ARGUMENT, "barycentric, face, render and vertex_normal outputs are required");
    if (a->target_image_out && !a->target_image)
        return fail(GVR_ERR_INVALID_ARGUMENT, "target_image_out needs target_image");
    DeviceGuard g(h->device);
    if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const FwdLayout need = fwd_layout(h, B, nullptr);
    CallScratch scratch;
    int rc = scratch.acquire(a->workspace, a->workspace_bytes, need.bytes, st);
    if (rc != GVR_OK) return rc;
    FwdLayout L = fwd_layout(h, B, scratch.ptr);
    gvr::FrameDims dims = dims_of(h, B, textured ? a->texture_height : 1, textured ? a->texture_width : 1);
    cudaError_t e = gvr::launch_forward(h->topo(), dims, L.s, a->vertex_pos, a->vertex_color, a->texture, a->sh_coeff,
                                        a->extrinsics, a->intrinsics, a->barycentric, a->face, a->render,
                                        a->vertex_normal, L.proj, st);
    if (e != cudaSuccess) return cuda_fail(e, "forward launch");
    const size_t img = (size_t)B * h->attrs.num_cameras * h->attrs.render_resolution_v * h->attrs.render_resolution_u * 3;
    if (a->target_image_out && a->target_image_out != a->target_image) {
        e = cudaMemcpyAsync(a->target_image_out, a->target_image, img * sizeof(float), cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return cuda_fail(e, "target_image_out copy");
    }
    if (a->normal_map && a->texture_height > 0 && a->texture_width > 0) {
        e = cudaMemsetAsync(a->normal_map, 0, (size_t)B * a->texture_height * a->texture_width * 3 * sizeof(float), st);
        if (e != cudaSuccess) return cuda_fail(e, "normal_map clear");
    }
    return GVR_OK;
}

int gvr_backward(GvrHandle *h, const GvrBackwardArgs *a, void *stream) {
    if (!h || !a) return fail(GVR_ERR_INVALID_ARGUMENT, "handle/args is NULL");
    const int B = a->batch;
    if (!batch_fits(h, B)) return fail(GVR_ERR_INVALID_ARGUMENT, "batch must be >= 1 and the call within int32 index range");
    const int mode = h->attrs.albedo_mode;
    const bool textured = mode == GVR_ALBEDO_TEXTURED;
    if (a->texture_height < 1 || a->texture_width < 1)
        return fail(GVR_ERR_INVALID_ARGUMENT, "texture_height/texture_width must be >= 1 (texture_grad shape)");
    if (!a->vertex_pos_grad || !a->vertex_color_grad || !a->texture_grad || !a->sh_coeff_grad)
        return fail(GVR_ERR_INVALID_ARGUMENT, "all four gradient outputs are required");
    const bool zeroMode = mode == GVR_ALBEDO_NORMAL || mode == GVR_ALBEDO_LIGHTING;
    if (!zeroMode) {
        if (!a->render_grad || !a->vertex_pos || !a->sh_coeff || !a->vertex_normal || !a->face || !a->extrinsics ||
            !a->intrinsics)
            return fail(GVR_ERR_INVALID_ARGUMENT, "render_grad, vertex_pos, sh_coeff, vertex_normal, face, extrinsics, intrinsics are required");
        if (mode == GVR_ALBEDO_VERTEX_COLOR && !a->vertex_color)
            return fail(GVR_ERR_INVALID_ARGUMENT, "vertexColor mode needs vertex_color");
        if (textured && !a->texture) return fail(GVR_ERR_INVALID_ARGUMENT, "textured mode needs texture");
        if (a->target_grad && !a->target_image)
            return fail(GVR_ERR_INVALID_ARGUMENT, "target_grad needs target_image");
    }
    DeviceGuard g(h->device);
    if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CallScratch scratch;
    if (!zeroMode) {
        int rc = scratch.acquire(a->workspace, a->workspace_bytes, bwd_layout(h, B, nullptr).bytes, st);
        if (rc != GVR_OK) return rc;
    }
    BwdLayout L = bwd_layout(h, B, scratch.ptr);
    gvr::FrameDims dims = dims_of(h, B, a->texture_height, a->texture_width);
    cudaError_t e = gvr::launch_backward(h->topo(), dims, L.s, *a, h->attrs.image_filter_size, st);
    if (e != cudaSuccess) return cuda_fail(e, "backward launch");
    return GVR_OK;
}

int gvr_debug_rays(GvrHandle *h, int32_t batch, const float *extr, const float *intr, float *rays, void *stream) {
    if (!h || !extr || !intr || !rays || batch < 1) return fail(GVR_ERR_INVALID_ARGUMENT, "bad gvr_debug_rays arguments");
    DeviceGuard g(h->device);
    if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int BC = batch * h->attrs.num_cameras;
    CallScratch scratch;
    int rc = scratch.acquire(nullptr, 0, sizeof(gvr::Camera) * BC, st);
    if (rc != GVR_OK) return rc;
    gvr::Camera *cams = static_cast<gvr::Camera *>(scratch.ptr);
    cudaError_t e = gvr::launch_cameras(extr, intr, cams, BC, st);
    if (e == cudaSuccess)
        e = gvr::launch_debug_rays(cams, rays, BC, h->attrs.render_resolution_u, h->attrs.render_resolution_v, st);
    if (e != cudaSuccess) return cuda_fail(e, "debug rays");
    return GVR_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------- backward without allocation
//
// Scratch for gvr_backward_noalloc: a fixed device array that every GPU
// loading this library holds until the process exits.  In host code the
// symbol is only a stand-in, so its device address is looked up once per
// device (with that device current) and cached.

namespace {

__device__ __align__(256) unsigned char g_noalloc_scratch[GVR_NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_mu;
std::vector<void *> g_noalloc_addr;  // per device ordinal

}  // namespace

extern "C" int gvr_backward_noalloc(GvrHandle *h, const GvrBackwardArgs *a, void *stream) {
    if (!h || !a) return fail(GVR_ERR_INVALID_ARGUMENT, "handle/args is NULL");
    const size_t need = gvr_backward_workspace_size(h, a->batch, a->texture_height, a->texture_width);
    if (need == 0) return fail(GVR_ERR_INVALID_ARGUMENT, "batch must be >= 1");
    if (need > GVR_NOALLOC_SCRATCH_BYTES)
        return fail(GVR_ERR_WORKSPACE, "gvr_backward_noalloc: this call needs " + std::to_string(need) +
                                           " bytes of scratch but the library's fixed scratch array holds " +
                                           std::to_string((size_t)GVR_NOALLOC_SCRATCH_BYTES) +
                                           "; use gvr_backward with a workspace");
    void *scratch = nullptr;
    {
        DeviceGuard g(h->device);
        if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (h->device < 0) return fail(GVR_ERR_INVALID_ARGUMENT, "bad device");
        if ((size_t)h->device >= g_noalloc_addr.size()) g_noalloc_addr.resize(h->device + 1, nullptr);
        if (!g_noalloc_addr[h->device]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
            g_noalloc_addr[h->device] = p;
        }
        scratch = g_noalloc_addr[h->device];
    }
    GvrBackwardArgs args = *a;
    args.workspace = scratch;
    args.workspace_bytes = GVR_NOALLOC_SCRATCH_BYTES;
    return gvr_backward(h, &args, stream);
}

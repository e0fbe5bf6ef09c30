// gvr_api.cu -- the C ABI (include/gvr.h): validation, topology upload,
// workspace layout and dispatch.  Errors are returned, never fatal.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
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
    int4 *d_vcsr;

    gvr::Topology topo() const { return gvr::Topology{d_faces, d_uvs, d_vstart, d_vfaces, d_vcsr, N, F}; }
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
    int *uvOwner;  // [Ht*Wt] face owning each texel (compute_normal_map only)
    size_t bytes;
};

// Tile shape (w x h = 256 pixels, w in {8, 16, 32}) and big-face threshold
// of the forward binning.  Every choice gives the same pixels.
struct TileCfg {
    int w = gvr::kTile, h = gvr::kTile, big = gvr::kBigTiles;
    int tilesX(const GvrHandle *hd) const { return (hd->attrs.render_resolution_u + w - 1) / w; }
    int tilesY(const GvrHandle *hd) const { return (hd->attrs.render_resolution_v + h - 1) / h; }
    bool valid() const { return (w == 8 || w == 16 || w == 32) && w * h == gvr::kTilePix && big >= 1 && big <= 64; }
};

// Buffers of one forward call except the per-call zeroed counters.
void fwd_carve_main(const GvrHandle *h, int B, int Ht, int Wt, const TileCfg &tc, Carver &c, FwdLayout &L) {
    const size_t BC = (size_t)B * h->attrs.num_cameras, T = (size_t)tc.tilesX(h) * tc.tilesY(h);
    L.s.cams = c.take<gvr::Camera>(BC);
    L.s.geo = c.take<gvr::FaceGeo>((size_t)B * h->F);
    L.s.fnormal = c.take<float4>((size_t)B * h->F);
    L.s.faceC = c.take<float4>((size_t)B * h->F);
    L.proj = c.take<float4>(BC * h->N);
    if (h->attrs.compute_normal_map) {  // no binning: the depth and shading passes do not run
        L.uvOwner = c.take<int>((size_t)(Ht > 0 ? Ht : 1) * (Wt > 0 ? Wt : 1));
        return;
    }
    L.s.vface = c.take<gvr::ViewFace>(BC * h->F);
    L.s.shadeRec = c.take<float4>((size_t)B * h->F * gvr::kShadeRows);
    L.s.tileStart = c.take<int>(BC * T + 1);
    L.s.bins = c.take<int>((size_t)tc.big * BC * h->F);
    L.s.bigList = c.take<int>(BC * h->F);
}

// The counters cleared before every call (tile counts and cursors, big-list
// counts, per-view depth ranges).
void fwd_carve_counters(const GvrHandle *h, int B, const TileCfg &tc, Carver &c, FwdLayout &L) {
    if (h->attrs.compute_normal_map) return;
    const size_t BC = (size_t)B * h->attrs.num_cameras, T = (size_t)tc.tilesX(h) * tc.tilesY(h);
    L.s.tileCount = c.take<int>(BC * T);
    L.s.tileCursor = c.take<int>(BC * T);
    L.s.bigCount = c.take<int>(BC);
    L.s.zRange = c.take<unsigned>(2 * BC);
}

FwdLayout fwd_layout(const GvrHandle *h, int B, int Ht, int Wt, void *base, const TileCfg &tc = TileCfg()) {
    Carver c(base);
    FwdLayout L{};
    fwd_carve_main(h, B, Ht, Wt, tc, c, L);
    c.take<char>(0);  // align
    const size_t z0 = c.off;
    fwd_carve_counters(h, B, tc, c, L);
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
    L.s.faceRec = c.take<float4>((size_t)B * h->F * gvr::kBwdFaceRows);
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
    if (attrs->albedo_mode < GVR_ALBEDO_VERTEX_COLOR || attrs->albedo_mode > GVR_ALBEDO_UV)
        return fail(GVR_ERR_INVALID_ARGUMENT, "INVALID ALBEDO MODE");
    if (attrs->shading_mode < GVR_SHADING_SHADED || attrs->shading_mode > GVR_SHADING_PHONG)
        return fail(GVR_ERR_INVALID_ARGUMENT, "INVALID SHADING MODE");
    // CudaRendererGrad.cpp:84-98
    if (attrs->image_filter_size <= 0) return fail(GVR_ERR_INVALID_ARGUMENT, "INVALID IMAGE FILTER SIZE");
    if (attrs->texture_filter_size <= 0) return fail(GVR_ERR_INVALID_ARGUMENT, "INVALID TEXTURE FILTER SIZE");
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
    std::vector<int4> csr(adj.size());
    for (int k = 0; k < nnz; ++k) {
        const int f = adj[k];
        csr[k] = make_int4(topo->faces[3 * f], topo->faces[3 * f + 1], topo->faces[3 * f + 2], f);
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
        {(void **)&h->d_vcsr, csr.data(), csr.size() * sizeof(int4)},
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
    cudaFree(h->d_vcsr);
    delete h;
}

size_t gvr_forward_workspace_size(const GvrHandle *h, int32_t batch, int32_t texture_height, int32_t texture_width) {
    if (!h || batch < 1) return 0;
    return fwd_layout(h, batch, texture_height, texture_width, nullptr).bytes;
}

size_t gvr_backward_workspace_size(const GvrHandle *h, int32_t batch, int32_t, int32_t) {
    if (!h || batch < 1) return 0;
    return bwd_layout(h, batch, nullptr).bytes;
}

static gvr::FrameDims dims_of(const GvrHandle *h, int B, int Ht, int Wt, const TileCfg &tc = TileCfg()) {
    gvr::FrameDims d;
    d.B = B;
    d.C = h->attrs.num_cameras;
    d.W = h->attrs.render_resolution_u;
    d.H = h->attrs.render_resolution_v;
    d.tilesX = tc.tilesX(h);
    d.tilesY = tc.tilesY(h);
    d.Ht = Ht;
    d.Wt = Wt;
    d.albedo = h->attrs.albedo_mode;
    d.shading = h->attrs.shading_mode;
    d.tileW = tc.w;
    d.tileH = tc.h;
    d.tileShift = tc.w == 8 ? 3 : tc.w == 16 ? 4 : 5;
    d.bigTiles = tc.big;
    return d;
}

// Checks the forward arguments against the handle (shared by the per-call
// and the batched forward).
static int check_forward_args(const GvrHandle *h, const GvrForwardArgs *a) {
    if (!h || !a) return fail(GVR_ERR_INVALID_ARGUMENT, "handle/args is NULL");
    if (!batch_fits(h, a->batch))
        return fail(GVR_ERR_INVALID_ARGUMENT, "batch must be >= 1 and the call within int32 index range");
    const int mode = h->attrs.albedo_mode;
    const bool textured = mode == GVR_ALBEDO_TEXTURED || mode == GVR_ALBEDO_TEXTURED_BILINEAR;
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
    if (h->attrs.compute_normal_map && (!a->normal_map || a->texture_height < 1 || a->texture_width < 1))
        return fail(GVR_ERR_INVALID_ARGUMENT,
                    "compute_normal_map needs the normal_map output and texture_height/width >= 1");
    return GVR_OK;
}

// Texture size the forward uses (1x1 when neither textured nor normal-map).
static void forward_texture_size(const GvrHandle *h, const GvrForwardArgs *a, int &Ht, int &Wt) {
    const bool used = h->attrs.albedo_mode == GVR_ALBEDO_TEXTURED || h->attrs.albedo_mode == GVR_ALBEDO_TEXTURED_BILINEAR ||
                      h->attrs.compute_normal_map;
    Ht = used ? a->texture_height : 1;
    Wt = used ? a->texture_width : 1;
}

static gvr::FwdJob make_job(const GvrHandle *h, const GvrForwardArgs *a, const FwdLayout &L,
                            const gvr::FrameDims &dims) {
    gvr::FwdJob J;
    J.topo = h->topo();
    J.dims = dims;
    J.ws = L.s;
    J.io = gvr::RasterIO{a->vertex_pos, a->vertex_color, a->texture, a->sh_coeff, a->vertex_normal,
                         a->barycentric, a->face, a->render};
    J.extr = a->extrinsics;
    J.intr = a->intrinsics;
    J.proj = L.proj;
    J.vnormal_out = a->vertex_normal;
    return J;
}

// The work of gvr_forward after the frame: the target copy and the unused normal map.
static int forward_epilogue(const GvrHandle *h, const GvrForwardArgs *a, cudaStream_t st) {
    const int B = a->batch;
    const size_t img = (size_t)B * h->attrs.num_cameras * h->attrs.render_resolution_v * h->attrs.render_resolution_u * 3;
    cudaError_t e;
    if (a->target_image_out && a->target_image_out != a->target_image) {
        e = cudaMemcpyAsync(a->target_image_out, a->target_image, img * sizeof(float), cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return cuda_fail(e, "target_image_out copy");
    }
    if (!h->attrs.compute_normal_map && a->normal_map && a->texture_height > 0 && a->texture_width > 0) {
        e = cudaMemsetAsync(a->normal_map, 0, (size_t)B * a->texture_height * a->texture_width * 3 * sizeof(float), st);
        if (e != cudaSuccess) return cuda_fail(e, "normal_map clear");
    }
    return GVR_OK;
}

int gvr_forward(GvrHandle *h, const GvrForwardArgs *a, void *stream) {
    int rc = check_forward_args(h, a);
    if (rc != GVR_OK) return rc;
    const int B = a->batch;
    DeviceGuard g(h->device);
    if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int Ht, Wt;
    forward_texture_size(h, a, Ht, Wt);
    const FwdLayout need = fwd_layout(h, B, Ht, Wt, nullptr);
    CallScratch scratch;
    rc = scratch.acquire(a->workspace, a->workspace_bytes, need.bytes, st);
    if (rc != GVR_OK) return rc;
    const FwdLayout L = fwd_layout(h, B, Ht, Wt, scratch.ptr);
    const gvr::FwdJob J = make_job(h, a, L, dims_of(h, B, Ht, Wt));
    const cudaError_t e = h->attrs.compute_normal_map ? gvr::launch_forward_normal_map(J, L.uvOwner, a->normal_map, st)
                                                      : gvr::launch_forward(J, st);
    if (e != cudaSuccess) return cuda_fail(e, "forward launch");
    return forward_epilogue(h, a, st);
}

// Checks the backward arguments against the handle (shared by the per-call
// and the batched backward).
static int check_backward_args(const GvrHandle *h, const GvrBackwardArgs *a) {
    if (!h || !a) return fail(GVR_ERR_INVALID_ARGUMENT, "handle/args is NULL");
    const int B = a->batch;
    if (!batch_fits(h, B)) return fail(GVR_ERR_INVALID_ARGUMENT, "batch must be >= 1 and the call within int32 index range");
    const int mode = h->attrs.albedo_mode;
    const bool textured = mode == GVR_ALBEDO_TEXTURED || mode == GVR_ALBEDO_TEXTURED_BILINEAR;
    if (a->texture_height < 1 || a->texture_width < 1)
        return fail(GVR_ERR_INVALID_ARGUMENT, "texture_height/texture_width must be >= 1 (texture_grad shape)");
    if (!a->vertex_pos_grad || !a->vertex_color_grad || !a->texture_grad || !a->sh_coeff_grad)
        return fail(GVR_ERR_INVALID_ARGUMENT, "all four gradient outputs are required");
    const bool zeroMode = mode == GVR_ALBEDO_NORMAL || mode == GVR_ALBEDO_LIGHTING || mode == GVR_ALBEDO_UV;
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
    return GVR_OK;
}

static bool zero_gradient_mode(const GvrHandle *h) {
    const int mode = h->attrs.albedo_mode;
    return mode == GVR_ALBEDO_NORMAL || mode == GVR_ALBEDO_LIGHTING || mode == GVR_ALBEDO_UV;
}

int gvr_backward(GvrHandle *h, const GvrBackwardArgs *a, void *stream) {
    int rc = check_backward_args(h, a);
    if (rc != GVR_OK) return rc;
    const int B = a->batch;
    const bool zeroMode = zero_gradient_mode(h);
    DeviceGuard g(h->device);
    if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CallScratch scratch;
    if (!zeroMode) {
        rc = scratch.acquire(a->workspace, a->workspace_bytes, bwd_layout(h, B, nullptr).bytes, st);
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
// symbol is only a stand-in, so its device address is looked up (with the
// handle's device current) on every call: the lookup is a table read once
// the module is loaded, and a device reset, after which the module is
// loaded again and the array may move, cannot leave a stale address behind.
// The first call on a device loads the module, so it should come before
// any stream capture.

namespace {

__device__ __align__(256) unsigned char g_noalloc_scratch[GVR_NOALLOC_SCRATCH_BYTES];

}  // namespace

extern "C" int gvr_backward_noalloc(GvrHandle *h, const GvrBackwardArgs *a, void *stream) {
    if (!h || !a) return fail(GVR_ERR_INVALID_ARGUMENT, "handle/args is NULL");
    if (!batch_fits(h, a->batch))
        return fail(GVR_ERR_INVALID_ARGUMENT, "batch must be >= 1 and the call within int32 index range");
    const int mode = h->attrs.albedo_mode;
    if (mode == GVR_ALBEDO_NORMAL || mode == GVR_ALBEDO_LIGHTING || mode == GVR_ALBEDO_UV) {
        // zero-gradient modes only clear the outputs: no scratch at all
        GvrBackwardArgs args = *a;
        args.workspace = nullptr;
        args.workspace_bytes = 0;
        return gvr_backward(h, &args, stream);
    }
    const size_t need = gvr_backward_workspace_size(h, a->batch, a->texture_height, a->texture_width);
    if (need > GVR_NOALLOC_SCRATCH_BYTES)
        return fail(GVR_ERR_WORKSPACE, "gvr_backward_noalloc: this call needs " + std::to_string(need) +
                                           " bytes of scratch but the library's fixed scratch array holds " +
                                           std::to_string((size_t)GVR_NOALLOC_SCRATCH_BYTES) +
                                           "; use gvr_backward with a workspace");
    void *scratch = nullptr;
    {
        DeviceGuard g(h->device);
        if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
        const cudaError_t e = cudaGetSymbolAddress(&scratch, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
    }
    GvrBackwardArgs args = *a;
    args.workspace = scratch;
    args.workspace_bytes = GVR_NOALLOC_SCRATCH_BYTES;
    return gvr_backward(h, &args, stream);
}

// ---------------------------------------------------------------------------- batched forward plans

// The backward half of a plan (gvr_plan_bind_backward): one backward call per job.
struct PlanBackward {
    std::vector<GvrBackwardArgs> args;
    void *d_mem = nullptr;  // every job's scratch and the tables
    gvr::BwdBatchLaunch launch{};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~PlanBackward() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (d_mem) cudaFree(d_mem);
    }
};

struct GvrPlan {
    int device = 0;
    std::vector<GvrJob> jobs;
    std::vector<TileCfg> tiles;
    void *d_mem = nullptr;  // every job's scratch, the job tables and the zeroed counters
    gvr::BatchLaunch launch{};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    PlanBackward *bwd = nullptr;
    // per-job rasters on parallel lanes (forked from and joined to the caller's
    // stream); no lanes with GVR_PLAN_PERSISTENT
    std::vector<gvr::FwdJob> hostJobs;
    std::vector<int> order;                 // jobs by decreasing pixel count
    std::vector<cudaStream_t> lanes;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> joins;
};

namespace {

// Candidate bin/tile configurations of the autotuner: tile shapes of 256
// pixels and the span (in tiles) above which a face goes to the view's
// big-face list.
const TileCfg kTuneCandidates[] = {{16, 16, 16}, {32, 8, 16}, {8, 32, 16}, {16, 16, 4}, {32, 8, 4}, {8, 32, 4}};

std::mutex g_tune_mu;
std::map<std::tuple<int, int, int>, TileCfg> g_tune_cache;  // (floor(log2 F), W, H) -> fastest

int log2_floor(int x) {
    int k = 0;
    while (k < 30 && (1 << (k + 1)) <= x) ++k;
    return k;
}

// Times one forward of a job under every candidate configuration on a
// private stream (CUDA events; one warm-up, median of three) and returns the
// fastest.  The job's outputs are written, as by a normal forward.
int autotune_job(const GvrHandle *h, const GvrForwardArgs *a, TileCfg &best) {
    int Ht, Wt;
    forward_texture_size(h, a, Ht, Wt);
    size_t bytes = 0;
    for (const TileCfg &c : kTuneCandidates) bytes = std::max(bytes, fwd_layout(h, a->batch, Ht, Wt, nullptr, c).bytes);
    void *ws = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaError_t e = cudaMalloc(&ws, bytes);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
    float bestMs = INFINITY;
    best = TileCfg();
    for (const TileCfg &c : kTuneCandidates) {
        if (e != cudaSuccess) break;
        const FwdLayout L = fwd_layout(h, a->batch, Ht, Wt, ws, c);
        const gvr::FwdJob J = make_job(h, a, L, dims_of(h, a->batch, Ht, Wt, c));
        float t[3];
        e = gvr::launch_forward(J, st);
        for (int r = 0; r < 3 && e == cudaSuccess; ++r) {
            e = cudaEventRecord(ev[0], st);
            if (e == cudaSuccess) e = gvr::launch_forward(J, st);
            if (e == cudaSuccess) e = cudaEventRecord(ev[1], st);
            if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&t[r], ev[0], ev[1]);
        }
        if (e != cudaSuccess) break;
        std::sort(t, t + 3);
        if (t[1] < bestMs) {
            bestMs = t[1];
            best = c;
        }
    }
    if (st) cudaStreamSynchronize(st);
    for (cudaEvent_t x : ev)
        if (x) cudaEventDestroy(x);
    if (st) cudaStreamDestroy(st);
    if (ws) cudaFree(ws);
    return e == cudaSuccess ? GVR_OK : cuda_fail(e, "autotune");
}

int tile_config_for(const GvrHandle *h, const GvrForwardArgs *a, bool tune, TileCfg &out) {
    out = TileCfg();
    if (!tune) return GVR_OK;
    const auto key = std::make_tuple(log2_floor(h->F), h->attrs.render_resolution_u, h->attrs.render_resolution_v);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            out = it->second;
            return GVR_OK;
        }
    }
    int rc = autotune_job(h, a, out);
    if (rc != GVR_OK) return rc;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = out;
    return GVR_OK;
}

// Device tables of a plan, carved after every job's scratch.
struct PlanTables {
    gvr::FwdJob *jobs;
    int *blockStart[gvr::kNumStages];
    int *itemStart;
    int *counter;
};

// Carves (or, with base == nullptr, measures) a plan's memory: every job's
// scratch, the tables, then one zeroed region holding every job's counters
// and the raster work counter.
size_t plan_carve(const GvrPlan &p, void *base, std::vector<FwdLayout> &lay, PlanTables &t, size_t &z0,
                  size_t &z1) {
    const int J = (int)p.jobs.size();
    Carver c(base);
    lay.assign(J, FwdLayout{});
    for (int j = 0; j < J; ++j) {
        const GvrJob &job = p.jobs[j];
        int Ht, Wt;
        forward_texture_size(job.handle, &job.forward, Ht, Wt);
        fwd_carve_main(job.handle, job.forward.batch, Ht, Wt, p.tiles[j], c, lay[j]);
    }
    t.jobs = c.take<gvr::FwdJob>(J);
    for (int s = 0; s < gvr::kNumStages; ++s) t.blockStart[s] = c.take<int>(J + 1);
    t.itemStart = c.take<int>(J + 1);
    c.take<char>(0);
    z0 = c.off;
    for (int j = 0; j < J; ++j) fwd_carve_counters(p.jobs[j].handle, p.jobs[j].forward.batch, p.tiles[j], c, lay[j]);
    t.counter = c.take<int>(1);
    z1 = c.off;
    return c.off + 256;
}

int plan_forward_body(GvrPlan *p, cudaStream_t st) {
    cudaError_t e = gvr::launch_forward_batched(p->launch, st, p->lanes.empty());
    if (e != cudaSuccess) return cuda_fail(e, "batched forward launch");
    if (!p->lanes.empty()) {
        e = cudaEventRecord(p->fork, st);
        for (size_t k = 0; k < p->lanes.size() && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(p->lanes[k], p->fork, 0);
        for (size_t i = 0; i < p->order.size() && e == cudaSuccess; ++i)
            e = gvr::launch_raster(p->hostJobs[p->order[i]], p->lanes[i % p->lanes.size()]);
        for (size_t k = 0; k < p->lanes.size() && e == cudaSuccess; ++k) {
            e = cudaEventRecord(p->joins[k], p->lanes[k]);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(st, p->joins[k], 0);
        }
        if (e != cudaSuccess) return cuda_fail(e, "per-job raster lanes");
    }
    for (const GvrJob &job : p->jobs) {
        const int rc = forward_epilogue(job.handle, &job.forward, st);
        if (rc != GVR_OK) return rc;
    }
    return GVR_OK;
}

}  // namespace

extern "C" {

int gvr_plan_create(const GvrJob *jobs, int32_t count, int32_t flags, GvrPlan **out_plan) {
    if (!out_plan) return fail(GVR_ERR_INVALID_ARGUMENT, "out_plan is NULL");
    *out_plan = nullptr;
    if (!jobs || count < 1) return fail(GVR_ERR_INVALID_ARGUMENT, "a plan needs at least one job");
    const int device = jobs[0].handle ? jobs[0].handle->device : -1;
    for (int j = 0; j < count; ++j) {
        if (jobs[j].handle && jobs[j].handle->attrs.compute_normal_map)
            return fail(GVR_ERR_UNSUPPORTED, "job " + std::to_string(j) + ": normal-map handles run through gvr_forward");
        const int rc = check_forward_args(jobs[j].handle, &jobs[j].forward);
        if (rc != GVR_OK) return fail(rc, "job " + std::to_string(j) + ": " + g_error);
        if (jobs[j].handle->device != device)
            return fail(GVR_ERR_INVALID_ARGUMENT, "job " + std::to_string(j) + " is on another device");
    }
    DeviceGuard g(device);
    if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
    GvrPlan *p = new GvrPlan();
    p->device = device;
    p->jobs.assign(jobs, jobs + count);
    p->tiles.resize(count);
    for (int j = 0; j < count; ++j) {
        const GvrJob &job = jobs[j];
        const bool forced = job.tile_width != 0 || job.big_tiles != 0;
        int rc = GVR_OK;
        if (forced) {
            TileCfg c;
            if (job.tile_width) {
                c.w = job.tile_width;
                c.h = job.tile_width > 0 ? gvr::kTilePix / job.tile_width : 0;
            }
            if (job.big_tiles) c.big = job.big_tiles;
            if (!c.valid() || c.big > gvr::kBigTiles)
                rc = fail(GVR_ERR_INVALID_ARGUMENT, "job " + std::to_string(j) +
                                                        ": tile_width must be 8, 16 or 32 and big_tiles 1..16");
            p->tiles[j] = c;
        } else {
            rc = tile_config_for(job.handle, &job.forward, (flags & GVR_PLAN_AUTOTUNE) != 0, p->tiles[j]);
        }
        if (rc != GVR_OK) {
            delete p;
            return rc;
        }
    }
    // host copies of the tables
    std::vector<int> start[gvr::kNumStages], items(count + 1, 0);
    for (auto &s : start) s.assign(count + 1, 0);
    long long totalItems = 0, totalBlocks[gvr::kNumStages] = {0};
    for (int j = 0; j < count; ++j) {
        const GvrHandle *h = jobs[j].handle;
        const long long B = jobs[j].forward.batch, C = h->attrs.num_cameras;
        const long long n[gvr::kNumStages] = {B * C, B * h->F, B * h->N, B * C * h->F, B * C * h->F};
        for (int s = 0; s < gvr::kNumStages; ++s) {
            start[s][j] = (int)totalBlocks[s];
            totalBlocks[s] += (n[s] + gvr::kBatchBlock - 1) / gvr::kBatchBlock;
        }
        items[j] = (int)totalItems;
        totalItems += B * C * p->tiles[j].tilesX(h) * p->tiles[j].tilesY(h);
        if (totalItems >= INT_MAX || totalBlocks[gvr::kStageBinCount] >= INT_MAX) {
            delete p;
            return fail(GVR_ERR_INVALID_ARGUMENT, "plan too large for int32 indexing");
        }
    }
    for (int s = 0; s < gvr::kNumStages; ++s) start[s][count] = (int)totalBlocks[s];
    items[count] = (int)totalItems;

    std::vector<FwdLayout> lay;
    PlanTables t{};
    size_t z0 = 0, z1 = 0;
    const size_t bytes = plan_carve(*p, nullptr, lay, t, z0, z1);
    cudaError_t e = cudaMalloc(&p->d_mem, bytes);
    if (e != cudaSuccess) {
        delete p;
        return cuda_fail(e, "cudaMalloc(plan)");
    }
    plan_carve(*p, p->d_mem, lay, t, z0, z1);
    std::vector<gvr::FwdJob> hostJobs(count);
    for (int j = 0; j < count; ++j) {
        const GvrJob &job = jobs[j];
        int Ht, Wt;
        forward_texture_size(job.handle, &job.forward, Ht, Wt);
        hostJobs[j] = make_job(job.handle, &job.forward, lay[j], dims_of(job.handle, job.forward.batch, Ht, Wt, p->tiles[j]));
    }
    e = cudaMemcpy(t.jobs, hostJobs.data(), sizeof(gvr::FwdJob) * count, cudaMemcpyHostToDevice);
    for (int s = 0; s < gvr::kNumStages && e == cudaSuccess; ++s)
        e = cudaMemcpy(t.blockStart[s], start[s].data(), sizeof(int) * (count + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t.itemStart, items.data(), sizeof(int) * (count + 1), cudaMemcpyHostToDevice);
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) {
        gvr_plan_destroy(p);
        return cuda_fail(e, "plan setup");
    }
    gvr::BatchLaunch &L = p->launch;
    L.jobs = t.jobs;
    for (int s = 0; s < gvr::kNumStages; ++s) {
        L.blockStart[s] = t.blockStart[s];
        L.blocks[s] = (int)totalBlocks[s];
    }
    L.itemStart = t.itemStart;
    L.counter = t.counter;
    L.nJobs = count;
    L.rasterGrid = (int)std::min<long long>((long long)sms * gvr::raster_persistent_blocks_per_sm(), totalItems);
    L.zeroBase = static_cast<char *>(p->d_mem) + z0;
    L.zeroBytes = z1 - z0;
    p->hostJobs = hostJobs;
    p->order.resize(count);
    for (int j = 0; j < count; ++j) p->order[j] = j;
    std::sort(p->order.begin(), p->order.end(), [&](int x, int y) {
        const auto px = (long long)hostJobs[x].dims.B * hostJobs[x].dims.C * hostJobs[x].dims.W * hostJobs[x].dims.H;
        const auto py = (long long)hostJobs[y].dims.B * hostJobs[y].dims.C * hostJobs[y].dims.W * hostJobs[y].dims.H;
        return px > py;
    });
    const int nLanes = (flags & GVR_PLAN_PERSISTENT) ? 0 : std::min(GVR_PLAN_LANES, count);
    if (nLanes > 0) e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming);
    for (int k = 0; k < nLanes && e == cudaSuccess; ++k) {
        cudaStream_t s = nullptr;
        cudaEvent_t ev = nullptr;
        e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e == cudaSuccess) {
            p->lanes.push_back(s);
            e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        }
        if (e == cudaSuccess) p->joins.push_back(ev);
    }
    if (e != cudaSuccess) {
        gvr_plan_destroy(p);
        return cuda_fail(e, "plan lanes");
    }
    *out_plan = p;
    return GVR_OK;
}

int gvr_plan_forward(GvrPlan *p, void *stream) {
    if (!p) return fail(GVR_ERR_INVALID_ARGUMENT, "plan is NULL");
    DeviceGuard g(p->device);
    if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
    return plan_forward_body(p, static_cast<cudaStream_t>(stream));
}

int gvr_plan_forward_graph(GvrPlan *p, void *stream) {
    if (!p) return fail(GVR_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (!stream) return fail(GVR_ERR_INVALID_ARGUMENT, "graph capture needs a created (non-default) stream");
    DeviceGuard g(p->device);
    if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!p->exec) {
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
        const int rc = plan_forward_body(p, st);
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(st, &graph);
        if (rc != GVR_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&p->exec, graph, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(graph);
            p->exec = nullptr;
            return cuda_fail(e, "cudaGraphInstantiate");
        }
        p->graph = graph;
    }
    const cudaError_t e = cudaGraphLaunch(p->exec, st);
    return e == cudaSuccess ? GVR_OK : cuda_fail(e, "cudaGraphLaunch");
}

int gvr_plan_tile_config(const GvrPlan *p, int32_t job, int32_t *tile_w, int32_t *tile_h, int32_t *big_tiles) {
    if (!p || job < 0 || job >= (int)p->tiles.size()) return fail(GVR_ERR_INVALID_ARGUMENT, "bad plan or job index");
    if (tile_w) *tile_w = p->tiles[job].w;
    if (tile_h) *tile_h = p->tiles[job].h;
    if (big_tiles) *big_tiles = p->tiles[job].big;
    return GVR_OK;
}

int gvr_plan_bind_backward(GvrPlan *p, const GvrBackwardArgs *args, int32_t count) {
    if (!p) return fail(GVR_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (!args || count != (int)p->jobs.size())
        return fail(GVR_ERR_INVALID_ARGUMENT, "one backward call per job of the plan, in the plan's job order");
    for (int j = 0; j < count; ++j) {
        const int rc = check_backward_args(p->jobs[j].handle, &args[j]);
        if (rc != GVR_OK) return fail(rc, "job " + std::to_string(j) + ": " + g_error);
    }
    DeviceGuard g(p->device);
    if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
    using gvr::BwdBatchLaunch;
    const int J = count;
    // host tables: per-stage block offsets, clearing regions and pixel groups
    std::vector<int> start[gvr::kNumBwdStages];
    for (auto &v : start) v.assign(J + 1, 0);
    long long total[gvr::kNumBwdStages] = {0};
    std::vector<int> variant(J);
    std::vector<std::vector<int>> groupJobs(gvr::kNumBwdVariants), groupStart(gvr::kNumBwdVariants);
    std::vector<long long> groupTotal(gvr::kNumBwdVariants, 0);
    for (int j = 0; j < J; ++j) {
        const GvrHandle *h = p->jobs[j].handle;
        const GvrBackwardArgs &a = args[j];
        const long long B = a.batch, C = h->attrs.num_cameras;
        variant[j] = gvr::backward_variant(h->attrs.albedo_mode, h->attrs.shading_mode, a.target_grad != nullptr,
                                           (a.flags & GVR_BACKWARD_ALBEDO_POSITION) != 0);
        const bool zero = variant[j] < 0;
        const long long n[gvr::kNumBwdStages] = {zero ? 0 : (B * C + gvr::kBatchBlock - 1) / gvr::kBatchBlock,
                                                 zero ? 0 : (B * h->F + gvr::kBatchBlock - 1) / gvr::kBatchBlock,
                                                 zero ? 0 : (B * h->N + 255) / 256, zero ? 0 : B * C * 27};
        for (int st = 0; st < gvr::kNumBwdStages; ++st) {
            start[st][j] = (int)total[st];
            total[st] += n[st];
        }
        if (!zero) {
            groupJobs[variant[j]].push_back(j);
            groupStart[variant[j]].push_back((int)groupTotal[variant[j]]);
            groupTotal[variant[j]] += B * C * h->tilesX * h->tilesY;
        }
    }
    for (int st = 0; st < gvr::kNumBwdStages; ++st) {
        if (total[st] >= INT_MAX) return fail(GVR_ERR_INVALID_ARGUMENT, "plan too large for int32 indexing");
        start[st][J] = (int)total[st];
    }
    for (int v = 0; v < gvr::kNumBwdVariants; ++v) {
        if (groupTotal[v] >= INT_MAX) return fail(GVR_ERR_INVALID_ARGUMENT, "plan too large for int32 indexing");
        groupStart[v].push_back((int)groupTotal[v]);
    }
    // device memory: every job's scratch, then the tables
    auto measure = [&](void *base, std::vector<BwdLayout> &lay, gvr::BwdJob *&djobs, int *(&dstart)[gvr::kNumBwdStages],
                       gvr::ZeroRegion *&dzero, int *&dzeroStart, int *&dgroups, size_t nZero, size_t nGroupInts) {
        Carver c(base);
        lay.assign(J, BwdLayout{});
        for (int j = 0; j < J; ++j) {
            if (variant[j] < 0) continue;
            Carver sub(base ? static_cast<char *>(base) + ((c.off + 255) & ~size_t(255)) : nullptr);
            const size_t bytes = bwd_layout(p->jobs[j].handle, args[j].batch, nullptr).bytes;
            lay[j] = bwd_layout(p->jobs[j].handle, args[j].batch, sub.base);
            c.take<char>(bytes);
        }
        djobs = c.take<gvr::BwdJob>(J);
        for (int st = 0; st < gvr::kNumBwdStages; ++st) dstart[st] = c.take<int>(J + 1);
        dzero = c.take<gvr::ZeroRegion>(nZero > 0 ? nZero : 1);
        dzeroStart = c.take<int>(nZero + 1);
        dgroups = c.take<int>(nGroupInts > 0 ? nGroupInts : 1);
        return c.off + 256;
    };
    std::vector<BwdLayout> lay;
    gvr::BwdJob *djobs = nullptr;
    int *dstart[gvr::kNumBwdStages] = {nullptr};
    gvr::ZeroRegion *dzero = nullptr;
    int *dzeroStart = nullptr, *dgroups = nullptr;
    size_t nZero = 0, nGroupInts = 0;
    for (int j = 0; j < J; ++j) nZero += variant[j] < 0 ? 4 : 2;
    for (int v = 0; v < gvr::kNumBwdVariants; ++v)
        if (!groupJobs[v].empty()) nGroupInts += 2 * groupJobs[v].size() + 1;
    const size_t bytes = measure(nullptr, lay, djobs, dstart, dzero, dzeroStart, dgroups, nZero, nGroupInts);
    PlanBackward *b = new PlanBackward();
    cudaError_t e = cudaMalloc(&b->d_mem, bytes);
    if (e != cudaSuccess) {
        delete b;
        return cuda_fail(e, "cudaMalloc(plan backward)");
    }
    measure(b->d_mem, lay, djobs, dstart, dzero, dzeroStart, dgroups, nZero, nGroupInts);
    // host copies of the job records, clearing regions and groups
    std::vector<gvr::BwdJob> hostJobs(J);
    std::vector<gvr::ZeroRegion> zeros;
    std::vector<int> zeroStart(1, 0);
    auto addZero = [&](void *ptr, long long floats) {
        zeros.push_back(gvr::ZeroRegion{static_cast<float *>(ptr), floats});
        zeroStart.push_back(zeroStart.back() + (int)((floats + gvr::kZeroPerBlock - 1) / gvr::kZeroPerBlock));
    };
    for (int j = 0; j < J; ++j) {
        const GvrHandle *h = p->jobs[j].handle;
        const GvrBackwardArgs &a = args[j];
        const long long B = a.batch, C = h->attrs.num_cameras;
        gvr::BwdJob &R = hostJobs[j];
        std::memset(&R, 0, sizeof(R));
        R.topo = h->topo();
        R.dims = dims_of(h, a.batch, a.texture_height, a.texture_width);
        R.ws = lay[j].s;
        const int phong = h->attrs.shading_mode == GVR_SHADING_PHONG && h->attrs.albedo_mode != GVR_ALBEDO_FOREGROUND_MASK;
        R.io = gvr::BwdIO{a.render_grad, a.vertex_pos, a.vertex_color, a.texture, a.sh_coeff, a.target_image,
                          a.vertex_normal, a.barycentric, a.face, a.target_grad, a.texture_grad,
                          h->attrs.image_filter_size, phong};
        R.extr = a.extrinsics;
        R.intr = a.intrinsics;
        R.vpos_grad = a.vertex_pos_grad;
        R.vcol_grad = a.vertex_color_grad;
        R.sh_grad = a.sh_coeff_grad;
        R.zeroMode = variant[j] < 0;
        R.shaded = h->attrs.shading_mode == GVR_SHADING_SHADED && h->attrs.albedo_mode != GVR_ALBEDO_FOREGROUND_MASK;
        R.useCol = h->attrs.albedo_mode == GVR_ALBEDO_VERTEX_COLOR;
        const long long tex = B * a.texture_height * a.texture_width * 3;
        if (R.zeroMode) {
            addZero(a.vertex_pos_grad, B * h->N * 3);
            addZero(a.vertex_color_grad, B * h->N * 3);
            addZero(a.texture_grad, tex);
            addZero(a.sh_coeff_grad, B * C * 27);
        } else {
            addZero(R.ws.faceAcc, B * h->F * gvr::kFaceAccFloats);
            addZero(a.texture_grad, tex);
        }
    }
    std::vector<int> groupInts;
    gvr::BwdBatchLaunch &L = b->launch;
    L.nGroups = 0;
    for (int v = 0; v < gvr::kNumBwdVariants; ++v) {
        if (groupJobs[v].empty()) continue;
        const int g = L.nGroups++;
        L.groupVariant[g] = v;
        L.groupCount[g] = (int)groupJobs[v].size();
        L.groupBlocks[g] = groupStart[v].back();
        L.groupJobs[g] = dgroups + groupInts.size();
        groupInts.insert(groupInts.end(), groupJobs[v].begin(), groupJobs[v].end());
        L.groupStart[g] = dgroups + groupInts.size();
        groupInts.insert(groupInts.end(), groupStart[v].begin(), groupStart[v].end());
    }
    e = cudaMemcpy(djobs, hostJobs.data(), sizeof(gvr::BwdJob) * J, cudaMemcpyHostToDevice);
    for (int st = 0; st < gvr::kNumBwdStages && e == cudaSuccess; ++st)
        e = cudaMemcpy(dstart[st], start[st].data(), sizeof(int) * (J + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !zeros.empty())
        e = cudaMemcpy(dzero, zeros.data(), sizeof(gvr::ZeroRegion) * zeros.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dzeroStart, zeroStart.data(), sizeof(int) * zeroStart.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !groupInts.empty())
        e = cudaMemcpy(dgroups, groupInts.data(), sizeof(int) * groupInts.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        delete b;
        return cuda_fail(e, "plan backward setup");
    }
    if (zeroStart.back() >= INT_MAX) {
        delete b;
        return fail(GVR_ERR_INVALID_ARGUMENT, "plan too large for int32 indexing");
    }
    L.jobs = djobs;
    for (int st = 0; st < gvr::kNumBwdStages; ++st) {
        L.blockStart[st] = dstart[st];
        L.blocks[st] = (int)total[st];
    }
    L.zeros = dzero;
    L.zeroStart = dzeroStart;
    L.nZero = (int)zeros.size();
    L.zeroBlocks = zeroStart.back();
    L.nJobs = J;
    b->args.assign(args, args + count);
    delete p->bwd;
    p->bwd = b;
    return GVR_OK;
}

int gvr_plan_backward(GvrPlan *p, void *stream) {
    if (!p) return fail(GVR_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (!p->bwd) return fail(GVR_ERR_INVALID_ARGUMENT, "no backward bound to the plan (gvr_plan_bind_backward)");
    DeviceGuard g(p->device);
    if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
    const cudaError_t e = gvr::launch_backward_batched(p->bwd->launch, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? GVR_OK : cuda_fail(e, "batched backward launch");
}

int gvr_plan_backward_graph(GvrPlan *p, void *stream) {
    if (!p) return fail(GVR_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (!p->bwd) return fail(GVR_ERR_INVALID_ARGUMENT, "no backward bound to the plan (gvr_plan_bind_backward)");
    if (!stream) return fail(GVR_ERR_INVALID_ARGUMENT, "graph capture needs a created (non-default) stream");
    DeviceGuard g(p->device);
    if (g.err != cudaSuccess) return cuda_fail(g.err, "cudaSetDevice");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    PlanBackward *b = p->bwd;
    if (!b->exec) {
        cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
        const cudaError_t le = gvr::launch_backward_batched(b->launch, st);
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(st, &graph);
        if (le != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return cuda_fail(le, "batched backward launch");
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&b->exec, graph, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(graph);
            b->exec = nullptr;
            return cuda_fail(e, "cudaGraphInstantiate");
        }
        b->graph = graph;
    }
    const cudaError_t e = cudaGraphLaunch(b->exec, st);
    return e == cudaSuccess ? GVR_OK : cuda_fail(e, "cudaGraphLaunch");
}

void gvr_plan_destroy(GvrPlan *p) {
    if (!p) return;
    DeviceGuard g(p->device);
    delete p->bwd;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->d_mem) cudaFree(p->d_mem);
    for (cudaStream_t s : p->lanes) cudaStreamDestroy(s);
    for (cudaEvent_t ev : p->joins) cudaEventDestroy(ev);
    if (p->fork) cudaEventDestroy(p->fork);
    delete p;
}

}  // extern "C"

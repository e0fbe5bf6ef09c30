/*
 * gvr.h -- C ABI of the GB300 differentiable mesh rasteriser.
 *
 * Drop-in boundary for the reference's CudaRenderer operator pair:
 *   gvr_create   <- CudaRenderer / CudaRendererGrad op construction
 *                   (cpp/src/TensorflowOperators/CudaRenderer/CudaRenderer.cpp:37-155,
 *                    CudaRendererGrad.cpp:43-101) and the renderer constructors
 *                   (cpp/src/Renderer/CUDABasedRasterization.cpp:11-106,
 *                    CUDABasedRasterizationGrad.cpp:7-87): attrs, topology,
 *                   vertex->face adjacency.
 *   gvr_forward  <- CudaRenderer::Compute (CudaRenderer.cpp:298-335) and the op
 *                   signature REGISTER_OP("CudaRendererGpu") (CudaRenderer.cpp:5-33).
 *   gvr_backward <- CudaRendererGrad::Compute (CudaRendererGrad.cpp:252-293) and
 *                   REGISTER_OP("CudaRendererGradGpu") (CudaRendererGrad.cpp:6-39).
 *   gvr_destroy  <- the renderer destructors (CUDABasedRasterization.cpp:110-121).
 *
 * Conventions: every tensor pointer is a device pointer to C-contiguous
 * float32 (int32 for faces) data in the reference's layouts; `stream` is a
 * cudaStream_t (NULL = legacy default stream).  Calls return a GvrStatus and
 * never abort; gvr_last_error() gives the calling thread's last message.
 * A handle is immutable after gvr_create and may be used from several
 * streams at once; per-call scratch is either the caller's workspace or
 * stream-ordered memory (cudaMallocAsync) owned by the call.
 */
#ifndef GVR_H
#define GVR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GVR_ABI_VERSION 1

typedef enum {
    GVR_OK = 0,
    GVR_ERR_INVALID_ARGUMENT = -1, /* bad size, pointer, index or mode             */
    GVR_ERR_CUDA = -2,             /* a CUDA runtime call or kernel launch failed  */
    GVR_ERR_OUT_OF_MEMORY = -3,    /* device allocation failed                     */
    GVR_ERR_WORKSPACE = -4,        /* caller workspace smaller than required       */
    GVR_ERR_UNSUPPORTED = -5       /* combination not supported by this build      */
} GvrStatus;

/* AlbedoMode / ShadingMode (cpp/src/Renderer/CUDABasedRasterizationInput.h:25-35).
 * Values 0-4 and shading 0-1 are the reference's.  The others have no
 * reference counterpart:
 *   GVR_ALBEDO_TEXTURED_BILINEAR  bilinear texture lookup at the same texture
 *       coordinate (texel centres at integer + 0.5, indices clamped to the
 *       texture); its texture gradient is the lookup's derivative (4 texels).
 *   GVR_ALBEDO_UV  the interpolated per-corner (u, v) as red and green, blue
 *       0, never shaded; zero gradients (like the normal mode).
 *   GVR_SHADING_PHONG  a headlight Phong term instead of SH:
 *       albedo * (0.2 + 0.7 max(0, n.l)) + 0.3 max(0, 2 (n.l)^2 - 1)^16 with
 *       l the direction to the camera; gradients for vertex colours and
 *       texture only (no SH, no position gradient). */
typedef enum {
    GVR_ALBEDO_VERTEX_COLOR = 0,
    GVR_ALBEDO_TEXTURED = 1,
    GVR_ALBEDO_NORMAL = 2,
    GVR_ALBEDO_LIGHTING = 3,
    GVR_ALBEDO_FOREGROUND_MASK = 4,
    GVR_ALBEDO_TEXTURED_BILINEAR = 5,
    GVR_ALBEDO_UV = 6
} GvrAlbedoMode;

typedef enum { GVR_SHADING_SHADED = 0, GVR_SHADING_SHADELESS = 1, GVR_SHADING_PHONG = 2 } GvrShadingMode;

typedef struct GvrHandle GvrHandle;

/* Op attrs `faces`, `texture_coordinates`, `number_of_vertices`
 * (CudaRenderer.cpp:23-25); host pointers, copied by gvr_create. */
typedef struct {
    const int32_t *faces;              /* [F*3] vertex ids                     */
    const float *texture_coordinates;  /* [F*6] per-corner (u, v); may be NULL */
    int32_t num_faces;                 /* F                                    */
    int32_t num_vertices;              /* N                                    */
} GvrTopology;

/* Remaining op attrs (CudaRenderer.cpp:26-33). */
typedef struct {
    int32_t num_cameras;          /* number_of_cameras                         */
    int32_t render_resolution_u;  /* W                                         */
    int32_t render_resolution_v;  /* H                                         */
    int32_t albedo_mode;          /* GvrAlbedoMode                             */
    int32_t shading_mode;         /* GvrShadingMode (foregroundMask forces shadeless) */
    int32_t image_filter_size;    /* >= 1, window half-size of the target-image gradient */
    int32_t texture_filter_size;  /* >= 1, accepted; unused by the reference kernels too */
    int32_t compute_normal_map;   /* 1: write the texture-space normal map instead of
                                     rendering; the frame outputs stay cleared (face -1,
                                     barycentrics 0, green), as in the reference */
} GvrAttrs;

/* CudaRendererGpu inputs 0-6 and outputs 0-5 (CudaRenderer.cpp:7-20). */
typedef struct {
    int32_t batch;                /* B                                          */
    int32_t texture_height;       /* Ht (texture dim 1)                         */
    int32_t texture_width;        /* Wt (texture dim 2)                         */
    const float *vertex_pos;      /* [B,N,3]                                    */
    const float *vertex_color;    /* [B,N,3]                                    */
    const float *texture;         /* [B,Ht,Wt,3]                                */
    const float *sh_coeff;        /* [B,C,27]                                   */
    const float *target_image;    /* [B,C,H,W,3]; read only for target_image_out */
    const float *extrinsics;      /* [B,C,12] world->camera 3x4 row-major       */
    const float *intrinsics;      /* [B,C,9] 3x3 row-major                      */
    float *barycentric;           /* out [B,C,H,W,2]                            */
    int32_t *face;                /* out [B,C,H,W], -1 = background             */
    float *render;                /* out [B,C,H,W,3]                            */
    float *vertex_normal;         /* out [B,C,N,3]                              */
    float *target_image_out;      /* out [B,C,H,W,3] copy of target_image, or NULL */
    float *normal_map;            /* out [B,Ht,Wt,3]; required with compute_normal_map,
                                     otherwise NULL or cleared to 0 */
    void *workspace;              /* optional device scratch, >= gvr_forward_workspace_size */
    size_t workspace_bytes;
} GvrForwardArgs;

/* CudaRendererGradGpu inputs 0-11 and outputs 0-3 (CudaRendererGrad.cpp:8-29). */
typedef struct {
    int32_t batch;
    int32_t texture_height;
    int32_t texture_width;
    const float *render_grad;     /* [B,C,H,W,3]                                */
    const float *vertex_pos;      /* [B,N,3]                                    */
    const float *vertex_color;    /* [B,N,3]                                    */
    const float *texture;         /* [B,Ht,Wt,3]                                */
    const float *sh_coeff;        /* [B,C,27]                                   */
    const float *target_image;    /* [B,C,H,W,3]; may be NULL if target_grad is NULL */
    const float *vertex_normal;   /* [B,C,N,3] (forward output)                 */
    const float *barycentric;     /* [B,C,H,W,2] (forward output); NULL = recomputed from `face` */
    const int32_t *face;          /* [B,C,H,W] (forward output)                 */
    const float *target_grad;     /* [B,C,H,W,3] upstream grad of target_image_out, or NULL = 0 */
    const float *extrinsics;      /* [B,C,12]                                   */
    const float *intrinsics;      /* [B,C,9]                                    */
    float *vertex_pos_grad;       /* out [B,N,3]                                */
    float *vertex_color_grad;     /* out [B,N,3]                                */
    float *texture_grad;          /* out [B,Ht,Wt,3]                            */
    float *sh_coeff_grad;         /* out [B,C,27]                               */
    void *workspace;
    size_t workspace_bytes;
    int32_t flags;                /* 0 = the reference's gradient; GVR_BACKWARD_* options */
} GvrBackwardArgs;

/* Backward option without reference counterpart (vertexColor mode only):
 * also propagate the change of the interpolated vertex colour through the
 * barycentrics into vertex_pos_grad.  The reference leaves this term out
 * (CUDABasedRasterizationGrad.cu:489), so its position gradient is the
 * loss's derivative only for constant colours; fitting with per-vertex
 * colours needs the term.  Ignored in the other modes. */
#define GVR_BACKWARD_ALBEDO_POSITION 1

/* Builds the device topology and vertex->face adjacency in O(F)
 * (replaces the O(N*F) getVertexFaces, CUDABasedRasterization.cpp:125-154).
 * Uses the current CUDA device. */
int gvr_create(const GvrTopology *topology, const GvrAttrs *attrs, GvrHandle **out_handle);

/* Frees everything the handle owns (and nothing else). NULL is a no-op. */
void gvr_destroy(GvrHandle *handle);

/* Forward render of all B x C views (CUDABasedRasterization.cu:449-473). */
int gvr_forward(GvrHandle *handle, const GvrForwardArgs *args, void *stream);

/* Gradients (CUDABasedRasterizationGrad.cu:624-635).  For albedo modes
 * normal/lighting it writes zeros, as python/CudaRenderer.py:207-213 returns. */
int gvr_backward(GvrHandle *handle, const GvrBackwardArgs *args, void *stream);

/* Device scratch a call needs for the given batch and texture size. */
size_t gvr_forward_workspace_size(const GvrHandle *handle, int32_t batch, int32_t texture_height,
                                  int32_t texture_width);
size_t gvr_backward_workspace_size(const GvrHandle *handle, int32_t batch, int32_t texture_height,
                                   int32_t texture_width);

/* Message of the calling thread's last failed call ("" if none). */
const char *gvr_last_error(void);

/* GVR_ABI_VERSION of the loaded library. */
int gvr_abi_version(void);

/* Test hook with no reference counterpart: the per-pixel FP32 ray directions
 * [B,C,H,W,3] exactly as the raster and backward kernels compute them
 * (getRayCuda2, cpp/src/Utils/CameraUtil.h:251-257). */
int gvr_debug_rays(GvrHandle *handle, int32_t batch, const float *extrinsics, const float *intrinsics,
                   float *rays_out, void *stream);

/* Backward pass that allocates nothing; it has no counterpart in the reference.
 *
 * For callers that must not allocate device memory while rendering: a host
 * that hands this library a fixed memory budget up front (an engine or
 * plugin host whose allocator owns the GPU), or code on a real-time path
 * where a cudaMalloc would synchronise the device and stall the frame.
 * The caller still passes every input and output buffer; the scratch the
 * backward needs (per-face gradient accumulators, SH partial sums, camera and
 * face records) lives in one device array of GVR_NOALLOC_SCRATCH_BYTES that
 * the library reserves on each GPU it is loaded on, for the life of the
 * process.  Calls needing more scratch than that (about 22 MiB for one batch
 * element of 8 views at 1024x1024 and 70,000 faces) return
 * GVR_ERR_WORKSPACE (the normal, lighting and UV modes need no scratch and
 * take any size).  Each call looks up the array's device address
 * (cudaGetSymbolAddress) with the handle's device current; the first call on
 * a device also loads the library's device code there, so make that first
 * call before any stream capture.  A device reset invalidates handles, not
 * this lookup.  Every call on a device shares the one array: calls that
 * overlap on the GPU (other streams, other threads) race and corrupt each
 * other's results; everything that must start at zero is cleared inside
 * each call. */
#define GVR_NOALLOC_SCRATCH_BYTES (32u << 20)
int gvr_backward_noalloc(GvrHandle *handle, const GvrBackwardArgs *args, void *stream);

/* ---- Image helpers: gradientImageKernel and gaussianImageKernel of the
 * reference (cpp/src/Renderer/gradientImage.cu:8-55, host entry
 * gradientImage :57-67), over a batch of float RGB images [B, H, W, 3].
 * Gradient: 1/8-scaled 3x3 Sobel in x and y, zero where x < 1, y < 1,
 * x >= W - 2 or y >= H - 2.  Blur: 3x3 binomial (1 2 1)^2 / 16; the border
 * ring (x < 1, y < 1, x > W - 2, y > H - 2) of `out` is not written.  The
 * reference writes past the image when W or H is not a multiple of 16;
 * these never do.  Asynchronous on `stream`. */
int gvr_image_gradient(const float *image, float *grad_x, float *grad_y, int32_t batch, int32_t width,
                       int32_t height, void *stream);
int gvr_image_gaussian3x3(const float *image, float *out, int32_t batch, int32_t width, int32_t height, void *stream);

/* ---- Batched forward of many meshes (no reference counterpart: the
 * reference renders one mesh per op call and loops over the batch on the
 * host, CudaRenderer.cpp:309).
 *
 * A plan binds a list of forward jobs -- each a handle (mesh topology,
 * views, resolution, modes) with one call's device buffers -- once, and
 * renders all of them with one launch per pipeline stage over every job,
 * then the raster: by default each job's raster kernel on one of
 * GVR_PLAN_LANES streams forked from and joined to the caller's stream
 * (largest jobs first; under graph capture they become parallel branches),
 * or, with GVR_PLAN_PERSISTENT, one persistent raster kernel that pulls
 * (job, view, tile) items from a shared counter.  Meshes of very different
 * sizes share the GPU either way.  Every job's outputs are bit-identical to gvr_forward
 * on the same buffers.  The plan owns all scratch (allocated at create);
 * gvr_plan_forward allocates nothing and never synchronises the host, and
 * gvr_plan_forward_graph captures it once into a CUDA graph and replays
 * that graph on later calls.  The buffers named in the jobs must stay valid
 * for the life of the plan; their contents may change between calls.
 * Handles with compute_normal_map are refused (GVR_ERR_UNSUPPORTED). */
typedef struct GvrPlan GvrPlan;

typedef struct {
    GvrHandle *handle;
    GvrForwardArgs forward;  /* workspace fields ignored */
    int32_t tile_width;      /* 8, 16 or 32 (tile height = 256 / width), or 0: chosen by the plan */
    int32_t big_tiles;       /* 1..16: faces spanning more tiles go to the view's big-face list; 0: chosen */
} GvrJob;

/* For jobs that leave the choice to the plan: with GVR_PLAN_AUTOTUNE the
 * plan picks, per (floor(log2 F), W, H) bucket, the fastest tile shape
 * (16x16, 32x8, 8x32) and big-face threshold (4 or 16 tiles) by timing the
 * first job of the bucket (the choice is cached for the process); without
 * it they use 16x16 and 16. */
#define GVR_PLAN_AUTOTUNE 1
/* One persistent raster kernel over every job instead of a raster kernel per
 * job on parallel lanes (the same outputs; the lanes measured faster). */
#define GVR_PLAN_PERSISTENT 2
#define GVR_PLAN_LANES 16

int gvr_plan_create(const GvrJob *jobs, int32_t count, int32_t flags, GvrPlan **out_plan);
int gvr_plan_forward(GvrPlan *plan, void *stream);
/* `stream` must be a created stream (graph capture cannot use the legacy default stream). */
int gvr_plan_forward_graph(GvrPlan *plan, void *stream);
/* The bin/tile configuration chosen for job `job`. */
int gvr_plan_tile_config(const GvrPlan *plan, int32_t job, int32_t *tile_w, int32_t *tile_h, int32_t *big_tiles);

/* Batched backward of the same jobs (no reference counterpart: the reference
 * runs its grad op once per batch element in a host loop,
 * cpp/src/TensorflowOperators/CudaRenderer/CudaRendererGrad.cpp:259-285).
 * gvr_plan_bind_backward binds one backward call per job of the plan, in
 * the plan's job order (`count` = the plan's job count; the arguments mean
 * what they mean for gvr_backward, workspace fields ignored) and allocates
 * every job's scratch; binding again replaces the earlier binding.
 * gvr_plan_backward then computes every job's gradients with one clearing
 * launch, one launch per stage over all jobs (cameras, face records, the
 * two vertex gathers, the SH sums) and one pixel-kernel launch per kernel
 * variant present among the jobs (albedo class x shaded x target gradient),
 * allocating nothing and never synchronising the host;
 * gvr_plan_backward_graph captures that sequence once into a CUDA graph and
 * replays it.  Each job's gradients equal gvr_backward's on the same
 * buffers up to the order of the FP32 atomic sums (SH gradients bit for
 * bit).  The bound buffers must stay valid for the life of the binding. */
int gvr_plan_bind_backward(GvrPlan *plan, const GvrBackwardArgs *args, int32_t count);
int gvr_plan_backward(GvrPlan *plan, void *stream);
/* `stream` must be a created stream (graph capture cannot use the legacy default stream). */
int gvr_plan_backward_graph(GvrPlan *plan, void *stream);
void gvr_plan_destroy(GvrPlan *plan);

/* Per-kernel timing, no reference counterpart.  While enabled, every kernel
 * the library launches is bracketed by a CUDA event pair on its stream;
 * gvr_profile_read waits for those events and reports, per kernel name, the
 * launches and summed milliseconds since the last gvr_profile_enable call. */
typedef struct {
    char name[48];
    long long launches;
    double total_ms;
} GvrKernelTime;

/* Turns timing on (1) or off (0), clears the tallies; returns the previous state. */
int gvr_profile_enable(int enable);

/* Fills up to `capacity` entries; returns the number of distinct kernels timed. */
int gvr_profile_read(GvrKernelTime *out, int capacity);

/* Kernels launched by this library since it was loaded (profiling on or off). */
long long gvr_launch_count(void);

/* Measurement of the L2's reduction rate, no reference counterpart: `grid`
 * blocks of 256 threads each issue `rounds` fire-and-forget FP32 additions
 * (vector4 = 0: one float; 1: one 16-byte float4, as the backward's per-face
 * accumulators take them) to pseudo-random 32-byte sectors of `buf`
 * (`words` floats, a multiple of 8), one sector per addition, so that every
 * addition is one L2 reduction request.  Returns GVR_OK or an error code. */
int gvr_probe_reductions(float *buf, long long words, int vector4, int rounds, int grid, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GVR_H */

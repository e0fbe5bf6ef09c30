// gvr_internal.cuh -- shared device code of the GB300 rasteriser.
//
// Two arithmetic regimes:
//  * "x" functions evaluate the reference's FP32 expression sequence with one
//    IEEE round-to-nearest operation per C operator (__fmul_rn/__fadd_rn/
//    __fsub_rn/__fdiv_rn/__fsqrt_rn never contract into FMA).  Everything that
//    decides a discrete outcome goes through them: vertex projection and face
//    boxes, the per-pixel ray, the ray/triangle test, barycentrics, quantised
//    depth, vertex normals, the normal flip and the nearest-texel pick.  The
//    result is bit-identical to the reference kernels built with -fmad=false.
//  * Continuous values (shading, gradients) use ordinary FP32 with FMA.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gvr.h"

namespace gvr {

constexpr int kTile = 16;                   // raster/backward tile edge in pixels
constexpr int kTilePix = kTile * kTile;     // one thread per tile pixel
constexpr int kBigTiles = 16;               // faces spanning more tiles use the per-view big list
constexpr unsigned long long kEmptyKey = ~0ull;
constexpr int kFaceAccFloats = 32;          // per-face gradient accumulator (see backward)

// ---------------------------------------------------------------------------- exact FP32

struct V3 {
    float x, y, z;
};

__device__ __forceinline__ float xm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float xd(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 xsub(V3 a, V3 b) { return v3(xs(a.x, b.x), xs(a.y, b.y), xs(a.z, b.z)); }
__device__ __forceinline__ float xdot(V3 a, V3 b) { return xa(xa(xm(a.x, b.x), xm(a.y, b.y)), xm(a.z, b.z)); }
__device__ __forceinline__ V3 xcross(V3 a, V3 b) {
    return v3(xs(xm(a.y, b.z), xm(a.z, b.y)), xs(xm(a.z, b.x), xm(a.x, b.z)), xs(xm(a.x, b.y), xm(a.y, b.x)));
}
__device__ __forceinline__ V3 ld3(const float *p) { return v3(p[0], p[1], p[2]); }

// ---------------------------------------------------------------------------- per-call records

// Per (batch, view) camera record, written by the set-up launch (camera_item).
struct Camera {
    float invE[16];   // inverse extrinsics (cofactor inverse, FP32)
    float invP[16];   // inverse of K*E
    float orig[4];    // ray origin (camera centre), mm
    float origS[4];   // origin / 1000
    float KE[12];     // K*E (3x4), used by the target-image Jacobian
    float K[9];       // intrinsics
    float E[12];      // extrinsics
    float origLen;    // |orig|, mm (the skip tests' error scale)
    float pad[58];    // 128 floats = 512 B
};

// Per (batch, face) geometry in the reference's scaled units (/1000).
struct FaceGeo {
    float4 a;   // v0s.xyz, v1s.x
    float4 b;   // v1s.yz, v2s.xy
    float4 c;   // v2s.z, N.xyz
    float4 d;   // dot(v0s, N), dot(N, N), pad, pad
};

// Per (batch, view, face) screen record (64 bytes).
//
// Besides the reference's pixel box and vertex depths it carries screen-space
// barycentrics lam(p) = (1 - l1 - l2, l1, l2) with l_k = a_k (px - x0) + b_k (py - y0),
// used only to SKIP work that cannot change the result: a pixel whose
// screen barycentrics are below -mOut is certainly rejected by the exact
// test; one whose barycentrics are all >= mIn is certainly accepted (when
// kCertain is set).  The margins bound the FP32 error of the exact test
// (grows as 1/|cos| and 1/face size), the error of the screen projection,
// and the perspective factor between screen and world barycentrics
// (z_max/z_min); dRel bounds the relative error of depth_approx.
struct ViewFace {
    int4 hdr;     // box x (x0 | x1 << 16), box y (y0 | y1 << 16), flags, dRel (float bits)
    float4 z;     // projected camera-space depth of v0, v1, v2; w = mIn
    float4 s0;    // screen x0, y0 of vertex 0, mOut, zLowSafe (a lower bound of any accepted depth)
    float4 s1;    // a1, b1, a2, b2
};

constexpr int kScreenValid = 1;  // all z >= 1 mm, z_max/z_min <= 64, non-degenerate screen triangle
constexpr int kCertain = 2;      // screen-valid, |cos(view ray, normal)| >= 0.02, clear of the parallel-ray test

__device__ __forceinline__ int vf_flags(const ViewFace &vf) { return vf.hdr.z; }
__device__ __forceinline__ float vf_drel(const ViewFace &vf) { return __int_as_float(vf.hdr.w); }

// Inclusive pixel box; empty boxes are stored as x0 = 1, x1 = 0.
__device__ __forceinline__ int4 vf_box(const ViewFace &vf) {
    return make_int4(vf.hdr.x & 0xffff, vf.hdr.y & 0xffff, (unsigned)vf.hdr.x >> 16, (unsigned)vf.hdr.y >> 16);
}

// Screen barycentrics of pixel centre (px, py).
__device__ __forceinline__ void screen_lambda(const ViewFace &vf, float px, float py, float &l0, float &l1, float &l2) {
    const float dx = px - vf.s0.x, dy = py - vf.s0.y;
    l1 = vf.s1.x * dx + vf.s1.y * dy;
    l2 = vf.s1.z * dx + vf.s1.w * dy;
    l0 = 1.0f - l1 - l2;
}

// Approximation of the reference's quantised depth 1e4 / sum(b_i / z_i) with
// world barycentrics b_i = (l_i / z_i) / sum(l_j / z_j): 1e4 * S / T with
// S = sum l_i / z_i, T = sum l_i / z_i^2.
__device__ __forceinline__ float depth_approx(const ViewFace &vf, float l0, float l1, float l2) {
    const float r0 = 1.0f / vf.z.x, r1 = 1.0f / vf.z.y, r2 = 1.0f / vf.z.z;
    const float S = l0 * r0 + l1 * r1 + l2 * r2;
    const float T = l0 * r0 * r0 + l1 * r1 * r1 + l2 * r2 * r2;
    return 10000.0f * __fdividef(S, T);
}

struct FaceSetup {
    V3 v0, v1, v2, n;
    float v0dn, denom;
};

__device__ __forceinline__ FaceSetup load_face(const FaceGeo *g) {
    float4 a = g->a, b = g->b, c = g->c, d = g->d;
    FaceSetup s;
    s.v0 = v3(a.x, a.y, a.z);
    s.v1 = v3(a.w, b.x, b.y);
    s.v2 = v3(b.z, b.w, c.x);
    s.n = v3(c.y, c.z, c.w);
    s.v0dn = d.x;
    s.denom = d.y;
    return s;
}

// ---------------------------------------------------------------------------- reference arithmetic

// Per-pixel ray direction: getRayCuda2 (cpp/src/Utils/CameraUtil.h:251-257)
// = normalize(backprojectPixelCuda((u+.5, v+.5, 1000)) - origin) with the
// device rsqrtf of normalize (cutil_math.h:1184-1188).
__device__ __forceinline__ V3 pixel_ray(const Camera &cam, int u, int v) {
    const float *P = cam.invP;
    float tx = xm(u + 0.5f, 1000.0f), ty = xm(v + 0.5f, 1000.0f), tz = 1000.0f;
    float bx = xa(xa(xa(xm(P[0], tx), xm(P[1], ty)), xm(P[2], tz)), xm(P[3], 1.0f));
    float by = xa(xa(xa(xm(P[4], tx), xm(P[5], ty)), xm(P[6], tz)), xm(P[7], 1.0f));
    float bz = xa(xa(xa(xm(P[8], tx), xm(P[9], ty)), xm(P[10], tz)), xm(P[11], 1.0f));
    V3 w = v3(xs(bx, cam.orig[0]), xs(by, cam.orig[1]), xs(bz, cam.orig[2]));
    float inv = rsqrtf(xdot(w, w));
    return v3(xm(w.x, inv), xm(w.y, inv), xm(w.z, inv));
}

// rayTriangleIntersect + uv2barycentric (cpp/src/Utils/RendererUtil.h:26-128)
// with the per-face terms precomputed (same values, same order).
// odn = dot(origin/1000, N).  Returns (a, b, c) or (-1, -1, -1).
__device__ __forceinline__ V3 barycentric(const FaceSetup &f, V3 origS, float odn, V3 d) {
    const V3 fail = v3(-1.0f, -1.0f, -1.0f);
    float nd = xdot(d, f.n);
    if (fabsf(nd) < 0.0000001f) return fail;
    float t = xd(xs(f.v0dn, odn), nd);
    if (t < 0.0f) return fail;
    V3 P = v3(xa(origS.x, xm(t, d.x)), xa(origS.y, xm(t, d.y)), xa(origS.z, xm(t, d.z)));
    if (xdot(f.n, xcross(xsub(f.v1, f.v0), xsub(P, f.v0))) < 0.0f) return fail;
    float a = xdot(f.n, xcross(xsub(f.v2, f.v1), xsub(P, f.v1)));
    if (a < 0.0f) return fail;
    float b = xdot(f.n, xcross(xsub(f.v0, f.v2), xsub(P, f.v2)));
    if (b < 0.0f) return fail;
    a = xd(a, f.denom);
    b = xd(b, f.denom);
    return v3(a, b, xs(xs(1.0f, a), b));
}

// isInsideTriangle (cpp/src/Renderer/CUDABasedRasterization.cu:243).
__device__ __forceinline__ bool inside(V3 abc) {
    return abc.x >= -0.001f && abc.y >= -0.001f && abc.z >= -0.001f && abc.x <= 1.001f && abc.y <= 1.001f &&
           abc.z <= 1.001f;
}

// Quantised perspective-correct depth (CUDABasedRasterization.cu:247-250);
// float->int is round-toward-zero and saturating, as the reference's
// implicit conversion in atomicMin(int*, float).
__device__ __forceinline__ int depth_quantised(V3 abc, float z0, float z1, float z2) {
    float z = xd(1.0f, xa(xa(xd(abc.x, z0), xd(abc.y, z1)), xd(abc.z, z2)));
    return __float2int_rz(xm(z, 10000.0f));
}

// Depth|face key: smaller depth wins, then smaller face id.
__device__ __forceinline__ unsigned long long depth_key(int depth, int face) {
    return ((unsigned long long)((unsigned)depth ^ 0x80000000u) << 32) | (unsigned)face;
}

// Pixel normal (un-normalised, FP32 exact) and flip decision
// (CUDABasedRasterization.cu:308-319, CUDABasedRasterizationGrad.cu:231-240).
__device__ __forceinline__ V3 pixel_normal_un(V3 n0, V3 n1, V3 n2, V3 abc) {
    return v3(xa(xa(xm(n0.x, abc.x), xm(n1.x, abc.y)), xm(n2.x, abc.z)),
              xa(xa(xm(n0.y, abc.x), xm(n1.y, abc.y)), xm(n2.y, abc.z)),
              xa(xa(xm(n0.z, abc.x), xm(n1.z, abc.y)), xm(n2.z, abc.z)));
}

// Unit pixel normal n = un / len and the reference's flip decision
// (n . d > 0 with n's components the IEEE quotients un_i / len,
// CUDABasedRasterization.cu:308-319).  n is formed with one correctly
// rounded reciprocal and three products, within 1 ulp of the quotients per
// component, which moves n . d by less than 1e-6; when |n . d| is below
// that, the decision is taken on the exact quotients, so it is always the
// reference's.  Returns n, flipped when `flipped`.
__device__ __forceinline__ V3 unit_normal(V3 un, float len, V3 d, bool &flipped) {
    const float inv = __frcp_rn(len);
    const V3 n = v3(__fmul_rn(un.x, inv), __fmul_rn(un.y, inv), __fmul_rn(un.z, inv));
    float nd = xdot(n, d);
    if (fabsf(nd) < 1e-6f) nd = xdot(v3(xd(un.x, len), xd(un.y, len), xd(un.z, len)), d);
    flipped = nd > 0.0f;
    return flipped ? v3(-n.x, -n.y, -n.z) : n;
}

// Nearest-texel texture coordinate (CUDABasedRasterization.cu:326-345):
// returns the clamped (U0, V0) in texels.
__device__ __forceinline__ float2 texel_coord6(float u0, float v0, float u1, float v1, float u2, float v2, V3 abc,
                                              int Wt, int Ht) {
    float t0x = u0, t0y = xs(1.0f, v0);
    float t1x = u1, t1y = xs(1.0f, v1);
    float t2x = u2, t2y = xs(1.0f, v2);
    float fx = xa(xa(xm(t0x, abc.x), xm(t1x, abc.y)), xm(t2x, abc.z));
    float fy = xa(xa(xm(t0y, abc.x), xm(t1y, abc.y)), xm(t2y, abc.z));
    fx = xm(fx, (float)Wt);
    fy = xm(fy, (float)Ht);
    fx = fminf(fmaxf(fx, 0.0f), (float)(Wt - 1));
    fy = fminf(fmaxf(fy, 0.0f), (float)(Ht - 1));
    return make_float2(fx, fy);
}

__device__ __forceinline__ float2 texel_coord(const float *uv6, V3 abc, int Wt, int Ht) {
    return texel_coord6(uv6[0], uv6[1], uv6[2], uv6[3], uv6[4], uv6[5], abc, Wt, Ht);
}

// SH irradiance per channel (getIllum, cpp/src/Utils/RendererUtil.h:179-214).
__device__ __forceinline__ void sh_basis(V3 n, float basis[9]) {
    basis[0] = 1.0f;
    basis[1] = n.y;
    basis[2] = n.z;
    basis[3] = n.x;
    basis[4] = n.x * n.y;
    basis[5] = n.z * n.y;
    basis[6] = 3.0f * n.z * n.z - 1.0f;
    basis[7] = n.x * n.z;
    basis[8] = n.x * n.x - n.y * n.y;
}

// ---------------------------------------------------------------------------- modes without reference counterpart

// Headlight Phong (GVR_SHADING_PHONG): colour = albedo * phong_factor + phong_specular,
// with ndl = n . l for l the unit direction to the camera.
constexpr float kPhongAmbient = 0.2f, kPhongDiffuse = 0.7f, kPhongSpecular = 0.3f;
__device__ __forceinline__ float phong_factor(float ndl) { return kPhongAmbient + kPhongDiffuse * fmaxf(ndl, 0.0f); }
__device__ __forceinline__ float phong_specular(float ndl) {
    float r = fmaxf(2.0f * ndl * ndl - 1.0f, 0.0f);  // (r . v) for the mirror direction r of l about n, v = l
    r *= r;
    r *= r;
    r *= r;
    r *= r;  // ^16
    return kPhongSpecular * r;
}

// Bilinear lookup (GVR_ALBEDO_TEXTURED_BILINEAR) at the clamped texture
// coordinate (U0, V0) of texel_coord: texel centres at integer + 0.5,
// neighbour indices clamped to the texture.  idx: texel offsets (in texels)
// of the four corners, w: their weights.
__device__ __forceinline__ void bilinear_taps(float U0, float V0, int Wt, int Ht, int idx[4], float w[4]) {
    const float x = U0 - 0.5f, y = V0 - 0.5f;
    const float x0 = floorf(x), y0 = floorf(y);
    const float fx = x - x0, fy = y - y0;
    const int ix0 = min(max((int)x0, 0), Wt - 1), ix1 = min(max((int)x0 + 1, 0), Wt - 1);
    const int iy0 = min(max((int)y0, 0), Ht - 1), iy1 = min(max((int)y0 + 1, 0), Ht - 1);
    idx[0] = iy0 * Wt + ix0;
    idx[1] = iy0 * Wt + ix1;
    idx[2] = iy1 * Wt + ix0;
    idx[3] = iy1 * Wt + ix1;
    w[0] = (1.0f - fx) * (1.0f - fy);
    w[1] = fx * (1.0f - fy);
    w[2] = (1.0f - fx) * fy;
    w[3] = fx * fy;
}

// ---------------------------------------------------------------------------- error-free FP32

// s + e == a + b exactly (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Compensated dot product (Ogita, Rump & Oishi's Dot2): as accurate as if
// computed in twice the working precision, then rounded.
template <int K>
__device__ __forceinline__ float dot2(const float (&x)[K], const float (&y)[K]) {
    float p = __fmul_rn(x[0], y[0]);
    float s = __fmaf_rn(x[0], y[0], -p);
#pragma unroll
    for (int i = 1; i < K; ++i) {
        const float h = __fmul_rn(x[i], y[i]);
        const float r = __fmaf_rn(x[i], y[i], -h);
        float q;
        two_sum(p, h, p, q);
        s = __fadd_rn(s, __fadd_rn(q, r));
    }
    return __fadd_rn(p, s);
}

// First statement of a kernel launched by launch_pdl: lets the next kernel
// on the stream be launched now (its blocks wait in their own pdl_enter),
// then waits until the previous kernel has completed and its memory writes
// are visible.  Without a programmatic predecessor both return at once.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// The job owning block `blk` of a batched launch: the last j with blockStart[j] <= blk.
__device__ __forceinline__ int job_of_block(const int *__restrict__ blockStart, int nJobs, int blk) {
    int lo = 0, hi = nJobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (blockStart[mid] <= blk) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------------------------- launch params

struct Topology {
    const int32_t *faces;   // [F*3]
    const float *uvs;       // [F*6]
    const int32_t *vstart;  // [N+1]
    const int32_t *vfaces;  // [nnz] faces around each vertex, ascending
    const int4 *vcsr;       // [nnz] the same faces as (i0, i1, i2, f): a gather reads the face's
                            // vertex ids (and so its corners at the vertex) with its id in one load
    int N, F;
};

// Per-call frame description.  The forward bins faces into tiles of
// tileW x tileH = 256 pixels (tileW in {8, 16, 32}; default 16 x 16) and
// sends faces spanning more than bigTiles tiles to a per-view list that
// every tile scans; tilesX/tilesY count those tiles.  The backward always
// works on 16 x 16 tiles.
struct FrameDims {
    int B, C, W, H, tilesX, tilesY, Ht, Wt;
    int albedo, shading;
    int tileW, tileH, tileShift, bigTiles;  // tileShift = log2(tileW)
};

// Forward scratch carved out of one workspace.
// Per (batch, face) record of what the forward's shading reads about a
// face, five 16-byte rows instead of 18 dependent scalar gathers:
//   r0 = N0.xyz, N1.x;  r1 = N1.yz, N2.xy;  r2 = N2.z, u0, v0, u1;
//   r3 = v1, u2, v2, 0;  r4 = i0, i1, i2 (int bits), 0
// (N: the un-normalised vertex normals of view 0, bit-identical to the
// vertex_normal output of every view; u, v: texture coordinates as stored).
constexpr int kShadeRows = 5;

struct FwdScratch {
    Camera *cams;        // [B*C]
    FaceGeo *geo;        // [B*F]
    float4 *fnormal;     // [B*F] un-normalised face normals; w = their length
    float4 *faceC;       // [B*F] centroid (mm) and smallest altitude (mm) of each face
    float4 *shadeRec;    // [B*F*kShadeRows], written by the binning pass
    ViewFace *vface;     // [B*C*F]
    int *tileCount;      // [B*C*T]
    int *tileStart;      // [B*C*T + 1]
    int *tileCursor;     // [B*C*T]
    int *bins;           // [kBigTiles*B*C*F]
    int *bigList;        // [B*C*F]
    int *bigCount;       // [B*C]
    unsigned *zRange;    // [B*C*2] per view: max of ~bits(zLowSafe) (= ~min) and max of bits(zLowSafe)
                         // over its faces with a finite, non-negative bound; 0 = none
    size_t zeroBytes;    // bytes from tileCount to clear per call (counts, cursors, big counts)
    void *zeroBase;
};

// Inputs/outputs of the raster + resolve kernel.
struct RasterIO {
    const float *verts;      // [B,N,3]
    const float *colors;     // [B,N,3]
    const float *texture;    // [B,Ht,Wt,3]
    const float *sh;         // [B,C,27]
    const float *vnormal;    // [B,C,N,3] (written by the vertex stage)
    float *bary;             // [B,C,H,W,2]
    int32_t *face;           // [B,C,H,W]
    float *render;           // [B,C,H,W,3]
};

// One forward job: one handle's topology and one call's frame, scratch and
// buffers.  The single-mesh kernels take it by value; the batched kernels
// read an array of them from device memory.
struct FwdJob {
    Topology topo;
    FrameDims dims;
    FwdScratch ws;
    RasterIO io;
    const float *extr;   // [B,C,12]
    const float *intr;   // [B,C,9]
    float4 *proj;        // [B*C*N] projected vertices
    float *vnormal_out;  // [B,C,N,3] (the buffer io.vnormal reads)
};

// Per (batch, face) record of what the backward's pixels read about their
// face, five 16-byte rows instead of 18 scalar gathers:
//   r0 = i0, i1, i2 (int bits), u0;  r1 = v0, u1, v1, u2;  r2 = v2, V0.xyz;
//   r3 = V1.xyz, V2.x;  r4 = V2.yz, 0, 0   (u, v: texture coordinates as
// stored; V: vertex positions, mm).
constexpr int kBwdFaceRows = 5;

struct BwdScratch {
    Camera *cams;        // [B*C]
    FaceGeo *geo;        // [B*F]
    float4 *faceRec;     // [B*F*kBwdFaceRows]
    float4 *faceAcc;     // [B*F*kFaceAccFloats/4]
    float4 *gN;          // [B*N] normal-gradient accumulator per vertex
    float *shPartial;    // [B*C][27][T] per-tile SH partial sums
};

// Inputs and outputs of the backward's pixel kernel.
struct BwdIO {
    const float *grad_render;  // [B,C,H,W,3]
    const float *verts;        // [B,N,3]
    const float *colors;       // [B,N,3]
    const float *texture;      // [B,Ht,Wt,3]
    const float *sh;           // [B,C,27]
    const float *target;       // [B,C,H,W,3]
    const float *vnormal;      // [B,C,N,3]
    const float *bary_in;      // [B,C,H,W,2] or null
    const int32_t *face;       // [B,C,H,W]
    const float *grad_target;  // [B,C,H,W,3] or null
    float *tex_grad;           // [B,Ht,Wt,3]
    int imageFilter;
    int phong;                 // GVR_SHADING_PHONG: albedo scaled by the headlight term, no SH
};

// One backward job of a batched plan: one handle's topology and one call's
// frame, scratch and buffers.  The batched kernels read an array of them
// from device memory.
struct BwdJob {
    Topology topo;
    FrameDims dims;        // 16 x 16 tiles
    BwdScratch ws;
    BwdIO io;
    const float *extr;     // [B,C,12]
    const float *intr;     // [B,C,9]
    float *vpos_grad;      // [B,N,3]
    float *vcol_grad;      // [B,N,3]
    float *sh_grad;        // [B,C,27]
    int zeroMode;          // normal / lighting / UV: the outputs are only cleared
    int shaded;            // SH terms and the normal-adjacency gather
    int useCol;            // vertex colours receive a gradient
};

}  // namespace gvr

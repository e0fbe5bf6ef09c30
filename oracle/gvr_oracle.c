/*
 * gvr_oracle.c -- CPU restatement of the reference renderer's forward and
 * backward kernels.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke
 * check and the CPU-baseline leg of bench.py call it as the checker.  The
 * product path never links or calls it.
 *
 * What it restates (reference paths relative to the reference project root):
 *   cpp/src/Renderer/CUDABasedRasterization.cu      forward kernels  :23-408
 *   cpp/src/Renderer/CUDABasedRasterizationGrad.cu  backward kernel  :114-617
 *   cpp/src/Utils/RendererUtil.h                    per-pixel math   :26-914
 *   cpp/src/Utils/CameraUtil.h                      camera math      :141-257
 *   cpp/src/Utils/float4x4.h                        cofactor inverse :78-101,160-282
 *   cpp/src/Renderer/CUDABasedRasterization.cpp     vertex->face CSR :125-154
 *
 * Two arithmetic regimes:
 *   - Every DISCRETE decision (pixel coverage, the quantised depth compare,
 *     the barycentric output, vertex normals, the normal flip, the texel
 *     picked by the nearest lookup) is evaluated in FP32 in exactly the
 *     reference's operation order.  This file must be compiled with
 *     -ffp-contract=off and without -ffast-math so each C float operation is
 *     one IEEE round-to-nearest operation, like device code built with
 *     -fmad=false.  The one operation that cannot be restated bit-exactly on
 *     a CPU is the device rsqrtf inside normalize() (cutil_math.h:1184-1188);
 *     the oracle uses 1.0f/sqrtf (the reference's own host definition,
 *     cutil_math.h:58-61) unless the caller passes the per-pixel ray
 *     directions produced on the device (orc_scene.rays).
 *   - Every CONTINUOUS value (shaded colours, all gradients) is evaluated in
 *     FP64 from those FP32 decisions.
 *
 * Ties: the reference resolves equal quantised depths by a write race
 * (CUDABasedRasterization.cu:295-301).  The oracle reports the minimal face id
 * among the faces with minimal quantised depth and the size of that tie set,
 * plus up to ORC_MAX_TIES of its members.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_TIES 4

enum { ORC_VERTEX_COLOR = 0, ORC_TEXTURED = 1, ORC_NORMAL = 2, ORC_LIGHTING = 3, ORC_FOREGROUND = 4,
       ORC_TEXTURED_BILINEAR = 5, ORC_UV = 6 };
enum { ORC_SHADED = 0, ORC_SHADELESS = 1, ORC_PHONG = 2 };

typedef struct {
    int N, F, C, W, H, Ht, Wt;
    int albedo_mode, shading_mode, image_filter_size;
    const int32_t *faces;   /* [F*3]                 */
    const float *uvs;       /* [F*6] per-corner (u,v) */
    const float *verts;     /* [N*3] world, mm        */
    const float *colors;    /* [N*3]                  */
    const float *texture;   /* [Ht*Wt*3]              */
    const float *sh;        /* [C*27]                 */
    const float *extr;      /* [C*12] world->camera   */
    const float *intr;      /* [C*9]                  */
    const float *rays;      /* optional [C*H*W*3] ray directions; NULL = 1/sqrtf */
} orc_scene;

/* ------------------------------------------------------------------------- */
/* FP32 helpers: one IEEE operation per C operator (compile with contraction off) */

typedef struct { float x, y, z; } f3;
static inline f3 mk3(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline f3 sub3(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline f3 add3(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline f3 smul3(float s, f3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
static inline f3 sdiv3(f3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
static inline float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline f3 cross3(f3 a, f3 b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline f3 ld3(const float *p) { return mk3(p[0], p[1], p[2]); }

/* Device float->int conversion semantics (round toward zero, saturate, NaN->0). */
static inline int f2i_rz(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT_MAX;
    if (x <= -2147483648.0f) return INT_MIN;
    return (int)x;
}

/* FP64 helpers */
typedef struct { double x, y, z; } d3;
static inline d3 dk3(double x, double y, double z) { d3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline d3 dsub(d3 a, d3 b) { return dk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline d3 dadd(d3 a, d3 b) { return dk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline d3 dscale(double s, d3 a) { return dk3(s * a.x, s * a.y, s * a.z); }
static inline double ddot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline d3 dcross(d3 a, d3 b) {
    return dk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline d3 dnormalize(d3 a) { double l = sqrt(ddot(a, a)); return dk3(a.x / l, a.y / l, a.z / l); }
static inline d3 f2d(f3 a) { return dk3(a.x, a.y, a.z); }
static inline d3 ldd3(const float *p) { return dk3(p[0], p[1], p[2]); }

/* ------------------------------------------------------------------------- */
/* Cameras: CUDABasedRasterization.cu:23-67 with float4x4 product (:78-101)
 * and the cofactor inverse getInverse (float4x4.h:160-282).  Matrices are
 * row-major 4x4 as float4x4::entries. */

static void mat4_mul(const float *a, const float *b, float *r) {
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            r[4 * i + j] = a[4 * i + 0] * b[0 * 4 + j] + a[4 * i + 1] * b[1 * 4 + j] +
                           a[4 * i + 2] * b[2 * 4 + j] + a[4 * i + 3] * b[3 * 4 + j];
}

static void mat4_inverse(const float *e, float *out) {
    float inv[16];
    inv[0] = e[5] * e[10] * e[15] - e[5] * e[11] * e[14] - e[9] * e[6] * e[15] + e[9] * e[7] * e[14] +
             e[13] * e[6] * e[11] - e[13] * e[7] * e[10];
    inv[4] = -e[4] * e[10] * e[15] + e[4] * e[11] * e[14] + e[8] * e[6] * e[15] - e[8] * e[7] * e[14] -
             e[12] * e[6] * e[11] + e[12] * e[7] * e[10];
    inv[8] = e[4] * e[9] * e[15] - e[4] * e[11] * e[13] - e[8] * e[5] * e[15] + e[8] * e[7] * e[13] +
             e[12] * e[5] * e[11] - e[12] * e[7] * e[9];
    inv[12] = -e[4] * e[9] * e[14] + e[4] * e[10] * e[13] + e[8] * e[5] * e[14] - e[8] * e[6] * e[13] -
              e[12] * e[5] * e[10] + e[12] * e[6] * e[9];
    inv[1] = -e[1] * e[10] * e[15] + e[1] * e[11] * e[14] + e[9] * e[2] * e[15] - e[9] * e[3] * e[14] -
             e[13] * e[2] * e[11] + e[13] * e[3] * e[10];
    inv[5] = e[0] * e[10] * e[15] - e[0] * e[11] * e[14] - e[8] * e[2] * e[15] + e[8] * e[3] * e[14] +
             e[12] * e[2] * e[11] - e[12] * e[3] * e[10];
    inv[9] = -e[0] * e[9] * e[15] + e[0] * e[11] * e[13] + e[8] * e[1] * e[15] - e[8] * e[3] * e[13] -
             e[12] * e[1] * e[11] + e[12] * e[3] * e[9];
    inv[13] = e[0] * e[9] * e[14] - e[0] * e[10] * e[13] - e[8] * e[1] * e[14] + e[8] * e[2] * e[13] +
              e[12] * e[1] * e[10] - e[12] * e[2] * e[9];
    inv[2] = e[1] * e[6] * e[15] - e[1] * e[7] * e[14] - e[5] * e[2] * e[15] + e[5] * e[3] * e[14] +
             e[13] * e[2] * e[7] - e[13] * e[3] * e[6];
    inv[6] = -e[0] * e[6] * e[15] + e[0] * e[7] * e[14] + e[4] * e[2] * e[15] - e[4] * e[3] * e[14] -
             e[12] * e[2] * e[7] + e[12] * e[3] * e[6];
    inv[10] = e[0] * e[5] * e[15] - e[0] * e[7] * e[13] - e[4] * e[1] * e[15] + e[4] * e[3] * e[13] +
              e[12] * e[1] * e[7] - e[12] * e[3] * e[5];
    inv[14] = -e[0] * e[5] * e[14] + e[0] * e[6] * e[13] + e[4] * e[1] * e[14] - e[4] * e[2] * e[13] -
              e[12] * e[1] * e[6] + e[12] * e[2] * e[5];
    inv[3] = -e[1] * e[6] * e[11] + e[1] * e[7] * e[10] + e[5] * e[2] * e[11] - e[5] * e[3] * e[10] -
             e[9] * e[2] * e[7] + e[9] * e[3] * e[6];
    inv[7] = e[0] * e[6] * e[11] - e[0] * e[7] * e[10] - e[4] * e[2] * e[11] + e[4] * e[3] * e[10] +
             e[8] * e[2] * e[7] - e[8] * e[3] * e[6];
    inv[11] = -e[0] * e[5] * e[11] + e[0] * e[7] * e[9] + e[4] * e[1] * e[11] - e[4] * e[3] * e[9] -
              e[8] * e[1] * e[7] + e[8] * e[3] * e[5];
    inv[15] = e[0] * e[5] * e[10] - e[0] * e[6] * e[9] - e[4] * e[1] * e[10] + e[4] * e[2] * e[9] +
              e[8] * e[1] * e[6] - e[8] * e[2] * e[5];
    float det = e[0] * inv[0] + e[1] * inv[4] + e[2] * inv[8] + e[3] * inv[12];
    float detr = 1.0f / det;
    for (int i = 0; i < 16; ++i) out[i] = inv[i] * detr;
}

/* invE[16], invP[16] for camera c (CUDABasedRasterization.cu:29-64). */
void orc_camera(const float *extr12, const float *intr9, float *invE, float *invP) {
    float K[16], E[16], KE[16];
    for (int i = 0; i < 16; ++i) { K[i] = (i % 5 == 0) ? 1.0f : 0.0f; E[i] = K[i]; }
    for (int row = 0; row < 3; ++row) {
        K[4 * row + 0] = intr9[3 * row + 0];
        K[4 * row + 1] = intr9[3 * row + 1];
        K[4 * row + 2] = intr9[3 * row + 2];
        K[4 * row + 3] = 0.0f;
        E[4 * row + 0] = extr12[4 * row + 0];
        E[4 * row + 1] = extr12[4 * row + 1];
        E[4 * row + 2] = extr12[4 * row + 2];
        E[4 * row + 3] = extr12[4 * row + 3];
    }
    mat4_inverse(E, invE);
    mat4_mul(K, E, KE);
    mat4_inverse(KE, invP);
}

/* getCamSpacePoint (CameraUtil.h:174-186) then projectPointFloat3 (:141-170). */
static f3 project_vertex(const float *extr12, const float *intr9, f3 p) {
    float cx = extr12[0] * p.x + extr12[1] * p.y + extr12[2] * p.z + extr12[3] * 1.0f;
    float cy = extr12[4] * p.x + extr12[5] * p.y + extr12[6] * p.z + extr12[7] * 1.0f;
    float cz = extr12[8] * p.x + extr12[9] * p.y + extr12[10] * p.z + extr12[11] * 1.0f;
    float x = cx * intr9[0] + cy * intr9[1] + cz * intr9[2];
    float y = cx * intr9[3] + cy * intr9[4] + cz * intr9[5];
    float z = cx * intr9[6] + cy * intr9[7] + cz * intr9[8];
    if (z > 0.0000001f) { x /= z; y /= z; }
    else { z = 0.00001f; x /= z; y /= z; }
    return mk3(x, y, z);
}

/* Camera origin: getRayCuda2 (CameraUtil.h:253-255). */
static f3 ray_origin(const float *invE) {
    float ox = invE[3], oy = invE[7], oz = invE[11], ow = invE[15];
    return mk3(ox / ow, oy / ow, oz / ow);
}

/* Un-normalised ray direction: backprojectPixelCuda (CameraUtil.h:223-236) minus the origin. */
static f3 ray_unnormalised(const float *invP, f3 ro, float px, float py) {
    float tx = px * 1000.0f, ty = py * 1000.0f, tz = 1000.0f;
    float bx = invP[0] * tx + invP[1] * ty + invP[2] * tz + invP[3] * 1.0f;
    float by = invP[4] * tx + invP[5] * ty + invP[6] * tz + invP[7] * 1.0f;
    float bz = invP[8] * tx + invP[9] * ty + invP[10] * tz + invP[11] * 1.0f;
    return sub3(mk3(bx, by, bz), ro);
}

static f3 ray_dir(const orc_scene *s, int c, const float *invP, f3 ro, int u, int v) {
    if (s->rays) return ld3(s->rays + (((size_t)c * s->H + v) * s->W + u) * 3);
    f3 w = ray_unnormalised(invP, ro, u + 0.5f, v + 0.5f);
    float invLen = 1.0f / sqrtf(dot3(w, w));
    return mk3(w.x * invLen, w.y * invLen, w.z * invLen);
}

/* rayTriangleIntersect (RendererUtil.h:26-101) + uv2barycentric (:108-128). */
static f3 barycentric(f3 orig, f3 dir, f3 v0, f3 v1, f3 v2) {
    v0 = sdiv3(v0, 1000.0f);
    v1 = sdiv3(v1, 1000.0f);
    v2 = sdiv3(v2, 1000.0f);
    orig = sdiv3(orig, 1000.0f);
    f3 N = cross3(sub3(v1, v0), sub3(v2, v0));
    float NdotRay = dot3(dir, N);
    f3 fail = mk3(-1.0f, -1.0f, -1.0f);
    if (fabsf(NdotRay) < 0.0000001f) return fail;
    float t = (dot3(v0, N) - dot3(orig, N)) / NdotRay;
    if (t < 0) return fail;
    f3 P = add3(orig, smul3(t, dir));
    f3 C = cross3(sub3(v1, v0), sub3(P, v0));
    if (dot3(N, C) < 0) return fail;
    C = cross3(sub3(v2, v1), sub3(P, v1));
    float a = dot3(N, C);
    if (a < 0) return fail;
    C = cross3(sub3(v0, v2), sub3(P, v2));
    float b = dot3(N, C);
    if (b < 0) return fail;
    float denom = dot3(N, N);
    a /= denom;
    b /= denom;
    return mk3(a, b, 1.0f - a - b);
}

static inline int inside_triangle(f3 abc) {
    return (abc.x >= -0.001f) && (abc.y >= -0.001f) && (abc.z >= -0.001f) && (abc.x <= 1.001f) &&
           (abc.y <= 1.001f) && (abc.z <= 1.001f);
}

/* Quantised depth (CUDABasedRasterization.cu:247-250). */
static inline int depth_int(f3 abc, float z0, float z1, float z2) {
    float z = 1.0f / (abc.x / z0 + abc.y / z1 + abc.z / z2);
    z *= 10000.0f;
    return f2i_rz(z);
}

/* ------------------------------------------------------------------------- */
/* Vertex->face adjacency, ascending face id, each face once per vertex
 * (CUDABasedRasterization.cpp:125-154), built in O(F). */

typedef struct { int *start; int *faces; } csr_t;

static void build_csr(int N, int F, const int32_t *faces, csr_t *csr) {
    int *count = (int *)calloc((size_t)N + 1, sizeof(int));
    for (int f = 0; f < F; ++f) {
        int a = faces[3 * f], b = faces[3 * f + 1], c = faces[3 * f + 2];
        count[a]++;
        if (b != a) count[b]++;
        if (c != a && c != b) count[c]++;
    }
    csr->start = (int *)malloc(((size_t)N + 1) * sizeof(int));
    csr->start[0] = 0;
    for (int v = 0; v < N; ++v) csr->start[v + 1] = csr->start[v] + count[v];
    csr->faces = (int *)malloc((size_t)csr->start[N] * sizeof(int) + 1);
    memset(count, 0, ((size_t)N + 1) * sizeof(int));
    for (int f = 0; f < F; ++f) {
        int a = faces[3 * f], b = faces[3 * f + 1], c = faces[3 * f + 2];
        csr->faces[csr->start[a] + count[a]++] = f;
        if (b != a) csr->faces[csr->start[b] + count[b]++] = f;
        if (c != a && c != b) csr->faces[csr->start[c] + count[c]++] = f;
    }
    free(count);
}

static void free_csr(csr_t *csr) { free(csr->start); free(csr->faces); }

/* Vertex normals (CUDABasedRasterization.cu:122-174): per-face cross product,
 * summed over the CSR in ascending face order; the same for every view.
 * Vertices without faces get 0 (the reference leaves them uninitialised). */
static void vertex_normals(const orc_scene *s, const csr_t *csr, float *vn /*[N*3]*/) {
    float *fn = (float *)malloc((size_t)s->F * 3 * sizeof(float));
    for (int f = 0; f < s->F; ++f) {
        f3 v0 = ld3(s->verts + 3 * s->faces[3 * f]);
        f3 v1 = ld3(s->verts + 3 * s->faces[3 * f + 1]);
        f3 v2 = ld3(s->verts + 3 * s->faces[3 * f + 2]);
        f3 n = cross3(sub3(v1, v0), sub3(v2, v0));
        fn[3 * f] = n.x; fn[3 * f + 1] = n.y; fn[3 * f + 2] = n.z;
    }
    for (int v = 0; v < s->N; ++v) {
        f3 acc = mk3(0.0f, 0.0f, 0.0f);
        for (int i = csr->start[v]; i < csr->start[v + 1]; ++i) {
            f3 n = ld3(fn + 3 * csr->faces[i]);
            if (i == csr->start[v]) acc = n;
            else acc = mk3(acc.x + n.x, acc.y + n.y, acc.z + n.z);
        }
        vn[3 * v] = acc.x; vn[3 * v + 1] = acc.y; vn[3 * v + 2] = acc.z;
    }
    free(fn);
}

/* ------------------------------------------------------------------------- */
/* Shading helpers */

/* getShading / getIllum (RendererUtil.h:135-214), FP64. */
static d3 sh_light_d(d3 n, const double *sh) {
    double basis[9] = {1.0, n.y, n.z, n.x, n.x * n.y, n.z * n.y, 3.0 * n.z * n.z - 1.0, n.x * n.z,
                       n.x * n.x - n.y * n.y};
    double l[3];
    for (int ch = 0; ch < 3; ++ch) {
        double acc = 0.0;
        for (int k = 0; k < 9; ++k) acc += sh[9 * ch + k] * basis[k];
        l[ch] = acc;
    }
    return dk3(l[0], l[1], l[2]);
}

static d3 sh_light(d3 n, const float *sh) {
    double basis[9] = {1.0, n.y, n.z, n.x, n.x * n.y, n.z * n.y, 3.0 * n.z * n.z - 1.0, n.x * n.z,
                       n.x * n.x - n.y * n.y};
    double l[3];
    for (int ch = 0; ch < 3; ++ch) {
        double acc = 0.0;
        for (int k = 0; k < 9; ++k) acc += (double)sh[9 * ch + k] * basis[k];
        l[ch] = acc;
    }
    return dk3(l[0], l[1], l[2]);
}

/* FP32 pixel normal + flip decision (CUDABasedRasterization.cu:308-319,
 * CUDABasedRasterizationGrad.cu:231-240). */
static int normal_flipped(f3 n0, f3 n1, f3 n2, f3 abc, f3 d) {
    f3 un = add3(add3(smul3(abc.x, n0), smul3(abc.y, n1)), smul3(abc.z, n2));
    float len = sqrtf(dot3(un, un));
    f3 n = sdiv3(un, len);
    return dot3(n, d) > 0.0f;
}

/* FP32 texture coordinate (CUDABasedRasterization.cu:326-336). */
static void tex_coord(const orc_scene *s, int f, f3 abc, float *U0, float *V0) {
    const float *t = s->uvs + (size_t)f * 6;
    float t0x = t[0], t0y = 1.0f - t[1];
    float t1x = t[2], t1y = 1.0f - t[3];
    float t2x = t[4], t2y = 1.0f - t[5];
    float fx = t0x * abc.x + t1x * abc.y + t2x * abc.z;
    float fy = t0y * abc.x + t1y * abc.y + t2y * abc.z;
    fx = fx * (float)s->Wt;
    fy = fy * (float)s->Ht;
    fx = fmaxf(fx, 0.0f);
    fx = fminf(fx, (float)(s->Wt - 1));
    fy = fmaxf(fy, 0.0f);
    fy = fminf(fy, (float)(s->Ht - 1));
    *U0 = fx;
    *V0 = fy;
}

/* Modes without reference counterpart (gvr.h): bilinear texture lookup,
 * headlight Phong, UV colour. */
static void bilinear_taps(float U0, float V0, int Wt, int Ht, int idx[4], double w[4]) {
    float x = U0 - 0.5f, y = V0 - 0.5f;
    float x0 = floorf(x), y0 = floorf(y);
    double fx = (double)(x - x0), fy = (double)(y - y0);
    int ix0 = (int)x0, iy0 = (int)y0, ix1 = ix0 + 1, iy1 = iy0 + 1;
    ix0 = ix0 < 0 ? 0 : ix0 > Wt - 1 ? Wt - 1 : ix0;
    ix1 = ix1 < 0 ? 0 : ix1 > Wt - 1 ? Wt - 1 : ix1;
    iy0 = iy0 < 0 ? 0 : iy0 > Ht - 1 ? Ht - 1 : iy0;
    iy1 = iy1 < 0 ? 0 : iy1 > Ht - 1 ? Ht - 1 : iy1;
    idx[0] = iy0 * Wt + ix0; idx[1] = iy0 * Wt + ix1; idx[2] = iy1 * Wt + ix0; idx[3] = iy1 * Wt + ix1;
    w[0] = (1.0 - fx) * (1.0 - fy); w[1] = fx * (1.0 - fy); w[2] = (1.0 - fx) * fy; w[3] = fx * fy;
}

static d3 bilinear_albedo(const orc_scene *s, float U0, float V0) {
    int idx[4];
    double w[4];
    bilinear_taps(U0, V0, s->Wt, s->Ht, idx, w);
    d3 c = dk3(0, 0, 0);
    for (int k = 0; k < 4; ++k) c = dadd(c, dscale(w[k], ldd3(s->texture + 3 * (size_t)idx[k])));
    return c;
}

static double phong_factor(double ndl) { return 0.2 + 0.7 * (ndl > 0.0 ? ndl : 0.0); }
static double phong_specular(double ndl) {
    double r = 2.0 * ndl * ndl - 1.0;
    if (r < 0.0) r = 0.0;
    r *= r; r *= r; r *= r; r *= r;
    return 0.3 * r;
}

static d3 uv_colour(const orc_scene *s, int f, double a, double b, double c) {
    const float *t = s->uvs + (size_t)f * 6;
    return dk3(a * t[0] + b * t[2] + c * t[4], a * t[1] + b * t[3] + c * t[5], 0.0);
}

/* ------------------------------------------------------------------------- */
/* Forward */

typedef struct { int x0, y0, x1, y1; float z0, z1, z2; } vface_t;

/*
 * orc_forward: renders every view of one batch element.
 * Outputs (any may be NULL):
 *   face [C*H*W] int32 (min face id among minimal-depth faces, -1 background)
 *   bary [C*H*W*2] float (the FP32 barycentrics of that face)
 *   render [C*H*W*3] double
 *   vnormal [C*N*3] float
 *   depth [C*H*W] int32 (INT_MAX background)
 *   ties [C*H*W] int32 (number of faces with the minimal quantised depth)
 *   tie_faces [C*H*W*ORC_MAX_TIES] int32 (first members of the tie set, -1 padded)
 */
void orc_forward(const orc_scene *s, int32_t *face_out, float *bary_out, double *render_out, float *vnormal_out,
                 int32_t *depth_out, int32_t *ties_out, int32_t *tie_faces_out) {
    const int N = s->N, F = s->F, W = s->W, H = s->H;
    csr_t csr;
    build_csr(N, F, s->faces, &csr);
    float *vn = (float *)malloc((size_t)N * 3 * sizeof(float));
    vertex_normals(s, &csr, vn);

    vface_t *vf = (vface_t *)malloc((size_t)F * sizeof(vface_t));
    f3 *proj = (f3 *)malloc((size_t)N * sizeof(f3));
    int *rowStart = (int *)malloc(((size_t)H + 1) * sizeof(int));
    int *rowCount = (int *)malloc(((size_t)H + 1) * sizeof(int));

    for (int c = 0; c < s->C; ++c) {
        const float *extr = s->extr + 12 * c, *intr = s->intr + 9 * c, *sh = s->sh + 27 * c;
        float invE[16], invP[16];
        orc_camera(extr, intr, invE, invP);
        f3 ro = ray_origin(invE);
        if (vnormal_out) memcpy(vnormal_out + (size_t)c * N * 3, vn, (size_t)N * 3 * sizeof(float));

        for (int v = 0; v < N; ++v) proj[v] = project_vertex(extr, intr, ld3(s->verts + 3 * v));
        /* projectFacesDevice (CUDABasedRasterization.cu:184-208) */
        for (int f = 0; f < F; ++f) {
            f3 p0 = proj[s->faces[3 * f]], p1 = proj[s->faces[3 * f + 1]], p2 = proj[s->faces[3 * f + 2]];
            vf[f].x0 = f2i_rz(fmaxf(fminf(p0.x, fminf(p1.x, p2.x)) - 0.5f, 0.0f));
            vf[f].y0 = f2i_rz(fmaxf(fminf(p0.y, fminf(p1.y, p2.y)) - 0.5f, 0.0f));
            vf[f].x1 = f2i_rz(fminf(fmaxf(p0.x, fmaxf(p1.x, p2.x)) + 0.5f, (float)(W - 1)));
            vf[f].y1 = f2i_rz(fminf(fmaxf(p0.y, fmaxf(p1.y, p2.y)) + 0.5f, (float)(H - 1)));
            vf[f].z0 = p0.z; vf[f].z1 = p1.z; vf[f].z2 = p2.z;
        }
        /* bucket faces by the rows their box spans so rows can run in parallel */
        memset(rowCount, 0, ((size_t)H + 1) * sizeof(int));
        for (int f = 0; f < F; ++f) {
            if (vf[f].x0 > vf[f].x1 || vf[f].y0 > vf[f].y1) continue;
            int ya = vf[f].y0 < 0 ? 0 : vf[f].y0, yb = vf[f].y1 >= H ? H - 1 : vf[f].y1;
            for (int y = ya; y <= yb; ++y) rowCount[y]++;
        }
        rowStart[0] = 0;
        for (int y = 0; y < H; ++y) rowStart[y + 1] = rowStart[y] + rowCount[y];
        int *rowFaces = (int *)malloc((size_t)rowStart[H] * sizeof(int) + 1);
        memset(rowCount, 0, ((size_t)H + 1) * sizeof(int));
        for (int f = 0; f < F; ++f) {
            if (vf[f].x0 > vf[f].x1 || vf[f].y0 > vf[f].y1) continue;
            int ya = vf[f].y0 < 0 ? 0 : vf[f].y0, yb = vf[f].y1 >= H ? H - 1 : vf[f].y1;
            for (int y = ya; y <= yb; ++y) rowFaces[rowStart[y] + rowCount[y]++] = f;
        }

#pragma omp parallel
        {
            int *bestDepth = (int *)malloc((size_t)W * sizeof(int));
            int *bestFace = (int *)malloc((size_t)W * sizeof(int));
            int *nTies = (int *)malloc((size_t)W * sizeof(int));
            int *tieList = (int *)malloc((size_t)W * ORC_MAX_TIES * sizeof(int));
#pragma omp for schedule(dynamic, 4)
            for (int v = 0; v < H; ++v) {
                for (int u = 0; u < W; ++u) { bestDepth[u] = INT_MAX; bestFace[u] = -1; nTies[u] = 0; }
                for (int k = rowStart[v]; k < rowStart[v + 1]; ++k) {
                    int f = rowFaces[k];
                    f3 v0 = ld3(s->verts + 3 * s->faces[3 * f]);
                    f3 v1 = ld3(s->verts + 3 * s->faces[3 * f + 1]);
                    f3 v2 = ld3(s->verts + 3 * s->faces[3 * f + 2]);
                    int ua = vf[f].x0 < 0 ? 0 : vf[f].x0, ub = vf[f].x1 >= W ? W - 1 : vf[f].x1;
                    for (int u = ua; u <= ub; ++u) {
                        f3 d = ray_dir(s, c, invP, ro, u, v);
                        f3 abc = barycentric(ro, d, v0, v1, v2);
                        if (!inside_triangle(abc)) continue;
                        int zi = depth_int(abc, vf[f].z0, vf[f].z1, vf[f].z2);
                        if (zi < bestDepth[u] || nTies[u] == 0) {
                            bestDepth[u] = zi; bestFace[u] = f; nTies[u] = 1;
                            tieList[u * ORC_MAX_TIES] = f;
                        } else if (zi == bestDepth[u]) {
                            if (nTies[u] < ORC_MAX_TIES) tieList[u * ORC_MAX_TIES + nTies[u]] = f;
                            nTies[u]++;
                            if (f < bestFace[u]) bestFace[u] = f;
                        }
                    }
                }
                for (int u = 0; u < W; ++u) {
                    size_t p = ((size_t)c * H + v) * W + u;
                    int f = bestFace[u];
                    if (face_out) face_out[p] = f;
                    if (depth_out) depth_out[p] = nTies[u] ? bestDepth[u] : INT_MAX;
                    if (ties_out) ties_out[p] = nTies[u];
                    if (tie_faces_out)
                        for (int k = 0; k < ORC_MAX_TIES; ++k)
                            tie_faces_out[p * ORC_MAX_TIES + k] = k < nTies[u] ? tieList[u * ORC_MAX_TIES + k] : -1;
                    if (f < 0) {
                        if (bary_out) { bary_out[2 * p] = 0.0f; bary_out[2 * p + 1] = 0.0f; }
                        if (render_out) { render_out[3 * p] = 0.0; render_out[3 * p + 1] = 1.0; render_out[3 * p + 2] = 0.0; }
                        continue;
                    }
                    /* renderBuffersDevice resolve + shading (CUDABasedRasterization.cu:295-403) */
                    int i0 = s->faces[3 * f], i1 = s->faces[3 * f + 1], i2 = s->faces[3 * f + 2];
                    f3 d = ray_dir(s, c, invP, ro, u, v);
                    f3 abc = barycentric(ro, d, ld3(s->verts + 3 * i0), ld3(s->verts + 3 * i1), ld3(s->verts + 3 * i2));
                    if (bary_out) { bary_out[2 * p] = abc.x; bary_out[2 * p + 1] = abc.y; }
                    if (!render_out) continue;
                    f3 n0 = ld3(vn + 3 * i0), n1 = ld3(vn + 3 * i1), n2 = ld3(vn + 3 * i2);
                    int flip = normal_flipped(n0, n1, n2, abc, d);
                    d3 un = dadd(dadd(dscale(abc.x, f2d(n0)), dscale(abc.y, f2d(n1))), dscale(abc.z, f2d(n2)));
                    d3 n = dnormalize(un);
                    if (flip) n = dscale(-1.0, n);
                    d3 col = dk3(0, 0, 0);
                    if (s->albedo_mode == ORC_TEXTURED) {
                        float U0, V0;
                        tex_coord(s, f, abc, &U0, &V0);
                        int LU = f2i_rz(U0 - 0.5f), LV = f2i_rz(V0 - 0.5f);
                        col = ldd3(s->texture + ((size_t)LV * s->Wt + LU) * 3);
                    } else if (s->albedo_mode == ORC_VERTEX_COLOR) {
                        d3 c0 = ldd3(s->colors + 3 * i0), c1 = ldd3(s->colors + 3 * i1), c2 = ldd3(s->colors + 3 * i2);
                        col = dadd(dadd(dscale(abc.x, c0), dscale(abc.y, c1)), dscale(abc.z, c2));
                    } else if (s->albedo_mode == ORC_NORMAL) {
                        col = dk3((1.0 + n.x) / 2.0, (1.0 + n.y) / 2.0, (1.0 + n.z) / 2.0);
                    } else if (s->albedo_mode == ORC_TEXTURED_BILINEAR) {
                        float U0, V0;
                        tex_coord(s, f, abc, &U0, &V0);
                        col = bilinear_albedo(s, U0, V0);
                    } else if (s->albedo_mode == ORC_UV) {
                        col = uv_colour(s, f, abc.x, abc.y, abc.z);
                    } else {
                        col = dk3(1, 1, 1);
                    }
                    int lit = s->albedo_mode != ORC_NORMAL && s->albedo_mode != ORC_UV;
                    int shaded = (s->shading_mode == ORC_SHADED && lit) || s->albedo_mode == ORC_LIGHTING;
                    if (s->albedo_mode == ORC_FOREGROUND) shaded = 0; /* forced shadeless, CudaRenderer.cpp:72-76 */
                    if (s->shading_mode == ORC_PHONG && lit && s->albedo_mode != ORC_LIGHTING &&
                        s->albedo_mode != ORC_FOREGROUND) {
                        double ndl = -ddot(n, f2d(d));
                        double k = phong_factor(ndl), sp = phong_specular(ndl);
                        col = dk3(col.x * k + sp, col.y * k + sp, col.z * k + sp);
                    } else if (shaded) {
                        d3 l = sh_light(n, sh);
                        col = dk3(l.x * col.x, l.y * col.y, l.z * col.z);
                    }
                    render_out[3 * p] = col.x; render_out[3 * p + 1] = col.y; render_out[3 * p + 2] = col.z;
                }
            }
            free(bestDepth); free(bestFace); free(nTies); free(tieList);
        }
        free(rowFaces);
    }
    free(vf); free(proj); free(rowStart); free(rowCount); free(vn);
    free_csr(&csr);
}

/* Per-pixel FP32 ray directions exactly as orc_forward uses them (for tests). */
void orc_rays(const orc_scene *s, float *rays_out /*[C*H*W*3]*/) {
    for (int c = 0; c < s->C; ++c) {
        float invE[16], invP[16];
        orc_camera(s->extr + 12 * c, s->intr + 9 * c, invE, invP);
        f3 ro = ray_origin(invE);
        for (int v = 0; v < s->H; ++v)
            for (int u = 0; u < s->W; ++u) {
                f3 d = ray_dir(s, c, invP, ro, u, v);
                float *o = rays_out + (((size_t)c * s->H + v) * s->W + u) * 3;
                o[0] = d.x; o[1] = d.y; o[2] = d.z;
            }
    }
}

/* Projected vertices and face boxes for view c (tests). */
void orc_project(const orc_scene *s, int c, float *proj_out /*[N*3]*/, int32_t *bbox_out /*[F*4]*/) {
    const float *extr = s->extr + 12 * c, *intr = s->intr + 9 * c;
    f3 *proj = (f3 *)malloc((size_t)s->N * sizeof(f3));
    for (int v = 0; v < s->N; ++v) {
        proj[v] = project_vertex(extr, intr, ld3(s->verts + 3 * v));
        if (proj_out) { proj_out[3 * v] = proj[v].x; proj_out[3 * v + 1] = proj[v].y; proj_out[3 * v + 2] = proj[v].z; }
    }
    if (bbox_out)
        for (int f = 0; f < s->F; ++f) {
            f3 p0 = proj[s->faces[3 * f]], p1 = proj[s->faces[3 * f + 1]], p2 = proj[s->faces[3 * f + 2]];
            bbox_out[4 * f + 0] = f2i_rz(fmaxf(fminf(p0.x, fminf(p1.x, p2.x)) - 0.5f, 0.0f));
            bbox_out[4 * f + 1] = f2i_rz(fmaxf(fminf(p0.y, fminf(p1.y, p2.y)) - 0.5f, 0.0f));
            bbox_out[4 * f + 2] = f2i_rz(fminf(fmaxf(p0.x, fmaxf(p1.x, p2.x)) + 0.5f, (float)(s->W - 1)));
            bbox_out[4 * f + 3] = f2i_rz(fminf(fmaxf(p0.y, fmaxf(p1.y, p2.y)) + 0.5f, (float)(s->H - 1)));
        }
    free(proj);
}

/* ------------------------------------------------------------------------- */
/* Backward: renderBuffersGradDevice (CUDABasedRasterizationGrad.cu:114-617) in FP64.
 * Small dense matrix helpers mirror the mat NxM chains of the reference. */

typedef struct { double m[3][3]; } m33;

static m33 m33_zero(void) { m33 r; memset(&r, 0, sizeof(r)); return r; }
static m33 m33_ident(void) { m33 r = m33_zero(); r.m[0][0] = r.m[1][1] = r.m[2][2] = 1.0; return r; }
static m33 m33_diag(d3 a) { m33 r = m33_zero(); r.m[0][0] = a.x; r.m[1][1] = a.y; r.m[2][2] = a.z; return r; }
/* row vector (1x3) times 3x3 */
static d3 rowmul(d3 g, m33 M) {
    return dk3(g.x * M.m[0][0] + g.y * M.m[1][0] + g.z * M.m[2][0],
               g.x * M.m[0][1] + g.y * M.m[1][1] + g.z * M.m[2][1],
               g.x * M.m[0][2] + g.y * M.m[1][2] + g.z * M.m[2][2]);
}
/* matrix whose columns are the given vectors */
static m33 m33_cols(d3 c0, d3 c1, d3 c2) {
    m33 r;
    r.m[0][0] = c0.x; r.m[1][0] = c0.y; r.m[2][0] = c0.z;
    r.m[0][1] = c1.x; r.m[1][1] = c1.y; r.m[2][1] = c1.z;
    r.m[0][2] = c2.x; r.m[1][2] = c2.y; r.m[2][2] = c2.z;
    return r;
}
static m33 m33_add(m33 a, m33 b) {
    m33 r;
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] + b.m[i][j];
    return r;
}

/* getJLiNo (RendererUtil.h:371-391) */
static m33 J_light_normal(d3 n, const float *sh) {
    m33 J;
    for (int i = 0; i < 3; ++i) {
        const float *c = sh + 9 * i;
        J.m[i][0] = c[3] + c[4] * n.y + c[7] * n.z + c[8] * 2.0 * n.x;
        J.m[i][1] = c[1] + c[4] * n.x + c[5] * n.z + c[8] * -2.0 * n.y;
        J.m[i][2] = c[2] + c[5] * n.y + c[6] * 6.0 * n.z + c[7] * n.x;
    }
    return J;
}

/* getJNoNu (RendererUtil.h:398-415) */
static m33 J_normalize(d3 u, double norm) {
    double p2 = norm * norm, p3 = p2 * norm;
    m33 J;
    J.m[0][0] = (p2 - u.x * u.x) / p3;
    J.m[1][1] = (p2 - u.y * u.y) / p3;
    J.m[2][2] = (p2 - u.z * u.z) / p3;
    J.m[0][1] = J.m[1][0] = -(u.x * u.y) / p3;
    J.m[0][2] = J.m[2][0] = -(u.x * u.z) / p3;
    J.m[1][2] = J.m[2][1] = -(u.y * u.z) / p3;
    return J;
}

/* getJ_vi / getJ_vj / getJ_vk (RendererUtil.h:422-539): d cross(vj-vi, vk-vi) / d v. */
static m33 J_vi(d3 vk, d3 vj, d3 vi) {
    d3 e[3] = {dk3(-1, 0, 0), dk3(0, -1, 0), dk3(0, 0, -1)};
    d3 d1 = dsub(vj, vi), d2 = dsub(vk, vi);
    m33 J1 = m33_cols(dcross(d1, e[0]), dcross(d1, e[1]), dcross(d1, e[2]));
    m33 J2 = m33_cols(dcross(e[0], d2), dcross(e[1], d2), dcross(e[2], d2));
    return m33_add(J1, J2);
}
static m33 J_vj(d3 vk, d3 vi) {
    d3 d1 = dsub(vk, vi);
    return m33_cols(dcross(dk3(1, 0, 0), d1), dcross(dk3(0, 1, 0), d1), dcross(dk3(0, 0, 1), d1));
}
static m33 J_vk(d3 vj, d3 vi) {
    d3 d2 = dsub(vj, vi);
    return m33_cols(dcross(d2, dk3(1, 0, 0)), dcross(d2, dk3(0, 1, 0)), dcross(d2, dk3(0, 0, 1)));
}

/* dJBCDVerpos (RendererUtil.h:670-861): d(a,b,c)/d(v0,v1,v2) for a fixed ray. */
static void J_bary_pos(d3 orig, d3 dir, d3 v0, d3 v1, d3 v2, double J[3][9]) {
    memset(J, 0, sizeof(double) * 27);
    d3 N = dcross(dsub(v1, v0), dsub(v2, v0));
    double denom = ddot(N, N);
    double NdotDir = ddot(dir, N);
    if (fabs(ddot(dnormalize(dir), dnormalize(N))) < 0.001 || fabs(denom * denom) < 0.001) return;
    double t = (ddot(v0, N) - ddot(orig, N)) / NdotDir;
    d3 P = dadd(orig, dscale(t, dir));
    d3 edge1 = dsub(v2, v1), vp1 = dsub(P, v1), C1 = dcross(edge1, vp1);
    d3 edge2 = dsub(v0, v2), vp2 = dsub(P, v2), C2 = dcross(edge2, vp2);
    m33 dNv0 = J_vi(v2, v1, v0), dNv1 = J_vj(v2, v0), dNv2 = J_vk(v1, v0);
    d3 dN[9];
    for (int k = 0; k < 3; ++k) {
        dN[k] = dk3(dNv0.m[0][k], dNv0.m[1][k], dNv0.m[2][k]);
        dN[3 + k] = dk3(dNv1.m[0][k], dNv1.m[1][k], dNv1.m[2][k]);
        dN[6 + k] = dk3(dNv2.m[0][k], dNv2.m[1][k], dNv2.m[2][k]);
    }
    d3 Cs[2] = {C1, C2}, vps[2] = {vp1, vp2}, Es[2] = {edge1, edge2};
    d3 dE[2][9], dV[3][9];
    for (int var = 0; var < 9; ++var) {
        d3 unit = dk3(var % 3 == 0, var % 3 == 1, var % 3 == 2);
        int vert = var / 3;
        dV[0][var] = vert == 0 ? unit : dk3(0, 0, 0);
        dV[1][var] = vert == 1 ? unit : dk3(0, 0, 0);
        dV[2][var] = vert == 2 ? unit : dk3(0, 0, 0);
        /* edge1 = v2 - v1, edge2 = v0 - v2 */
        dE[0][var] = vert == 1 ? dscale(-1, unit) : (vert == 2 ? unit : dk3(0, 0, 0));
        dE[1][var] = vert == 0 ? unit : (vert == 2 ? dscale(-1, unit) : dk3(0, 0, 0));
    }
    double dt[9];
    d3 v0o = dsub(v0, orig);
    for (int var = 0; var < 9; ++var)
        dt[var] = (-1.0 / (ddot(N, dir) * ddot(N, dir))) * ddot(dN[var], dir) * ddot(v0o, N) +
                  (1.0 / ddot(N, dir)) * (ddot(dV[0][var], N) + ddot(v0o, dN[var]));
    for (int abc = 0; abc < 2; ++abc)
        for (int var = 0; var < 9; ++var) {
            double tmp = ddot(N, Cs[abc]);
            d3 dvp = dsub(dscale(dt[var], dir), dV[abc + 1][var]);
            double dtmp = ddot(dN[var], Cs[abc]) +
                          ddot(N, dadd(dcross(dE[abc][var], vps[abc]), dcross(Es[abc], dvp)));
            J[abc][var] = dtmp / denom + tmp * (-1.0 / (denom * denom)) * (2.0 * ddot(N, dN[var]));
        }
    for (int var = 0; var < 9; ++var) J[2][var] = -J[0][var] - J[1][var];
}

/* imageGradient (RendererUtil.h:566-620) on a [H,W,3] float image; returns d/du in g[0], d/dv in g[1]. */
static void image_gradient(const float *img, int px, int py, int w, int h, int k, d3 g[2]) {
    g[0] = g[1] = dk3(0, 0, 0);
    if (!(px >= k + 1 && py >= k + 1 && px < w - (k + 1) && py < h - (k + 1))) return;
    double norm = 0.0;
    d3 du = dk3(0, 0, 0), dv = dk3(0, 0, 0);
    for (int y = -k; y <= k; ++y)
        for (int x = -k; x <= k; ++x) {
            d3 I = ldd3(img + ((size_t)(py + y) * w + (px + x)) * 3);
            double den = (double)(x * x + y * y), Gu = 0.0, Gv = 0.0;
            if (den != 0.0) { Gu = x / den; Gv = y / den; }
            du = dadd(du, dscale(Gu, I));
            dv = dadd(dv, dscale(Gv, I));
            norm += fabs(Gu);
        }
    g[0] = dscale(1.0 / norm, du);
    g[1] = dscale(1.0 / norm, dv);
}

/* getJProjection (RendererUtil.h:275-332): 2x3 d(pixel)/d(world point). */
static void J_projection(d3 X, const float *intr9, const float *extr12, double J[2][3]) {
    memset(J, 0, sizeof(double) * 6);
    double KE[3][4];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 4; ++j) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k) acc += (double)intr9[3 * i + k] * extr12[4 * k + j];
            KE[i][j] = acc;
        }
    double P[3];
    for (int i = 0; i < 3; ++i) P[i] = KE[i][0] * X.x + KE[i][1] * X.y + KE[i][2] * X.z + KE[i][3];
    if (!(fabs(P[2]) > 0.0001)) return;
    double D[2][3] = {{1.0 / P[2], 0.0, -P[0] / (P[2] * P[2])}, {0.0, 1.0 / P[2], -P[1] / (P[2] * P[2])}};
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 3; ++j) J[i][j] = D[i][0] * KE[0][j] + D[i][1] * KE[1][j] + D[i][2] * KE[2][j];
}

/*
 * orc_backward: gradients of one batch element.  Inputs face/bary/vnormal are
 * the forward outputs (as the reference grad op consumes them).  Outputs are
 * FP64 and fully overwritten:
 *   gpos [N*3], gcol [N*3], gtex [Ht*Wt*3], gsh [C*27].
 */
/* flags & 1 (GVR_BACKWARD_ALBEDO_POSITION, an option without reference
 * counterpart): vertexColor mode also moves the vertices by the change of
 * the interpolated colour through the barycentrics, the term the reference
 * zeroes (CUDABasedRasterizationGrad.cu:489). */
void orc_backward_ex(const orc_scene *s, const int32_t *face, const float *bary, const float *vnormal,
                     const float *grad_render, const float *target, const float *grad_target, double *gpos,
                     double *gcol, double *gtex, double *gsh, int flags) {
    const int N = s->N, W = s->W, H = s->H, C = s->C;
    csr_t csr;
    build_csr(N, s->F, s->faces, &csr);
    memset(gpos, 0, sizeof(double) * 3 * N);
    memset(gcol, 0, sizeof(double) * 3 * N);
    memset(gtex, 0, sizeof(double) * 3 * (size_t)s->Ht * s->Wt);
    memset(gsh, 0, sizeof(double) * 27 * C);
    const int shaded = s->shading_mode == ORC_SHADED && s->albedo_mode != ORC_FOREGROUND;
    if (s->albedo_mode == ORC_NORMAL || s->albedo_mode == ORC_LIGHTING || s->albedo_mode == ORC_UV) {
        free_csr(&csr);
        return;
    }
    const int phong = s->shading_mode == ORC_PHONG && s->albedo_mode != ORC_FOREGROUND;
    int nthreads = 1;
#ifdef _OPENMP
    nthreads = omp_get_max_threads();
#endif
    double *tpos = (double *)calloc((size_t)nthreads * 3 * N, sizeof(double));
    double *tcol = (double *)calloc((size_t)nthreads * 3 * N, sizeof(double));
    double *tsh = (double *)calloc((size_t)nthreads * 27 * C, sizeof(double));

    for (int c = 0; c < C; ++c) {
        const float *extr = s->extr + 12 * c, *intr = s->intr + 9 * c, *sh = s->sh + 27 * c;
        const float *vn = vnormal + (size_t)c * N * 3;
        float invE[16], invP[16];
        orc_camera(extr, intr, invE, invP);
        f3 ro = ray_origin(invE);
#pragma omp parallel
        {
            int tid = 0;
#ifdef _OPENMP
            tid = omp_get_thread_num();
#endif
            double *mypos = tpos + (size_t)tid * 3 * N, *mycol = tcol + (size_t)tid * 3 * N;
            double *mysh = tsh + (size_t)tid * 27 * C + 27 * c;
#pragma omp for schedule(dynamic, 4)
            for (int v = 0; v < H; ++v)
                for (int u = 0; u < W; ++u) {
                    size_t p = ((size_t)c * H + v) * W + u;
                    int f = face[p];
                    if (f == -1) continue;
                    f3 df = ray_dir(s, c, invP, ro, u, v);
                    d3 o = f2d(ro), d = f2d(df);
                    float ba = bary[2 * p], bb = bary[2 * p + 1];
                    f3 abc = mk3(ba, bb, 1.0f - ba - bb);
                    d3 bcc = f2d(abc);
                    int id[3] = {s->faces[3 * f], s->faces[3 * f + 1], s->faces[3 * f + 2]};
                    d3 P[3], Col[3], Nor[3];
                    for (int i = 0; i < 3; ++i) {
                        P[i] = ldd3(s->verts + 3 * id[i]);
                        Col[i] = ldd3(s->colors + 3 * id[i]);
                        Nor[i] = ldd3(vn + 3 * id[i]);
                    }
                    double b[3] = {bcc.x, bcc.y, bcc.z};
                    d3 frag = dadd(dadd(dscale(b[0], P[0]), dscale(b[1], P[1])), dscale(b[2], P[2]));
                    d3 un = dadd(dadd(dscale(b[0], Nor[0]), dscale(b[1], Nor[1])), dscale(b[2], Nor[2]));
                    double unLen = sqrt(ddot(un, un));
                    d3 n = dscale(1.0 / unLen, un);
                    int flipped = normal_flipped(ld3(vn + 3 * id[0]), ld3(vn + 3 * id[1]), ld3(vn + 3 * id[2]), abc, df);
                    if (flipped) n = dscale(-1.0, n);
                    if (s->albedo_mode == ORC_FOREGROUND) Col[0] = Col[1] = Col[2] = dk3(1, 1, 1);
                    float U0 = 0.0f, V0 = 0.0f;
                    if (s->albedo_mode == ORC_TEXTURED || s->albedo_mode == ORC_TEXTURED_BILINEAR)
                        tex_coord(s, f, abc, &U0, &V0);
                    d3 light = sh_light(n, sh);
                    m33 JCoAl = shaded ? m33_diag(light) : m33_ident();
                    if (phong) {
                        double k = phong_factor(-ddot(n, d));
                        JCoAl = m33_diag(dk3(k, k, k));
                    }
                    d3 alb = dk3(0, 0, 0);
                    int LUi = 0, LVi = 0;
                    if (s->albedo_mode == ORC_VERTEX_COLOR) {
                        alb = dadd(dadd(dscale(b[0], Col[0]), dscale(b[1], Col[1])), dscale(b[2], Col[2]));
                    } else if (s->albedo_mode == ORC_TEXTURED) {
                        /* CUDABasedRasterizationGrad.cu:282-312 (corner weights as written there) */
                        int iu = f2i_rz(U0 - 0.5f), iv = f2i_rz(V0 - 0.5f);
                        float LU = iu + 0.5f, HU = iu + 1.5f, LV = iv + 0.5f, HV = iv + 1.5f;
                        LUi = f2i_rz(LU); LVi = f2i_rz(LV);
                        int HUi = f2i_rz(HU), HVi = f2i_rz(HV);
                        d3 cLL = ldd3(s->texture + ((size_t)LVi * s->Wt + LUi) * 3);
                        d3 cLH = ldd3(s->texture + ((size_t)HVi * s->Wt + LUi) * 3);
                        d3 cHL = ldd3(s->texture + ((size_t)LVi * s->Wt + HUi) * 3);
                        d3 cHH = ldd3(s->texture + ((size_t)HVi * s->Wt + HUi) * 3);
                        double u0 = U0, v0 = V0;
                        alb = dadd(dscale(v0 - LV, dadd(dscale(u0 - LU, cLL), dscale(HU - u0, cHL))),
                                   dscale(HV - v0, dadd(dscale(u0 - LU, cLH), dscale(HU - u0, cHH))));
                    }
                    int bidx[4] = {0, 0, 0, 0};
                    double bw[4] = {0, 0, 0, 0};
                    if (s->albedo_mode == ORC_TEXTURED_BILINEAR) {
                        bilinear_taps(U0, V0, s->Wt, s->Ht, bidx, bw);
                        alb = bilinear_albedo(s, U0, V0);
                    }
                    m33 JCoLi = m33_diag(alb);
                    const float *gr = grad_render + 3 * p;
                    d3 G = dk3(gr[0], gr[1], gr[2]);
                    /* vertex colour / texture (:327-395) */
                    if (s->albedo_mode == ORC_VERTEX_COLOR) {
                        d3 gc = rowmul(G, JCoAl);
                        for (int i = 0; i < 3; ++i) {
                            mycol[3 * id[i] + 0] += b[i] * gc.x;
                            mycol[3 * id[i] + 1] += b[i] * gc.y;
                            mycol[3 * id[i] + 2] += b[i] * gc.z;
                        }
                    } else if (s->albedo_mode == ORC_TEXTURED && !flipped) {
                        d3 gt = rowmul(G, JCoAl);
                        double *dst = gtex + ((size_t)LVi * s->Wt + LUi) * 3;
#pragma omp atomic
                        dst[0] += gt.x;
#pragma omp atomic
                        dst[1] += gt.y;
#pragma omp atomic
                        dst[2] += gt.z;
                    } else if (s->albedo_mode == ORC_TEXTURED_BILINEAR) {
                        d3 gt = rowmul(G, JCoAl);
                        for (int k = 0; k < 4; ++k) {
                            double *dst = gtex + 3 * (size_t)bidx[k];
#pragma omp atomic
                            dst[0] += bw[k] * gt.x;
#pragma omp atomic
                            dst[1] += bw[k] * gt.y;
#pragma omp atomic
                            dst[2] += bw[k] * gt.z;
                        }
                    }
                    /* SH (:402-436) */
                    if (shaded) {
                        double basis[9] = {1.0, n.y, n.z, n.x, n.x * n.y, n.z * n.y, 3.0 * n.z * n.z - 1.0,
                                           n.x * n.z, n.x * n.x - n.y * n.y};
                        double ga[3] = {G.x * alb.x, G.y * alb.y, G.z * alb.z};
                        for (int ch = 0; ch < 3; ++ch)
                            for (int k = 0; k < 9; ++k) mysh[9 * ch + k] += ga[ch] * basis[k];
                    }
                    /* vertex position, shading term (:458-525) */
                    d3 w = dk3(0, 0, 0);
                    const int albpos = (flags & 1) && s->albedo_mode == ORC_VERTEX_COLOR;
                    if (shaded || albpos) {
                        d3 r = dk3(0, 0, 0);
                        if (shaded) {
                            m33 JLiNo = J_light_normal(n, sh);
                            m33 JNoNu = J_normalize(un, unLen);
                            w = rowmul(rowmul(rowmul(G, JCoLi), JLiNo), JNoNu);
                            r = rowmul(w, m33_cols(Nor[0], Nor[1], Nor[2]));
                        }
                        if (albpos) r = dadd(r, rowmul(rowmul(G, JCoAl), m33_cols(Col[0], Col[1], Col[2])));
                        double JB[3][9];
                        J_bary_pos(o, d, P[0], P[1], P[2], JB);
                        for (int var = 0; var < 9; ++var) {
                            double g = r.x * JB[0][var] + r.y * JB[1][var] + r.z * JB[2][var];
                            mypos[3 * id[var / 3] + var % 3] += g;
                        }
                    }
                    /* model-to-data term (:531-555) */
                    {
                        const float *gtp = grad_target + 3 * p;
                        d3 GT = dk3(gtp[0], gtp[1], gtp[2]);
                        d3 dT[2];
                        image_gradient(target + (size_t)c * H * W * 3, u, v, W, H, s->image_filter_size, dT);
                        double Jp[2][3];
                        J_projection(frag, intr, extr, Jp);
                        double gu = ddot(GT, dT[0]), gv = ddot(GT, dT[1]);
                        d3 m = dk3(gu * Jp[0][0] + gv * Jp[1][0], gu * Jp[0][1] + gv * Jp[1][1],
                                   gu * Jp[0][2] + gv * Jp[1][2]);
                        for (int i = 0; i < 3; ++i) {
                            mypos[3 * id[i] + 0] += b[i] * m.x;
                            mypos[3 * id[i] + 1] += b[i] * m.y;
                            mypos[3 * id[i] + 2] += b[i] * m.z;
                        }
                    }
                    /* normal-adjacency term (:559-615) */
                    if (shaded) {
                        for (int i = 0; i < 3; ++i) {
                            d3 wi = dscale(b[i], w);
                            int idv = id[i];
                            for (int j = csr.start[idv]; j < csr.start[idv + 1]; ++j) {
                                int g = csr.faces[j];
                                int a0 = s->faces[3 * g], a1 = s->faces[3 * g + 1], a2 = s->faces[3 * g + 2];
                                d3 vi = ldd3(s->verts + 3 * a0), vj = ldd3(s->verts + 3 * a1), vk = ldd3(s->verts + 3 * a2);
                                d3 gi = rowmul(wi, J_vi(vk, vj, vi));
                                d3 gj = rowmul(wi, J_vj(vk, vi));
                                d3 gk = rowmul(wi, J_vk(vj, vi));
                                mypos[3 * a0] += gi.x; mypos[3 * a0 + 1] += gi.y; mypos[3 * a0 + 2] += gi.z;
                                mypos[3 * a1] += gj.x; mypos[3 * a1 + 1] += gj.y; mypos[3 * a1 + 2] += gj.z;
                                mypos[3 * a2] += gk.x; mypos[3 * a2 + 1] += gk.y; mypos[3 * a2 + 2] += gk.z;
                            }
                        }
                    }
                }
        }
    }
    for (int t = 0; t < nthreads; ++t) {
        for (int i = 0; i < 3 * N; ++i) { gpos[i] += tpos[(size_t)t * 3 * N + i]; gcol[i] += tcol[(size_t)t * 3 * N + i]; }
        for (int i = 0; i < 27 * C; ++i) gsh[i] += tsh[(size_t)t * 27 * C + i];
    }
    free(tpos); free(tcol); free(tsh);
    free_csr(&csr);
}

void orc_backward(const orc_scene *s, const int32_t *face, const float *bary, const float *vnormal,
                  const float *grad_render, const float *target, const float *grad_target, double *gpos,
                  double *gcol, double *gtex, double *gsh) {
    orc_backward_ex(s, face, bary, vnormal, grad_render, target, grad_target, gpos, gcol, gtex, gsh, 0);
}

/* ------------------------------------------------------------------------- */
/* FP64 forward at fixed visibility, for finite-difference checks of the
 * gradient restatement: given face ids per pixel, every quantity (camera
 * inverse, ray, barycentrics, vertex normals, shading) is computed in FP64.
 * verts_d (optional) replaces the FP32 vertex positions with FP64 ones.
 * flags_out bit 0: normal flipped; bit 1: |cos(ray, face normal)| < 0.002
 * (near the reference Jacobian's 0.001 early-out). */
#define VD(i) (verts_d ? dk3(verts_d[3 * (i)], verts_d[3 * (i) + 1], verts_d[3 * (i) + 2]) : ldd3(s->verts + 3 * (i)))
#define CD(i) (colors_d ? dk3(colors_d[3 * (i)], colors_d[3 * (i) + 1], colors_d[3 * (i) + 2]) : ldd3(s->colors + 3 * (i)))

static void mat4_inverse_d(const double *m, double *inv) {
    double a[4][8];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 8; ++j) a[i][j] = j < 4 ? m[4 * i + j] : (j - 4 == i);
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int r = c + 1; r < 4; ++r)
            if (fabs(a[r][c]) > fabs(a[piv][c])) piv = r;
        for (int j = 0; j < 8; ++j) { double t = a[c][j]; a[c][j] = a[piv][j]; a[piv][j] = t; }
        double p = a[c][c];
        for (int j = 0; j < 8; ++j) a[c][j] /= p;
        for (int r = 0; r < 4; ++r)
            if (r != c) {
                double fct = a[r][c];
                for (int j = 0; j < 8; ++j) a[r][j] -= fct * a[c][j];
            }
    }
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) inv[4 * i + j] = a[i][4 + j];
}

/* FP64 render at fixed visibility; verts_d [N*3], colors_d [N*3] and sh_d
 * [C*27] optionally replace the scene's FP32 arrays (finite differences of
 * parameters that feed them). */
void orc_render_fp64_ex(const orc_scene *s, const double *verts_d, const double *colors_d, const double *sh_d,
                        const int32_t *face, double *render_out, int32_t *flags_out) {
    const int N = s->N, F = s->F, W = s->W, H = s->H;
    csr_t csr;
    build_csr(N, F, s->faces, &csr);
    d3 *fn = (d3 *)malloc((size_t)F * sizeof(d3));
    d3 *vn = (d3 *)malloc((size_t)N * sizeof(d3));
    for (int f = 0; f < F; ++f) {
        d3 v0 = VD(s->faces[3 * f]), v1 = VD(s->faces[3 * f + 1]);
        d3 v2 = VD(s->faces[3 * f + 2]);
        fn[f] = dcross(dsub(v1, v0), dsub(v2, v0));
    }
    for (int v = 0; v < N; ++v) {
        d3 acc = dk3(0, 0, 0);
        for (int i = csr.start[v]; i < csr.start[v + 1]; ++i) acc = dadd(acc, fn[csr.faces[i]]);
        vn[v] = acc;
    }
    for (int c = 0; c < s->C; ++c) {
        const float *e12 = s->extr + 12 * c, *k9 = s->intr + 9 * c;
        double sh[27];
        for (int k = 0; k < 27; ++k) sh[k] = sh_d ? sh_d[27 * c + k] : (double)s->sh[27 * c + k];
        double E[16] = {0}, K[16] = {0}, KE[16], invE[16], invP[16];
        for (int i = 0; i < 16; ++i) E[i] = K[i] = (i % 5 == 0);
        for (int r = 0; r < 3; ++r)
            for (int j = 0; j < 4; ++j) { E[4 * r + j] = e12[4 * r + j]; K[4 * r + j] = j < 3 ? k9[3 * r + j] : 0.0; }
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) {
                double acc = 0;
                for (int k = 0; k < 4; ++k) acc += K[4 * i + k] * E[4 * k + j];
                KE[4 * i + j] = acc;
            }
        mat4_inverse_d(E, invE);
        mat4_inverse_d(KE, invP);
        d3 o = dk3(invE[3] / invE[15], invE[7] / invE[15], invE[11] / invE[15]);
#pragma omp parallel for schedule(dynamic, 4)
        for (int v = 0; v < H; ++v)
            for (int u = 0; u < W; ++u) {
                size_t p = ((size_t)c * H + v) * W + u;
                int f = face[p];
                double *out = render_out + 3 * p;
                if (flags_out) flags_out[p] = 0;
                if (f < 0) { out[0] = 0.0; out[1] = 1.0; out[2] = 0.0; continue; }
                double px = (u + 0.5) * 1000.0, py = (v + 0.5) * 1000.0, pz = 1000.0;
                d3 bp = dk3(invP[0] * px + invP[1] * py + invP[2] * pz + invP[3],
                            invP[4] * px + invP[5] * py + invP[6] * pz + invP[7],
                            invP[8] * px + invP[9] * py + invP[10] * pz + invP[11]);
                d3 d = dnormalize(dsub(bp, o));
                int i0 = s->faces[3 * f], i1 = s->faces[3 * f + 1], i2 = s->faces[3 * f + 2];
                d3 v0 = VD(i0), v1 = VD(i1), v2 = VD(i2);
                d3 Nf = dcross(dsub(v1, v0), dsub(v2, v0));
                double t = ddot(dsub(v0, o), Nf) / ddot(d, Nf);
                d3 P = dadd(o, dscale(t, d));
                double den = ddot(Nf, Nf);
                double a = ddot(Nf, dcross(dsub(v2, v1), dsub(P, v1))) / den;
                double b = ddot(Nf, dcross(dsub(v0, v2), dsub(P, v2))) / den;
                double cc = 1.0 - a - b;
                d3 un = dadd(dadd(dscale(a, vn[i0]), dscale(b, vn[i1])), dscale(cc, vn[i2]));
                d3 n = dnormalize(un);
                int flip = ddot(n, d) > 0.0;
                if (flip) n = dscale(-1.0, n);
                if (flags_out) {
                    /* 1: normal flipped; 2: grazing face (|cos| < 0.002); 4: interpolated normal within
                     * 0.01 of perpendicular to the ray, where a small change of the inputs can flip it */
                    double cosv = fabs(ddot(d, Nf)) / sqrt(den);
                    flags_out[p] = flip | ((cosv < 0.002) << 1) | ((fabs(ddot(n, d)) < 0.01) << 2);
                }
                d3 col;
                if (s->albedo_mode == ORC_TEXTURED) {
                    const float *tt = s->uvs + (size_t)f * 6;
                    double U = (tt[0] * a + tt[2] * b + tt[4] * cc) * s->Wt;
                    double V = ((1.0 - tt[1]) * a + (1.0 - tt[3]) * b + (1.0 - tt[5]) * cc) * s->Ht;
                    U = fmin(fmax(U, 0.0), s->Wt - 1.0);
                    V = fmin(fmax(V, 0.0), s->Ht - 1.0);
                    int LU = (int)(U - 0.5), LV = (int)(V - 0.5);
                    col = ldd3(s->texture + ((size_t)LV * s->Wt + LU) * 3);
                } else if (s->albedo_mode == ORC_VERTEX_COLOR) {
                    col = dadd(dadd(dscale(a, CD(i0)), dscale(b, CD(i1))), dscale(cc, CD(i2)));
                } else if (s->albedo_mode == ORC_NORMAL) {
                    col = dk3((1.0 + n.x) / 2.0, (1.0 + n.y) / 2.0, (1.0 + n.z) / 2.0);
                } else if (s->albedo_mode == ORC_TEXTURED_BILINEAR) {
                    const float *tt = s->uvs + (size_t)f * 6;
                    double U = (tt[0] * a + tt[2] * b + tt[4] * cc) * s->Wt;
                    double V = ((1.0 - tt[1]) * a + (1.0 - tt[3]) * b + (1.0 - tt[5]) * cc) * s->Ht;
                    U = fmin(fmax(U, 0.0), s->Wt - 1.0) - 0.5;
                    V = fmin(fmax(V, 0.0), s->Ht - 1.0) - 0.5;
                    double x0 = floor(U), y0 = floor(V), fx = U - x0, fy = V - y0;
                    int ix[2] = {(int)x0, (int)x0 + 1}, iy[2] = {(int)y0, (int)y0 + 1};
                    for (int k = 0; k < 2; ++k) {
                        ix[k] = ix[k] < 0 ? 0 : ix[k] > s->Wt - 1 ? s->Wt - 1 : ix[k];
                        iy[k] = iy[k] < 0 ? 0 : iy[k] > s->Ht - 1 ? s->Ht - 1 : iy[k];
                    }
                    col = dk3(0, 0, 0);
                    for (int ky = 0; ky < 2; ++ky)
                        for (int kx = 0; kx < 2; ++kx) {
                            double w = (kx ? fx : 1.0 - fx) * (ky ? fy : 1.0 - fy);
                            col = dadd(col, dscale(w, ldd3(s->texture + ((size_t)iy[ky] * s->Wt + ix[kx]) * 3)));
                        }
                } else if (s->albedo_mode == ORC_UV) {
                    col = uv_colour(s, f, a, b, cc);
                } else {
                    col = dk3(1, 1, 1);
                }
                int lit = s->albedo_mode != ORC_NORMAL && s->albedo_mode != ORC_UV;
                int shaded = (s->shading_mode == ORC_SHADED && lit) || s->albedo_mode == ORC_LIGHTING;
                if (s->albedo_mode == ORC_FOREGROUND) shaded = 0;
                if (s->shading_mode == ORC_PHONG && lit && s->albedo_mode != ORC_LIGHTING &&
                    s->albedo_mode != ORC_FOREGROUND) {
                    double ndl = -ddot(n, d);
                    double k = phong_factor(ndl), sp = phong_specular(ndl);
                    col = dk3(col.x * k + sp, col.y * k + sp, col.z * k + sp);
                } else if (shaded) {
                    d3 l = sh_light_d(n, sh);
                    col = dk3(l.x * col.x, l.y * col.y, l.z * col.z);
                }
                out[0] = col.x; out[1] = col.y; out[2] = col.z;
            }
    }
    free(fn); free(vn);
    free_csr(&csr);
}

/* ------------------------------------------------------------------------- */
/* Normal-map mode (compute_normal_map). */

/* Texture-space face map (CUDABasedRasterization.cpp:241-294): each face's
 * UV triangle in texel units (Wt*u, Ht*(1-v), 0), its box widened by 2
 * texels, and per texel the host ray/triangle test (rayTriangleIntersectHost,
 * :158-236, the same arithmetic as barycentric() above) of the ray from
 * (x+.5, y+.5, 1) along -z.  Faces run in ascending order and a later face
 * overwrites, as the reference's loop does when run serially.
 * owner_out [Ht*Wt] = face or -1; abc_out [Ht*Wt*3] = (a, b, c) or 0. */
void orc_uv_face_map(const float *uvs, int F, int Ht, int Wt, int32_t *owner_out, float *abc_out) {
    for (long i = 0; i < (long)Ht * Wt; ++i) {
        owner_out[i] = -1;
        abc_out[3 * i] = abc_out[3 * i + 1] = abc_out[3 * i + 2] = 0.0f;
    }
    const f3 dir = mk3(0.0f, 0.0f, -1.0f);
    for (int f = 0; f < F; ++f) {
        const float *t = uvs + 6 * (size_t)f;
        f3 t0 = mk3((float)Wt * t[0], (float)Ht * (1.0f - t[1]), 0.0f);
        f3 t1 = mk3((float)Wt * t[2], (float)Ht * (1.0f - t[3]), 0.0f);
        f3 t2 = mk3((float)Wt * t[4], (float)Ht * (1.0f - t[5]), 0.0f);
        /* int(fmax(min - 2, 0)) .. int(fmin(max + 2, size)), exclusive upper bound */
        double lx = fmax(fminf(t0.x, fminf(t1.x, t2.x)) - 2.0f, 0.0);
        double hx = fmin(fmaxf(t0.x, fmaxf(t1.x, t2.x)) + 2.0f, (double)Wt);
        double ly = fmax(fminf(t0.y, fminf(t1.y, t2.y)) - 2.0f, 0.0);
        double hy = fmin(fmaxf(t0.y, fmaxf(t1.y, t2.y)) + 2.0f, (double)Ht);
        int x0 = (int)lx, y0 = (int)ly;
        int x1 = hx > 0.0 ? (int)hx : 0, y1 = hy > 0.0 ? (int)hy : 0;
        for (int x = x0; x < x1; ++x)
            for (int y = y0; y < y1; ++y) {
                f3 abc = barycentric(mk3(x + 0.5f, y + 0.5f, 1.0f), dir, t0, t1, t2);
                if (abc.x != -1.0f && abc.y != -1.0f && abc.z != -1.0f) {
                    long i = (long)y * Wt + x;
                    owner_out[i] = f;
                    abc_out[3 * i] = abc.x; abc_out[3 * i + 1] = abc.y; abc_out[3 * i + 2] = abc.z;
                }
            }
    }
}

/* renderNormalMapDevice (CUDABasedRasterization.cu:415-445) from a face map:
 * the barycentric blend of the owner's vertex normals vn [N*3], normalised
 * when non-zero, mapped to (n+1)/2.  Uncovered texels read face 0 with zero
 * weights, i.e. (0.5, 0.5, 0.5).  out [Ht*Wt*3], FP32 like the reference. */
void orc_normal_map_from(const int32_t *faces, const float *vn, const int32_t *owner, const float *abc, int Ht,
                         int Wt, float *out) {
    for (long i = 0; i < (long)Ht * Wt; ++i) {
        int f = owner[i] >= 0 ? owner[i] : 0;
        f3 w = mk3(abc[3 * i], abc[3 * i + 1], abc[3 * i + 2]);
        f3 n0 = ld3(vn + 3 * faces[3 * f]), n1 = ld3(vn + 3 * faces[3 * f + 1]), n2 = ld3(vn + 3 * faces[3 * f + 2]);
        f3 n = mk3(n0.x * w.x + n1.x * w.y + n2.x * w.z, n0.y * w.x + n1.y * w.y + n2.y * w.z,
                   n0.z * w.x + n1.z * w.y + n2.z * w.z);
        float len = sqrtf(dot3(n, n));
        if (len != 0.0f) n = sdiv3(n, len);
        out[3 * i] = (n.x + 1.0f) / 2.0f;
        out[3 * i + 1] = (n.y + 1.0f) / 2.0f;
        out[3 * i + 2] = (n.z + 1.0f) / 2.0f;
    }
}

/* The whole normal-map forward of one batch element: vertex normals of the
 * scene's vertices, face map at the scene's texture size, normal map. */
void orc_normal_map(const orc_scene *s, float *out /*[Ht*Wt*3]*/) {
    csr_t csr;
    build_csr(s->N, s->F, s->faces, &csr);
    float *vn = (float *)malloc((size_t)s->N * 3 * sizeof(float));
    vertex_normals(s, &csr, vn);
    int32_t *owner = (int32_t *)malloc((size_t)s->Ht * s->Wt * sizeof(int32_t));
    float *abc = (float *)malloc((size_t)s->Ht * s->Wt * 3 * sizeof(float));
    orc_uv_face_map(s->uvs, s->F, s->Ht, s->Wt, owner, abc);
    orc_normal_map_from(s->faces, vn, owner, abc, s->Ht, s->Wt, out);
    free(abc); free(owner); free(vn);
    free_csr(&csr);
}

void orc_render_fp64(const orc_scene *s, const double *verts_d, const int32_t *face, double *render_out,
                     int32_t *flags_out) {
    orc_render_fp64_ex(s, verts_d, NULL, NULL, face, render_out, flags_out);
}

int orc_max_ties(void) { return ORC_MAX_TIES; }

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

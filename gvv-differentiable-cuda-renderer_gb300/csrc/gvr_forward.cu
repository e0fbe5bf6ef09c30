// gvr_forward.cu -- forward render: cameras, face setup, vertex stage and
// tile binning; the raster + resolve + shade kernel is in gvr_raster.cu.
//
// Pipeline for all B x C views of one call (reference: the 7-kernel chain
// of cpp/src/Renderer/CUDABasedRasterization.cu:449-473, launched once per
// batch element there):
//   k_setup       camera inverses (:23-67), scaled face geometry and
//                 face normals (:122-141), cleared counters    B*F + B*C + clear
//   k_vertices    vertex normals (:148-174) + projection (:98-115) B*N*min(C,4)
//   k_bin_count   face boxes (:184-208), screen-space skip-test
//                 constants, per-tile counts                     B*C*F threads
//   k_scan_tiles  exclusive scan of the tile counts              8192 per block
//   k_bin_fill    per-tile face lists                            B*C*F threads
//   k_raster      one tile per block (replaces :215-408)
//
// Each stage is a per-item device function of a FwdJob.  The *_batched
// kernels run the same functions over many jobs (meshes of different sizes,
// modes and resolutions) in one launch per stage: blockStart[j] is the
// first block of job j, so every block belongs to one job.
#include "gvr_internal.cuh"
#include "gvr_kernels.h"
#include "gvr_profile.h"

namespace gvr {

// ---------------------------------------------------------------------------- cameras

__device__ static void mat4_mul_x(const float *a, const float *b, float *r) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
            r[4 * i + j] = xa(xa(xa(xm(a[4 * i + 0], b[j]), xm(a[4 * i + 1], b[4 + j])), xm(a[4 * i + 2], b[8 + j])),
                              xm(a[4 * i + 3], b[12 + j]));
}

// T3(a,b,c) = (a*b)*c, evaluated left to right as the reference's products.
__device__ __forceinline__ float T3(float a, float b, float c) { return xm(xm(a, b), c); }

// Cofactor inverse of a row-major 4x4 (float4x4::getInverse,
// cpp/src/Utils/float4x4.h:160-282): the same cofactor expressions summed
// left to right, then multiplied by 1/det.
__device__ static void mat4_inverse_x(const float *e, float *out) {
    float inv[16];
    inv[0] = xs(xa(xa(xs(xs(T3(e[5], e[10], e[15]), T3(e[5], e[11], e[14])), T3(e[9], e[6], e[15])), T3(e[9], e[7], e[14])),
                   T3(e[13], e[6], e[11])), T3(e[13], e[7], e[10]));
    inv[4] = xa(xs(xs(xa(xa(-T3(e[4], e[10], e[15]), T3(e[4], e[11], e[14])), T3(e[8], e[6], e[15])), T3(e[8], e[7], e[14])),
                   T3(e[12], e[6], e[11])), T3(e[12], e[7], e[10]));
    inv[8] = xs(xa(xa(xs(xs(T3(e[4], e[9], e[15]), T3(e[4], e[11], e[13])), T3(e[8], e[5], e[15])), T3(e[8], e[7], e[13])),
                   T3(e[12], e[5], e[11])), T3(e[12], e[7], e[9]));
    inv[12] = xa(xs(xs(xa(xa(-T3(e[4], e[9], e[14]), T3(e[4], e[10], e[13])), T3(e[8], e[5], e[14])), T3(e[8], e[6], e[13])),
                    T3(e[12], e[5], e[10])), T3(e[12], e[6], e[9]));
    inv[1] = xa(xs(xs(xa(xa(-T3(e[1], e[10], e[15]), T3(e[1], e[11], e[14])), T3(e[9], e[2], e[15])), T3(e[9], e[3], e[14])),
                   T3(e[13], e[2], e[11])), T3(e[13], e[3], e[10]));
    inv[5] = xs(xa(xa(xs(xs(T3(e[0], e[10], e[15]), T3(e[0], e[11], e[14])), T3(e[8], e[2], e[15])), T3(e[8], e[3], e[14])),
                   T3(e[12], e[2], e[11])), T3(e[12], e[3], e[10]));
    inv[9] = xa(xs(xs(xa(xa(-T3(e[0], e[9], e[15]), T3(e[0], e[11], e[13])), T3(e[8], e[1], e[15])), T3(e[8], e[3], e[13])),
                   T3(e[12], e[1], e[11])), T3(e[12], e[3], e[9]));
    inv[13] = xs(xa(xa(xs(xs(T3(e[0], e[9], e[14]), T3(e[0], e[10], e[13])), T3(e[8], e[1], e[14])), T3(e[8], e[2], e[13])),
                    T3(e[12], e[1], e[10])), T3(e[12], e[2], e[9]));
    inv[2] = xs(xa(xa(xs(xs(T3(e[1], e[6], e[15]), T3(e[1], e[7], e[14])), T3(e[5], e[2], e[15])), T3(e[5], e[3], e[14])),
                   T3(e[13], e[2], e[7])), T3(e[13], e[3], e[6]));
    inv[6] = xa(xs(xs(xa(xa(-T3(e[0], e[6], e[15]), T3(e[0], e[7], e[14])), T3(e[4], e[2], e[15])), T3(e[4], e[3], e[14])),
                   T3(e[12], e[2], e[7])), T3(e[12], e[3], e[6]));
    inv[10] = xs(xa(xa(xs(xs(T3(e[0], e[5], e[15]), T3(e[0], e[7], e[13])), T3(e[4], e[1], e[15])), T3(e[4], e[3], e[13])),
                    T3(e[12], e[1], e[7])), T3(e[12], e[3], e[5]));
    inv[14] = xa(xs(xs(xa(xa(-T3(e[0], e[5], e[14]), T3(e[0], e[6], e[13])), T3(e[4], e[1], e[14])), T3(e[4], e[2], e[13])),
                    T3(e[12], e[1], e[6])), T3(e[12], e[2], e[5]));
    inv[3] = xa(xs(xs(xa(xa(-T3(e[1], e[6], e[11]), T3(e[1], e[7], e[10])), T3(e[5], e[2], e[11])), T3(e[5], e[3], e[10])),
                   T3(e[9], e[2], e[7])), T3(e[9], e[3], e[6]));
    inv[7] = xs(xa(xa(xs(xs(T3(e[0], e[6], e[11]), T3(e[0], e[7], e[10])), T3(e[4], e[2], e[11])), T3(e[4], e[3], e[10])),
                   T3(e[8], e[2], e[7])), T3(e[8], e[3], e[6]));
    inv[11] = xa(xs(xs(xa(xa(-T3(e[0], e[5], e[11]), T3(e[0], e[7], e[9])), T3(e[4], e[1], e[11])), T3(e[4], e[3], e[9])),
                    T3(e[8], e[1], e[7])), T3(e[8], e[3], e[5]));
    inv[15] = xs(xa(xa(xs(xs(T3(e[0], e[5], e[10]), T3(e[0], e[6], e[9])), T3(e[4], e[1], e[10])), T3(e[4], e[2], e[9])),
                    T3(e[8], e[1], e[6])), T3(e[8], e[2], e[5]));
    float det = xa(xa(xa(xm(e[0], inv[0]), xm(e[1], inv[4])), xm(e[2], inv[8])), xm(e[3], inv[12]));
    float detr = xd(1.0f, det);
#pragma unroll
    for (int i = 0; i < 16; ++i) out[i] = xm(inv[i], detr);
}

__device__ __forceinline__ void camera_item(const float *__restrict__ extr, const float *__restrict__ intr,
                                            Camera *__restrict__ cams, int i) {
    const float *e12 = extr + 12 * (size_t)i, *k9 = intr + 9 * (size_t)i;
    float E[16], K[16], KE[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) E[j] = K[j] = (j % 5 == 0) ? 1.0f : 0.0f;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        K[4 * r + 0] = k9[3 * r + 0];
        K[4 * r + 1] = k9[3 * r + 1];
        K[4 * r + 2] = k9[3 * r + 2];
        K[4 * r + 3] = 0.0f;
        E[4 * r + 0] = e12[4 * r + 0];
        E[4 * r + 1] = e12[4 * r + 1];
        E[4 * r + 2] = e12[4 * r + 2];
        E[4 * r + 3] = e12[4 * r + 3];
    }
    Camera &cam = cams[i];
    mat4_inverse_x(E, cam.invE);
    mat4_mul_x(K, E, KE);
    mat4_inverse_x(KE, cam.invP);
    float ow = cam.invE[15];
    cam.orig[0] = xd(cam.invE[3], ow);
    cam.orig[1] = xd(cam.invE[7], ow);
    cam.orig[2] = xd(cam.invE[11], ow);
    cam.orig[3] = 1.0f;
#pragma unroll
    for (int j = 0; j < 3; ++j) cam.origS[j] = xd(cam.orig[j], 1000.0f);
    cam.origS[3] = 0.0f;
    cam.origLen = sqrtf(cam.orig[0] * cam.orig[0] + cam.orig[1] * cam.orig[1] + cam.orig[2] * cam.orig[2]);
#pragma unroll
    for (int j = 0; j < 12; ++j) { cam.KE[j] = KE[j]; cam.E[j] = e12[j]; }
#pragma unroll
    for (int j = 0; j < 9; ++j) cam.K[j] = k9[j];
}

// ---------------------------------------------------------------------------- face setup

// rec (backward only, else null): the face's BwdScratch::faceRec record;
// uvs may be null (no texture coordinates: zeros).
__device__ __forceinline__ void face_geo_item(const float *__restrict__ verts, const int32_t *__restrict__ faces,
                                              FaceGeo *__restrict__ geo, float4 *__restrict__ fnormal, int N, int F,
                                              int i, float4 *__restrict__ rec = nullptr,
                                              const float *__restrict__ uvs = nullptr,
                                              float4 *__restrict__ faceC = nullptr) {
    int b = i / F, f = i - b * F;
    const float *V = verts + (size_t)b * N * 3;
    int i0 = faces[3 * f], i1 = faces[3 * f + 1], i2 = faces[3 * f + 2];
    V3 p0 = ld3(V + 3 * i0), p1 = ld3(V + 3 * i1), p2 = ld3(V + 3 * i2);
    if (rec) {
        float t[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        if (uvs)
            for (int k = 0; k < 6; ++k) t[k] = uvs[6 * (size_t)f + k];
        float4 *R = rec + (size_t)i * kBwdFaceRows;
        R[0] = make_float4(__int_as_float(i0), __int_as_float(i1), __int_as_float(i2), t[0]);
        R[1] = make_float4(t[1], t[2], t[3], t[4]);
        R[2] = make_float4(t[5], p0.x, p0.y, p0.z);
        R[3] = make_float4(p1.x, p1.y, p1.z, p2.x);
        R[4] = make_float4(p2.y, p2.z, 0.0f, 0.0f);
    }
    V3 fn = xcross(xsub(p1, p0), xsub(p2, p0));
    const float fnLen = sqrtf(fn.x * fn.x + fn.y * fn.y + fn.z * fn.z);
    if (fnormal) fnormal[i] = make_float4(fn.x, fn.y, fn.z, fnLen);
    if (faceC) {  // what the binning pass's skip-test margins need of the face, whatever the view
        auto elen = [](V3 a, V3 c) {
            return sqrtf((a.x - c.x) * (a.x - c.x) + (a.y - c.y) * (a.y - c.y) + (a.z - c.z) * (a.z - c.z));
        };
        const float maxEdge = fmaxf(elen(p0, p1), fmaxf(elen(p1, p2), elen(p2, p0)));
        faceC[i] = make_float4((p0.x + p1.x + p2.x) * (1.0f / 3.0f), (p0.y + p1.y + p2.y) * (1.0f / 3.0f),
                               (p0.z + p1.z + p2.z) * (1.0f / 3.0f), fnLen / maxEdge);
    }
    // rayTriangleIntersect scales vertices by 1/1000 (RendererUtil.h:29-32)
    V3 s0 = v3(xd(p0.x, 1000.0f), xd(p0.y, 1000.0f), xd(p0.z, 1000.0f));
    V3 s1 = v3(xd(p1.x, 1000.0f), xd(p1.y, 1000.0f), xd(p1.z, 1000.0f));
    V3 s2 = v3(xd(p2.x, 1000.0f), xd(p2.y, 1000.0f), xd(p2.z, 1000.0f));
    V3 n = xcross(xsub(s1, s0), xsub(s2, s0));
    FaceGeo g;
    g.a = make_float4(s0.x, s0.y, s0.z, s1.x);
    g.b = make_float4(s1.y, s1.z, s2.x, s2.y);
    g.c = make_float4(s2.z, n.x, n.y, n.z);
    g.d = make_float4(xdot(s0, n), xdot(n, n), 0.0f, 0.0f);
    geo[i] = g;
}

// ---------------------------------------------------------------------------- vertex stage

// Vertex i for views sub, sub + lanes, ...: `lanes` threads share a vertex,
// each summing its normal (in the same order, so to the same bits; their
// loads are the same addresses) and projecting it into its share of views.
__device__ __forceinline__ void vertex_item(const FwdJob &J, int i, int sub = 0, int lanes = 1) {
    const Topology &topo = J.topo;
    const int N = topo.N, F = topo.F, C = J.dims.C;
    int b = i / N, v = i - b * N;
    // vertex normal = sum of adjacent face normals in ascending face order
    V3 acc = v3(0.0f, 0.0f, 0.0f);
    int s = topo.vstart[v], e = topo.vstart[v + 1];
    for (int k = s; k < e; ++k) {
        float4 n = J.ws.fnormal[(size_t)b * F + topo.vfaces[k]];
        if (k == s) acc = v3(n.x, n.y, n.z);
        else acc = v3(xa(acc.x, n.x), xa(acc.y, n.y), xa(acc.z, n.z));
    }
    V3 p = ld3(J.io.verts + (size_t)i * 3);
    for (int c = sub; c < C; c += lanes) {
        size_t o = ((size_t)b * C + c) * N + v;
        float *dst = J.vnormal_out + o * 3;
        dst[0] = acc.x;
        dst[1] = acc.y;
        dst[2] = acc.z;
        // getCamSpacePoint + projectPointFloat3 (CameraUtil.h:141-186)
        const Camera &cam = J.ws.cams[b * C + c];
        const float *E = cam.E, *K = cam.K;
        float cx = xa(xa(xa(xm(E[0], p.x), xm(E[1], p.y)), xm(E[2], p.z)), xm(E[3], 1.0f));
        float cy = xa(xa(xa(xm(E[4], p.x), xm(E[5], p.y)), xm(E[6], p.z)), xm(E[7], 1.0f));
        float cz = xa(xa(xa(xm(E[8], p.x), xm(E[9], p.y)), xm(E[10], p.z)), xm(E[11], 1.0f));
        float x = xa(xa(xm(cx, K[0]), xm(cy, K[1])), xm(cz, K[2]));
        float y = xa(xa(xm(cx, K[3]), xm(cy, K[4])), xm(cz, K[5]));
        float z = xa(xa(xm(cx, K[6]), xm(cy, K[7])), xm(cz, K[8]));
        if (z > 0.0000001f) {
            x = xd(x, z);
            y = xd(y, z);
        } else {
            z = 0.00001f;
            x = xd(x, z);
            y = xd(y, z);
        }
        J.proj[o] = make_float4(x, y, z, 0.0f);
    }
}

// ---------------------------------------------------------------------------- binning

__device__ __forceinline__ int4 face_box(float4 p0, float4 p1, float4 p2, int W, int H) {
    // projectFacesDevice (CUDABasedRasterization.cu:202-206): float boxes
    // converted to int by truncation.
    int4 r;
    r.x = __float2int_rz(fmaxf(xs(fminf(p0.x, fminf(p1.x, p2.x)), 0.5f), 0.0f));
    r.y = __float2int_rz(fmaxf(xs(fminf(p0.y, fminf(p1.y, p2.y)), 0.5f), 0.0f));
    r.z = __float2int_rz(fminf(xa(fmaxf(p0.x, fmaxf(p1.x, p2.x)), 0.5f), (float)(W - 1)));
    r.w = __float2int_rz(fminf(xa(fmaxf(p0.y, fmaxf(p1.y, p2.y)), 0.5f), (float)(H - 1)));
    return r;
}

// Runs of equal keys in consecutive lanes of the converged group `act`:
// whether this lane heads its run, its rank in the run, the run's length (in
// the head) and the head's lane.  Faces next to each other in index order
// are neighbours on the mesh, so the lanes of a warp meet a tile mostly in
// runs: one atomic per run stands in for one per lane, found with a shuffle
// and a ballot (a match over the warp keeps the address-divergence unit busy
// and stalls the binning kernels).
struct KeyRun {
    bool head;
    int rank, len, headLane;
};

__device__ __forceinline__ KeyRun key_run(unsigned act, long long key, int lane) {
    const unsigned below = act & ((1u << lane) - 1u);
    const int prevLane = below ? 31 - __clz(below) : lane;
    const long long prev = __shfl_sync(act, key, prevLane);
    KeyRun r;
    r.head = !below || prev != key;
    const unsigned heads = __ballot_sync(act, r.head);
    r.headLane = 31 - __clz(heads & ((2u << lane) - 1u));  // (2u << 31) - 1 = all lanes
    r.rank = __popc(below & ~((1u << r.headLane) - 1u));
    const unsigned after = heads & ~((2u << lane) - 1u);
    const int end = after ? __ffs(after) - 1 : 32;
    const unsigned upto = end == 32 ? 0xffffffffu : ((1u << end) - 1u);
    r.len = __popc(act & upto & ~((1u << lane) - 1u));
    return r;
}

__device__ __forceinline__ void bin_count_item(const FwdJob &J, int i) {
    const Topology &topo = J.topo;
    const FrameDims &dims = J.dims;
    const FwdScratch &ws = J.ws;
    const int F = topo.F, N = topo.N;
    int bc = i / F, f = i - bc * F, b = bc / dims.C;
    const int i0 = topo.faces[3 * f], i1 = topo.faces[3 * f + 1], i2 = topo.faces[3 * f + 2];
    const float4 *P = J.proj + (size_t)bc * N;
    float4 p0 = P[i0], p1 = P[i1], p2 = P[i2];
    int4 box = face_box(p0, p1, p2, dims.W, dims.H);
    if (box.x > box.z || box.y > box.w) box = make_int4(1, 1, 0, 0);
    // screen-space barycentric setup and the error bounds of the skip tests
    const float ex1 = p1.x - p0.x, ey1 = p1.y - p0.y, ex2 = p2.x - p0.x, ey2 = p2.y - p0.y;
    const float det = ex1 * ey2 - ey1 * ex2;
    const float zmn = fminf(p0.z, fminf(p1.z, p2.z)), zmx = fmaxf(p0.z, fmaxf(p1.z, p2.z));
    const Camera &cam = ws.cams[bc];
    const float4 fn = ws.fnormal[(size_t)b * F + f];  // w: its length
    const float4 fc = ws.faceC[(size_t)b * F + f];    // centroid, smallest altitude (mm)
    const float cx = fc.x, cy = fc.y, cz = fc.z, alt = fc.w, fnLen = fn.w;
    const float vx = cx - cam.orig[0], vy = cy - cam.orig[1], vz = cz - cam.orig[2];
    const float dist = sqrtf(vx * vx + vy * vy + vz * vz);
    const float cosv = fabsf(fn.x * vx + fn.y * vy + fn.z * vz) / (fnLen * dist);
    const float sEdge = fmaxf(sqrtf(ex1 * ex1 + ey1 * ey1), fmaxf(sqrtf(ex2 * ex2 + ey2 * ey2),
                              sqrtf((p2.x - p1.x) * (p2.x - p1.x) + (p2.y - p1.y) * (p2.y - p1.y))));
    const float altPx = fabsf(det) / sEdge;  // smallest screen altitude, pixels
    const float scale = cam.origLen + sqrtf(cx * cx + cy * cy + cz * cz) + dist;
    const bool valid = zmn >= 1.0f && zmx <= 64.0f * zmn && fabsf(det) > 1e-6f && isfinite(det) &&
                       isfinite(p0.x + p1.x + p2.x + p0.y + p1.y + p2.y) && isfinite(cosv) && alt > 0.0f;
    int flags = 0;
    float mIn = 2.0f, mOut = 0.0f, dRel = 1.0f;
    float4 s1 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (valid) {
        const float zr = zmx / zmn;
        const float idet = 1.0f / det;
        s1 = make_float4(ey2 * idet, -ex2 * idet, -ey1 * idet, ex1 * idet);
        // exact-test barycentric error: hit point off by ~eps*scale/cos along the ray
        const float eb = (4.0f * 6e-8f * scale / fmaxf(cosv, 1e-6f) + 4.0f * 6e-8f * scale) / alt + 1e-5f;
        // screen barycentric error: ~3e-4 px of projection and ray-direction error
        const float es = 3e-4f / altPx + 1e-6f;
        mIn = (2.0f * (eb + es) + 1e-4f) * zr;
        mOut = mIn + 2e-3f * zr;
        dRel = 2.0f * (eb + es) * (zr - 1.0f) + 1e-4f;
        // certainly accepted needs |N.d| (scaled units) clear of the 1e-7 parallel test
        const bool clear = fnLen * 1e-6f * cosv >= 4e-7f;
        flags = kScreenValid | ((cosv >= 0.02f && clear && mIn < 0.2f) ? kCertain : 0);
    }
    if (bc - b * dims.C == 0) {  // view 0 writes the face's shading record (vertex normals of view 0)
        const float *VN = J.vnormal_out + (size_t)bc * N * 3;
        const float *t = topo.uvs + 6 * (size_t)f;
        const V3 n0 = ld3(VN + 3 * i0), n1 = ld3(VN + 3 * i1), n2 = ld3(VN + 3 * i2);
        float4 *R = ws.shadeRec + ((size_t)b * F + f) * kShadeRows;
        R[0] = make_float4(n0.x, n0.y, n0.z, n1.x);
        R[1] = make_float4(n1.y, n1.z, n2.x, n2.y);
        R[2] = make_float4(n2.z, t[0], t[1], t[2]);
        R[3] = make_float4(t[3], t[4], t[5], 0.0f);
        R[4] = make_float4(__int_as_float(i0), __int_as_float(i1), __int_as_float(i2), 0.0f);
    }
    ViewFace vf;
    vf.hdr = make_int4(box.x | (box.z << 16), box.y | (box.w << 16), flags, __float_as_int(dRel));
    vf.z = make_float4(p0.z, p1.z, p2.z, mIn);
    // any accepted depth is >= zmin / 1.002 when all z > 0 and z_max / z_min is moderate
    // (barycentrics >= -0.001 summing to 1); otherwise no bound
    vf.s0 = make_float4(p0.x, p0.y, mOut, valid ? zmn * (10000.0f / 1.0025f) - 2.0f : -__int_as_float(0x7f800000));
    vf.s1 = s1;
    ws.vface[i] = vf;
    // the view's range of finite, non-negative depth bounds (the raster's
    // depth buckets span it): one pair of atomics per view per warp
    {
        const bool ranged = box.x <= box.z && box.y <= box.w && vf.s0.w >= 0.0f && vf.s0.w < __int_as_float(0x7f800000);
        const unsigned bits = __float_as_uint(vf.s0.w);
        const unsigned act = __activemask();
        const int lane = threadIdx.x & 31;
        unsigned pending = act;
        while (pending) {  // the distinct views of the warp's items (two at most when F >= 32)
            const int first = __ffs(pending) - 1;
            const bool mine = __shfl_sync(act, bc, first) == bc;
            const unsigned hiBits = __reduce_max_sync(act, mine && ranged ? bits : 0u);
            const unsigned loInv = __reduce_max_sync(act, mine && ranged ? ~bits : 0u);
            if (lane == first && hiBits) {
                atomicMax(&ws.zRange[2 * bc], loInv);
                atomicMax(&ws.zRange[2 * bc + 1], hiBits);
            }
            pending &= ~__ballot_sync(act, mine);
        }
    }
    if (box.x > box.z || box.y > box.w) return;
    const int sh = dims.tileShift, tH = dims.tileH;
    int tx0 = box.x >> sh, tx1 = box.z >> sh, ty0 = box.y / tH, ty1 = box.w / tH;
    int nt = (tx1 - tx0 + 1) * (ty1 - ty0 + 1);
    const int T = dims.tilesX * dims.tilesY;
    if (nt > dims.bigTiles) {
        int k = atomicAdd(&ws.bigCount[bc], 1);
        ws.bigList[(size_t)bc * F + k] = f;
        return;
    }
    // One atomic per run of lanes meeting the same tile in a round: the lanes
    // of a warp hold neighbouring faces, which share most of their tiles.
    const unsigned act = __activemask();
    const int lane = threadIdx.x & 31, w = tx1 - tx0 + 1;
    const int rounds = __reduce_max_sync(act, nt);
    for (int r = 0; r < rounds; ++r) {
        const long long key = r < nt ? (long long)bc * T + (ty0 + r / w) * dims.tilesX + tx0 + r % w : -1ll;
        const KeyRun R = key_run(act, key, lane);
        if (key >= 0 && R.head) atomicAdd(&ws.tileCount[key], R.len);
    }
}

// Exclusive scan of count[0..n) into start[0..n], start[n] = total, by one
// block of 1024 threads, 8192 counts per pass: each thread loads 8
// consecutive counts (two 16-byte loads when aligned), one block scan of
// the per-thread sums, then each thread writes its 8 starts.
__device__ __forceinline__ void scan_block(const int *__restrict__ count, int *__restrict__ start, int n) {
    __shared__ int warpSum[32];
    __shared__ int carry;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool vec = ((reinterpret_cast<uintptr_t>(count) | reinterpret_cast<uintptr_t>(start)) & 15) == 0;
    if (tid == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 8192) {
        const int i0 = base + 8 * tid;
        int x[8];
        if (vec && i0 + 8 <= n) {
            const int4 a = *reinterpret_cast<const int4 *>(count + i0), c = *reinterpret_cast<const int4 *>(count + i0 + 4);
            x[0] = a.x, x[1] = a.y, x[2] = a.z, x[3] = a.w, x[4] = c.x, x[5] = c.y, x[6] = c.z, x[7] = c.w;
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k) x[k] = i0 + k < n ? count[i0 + k] : 0;
        }
        int sum = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) sum += x[k];
        int incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warpSum[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const int w = warpSum[lane];
            int wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += y;
            }
            warpSum[lane] = wi - w;  // exclusive prefix of warp sums
        }
        __syncthreads();
        int run = carry + warpSum[warp] + incl - sum;
        int st[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            st[k] = run;
            run += x[k];
        }
        if (vec && i0 + 8 <= n) {
            *reinterpret_cast<int4 *>(start + i0) = make_int4(st[0], st[1], st[2], st[3]);
            *reinterpret_cast<int4 *>(start + i0 + 4) = make_int4(st[4], st[5], st[6], st[7]);
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k)
                if (i0 + k < n) start[i0 + k] = st[k];
        }
        __syncthreads();  // every thread has read carry
        if (tid == 1023) carry = run;
        __syncthreads();
    }
    if (tid == 0) start[n] = carry;
}

__device__ __forceinline__ void bin_fill_item(const FwdJob &J, int i) {
    const FrameDims &dims = J.dims;
    const FwdScratch &ws = J.ws;
    const int F = J.topo.F;
    int bc = i / F, f = i - bc * F;
    int4 box = vf_box(ws.vface[i]);
    if (box.x > box.z || box.y > box.w) return;
    const int sh = dims.tileShift, tH = dims.tileH;
    int tx0 = box.x >> sh, tx1 = box.z >> sh, ty0 = box.y / tH, ty1 = box.w / tH;
    const int w = tx1 - tx0 + 1, nt = w * (ty1 - ty0 + 1);
    if (nt > dims.bigTiles) return;
    const int T = dims.tilesX * dims.tilesY;
    // as in the count: one atomic per run of lanes meeting the same tile in a
    // round, the run's slots handed out by rank
    const unsigned act = __activemask();
    const int lane = threadIdx.x & 31;
    const int rounds = __reduce_max_sync(act, nt);
    for (int r = 0; r < rounds; ++r) {
        const long long key = r < nt ? (long long)bc * T + (ty0 + r / w) * dims.tilesX + tx0 + r % w : -1ll;
        const KeyRun R = key_run(act, key, lane);
        int slot = 0;
        if (key >= 0 && R.head) slot = atomicAdd(&ws.tileCursor[key], R.len);
        slot = __shfl_sync(act, slot, R.headLane) + R.rank;
        if (key >= 0) ws.bins[ws.tileStart[key] + slot] = f;
    }
}

// ---------------------------------------------------------------------------- single-call kernels

__global__ void k_cameras(const float *__restrict__ extr, const float *__restrict__ intr, Camera *__restrict__ cams,
                          int count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) camera_item(extr, intr, cams, i);
}

__global__ void k_face_geo(const float *__restrict__ verts, const int32_t *__restrict__ faces, FaceGeo *__restrict__ geo,
                           float4 *__restrict__ fnormal, int N, int F, int B, float4 *__restrict__ rec,
                           const float *__restrict__ uvs) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < B * F) face_geo_item(verts, faces, geo, fnormal, N, F, i, rec, uvs);
}

// `lanes` threads per vertex, each projecting into every lanes-th view.
__global__ void k_vertices(const FwdJob J, int lanes) {
    pdl_enter();
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int i = (int)(t / lanes), sub = (int)(t % lanes);
    if (i < J.dims.B * J.topo.N) vertex_item(J, i, sub, lanes);
}

__global__ void k_bin_count(const FwdJob J) {
    pdl_enter();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < J.dims.B * J.dims.C * J.topo.F) bin_count_item(J, i);
}

// The same scan by ceil(n / 8192) blocks of 1024 threads, none waiting on
// another: block j scans counts [8192 j, 8192 (j + 1)) as one pass of
// scan_block and offsets them by the sum of every count before them, which
// it adds up itself (a few 16-byte loads per thread, L2 hits, while the
// blocks are few; the launcher takes k_scan_tiles_one beyond kScanBlocks).
__global__ void __launch_bounds__(1024) k_scan_tiles(const int *__restrict__ count, int *__restrict__ start, int n) {
    pdl_enter();
    __shared__ int warpSum[32];
    __shared__ int offset;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int base = blockIdx.x * 8192;
    const bool vec = ((reinterpret_cast<uintptr_t>(count) | reinterpret_cast<uintptr_t>(start)) & 15) == 0;
    int before = 0;
    if (vec) {
        for (int k = 4 * tid; k < base; k += 4096) {  // base is a multiple of 4096
            const int4 q = *reinterpret_cast<const int4 *>(count + k);
            before += q.x + q.y + q.z + q.w;
        }
    } else {
        for (int k = tid; k < base; k += 1024) before += count[k];
    }
    before = __reduce_add_sync(0xffffffffu, before);
    if (lane == 0) warpSum[warp] = before;
    __syncthreads();
    if (warp == 0) {
        const int t = __reduce_add_sync(0xffffffffu, warpSum[lane]);
        if (lane == 0) offset = t;
    }
    __syncthreads();
    const int i0 = base + 8 * tid;
    int x[8];
    if (vec && i0 + 8 <= n) {
        const int4 a = *reinterpret_cast<const int4 *>(count + i0), c = *reinterpret_cast<const int4 *>(count + i0 + 4);
        x[0] = a.x, x[1] = a.y, x[2] = a.z, x[3] = a.w, x[4] = c.x, x[5] = c.y, x[6] = c.z, x[7] = c.w;
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = i0 + k < n ? count[i0 + k] : 0;
    }
    int sum = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) sum += x[k];
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    __syncthreads();  // every warp has read warpSum above
    if (lane == 31) warpSum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const int w = warpSum[lane];
        int wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        warpSum[lane] = wi - w;  // exclusive prefix of warp sums
    }
    __syncthreads();
    int run = offset + warpSum[warp] + incl - sum;
    int st[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        st[k] = run;
        run += x[k];
    }
    if (vec && i0 + 8 <= n) {
        *reinterpret_cast<int4 *>(start + i0) = make_int4(st[0], st[1], st[2], st[3]);
        *reinterpret_cast<int4 *>(start + i0 + 4) = make_int4(st[4], st[5], st[6], st[7]);
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k)
            if (i0 + k < n) start[i0 + k] = st[k];
    }
    if (blockIdx.x == gridDim.x - 1 && tid == 1023) start[n] = run;  // the last thread's run is the total
}

// One block for any n (linear work): the scan of calls with more than
// kScanBlocks * 8192 tiles, where the blocks of k_scan_tiles would each
// re-add too many counts.
__global__ void __launch_bounds__(1024) k_scan_tiles_one(const int *__restrict__ count, int *__restrict__ start, int n) {
    pdl_enter();
    scan_block(count, start, n);
}

__global__ void k_bin_fill(const FwdJob J) {
    pdl_enter();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < J.dims.B * J.dims.C * J.topo.F) bin_fill_item(J, i);
}

// ---------------------------------------------------------------------------- batched kernels

// Index spaces of the batched stages (BatchStage) and their per-job counts.
__device__ __forceinline__ int stage_count(const FwdJob &J, int stage) {
    switch (stage) {
        case kStageViews: return J.dims.B * J.dims.C;
        case kStageFaces: return J.dims.B * J.topo.F;
        case kStageVertices: return J.dims.B * J.topo.N;
        default: return J.dims.B * J.dims.C * J.topo.F;
    }
}

template <int STAGE>
__global__ void __launch_bounds__(kBatchBlock) k_stage_batched(const FwdJob *__restrict__ jobs,
                                                               const int *__restrict__ blockStart, int nJobs) {
    const int j = job_of_block(blockStart, nJobs, blockIdx.x);
    const FwdJob &J = jobs[j];
    const int i = (blockIdx.x - blockStart[j]) * kBatchBlock + threadIdx.x;
    if (i >= stage_count(J, STAGE)) return;
    if (STAGE == kStageViews) camera_item(J.extr, J.intr, J.ws.cams, i);
    else if (STAGE == kStageFaces)
        face_geo_item(J.io.verts, J.topo.faces, J.ws.geo, J.ws.fnormal, J.topo.N, J.topo.F, i, nullptr, nullptr,
                      J.ws.faceC);
    else if (STAGE == kStageVertices) vertex_item(J, i);
    else if (STAGE == kStageBinCount) bin_count_item(J, i);
    else bin_fill_item(J, i);
}

// The backward's camera and face stages over every job of a batched plan
// (zero-gradient jobs have no items).
template <int STAGE>
__global__ void __launch_bounds__(kBatchBlock) k_bwd_stage_batched(const BwdJob *__restrict__ jobs,
                                                                   const int *__restrict__ blockStart, int nJobs) {
    const int j = job_of_block(blockStart, nJobs, blockIdx.x);
    const BwdJob &J = jobs[j];
    const int i = (blockIdx.x - blockStart[j]) * kBatchBlock + threadIdx.x;
    if (J.zeroMode) return;
    if (STAGE == kBStageViews) {
        if (i < J.dims.B * J.dims.C) camera_item(J.extr, J.intr, J.ws.cams, i);
    } else if (i < J.dims.B * J.topo.F) {
        face_geo_item(J.io.verts, J.topo.faces, J.ws.geo, nullptr, J.topo.N, J.topo.F, i, J.ws.faceRec, J.topo.uvs);
    }
}

__global__ void __launch_bounds__(1024) k_scan_tiles_batched(const FwdJob *__restrict__ jobs) {
    const FwdJob &J = jobs[blockIdx.x];
    scan_block(J.ws.tileCount, J.ws.tileStart, J.dims.B * J.dims.C * J.dims.tilesX * J.dims.tilesY);
}

// The set-up of one call in one launch: the face pass (scaled geometry, face
// normals, and in the backward the face records and the cleared face
// accumulators), the camera records and a cleared region (the forward's
// per-call counters, or the backward's texture gradient).  Threads
// [0, faces) take faces, the next `views` take cameras, the rest clear.
__global__ void k_setup(const SetupArgs A) {
    pdl_enter();
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nF = (long long)A.B * A.F;
    if (i < nF) {
        face_geo_item(A.verts, A.faces, A.geo, A.fnormal, A.N, A.F, (int)i, A.rec, A.uvs, A.faceC);
        if (A.faceAcc) {
            float4 *acc = A.faceAcc + i * (kFaceAccFloats / 4);
#pragma unroll
            for (int q = 0; q < kFaceAccFloats / 4; ++q) acc[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        return;
    }
    const long long c = i - nF;
    if (c < A.views) {
        camera_item(A.extr, A.intr, A.cams, (int)c);
        return;
    }
    const long long z = c - A.views;  // four words per thread when the region is 16-byte aligned, else one
    float *w = reinterpret_cast<float *>(A.zero);
    if (A.zeroVec) {
        if (4 * z + 3 < A.zeroWords) reinterpret_cast<float4 *>(w)[z] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        else
            for (long long k = 4 * z; k < A.zeroWords; ++k) w[k] = 0.0f;
    } else if (z < A.zeroWords) {
        w[z] = 0.0f;
    }
}

// ---------------------------------------------------------------------------- host launch

static inline int blocks(size_t n, int t) { return (int)((n + t - 1) / t); }

cudaError_t launch_setup(SetupArgs a, cudaStream_t st) {
    a.zeroVec = ((reinterpret_cast<uintptr_t>(a.zero) & 15) == 0) ? 1 : 0;
    const long long zt = a.zero ? (a.zeroVec ? (a.zeroWords + 3) / 4 : a.zeroWords) : 0;
    const long long n = (long long)a.B * a.F + a.views + zt;
    if (n == 0) return cudaSuccess;
    cudaError_t err;
    GVR_LAUNCH(st, "k_setup", err = launch_pdl(k_setup, dim3((unsigned)((n + 127) / 128)), dim3(128), 0, st, a));
    return err;
}

cudaError_t launch_cameras(const float *extr, const float *intr, Camera *cams, int count, cudaStream_t st) {
    GVR_LAUNCH(st, "k_cameras", k_cameras<<<blocks(count, 64), 64, 0, st>>>(extr, intr, cams, count));
    return cudaGetLastError();
}

cudaError_t launch_face_geo(const float *verts, const Topology &topo, FaceGeo *geo, float4 *fnormal, int B,
                            cudaStream_t st, float4 *bwdRec) {
    GVR_LAUNCH(st, "k_face_geo",
               k_face_geo<<<blocks((size_t)B * topo.F, 256), 256, 0, st>>>(verts, topo.faces, geo, fnormal, topo.N,
                                                                            topo.F, B, bwdRec, topo.uvs));
    return cudaGetLastError();
}

static cudaError_t launch_vertices(const FwdJob &J, cudaStream_t st) {
    const int lanes = J.dims.C >= 4 ? 4 : J.dims.C;  // threads per vertex: the views split over them
    cudaError_t err;
    GVR_LAUNCH(st, "k_vertices",
               err = launch_pdl(k_vertices, dim3(blocks((size_t)J.dims.B * J.topo.N * lanes, 256)), dim3(256), 0, st,
                                J, lanes));
    return err;
}

cudaError_t launch_forward(const FwdJob &J, cudaStream_t st) {
    const FrameDims &dims = J.dims;
    const int B = dims.B, C = dims.C, T = dims.tilesX * dims.tilesY;
    SetupArgs sa{};
    sa.verts = J.io.verts;
    sa.faces = J.topo.faces;
    sa.uvs = J.topo.uvs;
    sa.N = J.topo.N;
    sa.F = J.topo.F;
    sa.B = B;
    sa.geo = J.ws.geo;
    sa.fnormal = J.ws.fnormal;
    sa.faceC = J.ws.faceC;
    sa.extr = J.extr;
    sa.intr = J.intr;
    sa.cams = J.ws.cams;
    sa.views = B * C;
    sa.zero = J.ws.zeroBase;
    sa.zeroWords = (long long)(J.ws.zeroBytes / 4);
    cudaError_t err = launch_setup(sa, st);
    if (err != cudaSuccess) return err;
    if ((err = launch_vertices(J, st)) != cudaSuccess) return err;
    const size_t nvf = (size_t)B * C * J.topo.F;
    GVR_LAUNCH(st, "k_bin_count", err = launch_pdl(k_bin_count, dim3(blocks(nvf, 128)), dim3(128), 0, st, J));
    if (err != cudaSuccess) return err;
    const int nt = B * C * T;
    constexpr int kScanBlocks = 16;  // beyond this many blocks the re-added prefixes outweigh the parallelism
    if ((nt + 8191) / 8192 <= kScanBlocks)
        GVR_LAUNCH(st, "k_scan_tiles",
                   err = launch_pdl(k_scan_tiles, dim3((nt + 8191) / 8192), dim3(1024), 0, st,
                                    (const int *)J.ws.tileCount, J.ws.tileStart, nt));
    else
        GVR_LAUNCH(st, "k_scan_tiles",
                   err = launch_pdl(k_scan_tiles_one, dim3(1), dim3(1024), 0, st, (const int *)J.ws.tileCount,
                                    J.ws.tileStart, nt));
    if (err != cudaSuccess) return err;
    GVR_LAUNCH(st, "k_bin_fill", err = launch_pdl(k_bin_fill, dim3(blocks(nvf, 128)), dim3(128), 0, st, J));
    if (err != cudaSuccess) return err;
    return launch_raster(J, st);
}

// compute_normal_map: cameras, vertex normals and projections as above, then
// the texture-space normal map instead of the depth and shading passes
// (renderBuffersGPU, CUDABasedRasterization.cu:449-473).
cudaError_t launch_forward_normal_map(const FwdJob &J, int *uvOwner, float *normal_map, cudaStream_t st) {
    const int B = J.dims.B, C = J.dims.C;
    cudaError_t err;
    if ((err = launch_cameras(J.extr, J.intr, J.ws.cams, B * C, st)) != cudaSuccess) return err;
    if ((err = launch_face_geo(J.io.verts, J.topo, J.ws.geo, J.ws.fnormal, B, st)) != cudaSuccess) return err;
    if ((err = launch_vertices(J, st)) != cudaSuccess) return err;
    return launch_normal_map(J.topo, J.dims, uvOwner, J.vnormal_out, normal_map, J.io.face, J.io.bary, J.io.render,
                             st);
}

// The batched forward of many jobs: one launch per stage over all jobs, then
// the persistent raster.  blockStart[s] holds nJobs + 1 block offsets of
// stage s (kBatchBlock threads per block); itemStart the raster items.
cudaError_t launch_forward_batched(const BatchLaunch &L, cudaStream_t st, bool raster) {
    cudaError_t err = cudaMemsetAsync(L.zeroBase, 0, L.zeroBytes, st);
    if (err != cudaSuccess) return err;
    GVR_LAUNCH(st, "k_cameras_batched",
               k_stage_batched<kStageViews><<<L.blocks[kStageViews], kBatchBlock, 0, st>>>(
                   L.jobs, L.blockStart[kStageViews], L.nJobs));
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    GVR_LAUNCH(st, "k_face_geo_batched",
               k_stage_batched<kStageFaces><<<L.blocks[kStageFaces], kBatchBlock, 0, st>>>(
                   L.jobs, L.blockStart[kStageFaces], L.nJobs));
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    GVR_LAUNCH(st, "k_vertices_batched",
               k_stage_batched<kStageVertices><<<L.blocks[kStageVertices], kBatchBlock, 0, st>>>(
                   L.jobs, L.blockStart[kStageVertices], L.nJobs));
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    GVR_LAUNCH(st, "k_bin_count_batched",
               k_stage_batched<kStageBinCount><<<L.blocks[kStageBinCount], kBatchBlock, 0, st>>>(
                   L.jobs, L.blockStart[kStageBinCount], L.nJobs));
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    GVR_LAUNCH(st, "k_scan_tiles_batched", k_scan_tiles_batched<<<L.nJobs, 1024, 0, st>>>(L.jobs));
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    GVR_LAUNCH(st, "k_bin_fill_batched",
               k_stage_batched<kStageBinFill><<<L.blocks[kStageBinCount], kBatchBlock, 0, st>>>(
                   L.jobs, L.blockStart[kStageBinCount], L.nJobs));
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
    if (!raster) return cudaSuccess;
    return launch_raster_persistent(L.jobs, L.itemStart, L.nJobs, L.counter, L.rasterGrid, st);
}

// Cameras and face records of every job of a batched backward.
cudaError_t launch_bwd_geo_batched(const BwdBatchLaunch &L, cudaStream_t st) {
    if (L.blocks[kBStageViews] > 0) {
        GVR_LAUNCH(st, "k_cameras_bwd_batched",
                   k_bwd_stage_batched<kBStageViews><<<L.blocks[kBStageViews], kBatchBlock, 0, st>>>(
                       L.jobs, L.blockStart[kBStageViews], L.nJobs));
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) return err;
    }
    if (L.blocks[kBStageFaces] > 0) {
        GVR_LAUNCH(st, "k_face_geo_bwd_batched",
                   k_bwd_stage_batched<kBStageFaces><<<L.blocks[kBStageFaces], kBatchBlock, 0, st>>>(
                       L.jobs, L.blockStart[kBStageFaces], L.nJobs));
    }
    return cudaGetLastError();
}

// Per-pixel rays for tests (same pixel_ray as the raster).
__global__ void k_debug_rays(const Camera *__restrict__ cams, float *__restrict__ out, int BC, int W, int H) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)BC * W * H) return;
    int u = (int)(i % W);
    int v = (int)((i / W) % H);
    int bc = (int)(i / ((size_t)W * H));
    V3 d = pixel_ray(cams[bc], u, v);
    out[3 * i + 0] = d.x;
    out[3 * i + 1] = d.y;
    out[3 * i + 2] = d.z;
}

cudaError_t launch_debug_rays(const Camera *cams, float *out, int BC, int W, int H, cudaStream_t st) {
    GVR_LAUNCH(st, "k_debug_rays", k_debug_rays<<<blocks((size_t)BC * W * H, 256), 256, 0, st>>>(cams, out, BC, W, H));
    return cudaGetLastError();
}

}  // namespace gvr

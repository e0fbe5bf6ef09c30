// gvr_backward.cu -- gradients of the render w.r.t. vertex positions,
// vertex colours, texture and SH coefficients.
//
// Reference: renderBuffersGradDevice (cpp/src/Renderer/CUDABasedRasterizationGrad.cu:114-617),
// one thread per pixel issuing ~210 float atomics per covered pixel.  Here:
//
//  k_bwd_pixels  one thread per pixel of a 16x16 tile.  Barycentrics come
//                from the forward's barycentric buffer, as the reference reads
//                them (without one they are recomputed from the face id with
//                the forward's exact FP32 ray/triangle test).  Per pixel the
//                chain rule gives
//                three 3-vectors weighted by the barycentric of each corner j:
//                  pos_j = b_j * (m - q)   shading + target-image terms
//                  gN_j  = b_j * w         d(loss)/d(un-normalised vertex normal)
//                  col_j = b_j * c         vertex colour
//                The warp pre-reduces them per face id (__match_any_sync +
//                a shuffle tree) and one lane per face adds them to a per-face
//                accumulator with 16-byte vector atomics.  SH gradients go
//                through a warp reduce-scatter into per-tile partials;
//                texels get atomics.  What a pixel reads about its face
//                (vertex indices, texture coordinates, vertex positions)
//                comes from one 80-byte record per face that the face pass
//                of the backward's set-up launch (k_setup) writes.
//  k_gather_a    per vertex, over its CSR faces: colour grad, position grad
//                (direct terms) and the vertex-normal gradient gN[v]; its
//                last B*C*27 blocks sum the per-tile SH partials in FP64 in
//                a fixed order (a separate launch, k_sh_finalize_batched, in
//                a batched plan).
//  k_gather_b    per vertex: the normal-adjacency term of :559-615.  The
//                reference applies, for every pixel, each corner's weight to
//                every face around that corner (~162 atomics); that sum is
//                linear in gN, so per face f=(a0,a1,a2) with
//                s_f = sum of gN over f's distinct vertices, corner r gets
//                (v[a(r+1)] - v[a(r+2)]) x s_f (= s_f . d cross(v1-v0, v2-v0)/d v_r).
//
// The shading-term Jacobian dJBCDVerpos (cpp/src/Utils/RendererUtil.h:670-861)
// is d(barycentrics)/d(vertices) for a fixed ray.  With e1 = v1-v0,
// e2 = v2-v0, N = e1 x e2 and the hit point o + t d, implicit
// differentiation of  b1 e1 + b2 e2 - t d = o - v0  gives
//   d b1 / d v_j = -b_j (e2 x d)/(N.d),  d b2 / d v_j = -b_j (d x e1)/(N.d),
//   d b0 / d v_j = -(d b1 + d b2)/d v_j,
// the same matrix in closed form; the reference's early-out
// (|cos(d, N)| < 0.001 or |N.N|^2 < 0.001) is kept.
#include "gvr_internal.cuh"
#include "gvr_kernels.h"
#include "gvr_profile.h"

namespace gvr {

// Sum of `val` over the lanes that share `peers` (a __match_any_sync mask):
// a pointer-jumping tree over the members, log2(largest group) steps.
// The result is valid in the group's lowest lane.
template <int NV>
__device__ __forceinline__ void group_reduce(float (&val)[NV], unsigned peers, int lane) {
    const unsigned full = 0xffffffffu;
    const int rank = __popc(peers & ((1u << lane) - 1u));
    const int maxSize = __reduce_max_sync(full, (unsigned)__popc(peers));
    const unsigned above = peers & ~((2u << lane) - 1u);
    int ptr = above ? __ffs(above) - 1 : -1;  // lane of the member with rank + d
    for (int d = 1; d < maxSize; d <<= 1) {
        const int src = ptr >= 0 ? ptr : lane;
        const bool take = ptr >= 0 && (rank & (2 * d - 1)) == 0;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            float o = __shfl_sync(full, val[k], src);
            if (take) val[k] += o;
        }
        int nxt = __shfl_sync(full, ptr, src);
        ptr = ptr >= 0 ? nxt : -1;
    }
}

// One butterfly step of a warp reduce-scatter: each lane carries C partial
// sums, swaps half of them with the lane C/2 away and keeps C/2.  Steps
// C = 32, 16, 8, 4, 2 leave lane k with the warp's sum of value k, in
// 16+8+4+2+1 = 31 shuffles (a shuffle tree per value takes 32 x 5).
template <int C>
__device__ __forceinline__ void reduce_scatter_step(float (&r)[32], int lane) {
    constexpr int H = C / 2;
    const bool upper = (lane & H) != 0;
#pragma unroll
    for (int i = 0; i < H; ++i) {
        const float send = upper ? r[i] : r[i + H];
        const float keep = upper ? r[i + H] : r[i];
        r[i] = keep + __shfl_xor_sync(0xffffffffu, send, H);
    }
}

// Adds (g0, g1, g2) to a texel's three floats with one 8-byte vector
// atomic and one scalar one: of two consecutive floats one starts on an
// 8-byte boundary.
__device__ __forceinline__ void add_texel(float *t, float g0, float g1, float g2) {
    if ((reinterpret_cast<uintptr_t>(t) & 7) == 0) {
        atomicAdd(reinterpret_cast<float2 *>(t), make_float2(g0, g1));
        atomicAdd(t + 2, g2);
    } else {
        atomicAdd(t, g0);
        atomicAdd(reinterpret_cast<float2 *>(t + 1), make_float2(g1, g2));
    }
}

// ALBPOS (vertexColor only, opt-in): add the change of the interpolated
// vertex colour through the barycentrics to the position gradient, which the
// reference leaves out (CUDABasedRasterizationGrad.cu:489).
// Tile (tx, ty) of view bc (= batch * C + camera).
template <int MODE, bool SHADED, bool TARGET, bool ALBPOS = false>
__device__ __forceinline__ void bwd_tile(const Topology &topo, const FrameDims &dims, const BwdScratch &ws,
                                         const BwdIO &io, const int bc, const int tx, const int ty) {
    constexpr bool COL = MODE == GVR_ALBEDO_VERTEX_COLOR;
    constexpr bool POS = SHADED || TARGET || ALBPOS;
    constexpr int NPOS = POS ? 9 : 0, NGN = SHADED ? 9 : 0, NCOL = COL ? 9 : 0;
    constexpr int NV = NPOS + NGN + NCOL > 0 ? NPOS + NGN + NCOL : 1;

    const int T = dims.tilesX * dims.tilesY;
    const int tile = ty * dims.tilesX + tx, b = bc / dims.C;
    const int tileX0 = tx * kTile, tileY0 = ty * kTile;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int u = tileX0 + (tid & (kTile - 1)), v = tileY0 + tid / kTile;
    const bool inImage = u < dims.W && v < dims.H;
    const size_t p = ((size_t)bc * dims.H + v) * dims.W + u;
    const int F = topo.F, N = topo.N;

    // the view's camera and SH coefficients, read by every pixel: staged
    // once per block (uniform global loads per pixel crowd the LSU pipe)
    __shared__ Camera sCam;
    __shared__ float sSH[27];
    {
        constexpr int kCamWords = (int)(sizeof(Camera) / sizeof(float));
        if (tid < kCamWords) reinterpret_cast<float *>(&sCam)[tid] = reinterpret_cast<const float *>(ws.cams + bc)[tid];
        else if (tid < kCamWords + 27) sSH[tid - kCamWords] = io.sh[(size_t)bc * 27 + (tid - kCamWords)];
    }
    int f = inImage ? __ldcs(io.face + p) : -1;
    if (f >= F) f = -1;  // ids outside [0, F) carry no face
    // the forward's barycentrics, as the reference's grad reads them
    // (CUDABasedRasterizationGrad.cu:210-211), and the upstream gradient,
    // loaded alongside the face id; the per-pixel inputs are read once, so
    // evict-first loads (ld.global.cs) leave the L2 to the face records,
    // vertex normals and texels that many pixels share
    const float2 bIn = inImage && io.bary_in ? __ldcs(reinterpret_cast<const float2 *>(io.bary_in) + p)
                                             : make_float2(0.0f, 0.0f);
    float G[3] = {0.0f, 0.0f, 0.0f};
    if (f >= 0) {
        G[0] = __ldcs(io.grad_render + 3 * p + 0);
        G[1] = __ldcs(io.grad_render + 3 * p + 1);
        G[2] = __ldcs(io.grad_render + 3 * p + 2);
    }
    __syncthreads();
    float shv[SHADED ? 32 : 1];  // 27 SH terms, padded to a warp for the reduce-scatter
#pragma unroll
    for (int k = 0; k < (SHADED ? 32 : 1); ++k) shv[k] = 0.0f;
    // what the position terms take from the shading phase: the ray, the
    // barycentrics, wv = d(loss)/d(un-normalised normal), rr[j] = d(loss)/d(b_j)
    // of the shading term and the colour weight gl = G * light
    V3 d = v3(0.0f, 0.0f, 0.0f), abc = v3(0.0f, 0.0f, 0.0f);
    float wv[3] = {0.0f, 0.0f, 0.0f}, rr[3] = {0.0f, 0.0f, 0.0f}, gl[3] = {0.0f, 0.0f, 0.0f};

    // ---- shading phase: normal, albedo and light; texel, SH and colour terms
    if (f >= 0) {
        const Camera &cam = sCam;
        d = pixel_ray(cam, u, v);
        abc = v3(bIn.x, bIn.y, xs(xs(1.0f, bIn.x), bIn.y));
        if (!io.bary_in) {
            // no barycentric buffer: recompute them from the face id with the
            // forward's exact test (a face the ray misses contributes nothing)
            const V3 origS = v3(cam.origS[0], cam.origS[1], cam.origS[2]);
            const FaceSetup fs = load_face(&ws.geo[(size_t)b * F + f]);
            abc = barycentric(fs, origS, xdot(origS, fs.n), d);
            if (abc.x == -1.0f && abc.y == -1.0f && abc.z == -1.0f) f = -1;
        }
        if (f >= 0) {
            const float4 *FR = ws.faceRec + ((size_t)b * F + f) * kBwdFaceRows;  // the face's record
            const float4 fr0 = FR[0];
            const int i0 = __float_as_int(fr0.x), i1 = __float_as_int(fr0.y), i2 = __float_as_int(fr0.z);
            const float *VN = io.vnormal + (size_t)bc * N * 3;
            const V3 N0 = ld3(VN + 3 * i0), N1 = ld3(VN + 3 * i1), N2 = ld3(VN + 3 * i2);
            const V3 un = pixel_normal_un(N0, N1, N2, abc);
            const float len = __fsqrt_rn(xdot(un, un));
            bool flipped;
            const V3 n = unit_normal(un, len, d, flipped);
            const float *sh = sSH;
            float basis[9];
            sh_basis(n, basis);
            float JCoAl[3] = {1.0f, 1.0f, 1.0f};
            if (!SHADED && io.phong) {  // d(colour)/d(albedo) of the headlight Phong term
                const float k = phong_factor(-(n.x * d.x + n.y * d.y + n.z * d.z));
                JCoAl[0] = JCoAl[1] = JCoAl[2] = k;
            }
            if (SHADED) {
#pragma unroll
                for (int ch = 0; ch < 3; ++ch) {
                    float l = 0.0f;
#pragma unroll
                    for (int k = 0; k < 9; ++k) l += sh[9 * ch + k] * basis[k];
                    JCoAl[ch] = l;
                }
            }
            // albedo as the gradient sees it (CUDABasedRasterizationGrad.cu:274-319)
            float alb[3] = {0.0f, 0.0f, 0.0f};
            if (MODE == GVR_ALBEDO_VERTEX_COLOR) {
                const float *Cb = io.colors + (size_t)b * N * 3;
#pragma unroll
                for (int ch = 0; ch < 3; ++ch)
                    alb[ch] = abc.x * Cb[3 * i0 + ch] + abc.y * Cb[3 * i1 + ch] + abc.z * Cb[3 * i2 + ch];
            }
            if (MODE == GVR_ALBEDO_TEXTURED) {
                const float4 fr1 = FR[1];
                const float2 tc = texel_coord6(fr0.w, fr1.x, fr1.y, fr1.z, fr1.w, FR[2].x, abc, dims.Wt, dims.Ht);
                const int iu = __float2int_rz(xs(tc.x, 0.5f)), iv = __float2int_rz(xs(tc.y, 0.5f));
                const int hu = min(iu + 1, dims.Wt - 1), hv = min(iv + 1, dims.Ht - 1);
                const float LU = iu + 0.5f, HU = iu + 1.5f, LV = iv + 0.5f, HV = iv + 1.5f;
                const float *tex = io.texture + (size_t)b * dims.Ht * dims.Wt * 3;
                const float *cLL = tex + ((size_t)iv * dims.Wt + iu) * 3, *cHL = tex + ((size_t)iv * dims.Wt + hu) * 3;
                const float *cLH = tex + ((size_t)hv * dims.Wt + iu) * 3, *cHH = tex + ((size_t)hv * dims.Wt + hu) * 3;
                // corner weights exactly as written at CUDABasedRasterizationGrad.cu:311-312
                const float wv0 = tc.y - LV, wv1 = HV - tc.y, wu0 = tc.x - LU, wu1 = HU - tc.x;
#pragma unroll
                for (int ch = 0; ch < 3; ++ch)
                    alb[ch] = wv0 * (wu0 * cLL[ch] + wu1 * cHL[ch]) + wv1 * (wu0 * cLH[ch] + wu1 * cHH[ch]);
                if (!flipped)
                    add_texel(io.tex_grad + (((size_t)b * dims.Ht + iv) * dims.Wt + iu) * 3, G[0] * JCoAl[0],
                              G[1] * JCoAl[1], G[2] * JCoAl[2]);
            }
            if (MODE == GVR_ALBEDO_TEXTURED_BILINEAR) {  // the lookup and its derivative: four texels
                const float4 fr1 = FR[1];
                const float2 tc = texel_coord6(fr0.w, fr1.x, fr1.y, fr1.z, fr1.w, FR[2].x, abc, dims.Wt, dims.Ht);
                int idx[4];
                float w[4];
                bilinear_taps(tc.x, tc.y, dims.Wt, dims.Ht, idx, w);
                const float *tex = io.texture + (size_t)b * dims.Ht * dims.Wt * 3;
                float *tgb = io.tex_grad + (size_t)b * dims.Ht * dims.Wt * 3;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
#pragma unroll
                    for (int ch = 0; ch < 3; ++ch) alb[ch] += w[k] * tex[3 * (size_t)idx[k] + ch];
                    add_texel(tgb + 3 * (size_t)idx[k], w[k] * (G[0] * JCoAl[0]), w[k] * (G[1] * JCoAl[1]),
                              w[k] * (G[2] * JCoAl[2]));
                }
            }
            if (SHADED) {
                const float ga[3] = {G[0] * alb[0], G[1] * alb[1], G[2] * alb[2]};
                // ga . d(light)/d(n)  (getJLiNo, RendererUtil.h:371-391)
                float wt[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
                for (int ch = 0; ch < 3; ++ch) {
                    const float *c9 = sh + 9 * ch;
                    wt[0] += ga[ch] * (c9[3] + c9[4] * n.y + c9[7] * n.z + 2.0f * c9[8] * n.x);
                    wt[1] += ga[ch] * (c9[1] + c9[4] * n.x + c9[5] * n.z - 2.0f * c9[8] * n.y);
                    wt[2] += ga[ch] * (c9[2] + c9[5] * n.y + 6.0f * c9[6] * n.z + c9[7] * n.x);
                }
                // . d(n)/d(un) = (|un|^2 I - un un^T) / |un|^3  (getJNoNu, :398-415)
                // the divisions of the continuous chain-rule terms use the hardware
                // reciprocal (2 ulp): the gradients' bar is 1e-4 relative
                const float len2 = len * len, inv3 = __fdividef(1.0f, len2 * len);
                const float wdot = wt[0] * un.x + wt[1] * un.y + wt[2] * un.z;
                wv[0] = (wt[0] * len2 - un.x * wdot) * inv3;
                wv[1] = (wt[1] * len2 - un.y * wdot) * inv3;
                wv[2] = (wt[2] * len2 - un.z * wdot) * inv3;
                // shading term through the barycentrics (:478-522): d(loss)/d(b_j) = wv . N_j
                rr[0] = wv[0] * N0.x + wv[1] * N0.y + wv[2] * N0.z;
                rr[1] = wv[0] * N1.x + wv[1] * N1.y + wv[2] * N1.z;
                rr[2] = wv[0] * N2.x + wv[1] * N2.y + wv[2] * N2.z;
                // the SH terms last: their 27 registers are live only up to the reduce-scatter
#pragma unroll
                for (int ch = 0; ch < 3; ++ch)
#pragma unroll
                    for (int k = 0; k < 9; ++k) shv[9 * ch + k] = ga[ch] * basis[k];
            }
            if (ALBPOS) {  // + sum_ch G light colour_j
                const float *Cb = io.colors + (size_t)b * N * 3;
#pragma unroll
                for (int ch = 0; ch < 3; ++ch) {
                    const float lg = G[ch] * JCoAl[ch];
                    rr[0] += lg * Cb[3 * i0 + ch];
                    rr[1] += lg * Cb[3 * i1 + ch];
                    rr[2] += lg * Cb[3 * i2 + ch];
                }
            }
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) gl[ch] = G[ch] * JCoAl[ch];
        }
    }

    // ---- SH partial sums of this tile, warp part: before the position
    // phase, so that the 32 per-lane terms are freed before the Jacobian
    __shared__ float red[kTilePix / 32][27];
    if constexpr (SHADED) {
        reduce_scatter_step<32>(shv, lane);
        reduce_scatter_step<16>(shv, lane);
        reduce_scatter_step<8>(shv, lane);
        reduce_scatter_step<4>(shv, lane);
        reduce_scatter_step<2>(shv, lane);
        if (lane < 27) red[warp][lane] = shv[0];
    }

    // ---- position phase: the shading term through the barycentrics
    // (closed-form Jacobian) and the target-image term
    float val[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) val[k] = 0.0f;
    if (f >= 0) {
        {
            const Camera &cam = sCam;
            const float4 *FR = ws.faceRec + ((size_t)b * F + f) * kBwdFaceRows;
            // Pv: per-pixel vector applied with the stored barycentrics (target term);
            // Qv[j]: shading term already weighted for corner j
            float Pv[3] = {0.0f, 0.0f, 0.0f};
            float Qv[3][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};
            if (SHADED || ALBPOS) {
                const float4 fr2 = FR[2], fr3 = FR[3], fr4 = FR[4];  // vertex positions
                const float3 V0 = make_float3(fr2.y, fr2.z, fr2.w);
                const float3 e1 = make_float3(fr3.x - V0.x, fr3.y - V0.y, fr3.z - V0.z);
                const float3 e2 = make_float3(fr3.w - V0.x, fr4.x - V0.y, fr4.y - V0.z);
                const float Nf[3] = {e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
                // N.d and the hit point in compensated arithmetic: near grazing
                // incidence both cancel badly in plain FP32 (error ~ eps/cos) and
                // the Jacobian scales with 1/cos.
                const float dv[3] = {d.x, d.y, d.z};
                const float nd = dot2<3>(Nf, dv);
                const float nn = Nf[0] * Nf[0] + Nf[1] * Nf[1] + Nf[2] * Nf[2];
                const float dd = d.x * d.x + d.y * d.y + d.z * d.z;
                if (nd * nd >= 1.0e-6f * nn * dd && nn * nn >= 0.001f) {
                    // P - V0 = t d - (V0 - o),  t = N.(V0 - o) / N.d, with V0 - o split exactly
                    float Dh[3], Dl[3];
                    two_sum(V0.x, -cam.orig[0], Dh[0], Dl[0]);
                    two_sum(V0.y, -cam.orig[1], Dh[1], Dl[1]);
                    two_sum(V0.z, -cam.orig[2], Dh[2], Dl[2]);
                    const float N6[6] = {Nf[0], Nf[1], Nf[2], Nf[0], Nf[1], Nf[2]};
                    const float D6[6] = {Dh[0], Dh[1], Dh[2], Dl[0], Dl[1], Dl[2]};
                    const float t = dot2<6>(N6, D6) / nd;
                    const float wx = __fmaf_rn(t, d.x, -Dh[0]) - Dl[0];
                    const float wy = __fmaf_rn(t, d.y, -Dh[1]) - Dl[1];
                    const float wz = __fmaf_rn(t, d.z, -Dh[2]) - Dl[2];
                    // barycentrics of the hit point: b1 = (w x e2).N / N.N, b2 = (e1 x w).N / N.N
                    const float inn = __fdividef(1.0f, nn);
                    const float hb1 = ((wy * e2.z - wz * e2.y) * Nf[0] + (wz * e2.x - wx * e2.z) * Nf[1] +
                                       (wx * e2.y - wy * e2.x) * Nf[2]) * inn;
                    const float hb2 = ((e1.y * wz - e1.z * wy) * Nf[0] + (e1.z * wx - e1.x * wz) * Nf[1] +
                                       (e1.x * wy - e1.y * wx) * Nf[2]) * inn;
                    const float hb[3] = {1.0f - hb1 - hb2, hb1, hb2};
                    const float inv = __fdividef(1.0f, nd);
                    const float3 g1 = make_float3((e2.y * d.z - e2.z * d.y) * inv, (e2.z * d.x - e2.x * d.z) * inv,
                                                  (e2.x * d.y - e2.y * d.x) * inv);
                    const float3 g2 = make_float3((d.y * e1.z - d.z * e1.y) * inv, (d.z * e1.x - d.x * e1.z) * inv,
                                                  (d.x * e1.y - d.y * e1.x) * inv);
                    const float k1 = rr[1] - rr[0], k2 = rr[2] - rr[0];
                    const float q[3] = {k1 * g1.x + k2 * g2.x, k1 * g1.y + k2 * g2.y, k1 * g1.z + k2 * g2.z};
#pragma unroll
                    for (int j = 0; j < 3; ++j)
#pragma unroll
                        for (int a = 0; a < 3; ++a) Qv[j][a] = -hb[j] * q[a];
                }
            }
            if (TARGET) {
                // model-to-data term (:531-555): g_target . dT/d(u,v) . d(u,v)/dX . dX/dv_j
                const float *gt = io.grad_target + 3 * p;
                const float GT[3] = {gt[0], gt[1], gt[2]};
                const int k = io.imageFilter;
                if ((GT[0] != 0.0f || GT[1] != 0.0f || GT[2] != 0.0f) && u >= k + 1 && v >= k + 1 &&
                    u < dims.W - (k + 1) && v < dims.H - (k + 1)) {
                    const float *img = io.target + (size_t)bc * dims.H * dims.W * 3;
                    float gu = 0.0f, gv = 0.0f, norm = 0.0f;
                    for (int y = -k; y <= k; ++y)
                        for (int x = -k; x <= k; ++x) {
                            const int den = x * x + y * y;
                            if (den == 0) continue;
                            const float Gu = (float)x / (float)den, Gv = (float)y / (float)den;
                            const float *I = img + ((size_t)(v + y) * dims.W + (u + x)) * 3;
                            const float gi = GT[0] * I[0] + GT[1] * I[1] + GT[2] * I[2];
                            gu += gi * Gu;
                            gv += gi * Gv;
                            norm += fabsf(Gu);
                        }
                    gu = __fdividef(gu, norm);
                    gv = __fdividef(gv, norm);
                    const float4 fr2 = FR[2], fr3 = FR[3], fr4 = FR[4];  // vertex positions
                    const float P0[3] = {fr2.y, fr2.z, fr2.w}, P1[3] = {fr3.x, fr3.y, fr3.z}, P2[3] = {fr3.w, fr4.x, fr4.y};
                    float X[3];
#pragma unroll
                    for (int a = 0; a < 3; ++a) X[a] = abc.x * P0[a] + abc.y * P1[a] + abc.z * P2[a];
                    const float *KE = cam.KE;
                    const float Px = KE[0] * X[0] + KE[1] * X[1] + KE[2] * X[2] + KE[3];
                    const float Py = KE[4] * X[0] + KE[5] * X[1] + KE[6] * X[2] + KE[7];
                    const float Pz = KE[8] * X[0] + KE[9] * X[1] + KE[10] * X[2] + KE[11];
                    if (fabsf(Pz) > 0.0001f) {
                        const float iz = __fdividef(1.0f, Pz), ax = Px * iz, ay = Py * iz;
#pragma unroll
                        for (int a = 0; a < 3; ++a)
                            Pv[a] += (gu * (KE[a] - ax * KE[8 + a]) + gv * (KE[4 + a] - ay * KE[8 + a])) * iz;
                    }
                }
            }
            const float bw[3] = {abc.x, abc.y, abc.z};
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    if (POS) val[3 * j + a] = bw[j] * Pv[a] + Qv[j][a];
                    if (SHADED) val[NPOS + 3 * j + a] = bw[j] * wv[a];
                    if (COL) val[NPOS + NGN + 3 * j + a] = bw[j] * gl[a];
                }
        }
    }

    // ---- per-face pre-reduction and accumulation
    if (NPOS + NGN + NCOL > 0) {
        const unsigned peers = __match_any_sync(0xffffffffu, f);
        group_reduce<NV>(val, peers, lane);
        const bool leader = (peers & ((1u << lane) - 1u)) == 0;
        if (leader && f >= 0) {
            float4 *acc = ws.faceAcc + ((size_t)b * F + f) * (kFaceAccFloats / 4);
            if (POS || SHADED) {
                float a[20];
#pragma unroll
                for (int k = 0; k < 20; ++k) a[k] = 0.0f;
#pragma unroll
                for (int k = 0; k < NPOS; ++k) a[k] = val[k];
#pragma unroll
                for (int k = 0; k < NGN; ++k) a[9 + k] = val[NPOS + k];
                constexpr int nA = SHADED ? 5 : 3;
#pragma unroll
                for (int q = 0; q < nA; ++q) atomicAdd(acc + q, make_float4(a[4 * q], a[4 * q + 1], a[4 * q + 2], a[4 * q + 3]));
            }
            if (COL) {
                float a[12];
#pragma unroll
                for (int k = 0; k < 12; ++k) a[k] = 0.0f;
#pragma unroll
                for (int k = 0; k < NCOL; ++k) a[k] = val[NPOS + NGN + k];
#pragma unroll
                for (int q = 0; q < 3; ++q) atomicAdd(acc + 5 + q, make_float4(a[4 * q], a[4 * q + 1], a[4 * q + 2], a[4 * q + 3]));
            }
        }
    }

    // ---- SH partial sums of this tile (block part)
    if constexpr (SHADED) {
        __syncthreads();
        if (tid < 27) {
            float s = 0.0f;
#pragma unroll
            for (int w = 0; w < kTilePix / 32; ++w) s += red[w][tid];
            ws.shPartial[((size_t)bc * 27 + tid) * T + tile] = s;  // coefficient-major: the finalize reads rows
        }
    }
}

// One block per 16 x 16 tile of one call: grid (tilesX, tilesY, views),
// views bcBase .. bcBase + gridDim.z - 1.
template <int MODE, bool SHADED, bool TARGET, bool ALBPOS = false>
__global__ void __launch_bounds__(kTilePix, 4) k_bwd_pixels(const Topology topo, const FrameDims dims, const BwdScratch ws,
                                                         const BwdIO io, int bcBase) {
    pdl_enter();
    bwd_tile<MODE, SHADED, TARGET, ALBPOS>(topo, dims, ws, io, bcBase + blockIdx.z, blockIdx.x, blockIdx.y);
}

// One block per 16 x 16 tile of every job of one variant in a batched plan:
// jobList[g] is the g-th job of the variant, its tiles start at block
// blockStart[g].  The job record is staged in shared memory once per block.
template <int MODE, bool SHADED, bool TARGET, bool ALBPOS = false>
__global__ void __launch_bounds__(kTilePix, 4) k_bwd_pixels_batched(const BwdJob *__restrict__ jobs,
                                                                 const int *__restrict__ jobList,
                                                                 const int *__restrict__ blockStart, int nJobs) {
    __shared__ BwdJob sJ;
    __shared__ int sBC, sTX, sTY;
    const int g = job_of_block(blockStart, nJobs, blockIdx.x);
    const BwdJob *J = jobs + jobList[g];
    constexpr int kWords = (int)(sizeof(BwdJob) / sizeof(int));
    for (int w = threadIdx.x; w < kWords; w += blockDim.x)
        reinterpret_cast<int *>(&sJ)[w] = reinterpret_cast<const int *>(J)[w];
    if (threadIdx.x == 0) {  // (view, tile) of the block, decomposed once
        const int local = blockIdx.x - blockStart[g], tilesX = J->dims.tilesX, T = tilesX * J->dims.tilesY;
        const int tile = local % T;
        sBC = local / T;
        sTX = tile % tilesX;
        sTY = tile / tilesX;
    }
    __syncthreads();
    bwd_tile<MODE, SHADED, TARGET, ALBPOS>(sJ.topo, sJ.dims, sJ.ws, sJ.io, sBC, sTX, sTY);
}

// ---------------------------------------------------------------------------- vertex gathers

// LANES consecutive threads share vertex i (sub = 0 .. LANES-1): thread sub
// takes faces sub, sub + LANES, ... of the vertex and the group adds its
// partial sums by a fixed butterfly (the same bits in every lane, whatever
// the schedule).  A vertex's few faces leave one thread per vertex with too
// little independent work to hide the gathers' latency.  All LANES threads
// of a group must reach the butterfly; `valid` is false past the last vertex.
template <int LANES, int NV>
__device__ __forceinline__ void lane_group_sum(float (&x)[NV]) {
#pragma unroll
    for (int o = 1; o < LANES; o <<= 1)
#pragma unroll
        for (int k = 0; k < NV; ++k) x[k] += __shfl_xor_sync(0xffffffffu, x[k], o);
}

constexpr int kGatherLanes = 8;

// Face-accumulator layout (floats): [0..8] position grad of corners 0..2,
// [9..17] vertex-normal grad of corners 0..2, [20..28] colour grad of corners 0..2.
template <int LANES>
__device__ __forceinline__ void gather_a_item(const Topology &topo, const float *__restrict__ faceAcc,
                                              float *__restrict__ vpos_grad, float *__restrict__ vcol_grad,
                                              float4 *__restrict__ gN, int useCol, int useGN, int i, int sub,
                                              bool valid) {
    const int N = topo.N, F = topo.F;
    const int b = i / N, v = i - b * N;
    float acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // position, normal and colour grads
    const float *Ab = faceAcc + (size_t)b * F * kFaceAccFloats;
    // the face's vertex ids and its id in one 16-byte load; the corners at v
    // follow from the ids, so the accumulator loads depend on one load only
    const int k0 = valid ? topo.vstart[v] + sub : 0, k1 = valid ? topo.vstart[v + 1] : 0;
    for (int k = k0; k < k1; k += LANES) {
        const int4 q = topo.vcsr[k];
        const float *A = Ab + (size_t)q.w * kFaceAccFloats;
        const int ids[3] = {q.x, q.y, q.z};
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            if (ids[r] != v) continue;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                acc[a] += A[3 * r + a];
                acc[3 + a] += A[9 + 3 * r + a];
                acc[6 + a] += A[20 + 3 * r + a];
            }
        }
    }
    if (LANES > 1) lane_group_sum<LANES>(acc);
    if (!valid || sub != 0) return;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        vpos_grad[3 * (size_t)i + a] = acc[a];
        vcol_grad[3 * (size_t)i + a] = useCol ? acc[6 + a] : 0.0f;
    }
    if (useGN) gN[i] = make_float4(acc[3], acc[4], acc[5], 0.0f);
}

// One block per (batch, view, coefficient), reading that coefficient's row
// of tile partials: thread i sums tiles i, i+256, ... (FP32 with
// compensation), then a fixed-order FP64 reduction (warp shuffles, then the
// eight warp sums in order) finishes, so the result is deterministic and
// FP64-accurate at FP32 cost.
__device__ __forceinline__ void sh_finalize_block(const float *__restrict__ partial, float *__restrict__ sh_grad,
                                                  int tilesPerView, int shaded, int blk) {
    __shared__ double red[8];
    const int bc = blk / 27, k = blk % 27;
    float s = 0.0f, comp = 0.0f;
    if (shaded)
        for (int t = threadIdx.x; t < tilesPerView; t += 256) {
            float hi, lo;
            two_sum(s, partial[((size_t)bc * 27 + k) * tilesPerView + t], hi, lo);
            s = hi;
            comp += lo;
        }
    double d = (double)s + (double)comp;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xffffffffu, d, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = d;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += red[w];
        sh_grad[(size_t)bc * 27 + k] = (float)t;
    }
}

// kGatherLanes threads per vertex (the first gatherBlocks blocks cover
// B*N*kGatherLanes threads); the blocks after them are the SH sums, one per
// (batch, view, coefficient), which need only the pixel kernel's partials
// too: run in this grid they leave the chain one launch shorter.
__global__ void __launch_bounds__(256) k_gather_a(const Topology topo, int B, const float *__restrict__ faceAcc,
                                                  float *__restrict__ vpos_grad, float *__restrict__ vcol_grad,
                                                  float4 *__restrict__ gN, int useCol, int useGN, int gatherBlocks,
                                                  const float *__restrict__ shPartial, float *__restrict__ sh_grad,
                                                  int tilesPerView, int shaded) {
    pdl_enter();
    if ((int)blockIdx.x >= gatherBlocks) {
        sh_finalize_block(shPartial, sh_grad, tilesPerView, shaded, blockIdx.x - gatherBlocks);
        return;
    }
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int i = (int)(t / kGatherLanes), sub = (int)(t % kGatherLanes);
    gather_a_item<kGatherLanes>(topo, faceAcc, vpos_grad, vcol_grad, gN, useCol, useGN, i, sub, i < B * topo.N);
}

template <int LANES>
__device__ __forceinline__ void gather_b_item(const Topology &topo, const float *__restrict__ verts,
                                              const float4 *__restrict__ gN, float *__restrict__ vpos_grad, int i,
                                              int sub, bool valid) {
    const int N = topo.N;
    const int b = i / N, v = i - b * N;
    const float *V = verts + (size_t)b * N * 3;
    const float4 *g = gN + (size_t)b * N;
    float acc[3] = {0, 0, 0};
    const int k0 = valid ? topo.vstart[v] + sub : 0, k1 = valid ? topo.vstart[v + 1] : 0;
    for (int k = k0; k < k1; k += LANES) {
        const int4 q = topo.vcsr[k];  // the face's vertex ids
        const int a[3] = {q.x, q.y, q.z};
        float4 s = g[a[0]];
        if (a[1] != a[0]) { float4 t = g[a[1]]; s.x += t.x; s.y += t.y; s.z += t.z; }
        if (a[2] != a[0] && a[2] != a[1]) { float4 t = g[a[2]]; s.x += t.x; s.y += t.y; s.z += t.z; }
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            if (a[r] != v) continue;
            const float *p1 = V + 3 * a[(r + 1) % 3], *p2 = V + 3 * a[(r + 2) % 3];
            float e[3] = {p1[0] - p2[0], p1[1] - p2[1], p1[2] - p2[2]};
            acc[0] += e[1] * s.z - e[2] * s.y;
            acc[1] += e[2] * s.x - e[0] * s.z;
            acc[2] += e[0] * s.y - e[1] * s.x;
        }
    }
    if (LANES > 1) lane_group_sum<LANES>(acc);
    if (!valid || sub != 0) return;
#pragma unroll
    for (int a = 0; a < 3; ++a) vpos_grad[3 * (size_t)i + a] += acc[a];
}

// kGatherLanes threads per vertex.
__global__ void k_gather_b(const Topology topo, int B, const float *__restrict__ verts, const float4 *__restrict__ gN,
                           float *__restrict__ vpos_grad) {
    pdl_enter();
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int i = (int)(t / kGatherLanes), sub = (int)(t % kGatherLanes);
    gather_b_item<kGatherLanes>(topo, verts, gN, vpos_grad, i, sub, i < B * topo.N);
}

// Both gathers over every job of a batched plan (WHICH 0: gather_a, 1: gather_b).
template <int WHICH>
__global__ void __launch_bounds__(256) k_gather_batched(const BwdJob *__restrict__ jobs,
                                                        const int *__restrict__ blockStart, int nJobs) {
    const int j = job_of_block(blockStart, nJobs, blockIdx.x);
    const BwdJob &J = jobs[j];
    const int i = (blockIdx.x - blockStart[j]) * 256 + threadIdx.x;
    if (J.zeroMode || i >= J.dims.B * J.topo.N) return;
    if (WHICH == 0)
        gather_a_item<1>(J.topo, reinterpret_cast<const float *>(J.ws.faceAcc), J.vpos_grad, J.vcol_grad, J.ws.gN,
                         J.useCol, J.shaded, i, 0, true);
    else if (J.shaded)
        gather_b_item<1>(J.topo, J.io.verts, J.ws.gN, J.vpos_grad, i, 0, true);
}

// One block per (job, batch, view, coefficient) of a batched plan.
__global__ void __launch_bounds__(256) k_sh_finalize_batched(const BwdJob *__restrict__ jobs,
                                                             const int *__restrict__ blockStart, int nJobs) {
    const int j = job_of_block(blockStart, nJobs, blockIdx.x);
    const BwdJob &J = jobs[j];
    if (J.zeroMode) return;
    sh_finalize_block(J.ws.shPartial, J.sh_grad, J.dims.tilesX * J.dims.tilesY, J.shaded, blockIdx.x - blockStart[j]);
}

// Clears every region of a batched backward: region r owns blocks
// [zeroStart[r], zeroStart[r + 1]), each clearing kZeroPerBlock floats.
__global__ void __launch_bounds__(256) k_zero_regions(const ZeroRegion *__restrict__ regions,
                                                      const int *__restrict__ zeroStart, int nRegions) {
    const int r = job_of_block(zeroStart, nRegions, blockIdx.x);
    const ZeroRegion R = regions[r];
    const long long base = (long long)(blockIdx.x - zeroStart[r]) * kZeroPerBlock;
    for (int k = threadIdx.x; k < kZeroPerBlock; k += 256) {
        const long long i = base + k;
        if (i < R.count) R.ptr[i] = 0.0f;
    }
}

// ---------------------------------------------------------------------------- host launch

static inline int blocks(size_t n, int t) { return (int)((n + t - 1) / t); }

// Calls v.run<MODE, SHADED, TARGET, ALBPOS>() for the pixel-kernel variant of
// a call: MODE is the albedo class (vertex colour, nearest texture, bilinear
// texture, or the constant white of foregroundMask), ALBPOS exists for
// vertex colours only.
template <int MODE, bool ALBPOS, class V>
static cudaError_t visit_st(bool shaded, bool target, V &v) {
    if (shaded) return target ? v.template run<MODE, true, true, ALBPOS>() : v.template run<MODE, true, false, ALBPOS>();
    return target ? v.template run<MODE, false, true, ALBPOS>() : v.template run<MODE, false, false, ALBPOS>();
}

template <class V>
static cudaError_t visit_variant(int albedo, bool shaded, bool target, bool albpos, V &v) {
    switch (albedo) {
        case GVR_ALBEDO_VERTEX_COLOR:
            return albpos ? visit_st<GVR_ALBEDO_VERTEX_COLOR, true>(shaded, target, v)
                          : visit_st<GVR_ALBEDO_VERTEX_COLOR, false>(shaded, target, v);
        case GVR_ALBEDO_TEXTURED: return visit_st<GVR_ALBEDO_TEXTURED, false>(shaded, target, v);
        case GVR_ALBEDO_TEXTURED_BILINEAR: return visit_st<GVR_ALBEDO_TEXTURED_BILINEAR, false>(shaded, target, v);
        default: return visit_st<GVR_ALBEDO_FOREGROUND_MASK, false>(false, target, v);
    }
}

// shaded: SH shading of a lit albedo (foregroundMask is forced shadeless)
static bool backward_shaded(int albedo, int shading) {
    return shading == GVR_SHADING_SHADED && albedo != GVR_ALBEDO_FOREGROUND_MASK;
}

int backward_variant(int albedo, int shading, bool target, bool albpos) {
    if (albedo == GVR_ALBEDO_NORMAL || albedo == GVR_ALBEDO_LIGHTING || albedo == GVR_ALBEDO_UV) return -1;
    const int cls = albedo == GVR_ALBEDO_VERTEX_COLOR ? 0 : albedo == GVR_ALBEDO_TEXTURED ? 1
                  : albedo == GVR_ALBEDO_TEXTURED_BILINEAR ? 2 : 3;
    const bool shaded = backward_shaded(albedo, shading);
    const bool ap = albpos && albedo == GVR_ALBEDO_VERTEX_COLOR;
    return ((cls * 2 + shaded) * 2 + target) * 2 + ap;
}

// The albedo mode, shading and options a variant number stands for.
static void variant_parts(int variant, int &albedo, bool &shaded, bool &target, bool &albpos) {
    static const int kCls[4] = {GVR_ALBEDO_VERTEX_COLOR, GVR_ALBEDO_TEXTURED, GVR_ALBEDO_TEXTURED_BILINEAR,
                                GVR_ALBEDO_FOREGROUND_MASK};
    albpos = variant & 1;
    target = (variant >> 1) & 1;
    shaded = (variant >> 2) & 1;
    albedo = kCls[(variant >> 3) & 3];
}

struct CallPixels {
    const Topology &topo;
    const FrameDims &dims;
    const BwdScratch &ws;
    const BwdIO &io;
    cudaStream_t st;
    template <int MODE, bool SHADED, bool TARGET, bool ALBPOS>
    cudaError_t run() {
        const int BC = dims.B * dims.C;
        for (int bc0 = 0; bc0 < BC; bc0 += 65535) {  // gridDim.z holds at most 65535 views
            const dim3 grid(dims.tilesX, dims.tilesY, min(65535, BC - bc0));
            cudaError_t e;
            GVR_LAUNCH(st, "k_bwd_pixels",
                       e = launch_pdl(k_bwd_pixels<MODE, SHADED, TARGET, ALBPOS>, grid, dim3(kTilePix), 0, st, topo, dims,
                                      ws, io, bc0));
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
};

struct BatchedPixels {
    const BwdBatchLaunch &L;
    int g;
    cudaStream_t st;
    template <int MODE, bool SHADED, bool TARGET, bool ALBPOS>
    cudaError_t run() {
        GVR_LAUNCH(st, "k_bwd_pixels_batched",
                   (k_bwd_pixels_batched<MODE, SHADED, TARGET, ALBPOS><<<L.groupBlocks[g], kTilePix, 0, st>>>(
                       L.jobs, L.groupJobs[g], L.groupStart[g], L.groupCount[g])));
        return cudaGetLastError();
    }
};

cudaError_t launch_backward(const Topology &topo, const FrameDims &dims, const BwdScratch &ws, const GvrBackwardArgs &a,
                            int imageFilter, cudaStream_t st) {
    const int B = dims.B, C = dims.C, N = topo.N, F = topo.F, T = dims.tilesX * dims.tilesY;
    const size_t texBytes = (size_t)B * dims.Ht * dims.Wt * 3 * sizeof(float);
    cudaError_t err;
    if (dims.albedo == GVR_ALBEDO_NORMAL || dims.albedo == GVR_ALBEDO_LIGHTING || dims.albedo == GVR_ALBEDO_UV) {
        // python/CudaRenderer.py:207-213: zero gradients for these modes (and for the UV mode)
        if ((err = cudaMemsetAsync(a.vertex_pos_grad, 0, (size_t)B * N * 3 * sizeof(float), st))) return err;
        if ((err = cudaMemsetAsync(a.vertex_color_grad, 0, (size_t)B * N * 3 * sizeof(float), st))) return err;
        if ((err = cudaMemsetAsync(a.texture_grad, 0, texBytes, st))) return err;
        return cudaMemsetAsync(a.sh_coeff_grad, 0, (size_t)B * C * 27 * sizeof(float), st);
    }
    const bool shaded = backward_shaded(dims.albedo, dims.shading);
    const bool target = a.target_grad != nullptr;
    SetupArgs sa{};  // cameras, face records, cleared face accumulators and texture gradient: one launch
    sa.verts = a.vertex_pos;
    sa.faces = topo.faces;
    sa.uvs = topo.uvs;
    sa.N = N;
    sa.F = F;
    sa.B = B;
    sa.geo = ws.geo;
    sa.rec = ws.faceRec;
    sa.faceAcc = ws.faceAcc;
    sa.extr = a.extrinsics;
    sa.intr = a.intrinsics;
    sa.cams = ws.cams;
    sa.views = B * C;
    sa.zero = a.texture_grad;
    sa.zeroWords = (long long)(texBytes / sizeof(float));
    if ((err = launch_setup(sa, st))) return err;
    const int phong = dims.shading == GVR_SHADING_PHONG && dims.albedo != GVR_ALBEDO_FOREGROUND_MASK;
    BwdIO io{a.render_grad, a.vertex_pos, a.vertex_color, a.texture, a.sh_coeff, a.target_image, a.vertex_normal,
             a.barycentric, a.face, a.target_grad, a.texture_grad, imageFilter, phong};
    const bool albpos = (a.flags & GVR_BACKWARD_ALBEDO_POSITION) != 0;
    CallPixels call{topo, dims, ws, io, st};
    if ((err = visit_variant(dims.albedo, shaded, target, albpos, call))) return err;
    const int useCol = dims.albedo == GVR_ALBEDO_VERTEX_COLOR, useGN = shaded, shadedFlag = shaded;
    const int gatherBlocks = blocks((size_t)B * N * kGatherLanes, 256);
    GVR_LAUNCH(st, "k_gather_a",
               err = launch_pdl(k_gather_a, dim3(gatherBlocks + B * C * 27), dim3(256), 0, st, topo, B,
                                reinterpret_cast<const float *>(ws.faceAcc), a.vertex_pos_grad, a.vertex_color_grad,
                                ws.gN, useCol, useGN, gatherBlocks, (const float *)ws.shPartial, a.sh_coeff_grad, T,
                                shadedFlag));
    if (err) return err;
    if (shaded) {
        GVR_LAUNCH(st, "k_gather_b",
                   err = launch_pdl(k_gather_b, dim3(blocks((size_t)B * N * kGatherLanes, 256)), dim3(256), 0, st,
                                    topo, B, a.vertex_pos, (const float4 *)ws.gN, a.vertex_pos_grad));
    }
    return err;
}

// The batched backward of many jobs: one clearing launch, the camera and face
// stages over every job, one pixel launch per variant present, both gathers
// and the SH sums over every job.
cudaError_t launch_backward_batched(const BwdBatchLaunch &L, cudaStream_t st) {
    cudaError_t err;
    if (L.zeroBlocks > 0) {
        GVR_LAUNCH(st, "k_zero_regions", k_zero_regions<<<L.zeroBlocks, 256, 0, st>>>(L.zeros, L.zeroStart, L.nZero));
        if ((err = cudaGetLastError())) return err;
    }
    if ((err = launch_bwd_geo_batched(L, st))) return err;
    for (int g = 0; g < L.nGroups; ++g) {
        int albedo;
        bool shaded, target, albpos;
        variant_parts(L.groupVariant[g], albedo, shaded, target, albpos);
        BatchedPixels launch{L, g, st};
        if ((err = visit_variant(albedo, shaded, target, albpos, launch))) return err;
    }
    if (L.blocks[kBStageVertices] > 0) {
        GVR_LAUNCH(st, "k_gather_a_batched",
                   k_gather_batched<0><<<L.blocks[kBStageVertices], 256, 0, st>>>(L.jobs, L.blockStart[kBStageVertices],
                                                                                   L.nJobs));
        if ((err = cudaGetLastError())) return err;
        GVR_LAUNCH(st, "k_gather_b_batched",
                   k_gather_batched<1><<<L.blocks[kBStageVertices], 256, 0, st>>>(L.jobs, L.blockStart[kBStageVertices],
                                                                                   L.nJobs));
        if ((err = cudaGetLastError())) return err;
    }
    if (L.blocks[kBStageSH] > 0) {
        GVR_LAUNCH(st, "k_sh_finalize_batched",
                   k_sh_finalize_batched<<<L.blocks[kBStageSH], 256, 0, st>>>(L.jobs, L.blockStart[kBStageSH], L.nJobs));
        if ((err = cudaGetLastError())) return err;
    }
    return cudaSuccess;
}

}  // namespace gvr

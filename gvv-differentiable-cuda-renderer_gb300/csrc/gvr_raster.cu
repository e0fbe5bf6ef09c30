// gvr_raster.cu -- visibility, resolve and shading of one 256-pixel tile
// (16x16 by default; 32x8 or 8x32 when a batched plan picks them) per block
// (the work of renderDepthBufferDevice + renderBuffersDevice,
// cpp/src/Renderer/CUDABasedRasterization.cu:215-408).
//
// The reference tests every pixel of every face's box with its FP32
// world-space ray/triangle test and keeps the smallest quantised depth.
// Here each thread owns one pixel and each warp an 8x4 block of the tile;
// the tile's face entries are staged in shared memory, counting-sorted front
// to back into depth buckets spanning the view's range of depth lower bounds,
// and each warp walks them once -- 32 at a time, a ballot keeping only the
// entries whose triangle may cover a pixel centre of its block -- with cheap
// screen-space bounds:
//
//   - a face that certainly covers the pixel lowers the pixel's depth bound
//     zup (the face's exact quantised depth is <= zup);
//   - a face that may still win (not certainly outside, not certainly
//     deeper than zup) is kept as a candidate (face, lower depth bound);
//   - once the next entry's depth lower bound exceeds zup at every pixel of
//     the warp, no later entry can matter and the warp stops.
//
// The resolve runs the reference's exact test on the surviving candidates
// only and keeps the packed depth|face minimum.  Every skipped face provably
// has a larger quantised depth than a face the exact test accepts, so face
// ids and barycentrics equal those of testing every face (ties between
// equal depths go to the smallest face id; the reference resolves them by a
// write race).
#include "gvr_internal.cuh"
#include "gvr_kernels.h"
#include "gvr_profile.h"

namespace gvr {
namespace {

constexpr int kChunk = kTilePix;  // face entries staged per pass: one per thread
constexpr int kBuckets = 128;     // depth buckets of the front-to-back order
constexpr int kMaxCand = 8;       // candidates a pixel keeps (shared-memory slots per pixel)

// Face entry with its skip-test constants and its box clipped to the tile
// (80 bytes).  Fields are grouped in 16-byte rows in the order the walk
// tests them, so an entry rejected by its box costs one shared-memory load.
struct __align__(16) Entry {
    int bx0, by0, bx1, by1;
    float zLowSafe, mOut;
    int flags, f;
    float x0, y0, a1, b1;
    float a2, b2, mIn, dRel;
    float r0, r1, r2, pad;
};

// The records this kernel reads (screen and face records, shading records,
// big-face lists, texels) were written by earlier launches and stay
// unchanged while it runs: they go through the non-coherent read-only path
// (ld.global.nc), which also left the compiler fewer live registers to
// spill.  The tile's bin entries, read once, are evict-first loads.
__device__ __forceinline__ ViewFace ldg_vf(const ViewFace *p) {
    ViewFace v;
    v.hdr = __ldg(&p->hdr);
    v.z = __ldg(&p->z);
    v.s0 = __ldg(&p->s0);
    v.s1 = __ldg(&p->s1);
    return v;
}

__device__ __forceinline__ FaceSetup ldg_face(const FaceGeo *p) {
    FaceGeo g;
    g.a = __ldg(&p->a);
    g.b = __ldg(&p->b);
    g.c = __ldg(&p->c);
    g.d = __ldg(&p->d);
    return load_face(&g);
}

__device__ __forceinline__ Entry make_entry(const ViewFace &vf, int f, int tileX0, int tileY0, int tileW, int tileH) {
    Entry E;
    E.x0 = vf.s0.x;
    E.y0 = vf.s0.y;
    E.a1 = vf.s1.x;
    E.b1 = vf.s1.y;
    E.a2 = vf.s1.z;
    E.b2 = vf.s1.w;
    // reciprocal depths feed only the depth estimate of the skip tests, whose
    // margin dRel is orders of magnitude above this approximation's error
    E.r0 = __fdividef(1.0f, vf.z.x);
    E.r1 = __fdividef(1.0f, vf.z.y);
    E.r2 = __fdividef(1.0f, vf.z.z);
    E.mIn = vf.z.w;
    E.mOut = vf.s0.z;
    E.dRel = vf_drel(vf);
    E.zLowSafe = vf.s0.w;
    E.flags = vf_flags(vf);
    E.f = f;
    E.pad = 0.0f;
    const int4 box = vf_box(vf);
    E.bx0 = max(box.x, tileX0);
    E.by0 = max(box.y, tileY0);
    E.bx1 = min(box.z, tileX0 + tileW - 1);
    E.by1 = min(box.w, tileY0 + tileH - 1);
    return E;
}

// Screen barycentrics of pixel centre (px, py) and the depth estimate 1e4*S/T
// (the reference's 1e4 / sum(b_i / z_i) with b_i its world barycentrics).
// g0 = (x0, y0, a1, b1), (a2, b2) of the entry.
__device__ __forceinline__ void lambda_at(const float4 &g0, float a2, float b2, float px, float py, float &l0, float &l1,
                                          float &l2) {
    const float dx = px - g0.x, dy = py - g0.y;
    l1 = g0.z * dx + g0.w * dy;
    l2 = a2 * dx + b2 * dy;
    l0 = 1.0f - l1 - l2;
}

// r = (r0, r1, r2): reciprocal vertex depths.
__device__ __forceinline__ float depth_at(const float4 &r, float l0, float l1, float l2) {
    const float S = l0 * r.x + l1 * r.y + l2 * r.z;
    const float T = l0 * r.x * r.x + l1 * r.y * r.y + l2 * r.z * r.z;
    return 10000.0f * __fdividef(S, T);
}

__device__ __forceinline__ void entry_lambda(const Entry &E, float px, float py, float &l0, float &l1, float &l2) {
    lambda_at(make_float4(E.x0, E.y0, E.a1, E.b1), E.a2, E.b2, px, py, l0, l1, l2);
}

__device__ __forceinline__ float entry_depth(const Entry &E, float l0, float l1, float l2) {
    return depth_at(make_float4(E.r0, E.r1, E.r2, 0.0f), l0, l1, l2);
}

// False when no pixel centre of the box [x0, x1] x [y0, y1] can pass the
// "not certainly outside" test of a screen-valid entry: each screen
// barycentric is affine, so its maximum over the box is at the corner
// picked by the signs of its slopes.  (The margin mOut leaves slack far
// above FP32 rounding, so a corner and a pixel evaluated with different
// rounding cannot disagree on a face the exact test could accept.)
__device__ __forceinline__ bool may_cover_box(const float4 &g0, float a2, float b2, float mOut, int x0, int x1, int y0,
                                              int y1) {
    const float xl = x0 + 0.5f, xh = x1 + 0.5f, yl = y0 + 0.5f, yh = y1 + 0.5f;
    const float a0 = -(g0.z + a2), b0 = -(g0.w + b2);
    float l0, l1, l2, s, t;
    lambda_at(g0, a2, b2, a0 >= 0.0f ? xh : xl, b0 >= 0.0f ? yh : yl, l0, s, t);
    lambda_at(g0, a2, b2, g0.z >= 0.0f ? xh : xl, g0.w >= 0.0f ? yh : yl, s, l1, t);
    lambda_at(g0, a2, b2, a2 >= 0.0f ? xh : xl, b2 >= 0.0f ? yh : yl, s, t, l2);
    return !(l0 < -mOut || l1 < -mOut || l2 < -mOut);
}

// The same test over the entry's whole clipped box.
__device__ __forceinline__ bool may_cover_rect(const Entry &E) {
    if (!(E.flags & kScreenValid)) return true;
    return may_cover_box(make_float4(E.x0, E.y0, E.a1, E.b1), E.a2, E.b2, E.mOut, E.bx0, E.bx1, E.by0, E.by1);
}

// May the face win the pixel against the certain depth bound zup?
__device__ __forceinline__ bool may_win(const Entry &E, float px, float py, float zup) {
    if (!(E.flags & kScreenValid)) return true;
    float l0, l1, l2;
    entry_lambda(E, px, py, l0, l1, l2);
    if (l0 < -E.mOut || l1 < -E.mOut || l2 < -E.mOut) return false;  // certainly outside
    float zlow = E.zLowSafe;  // lower bound of its quantised depth if accepted
    if (E.dRel < 0.25f) zlow = fmaxf(zlow, entry_depth(E, l0, l1, l2) * (1.0f - E.dRel) - 2.0f);
    return !(zlow > zup);
}

struct ExactCtx {
    const FaceGeo *geo;      // [F] of this batch element
    const ViewFace *vface;   // [F] of this view
    V3 origS;
    V3 d;
};

// The reference's exact test of face f at this pixel; key = kEmptyKey if
// rejected.  With needDepth = false (a single candidate) the key of an
// accepted face is just its id: only acceptance matters then.
__device__ __forceinline__ unsigned long long exact_key(const ExactCtx &x, int f, V3 &abc, bool needDepth) {
    const FaceSetup fs = ldg_face(&x.geo[f]);
    abc = barycentric(fs, x.origS, xdot(x.origS, fs.n), x.d);
    if (!inside(abc)) return kEmptyKey;
    if (!needDepth) return (unsigned long long)(unsigned)f;
    const float4 z = __ldg(&x.vface[f].z);
    return depth_key(depth_quantised(abc, z.x, z.y, z.z), f);
}

// Tile (tx, ty) of view bc (= batch * C + camera) of job J (256 threads, one
// pixel each).  Shared by the per-call grid kernel and the persistent
// batched kernel, so both produce the same bits.  ALB >= 0 compiles the
// shading for that albedo mode only (fewer live registers in the kernel);
// ALB = -1 reads the mode from the job at run time.
template <int ALB>
__device__ __forceinline__ void raster_tile(const FwdJob &J, const int bc, const int tx, const int ty) {
    const Topology &topo = J.topo;
    const FrameDims &dims = J.dims;
    const FwdScratch &ws = J.ws;
    const RasterIO &io = J.io;
    __shared__ Entry sE[kChunk];
    __shared__ float sBucketLo[kChunk];
    __shared__ int sHist[kBuckets + 1];
    const int T = dims.tilesX * dims.tilesY;
    const int tile = ty * dims.tilesX + tx, b = bc / dims.C;
    const int tileW = dims.tileW, tileH = dims.tileH;
    const int tileX0 = tx * tileW, tileY0 = ty * tileH;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // Each warp owns an 8x4 block of the tile (tileW / 8 = 2^wShift blocks
    // across): fewer faces overlap it than a full-width strip of 32 pixels.
    const int wShift = dims.tileShift - 3;
    const int colLo = tileX0 + ((warp & ((1 << wShift) - 1)) << 3), rowLo = tileY0 + ((warp >> wShift) << 2);
    const int colHi = colLo + 7, rowHi = rowLo + 3;
    const int u = colLo + (lane & 7), v = rowLo + (lane >> 3);
    const float px = u + 0.5f, py = v + 0.5f;
    const int F = topo.F;
    const ViewFace *VF = ws.vface + (size_t)bc * F;
    const int *bigList = ws.bigList + (size_t)bc * F;
    const size_t tIdx = (size_t)bc * T + tile;
    const int s0 = ws.tileStart[tIdx], nTile = ws.tileStart[tIdx + 1] - s0;
    const int nAll = nTile + ws.bigCount[bc];
    const float kInf = __int_as_float(0x7f800000);

    // One pass front to back: `zup` is the smallest certain depth bound so
    // far; candidates (face, lower depth bound) are kept while their bound
    // does not exceed it.  A bound only decreases, so a face dropped early
    // could never win; the survivors are filtered again by the final bound.
    // The tile's entries go through shared memory in chunks of kChunk (dense
    // meshes at low resolution put thousands of faces in a tile); zup and
    // the candidates carry over from chunk to chunk.
    // Candidates live in shared memory, slot j of pixel tid at [j][tid]
    // (conflict-free): appending is two stores, and the resolve walks them
    // with one copy of the exact test instead of one per register slot.
    __shared__ int sCandF[kMaxCand][kTilePix];
    __shared__ float sCandZ[kMaxCand][kTilePix];
    float zup = kInf;
    int nCand = 0;
    bool spill = false;
    // The view's range of finite, non-negative depth bounds, from the binning
    // pass: every kept entry with such a bound lies in it.
    const unsigned zr0 = ws.zRange[2 * bc], zr1 = ws.zRange[2 * bc + 1];
    const float lo = zr1 ? __uint_as_float(~zr0) : kInf, hi = zr1 ? __uint_as_float(zr1) : 0.0f;
    // bucket scale and the bucket width pulled down by 0.1% (below): any
    // rounding here is far inside the 0.25% slack of the bounds themselves
    const float scale = hi > lo ? __fdividef((float)kBuckets, hi - lo) : 0.0f;
    const float edge = scale > 0.0f ? __fdividef(0.999f, scale) : 0.0f;
    for (int k = tid; k <= kBuckets; k += kTilePix) sHist[k] = 0;
    // the view's camera and SH coefficients, read by every pixel of the
    // resolve and shading: staged once per tile
    __shared__ Camera sCam;
    __shared__ float sSH[27];
    {
        constexpr int kCamWords = (int)(sizeof(Camera) / sizeof(float));
        if (tid < kCamWords) reinterpret_cast<float *>(&sCam)[tid] = reinterpret_cast<const float *>(ws.cams + bc)[tid];
        else if (tid < kCamWords + 27) sSH[tid - kCamWords] = io.sh[(size_t)bc * 27 + (tid - kCamWords)];
    }
    if (nAll == 0) __syncthreads();  // (otherwise the first chunk's barriers order these stores)
    for (int c0 = 0; c0 < nAll; c0 += kChunk) {
        // Each thread builds one entry of the chunk, keeps only its face id
        // and depth bucket while the block counting-sorts the chunk into
        // kBuckets depth buckets spanning the view's depth bounds (faces
        // without a bound go first), then builds the entry again from the
        // record it just loaded (an L1 hit) and stores it in its sorted slot:
        // holding the 80-byte entry across the sort's barriers cost spills.
        // sBucketLo[i] is a lower bound of the depth bound of entry i and of
        // every entry after it, which is all the early exit needs.
        const int e = c0 + tid;
        bool keep = false;
        int fE = -1;
        int q = 0;  // 0: no usable bound; 1..kBuckets by depth
        if (e < nAll) {
            fE = e < nTile ? __ldcs(ws.bins + s0 + e) : __ldg(bigList + e - nTile);
            const Entry E = make_entry(ldg_vf(VF + fE), fE, tileX0, tileY0, tileW, tileH);
            keep = E.bx0 <= E.bx1 && E.by0 <= E.by1 && may_cover_rect(E);
            q = !keep || !(E.zLowSafe >= lo) ? 0 : 1 + min(kBuckets - 1, (int)((E.zLowSafe - lo) * scale));
        }
        __syncthreads();  // every warp is done walking the previous chunk; the histogram is clear
        if (keep) atomicAdd(&sHist[q], 1);
        const int nE = __syncthreads_count(keep);
        if (tid < 32) {  // exclusive prefix of the kBuckets + 1 counts: kPer per lane, one warp scan
            constexpr int kPer = (kBuckets + 1 + 31) / 32;
            int h[kPer];
            int own = 0;
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                const int qk = kPer * tid + k;
                h[k] = qk <= kBuckets ? sHist[qk] : 0;
                own += h[k];
            }
            int incl = own;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (tid >= o) incl += y;
            }
            int run = incl - own;
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                const int qk = kPer * tid + k;
                if (qk <= kBuckets) sHist[qk] = run;
                run += h[k];
            }
        }
        __syncthreads();
        if (keep) {
            const int pos = atomicAdd(&sHist[q], 1);  // < nE <= kChunk
            sE[pos] = make_entry(ldg_vf(VF + fE), fE, tileX0, tileY0, tileW, tileH);
            // the bucket's lower edge, pulled down by 0.1% of its offset so rounding
            // in the bucket index can never leave a member below it
            sBucketLo[pos] = q == 0 ? -kInf : q == 1 ? lo : lo + (float)(q - 1) * edge;
        }
        __syncthreads();
        for (int k = tid; k <= kBuckets; k += kTilePix) sHist[k] = 0;  // free until the next chunk's first barrier

        // The warp takes the sorted entries 32 at a time, one per lane: a
        // ballot marks those whose triangle may cover a pixel centre of the
        // warp's 8x4 block (box overlap, then the corner test over the part
        // of the box inside the block), and only they are visited.
        bool stop = false;
        for (int base = 0; base < nE && !stop; base += 32) {
            const int k = base + lane;
            bool meets = false;
            if (k < nE) {
                const float4 *rk = reinterpret_cast<const float4 *>(&sE[k]);
                const int4 bx = *reinterpret_cast<const int4 *>(rk);
                const int xl = max(bx.x, colLo), xh = min(bx.z, colHi), yl = max(bx.y, rowLo), yh = min(bx.w, rowHi);
                meets = xl <= xh && yl <= yh;
                if (meets) {
                    const float4 hk = rk[1];  // zLowSafe, mOut, flags, f
                    if (__float_as_int(hk.z) & kScreenValid) {
                        const float4 g1 = rk[3];
                        meets = may_cover_box(rk[2], g1.x, g1.y, hk.y, xl, xh, yl, yh);
                    }
                }
            }
            unsigned todo = __ballot_sync(0xffffffffu, meets);
            while (todo) {
            const int i = base + __ffs(todo) - 1;
            todo &= todo - 1;
            // every later entry of the chunk lies behind every pixel of this warp: stop
            if (sBucketLo[i] > __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(zup)))) {
                stop = true;
                break;
            }
            const float4 *row = reinterpret_cast<const float4 *>(&sE[i]);
            const int4 bx = *reinterpret_cast<const int4 *>(row);
            if (u < bx.x || u > bx.z || v < bx.y || v > bx.w) continue;
            const float4 h = row[1];  // zLowSafe, mOut, flags, f
            if (h.x > zup) continue;  // behind this pixel's covering face (and so is every later entry)
            const int flags = __float_as_int(h.z);
            float zlow = -kInf;
            if (flags & kScreenValid) {
                const float4 g0 = row[2], g1 = row[3];  // (x0, y0, a1, b1), (a2, b2, mIn, dRel)
                float l0, l1, l2;
                lambda_at(g0, g1.x, g1.y, px, py, l0, l1, l2);
                if (l0 < -h.y || l1 < -h.y || l2 < -h.y) continue;  // certainly outside
                const float zq = depth_at(row[4], l0, l1, l2);
                if ((flags & kCertain) && l0 >= g1.z && l1 >= g1.z && l2 >= g1.z)
                    zup = fminf(zup, zq * (1.0f + g1.w) + 2.0f);
                zlow = h.x;
                if (g1.w < 0.25f) zlow = fmaxf(zlow, zq * (1.0f - g1.w) - 2.0f);
                if (zlow > zup) continue;  // certainly behind a covering face
            }
            if (nCand == kMaxCand) {  // make room: drop candidates now known to lose
                int m = 0;
#pragma unroll 1
                for (int j = 0; j < kMaxCand; ++j) {
                    const float zj = sCandZ[j][tid];
                    if (!(zj > zup)) {
                        sCandF[m][tid] = sCandF[j][tid];
                        sCandZ[m][tid] = zj;
                        ++m;
                    }
                }
                nCand = m;
            }
            if (nCand == kMaxCand) {
                spill = true;
                continue;
            }
            sCandF[nCand][tid] = __float_as_int(h.w);
            sCandZ[nCand][tid] = zlow;
            ++nCand;
            }  // entries of the group that meet the block
        }
    }  // chunks

    if (u >= dims.W || v >= dims.H) return;

    // resolve: the reference's exact test on the candidates
    const Camera &cam = sCam;
    ExactCtx x;
    x.geo = ws.geo + (size_t)b * F;
    x.vface = VF;
    x.origS = v3(cam.origS[0], cam.origS[1], cam.origS[2]);
    x.d = pixel_ray(cam, u, v);
    unsigned long long best = kEmptyKey;
    V3 abc = v3(0.0f, 0.0f, 0.0f);
    if (!spill) {
        // the live candidates (bound not above the final zup) first, so that
        // the warp's exact tests line up: pass j tests every pixel's j-th
        int nLive = 0;
#pragma unroll 1
        for (int j = 0; j < nCand; ++j)
            if (!(sCandZ[j][tid] > zup)) sCandF[nLive++][tid] = sCandF[j][tid];
#pragma unroll 1
        for (int j = 0; j < nLive; ++j) {
            V3 t;
            const unsigned long long k = exact_key(x, sCandF[j][tid], t, nLive > 1);
            if (k < best) {
                best = k;
                abc = t;
            }
        }
    } else {
        // more candidates than slots (rare): test every entry of the tile
        // that may win against the final bound, rebuilt from the bins.  (A
        // second form over the staged entries, for tiles of one chunk, made
        // the common path spill.)
        for (int e = 0; e < nAll; ++e) {
            const int f = e < nTile ? ws.bins[s0 + e] : bigList[e - nTile];
            const Entry E = make_entry(VF[f], f, tileX0, tileY0, tileW, tileH);
            if (u < E.bx0 || u > E.bx1 || v < E.by0 || v > E.by1) continue;
            if (!may_win(E, px, py, zup)) continue;
            V3 t;
            const unsigned long long k = exact_key(x, E.f, t, true);
            if (k < best) {
                best = k;
                abc = t;
            }
        }
    }

    // the outputs are written once and not read again by this launch:
    // evict-first stores (st.global.cs) leave the L2 to the face records,
    // shading records and texels that neighbouring tiles read again
    const size_t p = ((size_t)bc * dims.H + v) * dims.W + u;
    if (best == kEmptyKey) {
        __stcs(io.face + p, -1);
        __stcs(reinterpret_cast<float2 *>(io.bary) + p, make_float2(0.0f, 0.0f));
        __stcs(io.render + 3 * p + 0, 0.0f);
        __stcs(io.render + 3 * p + 1, 1.0f);
        __stcs(io.render + 3 * p + 2, 0.0f);
        return;
    }
    const int f = (int)(unsigned)(best & 0xffffffffull);
    __stcs(io.face + p, f);
    __stcs(reinterpret_cast<float2 *>(io.bary) + p, make_float2(abc.x, abc.y));

    // shading (CUDABasedRasterization.cu:307-403) from the face's shading record
    const float4 *SR = ws.shadeRec + ((size_t)b * F + f) * kShadeRows;
    const float4 r0 = __ldg(SR), r1 = __ldg(SR + 1);
    const V3 d = x.d;
    V3 un = pixel_normal_un(v3(r0.x, r0.y, r0.z), v3(r0.w, r1.x, r1.y), v3(r1.z, r1.w, __ldg(&SR[2].x)), abc);
    bool flippedN;
    const V3 n = unit_normal(un, __fsqrt_rn(xdot(un, un)), d, flippedN);
    const int albedo = ALB >= 0 ? ALB : dims.albedo;
    float3 col;
    switch (albedo) {
        case GVR_ALBEDO_TEXTURED: {
            const float4 r2 = __ldg(SR + 2), r3 = __ldg(SR + 3);
            const float2 tc = texel_coord6(r2.y, r2.z, r2.w, r3.x, r3.y, r3.z, abc, dims.Wt, dims.Ht);
            int LU = __float2int_rz(xs(tc.x, 0.5f)), LV = __float2int_rz(xs(tc.y, 0.5f));
            const float *t = io.texture + (((size_t)b * dims.Ht + LV) * dims.Wt + LU) * 3;
            col = make_float3(__ldg(t), __ldg(t + 1), __ldg(t + 2));
            break;
        }
        case GVR_ALBEDO_VERTEX_COLOR: {
            const float4 r4 = SR[4];
            const int i0 = __float_as_int(r4.x), i1 = __float_as_int(r4.y), i2 = __float_as_int(r4.z);
            const float *Cb = io.colors + (size_t)b * topo.N * 3;
            const float *q0 = Cb + 3 * i0, *q1 = Cb + 3 * i1, *q2 = Cb + 3 * i2;
            col = make_float3(q0[0] * abc.x + q1[0] * abc.y + q2[0] * abc.z, q0[1] * abc.x + q1[1] * abc.y + q2[1] * abc.z,
                              q0[2] * abc.x + q1[2] * abc.y + q2[2] * abc.z);
            break;
        }
        case GVR_ALBEDO_NORMAL:
            col = make_float3((1.0f + n.x) * 0.5f, (1.0f + n.y) * 0.5f, (1.0f + n.z) * 0.5f);
            break;
        case GVR_ALBEDO_TEXTURED_BILINEAR: {
            const float4 r2 = SR[2], r3 = SR[3];
            const float2 tc = texel_coord6(r2.y, r2.z, r2.w, r3.x, r3.y, r3.z, abc, dims.Wt, dims.Ht);
            int idx[4];
            float w[4];
            bilinear_taps(tc.x, tc.y, dims.Wt, dims.Ht, idx, w);
            const float *tex = io.texture + (size_t)b * dims.Ht * dims.Wt * 3;
            col = make_float3(0.0f, 0.0f, 0.0f);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float *t = tex + 3 * (size_t)idx[k];
                col = make_float3(col.x + w[k] * t[0], col.y + w[k] * t[1], col.z + w[k] * t[2]);
            }
            break;
        }
        case GVR_ALBEDO_UV: {
            const float4 r2 = SR[2], r3 = SR[3];
            col = make_float3(abc.x * r2.y + abc.y * r2.w + abc.z * r3.y, abc.x * r2.z + abc.y * r3.x + abc.z * r3.z,
                              0.0f);
            break;
        }
        default:
            col = make_float3(1.0f, 1.0f, 1.0f);
            break;
    }
    const bool lit = albedo != GVR_ALBEDO_NORMAL && albedo != GVR_ALBEDO_UV;
    const bool shaded = (dims.shading == GVR_SHADING_SHADED && lit) || albedo == GVR_ALBEDO_LIGHTING;
    if (dims.shading == GVR_SHADING_PHONG && lit && albedo != GVR_ALBEDO_LIGHTING) {
        const float ndl = -(n.x * d.x + n.y * d.y + n.z * d.z);
        const float k = phong_factor(ndl), s = phong_specular(ndl);
        col = make_float3(col.x * k + s, col.y * k + s, col.z * k + s);
    } else if (shaded) {
        const float *sh = sSH;
        float basis[9];
        sh_basis(n, basis);
        float l0 = 0.0f, l1 = 0.0f, l2 = 0.0f;
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            l0 += sh[k] * basis[k];
            l1 += sh[9 + k] * basis[k];
            l2 += sh[18 + k] * basis[k];
        }
        col = make_float3(col.x * l0, col.y * l1, col.z * l2);
    }
    __stcs(io.render + 3 * p + 0, col.x);
    __stcs(io.render + 3 * p + 1, col.y);
    __stcs(io.render + 3 * p + 2, col.z);
}

}  // namespace

// One block per tile of one call: grid (tilesX, tilesY, views), views
// bcBase .. bcBase + gridDim.z - 1.  Compiled for the vertex-colour and the
// textured albedo and for any mode (ALB = -1).
template <int ALB>
__global__ void __launch_bounds__(kTilePix, 5) k_raster(const FwdJob J, int bcBase) {
    pdl_enter();
    raster_tile<ALB>(J, bcBase + blockIdx.z, blockIdx.x, blockIdx.y);
}

// Persistent: a grid sized to the resident capacity pulls (job, view, tile)
// items from one counter until all jobs' tiles are done.  itemStart[j] is the
// first item of job j (exclusive prefix of its B*C*tiles).
__global__ void __launch_bounds__(kTilePix, 4) k_raster_persistent(const FwdJob *__restrict__ jobs,
                                                                const int *__restrict__ itemStart, int nJobs,
                                                                int *__restrict__ counter) {
    __shared__ int sItem, sJob, sBC, sTX, sTY;
    __shared__ FwdJob sJ;
    const int total = itemStart[nJobs];
    for (;;) {
        if (threadIdx.x == 0) {
            const int item = atomicAdd(counter, 1);
            int j = 0;
            if (item < total) {
                int lo = 0, hi = nJobs - 1;  // last job whose first item is <= item
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (itemStart[mid] <= item) lo = mid;
                    else hi = mid - 1;
                }
                j = lo;
                // (view, tile) of the item, decomposed once for the block
                const FrameDims &d = jobs[j].dims;
                const int local = item - itemStart[j], T = d.tilesX * d.tilesY, tile = local % T;
                sBC = local / T;
                sTX = tile % d.tilesX;
                sTY = tile / d.tilesX;
            }
            sItem = item;
            sJob = j;
        }
        __syncthreads();
        const int item = sItem, j = sJob;
        if (item >= total) break;
        // the job record, staged once per item for uniform shared-memory reads
        const int words = (int)(sizeof(FwdJob) / sizeof(int));
        for (int w = threadIdx.x; w < words; w += blockDim.x)
            reinterpret_cast<int *>(&sJ)[w] = reinterpret_cast<const int *>(jobs + j)[w];
        __syncthreads();
        raster_tile<-1>(sJ, sBC, sTX, sTY);
        __syncthreads();  // shared memory and sItem are reused by the next item
    }
}

cudaError_t launch_raster(const FwdJob &J, cudaStream_t st) {
    const int BC = J.dims.B * J.dims.C;
    void (*kernel)(const FwdJob, int) = J.dims.albedo == GVR_ALBEDO_TEXTURED        ? k_raster<GVR_ALBEDO_TEXTURED>
                                        : J.dims.albedo == GVR_ALBEDO_VERTEX_COLOR ? k_raster<GVR_ALBEDO_VERTEX_COLOR>
                                                                                   : k_raster<-1>;
    for (int bc0 = 0; bc0 < BC; bc0 += 65535) {  // gridDim.z holds at most 65535 views
        const dim3 grid(J.dims.tilesX, J.dims.tilesY, min(65535, BC - bc0));
        cudaError_t e;
        GVR_LAUNCH(st, "k_raster", e = launch_pdl(kernel, grid, dim3(kTilePix), 0, st, J, bc0));
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_raster_persistent(const FwdJob *jobs, const int *itemStart, int nJobs, int *counter, int grid,
                                     cudaStream_t st) {
    GVR_LAUNCH(st, "k_raster_persistent",
               k_raster_persistent<<<grid, kTilePix, 0, st>>>(jobs, itemStart, nJobs, counter));
    return cudaGetLastError();
}

int raster_persistent_blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_raster_persistent, kTilePix, 0) != cudaSuccess) return 1;
    return n > 0 ? n : 1;
}

}  // namespace gvr

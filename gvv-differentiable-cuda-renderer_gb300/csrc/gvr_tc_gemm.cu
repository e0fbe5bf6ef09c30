// gvr_tc_gemm.cu -- BF16 GEMM on the 5th-generation tensor cores (tcgen05)
// with FP32 accumulation in tensor memory, plus the im2col / col2im kernels
// that turn the proposal network's 3x3 stride-2 convolutions into GEMMs.
//
// C[M, N] = A[M, K] * B[N, K]^T (+ bias[N], optional ReLU), A and B
// row-major with K contiguous ("K-major"), C row-major FP32 or BF16.
//
// One CTA of 128 threads computes a 128 x BN tile (BN in {32, 64, 128, 256},
// the smallest that covers N, else 256) through a pipeline of S stages:
//   * thread 0 (producer) issues, per K step of 64, two TMA tile loads
//     (cp.async.bulk.tensor, 128-byte swizzle: rows of 128 B, 16-byte chunks
//     XOR-permuted within 8-row atoms of 1 KB) into stage s and arms the
//     stage's `full` mbarrier with their byte count; before reusing a stage
//     it waits on the stage's `empty` mbarrier;
//   * thread 32 (MMA issuer) waits on `full`, issues four
//     tcgen05.mma.cta_group::1.kind::f16 (K = 16 each: the shared-memory
//     descriptors of the swizzled K-major tiles advance 32 B per K slice)
//     and a tcgen05.commit that arrives on `empty` when they have read the
//     stage; after the last step a commit arrives on `done`;
//   * warp 0 allocates BN columns of tensor memory; after `done`, the four
//     warps read the accumulator with tcgen05.ld (warp w = TMEM lanes
//     32w..32w+31 = rows), add the bias, apply ReLU and store 16 bytes at a
//     time (or add FP32 partials with vector atomics when K is split).
// Rows and columns outside the matrices are zero-filled by the TMA.  Every
// mbarrier wait is bounded (about one second of %globaltimer); a timeout
// sets an error flag in shared memory, the block drains the TMA loads it
// issued and the MMAs it committed (bounded), skips the epilogue, records
// the error in g_tc_error, frees its tensor memory and returns.
#include <cuda.h>  // CUtensorMap and its enums (the encoder is looked up at run time)
#include <cuda_bf16.h>
#include <stdint.h>

#include "gvr_nn.h"
#include "gvr_profile.h"

namespace gvr {
namespace {

constexpr int kBM = 128, kBK = 64, kThreads = 128, kMaxStages = 4;
constexpr int kATileBytes = kBM * kBK * 2;  // one 128 x 64 BF16 operand tile (16 KB)
constexpr uint64_t kWaitNs = 1000000000ull;

__device__ int g_tc_error;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase with `parity` to complete, at most limit_ns (~1 s).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint64_t limit_ns = kWaitNs) {
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > limit_ns) return false;
    return true;
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// One 2D TMA tile load (x = K element offset, y = row) completing on `bar`.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Test hook of the bounded waits: one warp waits on an mbarrier that nothing
// arrives on, gives up after limit_ns, records error code 2 and returns (no
// tensor memory or MMA involved, so nothing is left in flight).
__global__ void k_tc_wait_probe(unsigned long long limit_ns) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    __syncthreads();
    const bool done = mbar_wait(&bar, 0, limit_ns);
    if (!done && threadIdx.x == 0) atomicExch(&g_tc_error, 2);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor of a K-major tile with 128-byte swizzle:
// start address, leading byte offset 16 (unused for swizzled K-major),
// stride byte offset 1024 (between 8-row atoms), descriptor version 1,
// swizzle mode 2 (128 B).  Tiles start on 1 KB boundaries.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(16 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
           (1ull << 46) | (2ull << 61);
}

// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

template <int BN>
__global__ void __launch_bounds__(kThreads) k_gemm_bf16(const __grid_constant__ CUtensorMap tmA,
                                                        const __grid_constant__ CUtensorMap tmB, void *__restrict__ C,
                                                        const float *__restrict__ bias, int M, int N, int K, int ldc,
                                                        int flags, int stages) {
    constexpr int kBTileBytes = BN * kBK * 2;
    extern __shared__ uint8_t smemRaw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smemRaw) + 1023) & ~uintptr_t(1023));
    uint8_t *sA = smem;                         // stages x 16 KB
    uint8_t *sB = smem + stages * kATileBytes;  // stages x BN x 128 B
    __shared__ __align__(8) uint64_t fullBar[kMaxStages], emptyBar[kMaxStages], doneBar;
    __shared__ uint32_t tmemBase;
    __shared__ int sErr, sIssued, sConsumed;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * BN;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmemBase)),
                     "r"((uint32_t)BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < stages; ++s) {
            mbar_init(&fullBar[s], 1);
            mbar_init(&emptyBar[s], 1);
        }
        mbar_init(&doneBar, 1);
        sErr = 0;
        sIssued = 0;
        sConsumed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmemBase;
    constexpr uint32_t idesc = instr_desc(kBM, BN);

    // this CTA's share of the K steps (all of them unless K is split over gridDim.z CTAs)
    const int KTall = K / kBK, per = (KTall + gridDim.z - 1) / gridDim.z;
    const int ktBegin = blockIdx.z * per, ktEnd = min(KTall, ktBegin + per);
    const int KT = max(0, ktEnd - ktBegin);

    if (tid == 0) {  // producer: stage s of round r is free once round r - 1's MMAs have read it
        int kt = 0;
        for (; kt < KT; ++kt) {
            const int s = kt % stages, r = kt / stages;
            if (r > 0 && !mbar_wait(&emptyBar[s], (r - 1) & 1)) {
                sErr = 1;
                break;
            }
            mbar_arrive_expect_tx(&fullBar[s], (uint32_t)(kATileBytes + kBTileBytes));
            const int k0 = (ktBegin + kt) * kBK;
            tma_load_2d(sA + s * kATileBytes, &tmA, &fullBar[s], k0, m0);
            tma_load_2d(sB + s * kBTileBytes, &tmB, &fullBar[s], k0, n0);
        }
        sIssued = kt;
    } else if (tid == 32) {  // MMA issuer
        int kt = 0;
        for (; kt < KT; ++kt) {
            const int s = kt % stages, r = kt / stages;
            if (!mbar_wait(&fullBar[s], r & 1)) {
                sErr = 1;
                break;
            }
            tc_fence_after();
            const uint32_t a0 = smem_u32(sA + s * kATileBytes), b0 = smem_u32(sB + s * kBTileBytes);
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk) {  // K = 16 per MMA: 32 B further along the swizzled rows
                const uint64_t ad = sw128_desc(a0 + kk * 32), bd = sw128_desc(b0 + kk * 32);
                const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&emptyBar[s]))
                         : "memory");
        }
        sConsumed = kt;
        if (kt > 0)  // tracks every MMA issued before it
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&doneBar))
                         : "memory");
    }
    __syncthreads();
    bool ok = true;
    if (tid == 0) {
        // loads issued but never consumed (only after a timeout) land before the block moves on
        for (int kt = sConsumed; kt < sIssued; ++kt) mbar_wait(&fullBar[kt % stages], (kt / stages) & 1);
        ok = (sConsumed == 0 || mbar_wait(&doneBar, 0)) && sErr == 0;
        if (!ok) atomicExch(&g_tc_error, 1);
    }
    ok = __syncthreads_and(ok) != 0;
    tc_fence_after();

    if (ok && KT > 0) {
        const int row = m0 + warp * 32 + lane;
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
        const bool relu = flags & GVR_GEMM_RELU, outBf16 = flags & GVR_GEMM_OUT_BF16;
        const bool split = gridDim.z > 1, addBias = bias && blockIdx.z == 0;
        const bool vec = (ldc % 8) == 0 && (reinterpret_cast<uintptr_t>(C) & 15) == 0;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            uint32_t v[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                "%13, %14, %15}, [%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(taddr + (uint32_t)c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            const int col0 = n0 + c0;
            if (row >= M || col0 >= N) continue;
            float x[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                x[j] = __uint_as_float(v[j]);
                if (addBias && col0 + j < N) x[j] += bias[col0 + j];
                if (!split && relu) x[j] = fmaxf(x[j], 0.0f);
            }
            const bool full = col0 + 16 <= N && vec;
            if (split) {
                float *Cr = reinterpret_cast<float *>(C) + (size_t)row * ldc + col0;
                if (full) {
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        atomicAdd(reinterpret_cast<float4 *>(Cr) + q, make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]));
                } else {
                    for (int j = 0; j < 16 && col0 + j < N; ++j) atomicAdd(Cr + j, x[j]);
                }
            } else if (outBf16) {
                __nv_bfloat16 *Cr = reinterpret_cast<__nv_bfloat16 *>(C) + (size_t)row * ldc + col0;
                if (full) {
                    uint32_t w[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const __nv_bfloat162 h = __floats2bfloat162_rn(x[2 * q], x[2 * q + 1]);
                        w[q] = *reinterpret_cast<const uint32_t *>(&h);
                    }
                    reinterpret_cast<uint4 *>(Cr)[0] = make_uint4(w[0], w[1], w[2], w[3]);
                    reinterpret_cast<uint4 *>(Cr)[1] = make_uint4(w[4], w[5], w[6], w[7]);
                } else {
                    for (int j = 0; j < 16 && col0 + j < N; ++j) Cr[j] = __float2bfloat16_rn(x[j]);
                }
            } else {
                float *Cr = reinterpret_cast<float *>(C) + (size_t)row * ldc + col0;
                if (full) {
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        reinterpret_cast<float4 *>(Cr)[q] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
                } else {
                    for (int j = 0; j < 16 && col0 + j < N; ++j) Cr[j] = x[j];
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)BN)
                                : "memory");
}

// im2col of a 3x3, stride-2, padding-1 convolution over an NHWC BF16 input:
// row (b, oy, ox), column (ky * 3 + kx) * Cin + c, zero-padded to Kpad.
__global__ void k_im2col_3x3s2(const __nv_bfloat16 *__restrict__ x, __nv_bfloat16 *__restrict__ col, int B, int H,
                               int W, int Cin, int Ho, int Wo, int Kpad) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t total = (size_t)B * Ho * Wo * Kpad;
    if (i >= total) return;
    const int k = (int)(i % Kpad);
    const size_t m = i / Kpad;
    const int ox = (int)(m % Wo), oy = (int)((m / Wo) % Ho), b = (int)(m / ((size_t)Wo * Ho));
    __nv_bfloat16 v = __float2bfloat16_rn(0.0f);
    if (k < 9 * Cin) {
        const int tap = k / Cin, c = k - tap * Cin;
        const int iy = 2 * oy + tap / 3 - 1, ix = 2 * ox + tap % 3 - 1;
        if (iy >= 0 && iy < H && ix >= 0 && ix < W) v = x[(((size_t)b * H + iy) * W + ix) * Cin + c];
    }
    col[i] = v;
}

// col2im (the adjoint of k_im2col_3x3s2): every input element sums the
// column entries that read it; FP32 in, FP32 out.
__global__ void k_col2im_3x3s2(const float *__restrict__ col, float *__restrict__ dx, int B, int H, int W, int Cin,
                               int Ho, int Wo, int Kpad) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t total = (size_t)B * H * W * Cin;
    if (i >= total) return;
    const int c = (int)(i % Cin);
    const int ix = (int)((i / Cin) % W), iy = (int)((i / ((size_t)Cin * W)) % H), b = (int)(i / ((size_t)Cin * W * H));
    float acc = 0.0f;
#pragma unroll
    for (int ky = 0; ky < 3; ++ky) {
        const int ty = iy + 1 - ky;  // = 2 * oy
        if (ty < 0 || (ty & 1) || (ty >> 1) >= Ho) continue;
#pragma unroll
        for (int kx = 0; kx < 3; ++kx) {
            const int tx = ix + 1 - kx;
            if (tx < 0 || (tx & 1) || (tx >> 1) >= Wo) continue;
            const size_t m = ((size_t)b * Ho + (ty >> 1)) * Wo + (tx >> 1);
            acc += col[m * Kpad + (ky * 3 + kx) * Cin + c];
        }
    }
    dx[i] = acc;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled, looked up once through the runtime (no link-time
// dependency on the driver library).
EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// Tensor map of a row-major BF16 matrix [rows, K] with row stride ld
// elements, read in boxes of `boxRows` rows x 64 K-elements (128 B) with
// 128-byte swizzle; out-of-range rows read as zeros.
bool make_map(CUtensorMap *map, const void *base, int rows, int K, int ld, int boxRows) {
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)boxRows};
    const cuuint32_t elem[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, elem,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
cudaError_t launch_gemm(const GvrGemmArgs &a, cudaStream_t st, bool &mapFailed) {
    constexpr int stageBytes = kATileBytes + BN * kBK * 2;
    // about 100 KB of stages in flight per CTA (two CTAs per SM), 2..4 deep,
    // no deeper than this CTA's K steps
    const int KTall = a.K / kBK, splits = a.k_splits > 1 ? a.k_splits : 1;
    const int per = (KTall + splits - 1) / splits;
    const int stages = max(1, min(min(kMaxStages, max(2, (100 * 1024) / stageBytes)), per));
    // + alignment slack for the 1 KB swizzle atoms; at least enough that no
    // more CTAs fit on an SM than its 512 tensor-memory columns hold
    constexpr int kSmemPerSM = 233472, kTmemCols = 512;
    const int smem = max(stages * stageBytes + 1024, kSmemPerSM / (kTmemCols / BN + 1) - 1024 + 16);
    // the kernel's shared-memory limit is a per-device attribute: raise it once per device
    static bool raised[64] = {false};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64 || !raised[dev]) {
        e = cudaFuncSetAttribute(k_gemm_bf16<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kMaxStages * stageBytes + 1024);
        if (e != cudaSuccess) return e;
        if (dev >= 0 && dev < 64) raised[dev] = true;
    }
    CUtensorMap mA, mB;
    if (!make_map(&mA, a.A, a.M, a.K, a.lda, kBM) || !make_map(&mB, a.B, a.N, a.K, a.ldb, BN)) {
        mapFailed = true;
        return cudaErrorInvalidValue;
    }
    dim3 grid((a.N + BN - 1) / BN, (a.M + kBM - 1) / kBM, splits);
    GVR_LAUNCH(st, BN == 256 ? "k_gemm_bf16_n256" : BN == 128 ? "k_gemm_bf16_n128" : BN == 64 ? "k_gemm_bf16_n64"
                                                                                               : "k_gemm_bf16_n32",
               (k_gemm_bf16<BN><<<grid, kThreads, smem, st>>>(mA, mB, a.C, a.bias, a.M, a.N, a.K, a.ldc, a.flags,
                                                               stages)));
    return cudaGetLastError();
}

}  // namespace
}  // namespace gvr

namespace {
thread_local const char *g_nn_error = "";
int nn_fail(int code, const char *msg) {
    g_nn_error = msg;
    return code;
}
}  // namespace

extern "C" {

const char *gvr_nn_last_error(void) { return g_nn_error; }

int gvr_gemm_bf16(const GvrGemmArgs *a, void *stream) {
    if (!a || !a->A || !a->B || !a->C) return nn_fail(GVR_ERR_INVALID_ARGUMENT, "gemm: null pointer");
    if (a->M < 1 || a->N < 1 || a->K < 64 || a->K % 64)
        return nn_fail(GVR_ERR_INVALID_ARGUMENT, "gemm: M, N >= 1 and K a positive multiple of 64");
    if (a->lda < a->K || a->ldb < a->K || a->lda % 8 || a->ldb % 8 || a->ldc < a->N)
        return nn_fail(GVR_ERR_INVALID_ARGUMENT, "gemm: lda, ldb >= K and multiples of 8; ldc >= N");
    if ((reinterpret_cast<uintptr_t>(a->A) | reinterpret_cast<uintptr_t>(a->B)) % 16)
        return nn_fail(GVR_ERR_INVALID_ARGUMENT, "gemm: A and B must be 16-byte aligned");
    if ((long long)(a->M + 127) / 128 > 65535) return nn_fail(GVR_ERR_INVALID_ARGUMENT, "gemm: M too large");
    if (a->k_splits > 1 && (a->k_splits > 65535 || (a->flags & (GVR_GEMM_RELU | GVR_GEMM_OUT_BF16))))
        return nn_fail(GVR_ERR_INVALID_ARGUMENT, "gemm: k_splits needs FP32 output without ReLU (and <= 65535)");
    if ((long long)(a->N + 255) / 256 > 2147483647LL || a->M > 2147483647 - 127)
        return nn_fail(GVR_ERR_INVALID_ARGUMENT, "gemm: N or M too large");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    bool mapFailed = false;
    const cudaError_t e = a->N <= 32    ? gvr::launch_gemm<32>(*a, st, mapFailed)
                          : a->N <= 64  ? gvr::launch_gemm<64>(*a, st, mapFailed)
                          : a->N <= 128 ? gvr::launch_gemm<128>(*a, st, mapFailed)
                                        : gvr::launch_gemm<256>(*a, st, mapFailed);
    if (mapFailed) return nn_fail(GVR_ERR_CUDA, "gemm: tensor map encoding failed (cuTensorMapEncodeTiled)");
    return e == cudaSuccess ? GVR_OK : nn_fail(GVR_ERR_CUDA, cudaGetErrorString(e));
}

int gvr_tc_error(int clear) {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, gvr::g_tc_error, sizeof(int)) != cudaSuccess) return -1;
    if (clear && v) {
        const int z = 0;
        cudaMemcpyToSymbol(gvr::g_tc_error, &z, sizeof(int));
    }
    return v;
}

int gvr_tc_wait_probe(unsigned long long limit_ns, void *stream) {
    if (limit_ns == 0 || limit_ns > 2000000000ull)
        return nn_fail(GVR_ERR_INVALID_ARGUMENT, "wait probe: limit must be in (0, 2 s]");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    gvr::k_tc_wait_probe<<<1, 32, 0, st>>>(limit_ns);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GVR_OK : nn_fail(GVR_ERR_CUDA, cudaGetErrorString(e));
}

int gvr_im2col_3x3s2(const void *x, void *col, int B, int H, int W, int Cin, int Kpad, void *stream) {
    if (!x || !col || B < 1 || H < 1 || W < 1 || Cin < 1 || Kpad < 9 * Cin)
        return nn_fail(GVR_ERR_INVALID_ARGUMENT, "im2col: bad arguments");
    const int Ho = (H + 1) / 2, Wo = (W + 1) / 2;
    const size_t total = (size_t)B * Ho * Wo * Kpad;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    GVR_LAUNCH(st, "k_im2col_3x3s2",
               (gvr::k_im2col_3x3s2<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(
                   static_cast<const __nv_bfloat16 *>(x), static_cast<__nv_bfloat16 *>(col), B, H, W, Cin, Ho, Wo,
                   Kpad)));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GVR_OK : nn_fail(GVR_ERR_CUDA, cudaGetErrorString(e));
}

int gvr_col2im_3x3s2(const float *col, float *dx, int B, int H, int W, int Cin, int Kpad, void *stream) {
    if (!col || !dx || B < 1 || H < 1 || W < 1 || Cin < 1 || Kpad < 9 * Cin)
        return nn_fail(GVR_ERR_INVALID_ARGUMENT, "col2im: bad arguments");
    const int Ho = (H + 1) / 2, Wo = (W + 1) / 2;
    const size_t total = (size_t)B * H * W * Cin;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    GVR_LAUNCH(st, "k_col2im_3x3s2",
               (gvr::k_col2im_3x3s2<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(col, dx, B, H, W, Cin, Ho, Wo,
                                                                                     Kpad)));
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GVR_OK : nn_fail(GVR_ERR_CUDA, cudaGetErrorString(e));
}

}  // extern "C"

// gvr_tc_gemm.cu -- BF16 GEMM on the 5th-generation tensor cores (tcgen05)
// with FP32 accumulation in tensor memory, plus the im2col / col2im kernels
// that turn the proposal network's 3x3 stride-2 convolutions into GEMMs.
//
// C[M, N] = A[M, K] * B[N, K]^T (+ bias[N], optional ReLU), A and B
// row-major with K contiguous ("K-major"), C row-major FP32 or BF16.
//
// One CTA of 128 threads computes a 128 x BN tile:
//   * warp 0 allocates BN columns of tensor memory (128 lanes x BN FP32);
//   * every K step of 64, all threads copy the A and B tiles from global
//     memory into shared memory in the canonical no-swizzle K-major layout
//     (8-row x 16-byte core matrices; core matrices adjacent in K are 128 B
//     apart, 8-row groups 1024 B apart), fence them to the async proxy and
//     sync; thread 0 issues four tcgen05.mma (K = 16 each) and a
//     tcgen05.commit that arrives on the stage's mbarrier when they finish;
//   * two stages: the copy of step k overlaps the MMAs of step k-1, and a
//     stage is overwritten only after its mbarrier reports the MMAs that
//     read it complete;
//   * the epilogue waits for the last commit, reads the accumulator with
//     tcgen05.ld (warp w owns lanes 32w..32w+31 = rows), adds the bias,
//     applies ReLU and stores.
// Every mbarrier wait is bounded (about one second of %globaltimer) and is
// done by thread 0 alone; the block then agrees on the outcome with
// __syncthreads_and, so every thread leaves the K loop, skips the epilogue
// and reaches the tensor-memory free together.  On timeout the kernel
// records an error code in g_tc_error, waits once more (bounded) for its
// MMAs, frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <stdint.h>

#include "gvr_nn.h"
#include "gvr_profile.h"

namespace gvr {
namespace {

constexpr int kBM = 128, kBK = 64, kThreads = 128, kStages = 2;
constexpr int kTileBytes = kBM * kBK * 2;  // one 128 x 64 BF16 operand tile (16 KB)

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
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint64_t limit_ns = 1000000000ull) {
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > limit_ns) return false;
    return true;
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

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (8-row group) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Copies rows [r0, r0 + 128) x K columns [k0, k0 + 64) of a K-major BF16
// matrix into one canonical tile; rows at or beyond `rows` are zero.
__device__ __forceinline__ void load_tile(uint8_t *tile, const __nv_bfloat16 *__restrict__ X, int r0, int rows, int k0,
                                          int ld) {
    for (int c = threadIdx.x; c < kBM * (kBK / 8); c += kThreads) {
        const int r = c >> 3, kc = c & 7;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (r0 + r < rows) v = *reinterpret_cast<const uint4 *>(X + (size_t)(r0 + r) * ld + k0 + kc * 8);
        *reinterpret_cast<uint4 *>(tile + ((r >> 3) * 8 + kc) * 128 + (r & 7) * 16) = v;
    }
}

template <int BN>
__global__ void __launch_bounds__(kThreads) k_gemm_bf16(const __nv_bfloat16 *__restrict__ A,
                                                        const __nv_bfloat16 *__restrict__ B, void *__restrict__ C,
                                                        const float *__restrict__ bias, int M, int N, int K, int lda,
                                                        int ldb, int ldc, int flags) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA = smem;                          // kStages x 16 KB
    uint8_t *sB = smem + kStages * kTileBytes;   // kStages x (BN x 64 x 2) bytes
    constexpr int kBTile = BN * kBK * 2;
    __shared__ __align__(8) uint64_t mbar[kStages];
    __shared__ uint32_t tmemBase;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * BN;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmemBase)),
                     "r"((uint32_t)BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(&mbar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
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
    // The commit of step j arrives on mbar[j % 2]; it completes that
    // barrier's phase j / 2, so its wait parity is (j / 2) & 1.
    bool ok = true;
    int issued = 0;  // steps whose MMAs were committed
    for (int kt = 0; kt < KT; ++kt) {
        const int s = kt & 1;
        if (kt >= kStages) {  // the MMAs of step kt - 2 read this stage
            bool done = true;
            if (tid == 0) done = mbar_wait(&mbar[s], ((kt - kStages) >> 1) & 1);
            if (!__syncthreads_and(done)) {  // one decision for the whole block
                ok = false;
                break;
            }
        }
        const int k0 = (ktBegin + kt) * kBK;
        load_tile(sA + s * kTileBytes, A, m0, M, k0, lda);
        for (int c = tid; c < BN * (kBK / 8); c += kThreads) {
            const int r = c >> 3, kc = c & 7;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (n0 + r < N) v = *reinterpret_cast<const uint4 *>(B + (size_t)(n0 + r) * ldb + k0 + kc * 8);
            *reinterpret_cast<uint4 *>(sB + s * kBTile + ((r >> 3) * 8 + kc) * 128 + (r & 7) * 16) = v;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t a0 = smem_u32(sA + s * kTileBytes), b0 = smem_u32(sB + s * kBTile);
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk) {  // K = 16 per MMA: two core matrices along K
                const uint64_t ad = smem_desc(a0 + kk * 256, 128, 1024);
                const uint64_t bd = smem_desc(b0 + kk * 256, 128, 1024);
                const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&mbar[s]))
                         : "memory");
        }
        issued = kt + 1;
    }
    // the last commit tracks every MMA issued before it
    if (issued > 0) {
        const int j = issued - 1;
        bool done = true;
        if (tid == 0) {
            done = ok && mbar_wait(&mbar[j & 1], (j >> 1) & 1);
            if (!done) {  // record, then give the MMAs in flight one more bounded wait before the free
                atomicExch(&g_tc_error, 1);
                mbar_wait(&mbar[j & 1], (j >> 1) & 1);
            }
        }
        ok = __syncthreads_and(done) != 0;
    }
    tc_fence_after();

    if (ok && KT > 0) {
        const int row = m0 + warp * 32 + lane;
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
        const bool relu = flags & GVR_GEMM_RELU, outBf16 = flags & GVR_GEMM_OUT_BF16;
        const bool split = gridDim.z > 1, addBias = bias && blockIdx.z == 0;
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
            if (row < M) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int col = n0 + c0 + j;
                    if (col >= N) break;
                    float x = __uint_as_float(v[j]);
                    if (addBias) x += bias[col];
                    if (split) {
                        atomicAdd(reinterpret_cast<float *>(C) + (size_t)row * ldc + col, x);
                        continue;
                    }
                    if (relu) x = fmaxf(x, 0.0f);
                    if (outBf16) reinterpret_cast<__nv_bfloat16 *>(C)[(size_t)row * ldc + col] = __float2bfloat16_rn(x);
                    else reinterpret_cast<float *>(C)[(size_t)row * ldc + col] = x;
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

template <int BN>
cudaError_t launch_gemm(const GvrGemmArgs &a, cudaStream_t st) {
    const int smem = kStages * (kTileBytes + BN * kBK * 2);
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_gemm_bf16<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    dim3 grid((a.N + BN - 1) / BN, (a.M + kBM - 1) / kBM, a.k_splits > 1 ? a.k_splits : 1);
    GVR_LAUNCH(st, BN == 128 ? "k_gemm_bf16_n128" : "k_gemm_bf16_n64",
               (k_gemm_bf16<BN><<<grid, kThreads, smem, st>>>(
                   static_cast<const __nv_bfloat16 *>(a.A), static_cast<const __nv_bfloat16 *>(a.B), a.C, a.bias,
                   a.M, a.N, a.K, a.lda, a.ldb, a.ldc, a.flags)));
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
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = a->N <= 64 ? gvr::launch_gemm<64>(*a, st) : gvr::launch_gemm<128>(*a, st);
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

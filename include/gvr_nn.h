/*
 * gvr_nn.h -- tensor-core kernels of the learned proposal network.
 *
 * No reference counterpart: the reference has no learned component.  The
 * proposal network (a 3x3 stride-2 convolution encoder and an MLP that
 * regresses morphable-model, pose and SH parameters from renders) runs its
 * convolutions as im2col + GEMM and its linear layers as GEMM, all through
 * gvr_gemm_bf16: BF16 operands on the tcgen05 tensor cores, FP32
 * accumulation in tensor memory.
 *
 * All pointers are device pointers; `stream` is a cudaStream_t.  Calls
 * return a GvrStatus (gvr.h); gvr_nn_last_error() gives the message.
 */
#ifndef GVR_NN_H
#define GVR_NN_H

#include <stddef.h>
#include <stdint.h>

#include "gvr.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GVR_GEMM_RELU 1     /* C = max(C, 0) after the bias              */
#define GVR_GEMM_OUT_BF16 2 /* C is stored as BF16 (default FP32)        */

/* C[M, N] = A[M, K] * B[N, K]^T + bias[N].  A and B are row-major BF16 with
 * K contiguous; K a positive multiple of 64; lda, ldb multiples of 8 (rows
 * 16-byte aligned); A and B 16-byte aligned; bias FP32 or NULL.
 * k_splits > 1 splits K over that many CTAs per output tile, each adding
 * its FP32 partial product into C with atomics (for the weight gradients,
 * whose outputs are small and K is the batch's pixel count): C must hold
 * zeros (or a sum to add to) and be FP32, without ReLU. */
typedef struct {
    const void *A;
    const void *B;
    void *C;
    const float *bias;
    int32_t M, N, K;
    int32_t lda, ldb, ldc;
    int32_t flags;
    int32_t k_splits;  /* 0 or 1: no split */
} GvrGemmArgs;

int gvr_gemm_bf16(const GvrGemmArgs *args, void *stream);

/* Nonzero if a GEMM gave up waiting for its tensor-core work (and so left
 * its tile unwritten); `clear` resets the flag.  -1 if it cannot be read. */
int gvr_tc_error(int clear);

/* Test hook of the bounded waits that gvr_tc_error reports: one warp waits
 * on an mbarrier that nothing arrives on, gives up after limit_ns
 * (0 < limit_ns <= 2e9), sets the flag to 2 and returns; the context stays
 * usable.  Asynchronous on `stream`. */
int gvr_tc_wait_probe(unsigned long long limit_ns, void *stream);

/* im2col of a 3x3, stride-2, padding-1 convolution: x NHWC BF16 [B,H,W,Cin]
 * -> col BF16 [B*Ho*Wo, Kpad] with Ho = ceil(H/2), Wo = ceil(W/2), column
 * (ky*3 + kx)*Cin + c, columns >= 9*Cin zero. */
int gvr_im2col_3x3s2(const void *x, void *col, int B, int H, int W, int Cin, int Kpad, void *stream);

/* The adjoint: dx FP32 [B,H,W,Cin] = sum of the FP32 col entries that read each element. */
int gvr_col2im_3x3s2(const float *col, float *dx, int B, int H, int W, int Cin, int Kpad, void *stream);

const char *gvr_nn_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* GVR_NN_H */

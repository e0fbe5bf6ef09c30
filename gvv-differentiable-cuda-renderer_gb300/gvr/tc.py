"""Tensor-core layers of the proposal network (include/gvr_nn.h).

Every matrix product -- the forward of a convolution or linear layer and
both products of its backward -- runs on gvr_gemm_bf16 (tcgen05, BF16
operands, FP32 accumulation in tensor memory).  Convolutions are 3x3,
stride 2, padding 1 over NHWC BF16 activations, done as im2col + GEMM; their
input gradient is GEMM + col2im.  Operands whose K is not a multiple of 64
are zero-padded; transposes of the backward operands are torch copies.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib

BF16 = torch.bfloat16


class GvrGemmArgs(ctypes.Structure):
    _fields_ = [("A", ctypes.c_void_p), ("B", ctypes.c_void_p), ("C", ctypes.c_void_p), ("bias", ctypes.c_void_p),
                ("M", ctypes.c_int32), ("N", ctypes.c_int32), ("K", ctypes.c_int32), ("lda", ctypes.c_int32),
                ("ldb", ctypes.c_int32), ("ldc", ctypes.c_int32), ("flags", ctypes.c_int32),
                ("k_splits", ctypes.c_int32)]

_SMS = None


def _target_ctas(dev):
    """Two CTAs per SM: enough tiles to fill the GPU."""
    global _SMS
    if _SMS is None:
        _SMS = torch.cuda.get_device_properties(dev).multi_processor_count
    return 2 * _SMS


RELU, OUT_BF16 = 1, 2
_L = None


def _lib_nn():
    global _L
    if _L is None:
        L = _lib.load()
        L.gvr_gemm_bf16.argtypes = [ctypes.POINTER(GvrGemmArgs), ctypes.c_void_p]
        L.gvr_gemm_bf16.restype = ctypes.c_int
        L.gvr_tc_error.argtypes = [ctypes.c_int]
        L.gvr_tc_error.restype = ctypes.c_int
        L.gvr_tc_wait_probe.argtypes = [ctypes.c_ulonglong, ctypes.c_void_p]
        L.gvr_tc_wait_probe.restype = ctypes.c_int
        L.gvr_im2col_3x3s2.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 5 + [ctypes.c_void_p]
        L.gvr_im2col_3x3s2.restype = ctypes.c_int
        L.gvr_col2im_3x3s2.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 5 + [ctypes.c_void_p]
        L.gvr_col2im_3x3s2.restype = ctypes.c_int
        L.gvr_nn_last_error.restype = ctypes.c_char_p
        _L = L
    return _L


def _check(rc):
    if rc != 0:
        raise _lib.GvrError(rc, _lib_nn().gvr_nn_last_error().decode())


def _stream(dev):
    return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def pad_k(x, mult=64):
    """x [R, K] -> [R, ceil(K / mult) * mult] contiguous, zero columns appended."""
    K = x.shape[1]
    Kp = (K + mult - 1) // mult * mult
    if Kp == K and x.is_contiguous():
        return x
    out = torch.zeros((x.shape[0], Kp), dtype=x.dtype, device=x.device)
    out[:, :K] = x
    return out


def gemm(A, B, bias=None, relu=False, out_dtype=torch.float32):
    """A [M, K] @ B [N, K]^T (+ bias, ReLU) on the tensor cores; BF16 operands."""
    A = pad_k(A.to(BF16))
    B = pad_k(B.to(BF16))
    if A.shape[1] != B.shape[1]:
        raise ValueError("inner dimensions differ")
    M, K = A.shape
    N = B.shape[0]
    tiles = ((M + 127) // 128) * ((N + (63 if N <= 64 else 127)) // (64 if N <= 64 else 128))
    # few output tiles and a long K (weight gradients, the first MLP layer):
    # split K over CTAs that add FP32 partials; ReLU / BF16 output follow in torch
    splits = 1
    if tiles < _target_ctas(A.device):
        splits = max(1, min(K // 64, _target_ctas(A.device) // tiles, 4096))
    if splits > 1 and (relu or out_dtype != torch.float32):
        C = gemm(A, B, bias=bias)
        C = torch.relu(C) if relu else C
        return C.to(out_dtype)
    C = (torch.zeros if splits > 1 else torch.empty)((M, N), dtype=out_dtype, device=A.device)
    bias_t = None if bias is None else bias.float().contiguous()
    flags = (RELU if relu else 0) | (OUT_BF16 if out_dtype == BF16 else 0)
    args = GvrGemmArgs(A.data_ptr(), B.data_ptr(), C.data_ptr(), None if bias_t is None else bias_t.data_ptr(),
                       M, N, K, K, K, N, flags, splits)
    _check(_lib_nn().gvr_gemm_bf16(ctypes.byref(args), _stream(A.device)))
    return C


def tc_error(clear=True):
    """Nonzero if a GEMM timed out waiting for its tensor-core work."""
    return int(_lib_nn().gvr_tc_error(1 if clear else 0))


def wait_probe(limit_ms, device):
    """Runs the bounded-wait test hook (an mbarrier wait that nothing ends,
    given up after `limit_ms`) on `device`'s current stream."""
    _check(_lib_nn().gvr_tc_wait_probe(int(limit_ms * 1e6), _stream(torch.device(device))))


def im2col(x, kpad):
    """x NHWC BF16 [B, H, W, C] -> [B * Ho * Wo, kpad] (3x3, stride 2, padding 1)."""
    B, H, W, C = x.shape
    Ho, Wo = (H + 1) // 2, (W + 1) // 2
    x = x.contiguous()
    col = torch.empty((B * Ho * Wo, kpad), dtype=BF16, device=x.device)
    _check(_lib_nn().gvr_im2col_3x3s2(x.data_ptr(), col.data_ptr(), B, H, W, C, kpad, _stream(x.device)))
    return col


def col2im(col, shape):
    """Adjoint of im2col: FP32 col [B * Ho * Wo, kpad] -> FP32 NHWC `shape`."""
    B, H, W, C = shape
    col = col.float().contiguous()
    dx = torch.empty(shape, dtype=torch.float32, device=col.device)
    _check(_lib_nn().gvr_col2im_3x3s2(col.data_ptr(), dx.data_ptr(), B, H, W, C, col.shape[1], _stream(col.device)))
    return dx


class Conv3x3s2(torch.autograd.Function):
    """y = ReLU(conv3x3s2(x, W) + b) with x, y NHWC; W [Cout, 9 * Cin] in
    (ky, kx, c) column order (FP32 master weights, BF16 on the tensor cores)."""

    @staticmethod
    def forward(ctx, x, w, b):
        B, H, W, C = x.shape
        Cout = w.shape[0]
        kpad = (9 * C + 63) // 64 * 64
        col = im2col(x.to(BF16), kpad)
        wb = pad_k(w.to(BF16), 64)
        y = gemm(col, wb, bias=b, relu=True, out_dtype=BF16)
        Ho, Wo = (H + 1) // 2, (W + 1) // 2
        y = y.view(B, Ho, Wo, Cout)
        ctx.save_for_backward(col, wb, y)
        ctx.shape = (B, H, W, C)
        ctx.x_dtype = x.dtype
        return y

    @staticmethod
    def backward(ctx, gy):
        col, wb, y = ctx.saved_tensors
        B, H, W, C = ctx.shape
        Cout = wb.shape[0]
        g = (gy.float() * (y > 0)).reshape(-1, Cout)           # through the ReLU
        gb = g.sum(0)
        g16 = g.to(BF16)
        # dW [Cout, K] = g^T [Cout, M] @ col [M, K]: operands K-major along M
        gw = gemm(g16.t().contiguous(), col.t().contiguous())[:, :9 * C]
        # dcol [M, K] = g [M, Cout] @ W [Cout, K]
        dcol = gemm(g16, wb.t().contiguous())
        gx = col2im(dcol, (B, H, W, C)).to(ctx.x_dtype)
        return gx, gw, gb


class Linear(torch.autograd.Function):
    """y = x @ W^T + b (ReLU optional) with W [out, in] (FP32 master)."""

    @staticmethod
    def forward(ctx, x, w, b, relu):
        xb, wb = x.to(BF16).contiguous(), w.to(BF16).contiguous()
        y = gemm(xb, wb, bias=b, relu=relu, out_dtype=torch.float32)
        ctx.save_for_backward(xb, wb, y)
        ctx.relu = relu
        ctx.x_dtype = x.dtype
        return y

    @staticmethod
    def backward(ctx, gy):
        xb, wb, y = ctx.saved_tensors
        g = gy.float() * (y > 0) if ctx.relu else gy.float()
        gb = g.sum(0)
        g16 = g.to(BF16)
        gw = gemm(g16.t().contiguous(), xb.t().contiguous())[:, :xb.shape[1]]
        gx = gemm(g16, wb.t().contiguous())[:, :xb.shape[1]].to(ctx.x_dtype)
        return gx, gw, gb, None

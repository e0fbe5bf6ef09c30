"""Image-space helpers on the GPU (gvr_image_gradient, gvr_image_gaussian3x3;
the reference's cpp/src/Renderer/gradientImage.cu:8-67)."""
from __future__ import annotations

import ctypes

import torch

from . import _lib


def _prep(img):
    img = img.float().contiguous()
    if img.dim() == 3:
        img = img.unsqueeze(0)
    if img.dim() != 4 or img.shape[-1] != 3 or not img.is_cuda:
        raise ValueError("expected a CUDA float tensor [B, H, W, 3] or [H, W, 3]")
    return img


def image_gradient(img):
    """(gx, gy) of [B, H, W, 3] images: 1/8-scaled Sobel, zero border
    (x < 1, y < 1, x >= W - 2, y >= H - 2)."""
    img = _prep(img)
    B, H, W, _ = img.shape
    gx, gy = torch.empty_like(img), torch.empty_like(img)
    st = ctypes.c_void_p(torch.cuda.current_stream(img.device).cuda_stream)
    _lib.check(_lib.load().gvr_image_gradient(ctypes.c_void_p(img.data_ptr()), ctypes.c_void_p(gx.data_ptr()),
                                              ctypes.c_void_p(gy.data_ptr()), B, W, H, st))
    return gx, gy


def gaussian3x3(img, out=None):
    """3x3 binomial blur of [B, H, W, 3] images; the one-pixel border of the
    result keeps the values of `out` (default: the input)."""
    img = _prep(img)
    B, H, W, _ = img.shape
    out = img.clone() if out is None else out
    st = ctypes.c_void_p(torch.cuda.current_stream(img.device).cuda_stream)
    _lib.check(_lib.load().gvr_image_gaussian3x3(ctypes.c_void_p(img.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                                 B, W, H, st))
    return out

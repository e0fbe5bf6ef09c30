"""tcgen05 BF16 GEMM and the proposal network's layers against a plain
PyTorch FP32 reference of the same op on the same BF16-rounded operands.

GEMM: max |C - C_ref| <= 2e-3 * max |C_ref| (FP32 accumulation in a
different order).  Layers (forward and both gradients): the same relative
bound, with the reference computed in FP32 from the BF16 operands the
kernels see.
"""
import pytest

pytestmark = pytest.mark.gpu

TOL = 2e-3


def _rel(a, b):
    a, b = a.double(), b.double()
    return float((a - b).abs().max() / b.abs().max().clamp_min(1e-30))


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (300, 200, 192), (1000, 64, 576), (77, 193, 512), (4096, 256, 2304),
                                   (4096, 32, 64), (513, 1000, 128), (260, 2304, 320), (129, 48, 4096)])
def test_gemm_matches_fp32_reference(M, N, K):
    import torch
    from gvr import tc
    torch.manual_seed(M + N + K)
    dev = torch.device("cuda", 0)
    A = torch.randn(M, K, device=dev).to(torch.bfloat16)
    B = torch.randn(N, K, device=dev).to(torch.bfloat16)
    bias = torch.randn(N, device=dev)
    C = tc.gemm(A, B, bias=bias)
    ref = A.float() @ B.float().t() + bias
    torch.cuda.synchronize()
    assert tc.tc_error() == 0
    assert _rel(C, ref) <= TOL
    Cr = tc.gemm(A, B, bias=bias, relu=True, out_dtype=torch.bfloat16)
    assert _rel(Cr.float(), torch.relu(ref)) <= 1e-2  # BF16 output rounding


def test_gemm_split_k_for_small_outputs():
    """Few output tiles and a long K: the K range is split over CTAs that
    add FP32 partials (the weight-gradient shape)."""
    import torch
    from gvr import tc
    torch.manual_seed(5)
    dev = torch.device("cuda", 0)
    A = torch.randn(40, 64 * 700, device=dev).to(torch.bfloat16)
    B = torch.randn(96, 64 * 700, device=dev).to(torch.bfloat16)
    bias = torch.randn(96, device=dev)
    C = tc.gemm(A, B, bias=bias)
    ref = A.float() @ B.float().t() + bias
    torch.cuda.synchronize()
    assert tc.tc_error() == 0
    assert _rel(C, ref) <= TOL
    Cr = tc.gemm(A, B, bias=bias, relu=True, out_dtype=torch.bfloat16)
    assert _rel(Cr.float(), torch.relu(ref)) <= 1e-2


def test_gemm_pads_k():
    import torch
    from gvr import tc
    dev = torch.device("cuda", 0)
    A = torch.randn(50, 27, device=dev).to(torch.bfloat16)
    B = torch.randn(32, 27, device=dev).to(torch.bfloat16)
    assert _rel(tc.gemm(A, B), A.float() @ B.float().t()) <= TOL


def test_im2col_col2im_are_adjoint_and_match_unfold():
    import torch
    import torch.nn.functional as Fn
    from gvr import tc
    dev = torch.device("cuda", 0)
    x = torch.randn(2, 9, 12, 5, device=dev).to(torch.bfloat16)
    kpad = 64
    col = tc.im2col(x, kpad)
    # unfold over NCHW gives (c, ky, kx) order; ours is (ky, kx, c)
    u = Fn.unfold(x.float().permute(0, 3, 1, 2), 3, padding=1, stride=2)     # [B, C*9, L]
    u = u.view(2, 5, 9, -1).permute(0, 3, 2, 1).reshape(-1, 45)
    assert torch.equal(col[:, :45].float(), u)
    assert torch.all(col[:, 45:] == 0)
    g = torch.randn(col.shape, device=dev)
    g[:, 45:] = 0
    dx = tc.col2im(g, tuple(x.shape))
    lhs = (col.float() * g).sum()
    rhs = (x.float() * dx).sum()
    assert abs(float(lhs - rhs)) <= 1e-4 * float(lhs.abs() + rhs.abs())


def test_conv_and_linear_layers_match_fp32_reference():
    import torch
    import torch.nn.functional as Fn
    from gvr import tc
    torch.manual_seed(0)
    dev = torch.device("cuda", 0)
    x = torch.randn(3, 16, 20, 24, device=dev).to(torch.bfloat16).requires_grad_(True)
    w = (torch.randn(40, 9 * 24, device=dev) * 0.1).requires_grad_(True)
    b = torch.randn(40, device=dev).requires_grad_(True)
    y = tc.Conv3x3s2.apply(x, w, b)
    gy = torch.randn(y.shape, device=dev)
    (y.float() * gy).sum().backward()
    # reference: FP32 conv on the BF16-rounded operands, weights from (ky, kx, c) order to OIHW
    xr = x.detach().float().permute(0, 3, 1, 2).requires_grad_(True)
    wr = w.detach().to(torch.bfloat16).float().view(40, 3, 3, 24).permute(0, 3, 1, 2).contiguous().requires_grad_(True)
    br = b.detach().clone().requires_grad_(True)
    yr = torch.relu(Fn.conv2d(xr, wr, br, stride=2, padding=1)).permute(0, 2, 3, 1)
    (yr * gy).sum().backward()
    assert _rel(y.float(), yr) <= 1e-2                      # y is stored in BF16
    assert _rel(x.grad.float(), xr.grad.permute(0, 2, 3, 1)) <= 1e-2
    assert _rel(w.grad, wr.grad.permute(0, 2, 3, 1).reshape(40, -1)) <= 1e-2
    assert _rel(b.grad, br.grad) <= 1e-2
    # linear
    xl = torch.randn(96, 300, device=dev).requires_grad_(True)
    wl = (torch.randn(193, 300, device=dev) * 0.05).requires_grad_(True)
    bl = torch.randn(193, device=dev).requires_grad_(True)
    yl = tc.Linear.apply(xl, wl, bl, True)
    gl = torch.randn(yl.shape, device=dev)
    (yl * gl).sum().backward()
    xq = xl.detach().to(torch.bfloat16).float().requires_grad_(True)
    wq = wl.detach().to(torch.bfloat16).float().requires_grad_(True)
    bq = bl.detach().clone().requires_grad_(True)
    yq = torch.relu(xq @ wq.t() + bq)
    (yq * gl).sum().backward()
    assert _rel(yl, yq) <= TOL
    assert _rel(xl.grad, xq.grad) <= 1e-2
    assert _rel(wl.grad, wq.grad) <= 1e-2
    assert tc.tc_error() == 0


def test_bounded_wait_times_out_and_leaves_the_context_usable():
    """A kernel waiting on an mbarrier that nothing arrives on gives up after
    its limit and reports it through gvr_tc_error; the GEMM still works and
    the flag stays clear afterwards."""
    import torch
    from gvr import tc
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    tc.tc_error(clear=True)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    tc.wait_probe(5.0, dev)
    t1.record()
    t1.synchronize()
    assert tc.tc_error(clear=True) == 2
    assert t0.elapsed_time(t1) >= 4.0       # it did wait about its limit
    A = torch.randn(128, 64, device=dev).to(torch.bfloat16)
    B = torch.randn(64, 64, device=dev).to(torch.bfloat16)
    C = tc.gemm(A, B)
    torch.cuda.synchronize()
    ref = A.float() @ B.float().t()
    assert torch.allclose(C, ref, rtol=2e-3, atol=2e-3)
    assert tc.tc_error(clear=False) == 0

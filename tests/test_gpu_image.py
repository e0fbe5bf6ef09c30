"""Image helpers (gradientImage.cu:8-55 of the reference) against a float32
numpy restatement with the same operation order: bit-exact, on sizes that
are and are not multiples of the 16 x 16 block."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _np_gradient(I):
    B, H, W, _ = I.shape
    gx, gy = np.zeros_like(I), np.zeros_like(I)
    f = np.float32
    for y in range(1, H - 2):
        for x in range(1, W - 2):
            i00, i01, i02 = I[:, y - 1, x - 1], I[:, y - 1, x], I[:, y - 1, x + 1]
            i10, i12 = I[:, y, x - 1], I[:, y, x + 1]
            i20, i21, i22 = I[:, y + 1, x - 1], I[:, y + 1, x], I[:, y + 1, x + 1]
            gx[:, y, x] = f(0.125) * (((i02 - i00) + f(2) * (i12 - i10)) + (i22 - i20))
            gy[:, y, x] = f(0.125) * (((i20 - i00) + f(2) * (i21 - i01)) + (i22 - i02))
    return gx, gy


def _np_gaussian(I):
    out = I.copy()
    B, H, W, _ = I.shape
    f = np.float32
    for y in range(1, H - 1):
        for x in range(1, W - 1):
            c = ((I[:, y - 1, x - 1] + I[:, y - 1, x + 1]) + I[:, y + 1, x - 1]) + I[:, y + 1, x + 1]
            e = ((I[:, y - 1, x] + I[:, y, x - 1]) + I[:, y, x + 1]) + I[:, y + 1, x]
            out[:, y, x] = (f(0.0625) * c + f(0.125) * e) + f(0.25) * I[:, y, x]
    return out


@pytest.mark.parametrize("H,W", [(16, 32), (23, 37)])
def test_image_gradient_and_gaussian_bit_exact(H, W):
    import torch
    from gvr import image
    rng = np.random.default_rng(H * W)
    I = rng.uniform(0, 1, (2, H, W, 3)).astype(np.float32)
    t = torch.from_numpy(I).cuda()
    gx, gy = image.image_gradient(t)
    bl = image.gaussian3x3(t)
    torch.cuda.synchronize()
    rx, ry = _np_gradient(I)
    assert np.array_equal(gx.cpu().numpy().view(np.uint32), rx.view(np.uint32))
    assert np.array_equal(gy.cpu().numpy().view(np.uint32), ry.view(np.uint32))
    assert np.array_equal(bl.cpu().numpy().view(np.uint32), _np_gaussian(I).view(np.uint32))

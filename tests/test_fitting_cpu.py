"""Host-side pieces of gvr.fitting that need no GPU: the outline distance
field and the outline mask of the silhouette term, the Rodrigues rotation,
and the parameter draws."""
import math

import numpy as np
import torch

from gvr import fitting


def _square(n=12, lo=3, hi=9):
    fg = torch.zeros(1, 1, n, n, dtype=torch.bool)
    fg[0, 0, lo:hi, lo:hi] = True
    return fg


def test_contour_field_is_zero_on_the_outline_and_grows_by_one_per_pixel():
    fg = _square()
    f = fitting.contour_field(fg, 6)[0, 0]
    out = fitting.silhouette_pixels(fg)[0, 0] > 0
    assert torch.all(f[out] == 0)                       # minimum exactly on the outline pixels
    assert torch.all(f[~out] >= 1)
    assert f[5, 5] == 2 and f[4, 4] == 1                  # inside: d - 1 (chessboard)
    assert f[2, 5] == 1 and f[0, 5] == 3                  # outside: d
    # symmetric about the outline: the centred difference across it is zero
    assert f[3, 6 - 1] == 0 and f[2, 5] == f[4, 5]


def test_contour_field_is_capped_at_the_radius():
    fg = _square(n=40, lo=18, hi=22)
    f = fitting.contour_field(fg, 5)[0, 0]
    assert float(f.max()) == 5.0


def test_silhouette_pixels_are_foreground_with_a_background_neighbour():
    fg = _square()
    m = fitting.silhouette_pixels(fg)[0, 0] > 0
    assert int(m.sum()) == 6 * 4 - 4                      # the ring of a 6x6 square
    assert not m[5, 5] and m[3, 3] and not m[2, 2]


def test_rotation_matrix_is_rodrigues_and_smooth_at_zero():
    r = torch.tensor([[0.0, 0.0, 0.0], [0.0, math.pi / 2, 0.0], [0.3, -0.2, 0.5]], dtype=torch.float64)
    R = fitting.rotation_matrix(r)
    assert torch.allclose(R[0], torch.eye(3, dtype=torch.float64))
    assert torch.allclose(R[1] @ torch.tensor([1.0, 0, 0], dtype=torch.float64),
                          torch.tensor([0, 0, -1.0], dtype=torch.float64), atol=1e-12)
    assert torch.allclose(R[2] @ R[2].T, torch.eye(3, dtype=torch.float64), atol=1e-12)
    assert abs(float(torch.det(R[2])) - 1.0) < 1e-12
    x = torch.zeros(1, 3, dtype=torch.float64, requires_grad=True)
    g, = torch.autograd.grad(fitting.rotation_matrix(x)[0, 0, 1], x)
    assert torch.allclose(g, torch.tensor([[0.0, 0.0, -1.0]], dtype=torch.float64))


def test_parameter_draws_follow_the_fitting_distribution():
    p = fitting.sample_params(np.random.default_rng(0), 2000)
    assert p.shape == (2000, fitting.N_PARAMS)
    assert abs(p[:, :160].std() - 1.0) < 0.02
    yaw = np.degrees(p[:, 161])
    assert yaw.min() >= -45 and yaw.max() <= 45
    assert np.all(p[:, [160, 162, 163, 164, 165]] == 0)
    band0 = p[:, [166, 175, 184]]
    assert band0.min() >= 0.5 and band0.max() <= 1.2
    m = fitting.mean_params(3)
    assert np.all(m[:, [166, 175, 184]] == 0.85) and np.count_nonzero(m) == 9

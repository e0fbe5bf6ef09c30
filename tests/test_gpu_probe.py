"""The L2 reduction-rate probe behind the scatter kernels' atomics summary:
every addition lands in the buffer exactly once (its argument checks are
tested without a GPU in test_abi.py)."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("vector4", [0, 1])
def test_probe_adds_each_addition_once(vector4):
    import torch
    from gvr import _lib
    L = _lib.load()
    dev = torch.device("cuda", 0)
    words, rounds, grid = 8 * 1024, 4, 3
    buf = torch.zeros(words, dtype=torch.float32, device=dev)
    st = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    _lib.check(L.gvr_probe_reductions(ctypes.c_void_p(buf.data_ptr()), words, vector4, rounds, grid, st))
    torch.cuda.synchronize()
    additions = grid * 256 * rounds
    # small integers: the FP32 sums are exact whatever the order
    assert float(buf.sum()) == additions * (4 if vector4 else 1)
    # only the first float (or float4) of each 32-byte sector is touched
    per_sector = buf.view(-1, 8)
    assert float(per_sector[:, (4 if vector4 else 1):].abs().sum()) == 0.0

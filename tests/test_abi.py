"""C-ABI checks that need no GPU: libgvr.so builds, loads, exports every
symbol the headers in include/ declare, and rejects bad arguments with a
status code (validation runs on the host before any CUDA call)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "gvr.h")
HEADERS = sorted(glob.glob(os.path.join(REPO, "include", "*.h")))


def _declared():
    src = "\n".join(open(h).read() for h in HEADERS)
    return sorted(set(re.findall(r"^\s*(?:int|void|size_t|long long|const char \*)\s*\*?\s*(gvr_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    from gvr import _lib
    return _lib.load()


def test_header_symbols_exported(lib):
    from gvr import _lib
    names = _declared()
    assert len(names) >= 8
    assert set(names) == set(_lib.EXPORTS)
    for n in names:
        assert hasattr(lib, n), n


def test_abi_version(lib):
    src = open(HEADER).read()
    v = int(re.search(r"#define GVR_ABI_VERSION (\d+)", src).group(1))
    assert lib.gvr_abi_version() == v


def _create(lib, faces, N, C=1, W=8, H=8, albedo=0, shading=0, img_filter=1, tex_filter=1, nmap=0, uvs=None):
    from gvr import _lib
    f = np.ascontiguousarray(faces, np.int32).reshape(-1)
    t = None if uvs is None else np.ascontiguousarray(uvs, np.float32)
    topo = _lib.GvrTopology(f.ctypes.data, None if t is None else t.ctypes.data, f.size // 3, N)
    attrs = _lib.GvrAttrs(C, W, H, albedo, shading, img_filter, tex_filter, nmap)
    h = ctypes.c_void_p()
    rc = lib.gvr_create(ctypes.byref(topo), ctypes.byref(attrs), ctypes.byref(h))
    return rc, h, lib.gvr_last_error().decode()


@pytest.mark.parametrize("kw,msg", [
    (dict(N=0), "number_of_vertices"),
    (dict(C=0), "number_of_cameras"),
    (dict(W=0), "render_resolution_u"),
    (dict(H=0), "render_resolution_v"),
    (dict(albedo=7), "ALBEDO"),
    (dict(shading=3), "SHADING"),
    (dict(img_filter=0), "IMAGE FILTER"),
    (dict(tex_filter=0), "TEXTURE FILTER"),
])
def test_create_rejects_bad_attrs(lib, kw, msg):
    args = dict(faces=[0, 1, 2], N=3)
    args.update(kw)
    rc, h, err = _create(lib, **args)
    assert rc == -1 and not h.value and msg in err


def test_create_rejects_out_of_range_face(lib):
    rc, h, err = _create(lib, [0, 1, 5], 3)
    assert rc == -1 and "outside" in err


def test_calls_reject_null(lib):
    from gvr import _lib
    assert lib.gvr_forward(None, None, None) == -1
    assert lib.gvr_backward(None, None, None) == -1
    assert lib.gvr_forward_workspace_size(None, 1, 1, 1) == 0
    lib.gvr_destroy(None)  # no-op
    assert lib.gvr_debug_rays(None, 1, None, None, None, None) == -1
    assert "bad" in lib.gvr_last_error().decode()


def test_reduction_probe_checks_arguments_before_any_launch(lib):
    # the checks read only the pointer's value: a fake, 32-byte aligned address
    fake = ctypes.c_void_p(1 << 20)
    assert lib.gvr_probe_reductions(None, 64, 0, 1, 1, None) == -1
    assert lib.gvr_probe_reductions(fake, 60, 0, 1, 1, None) == -1           # not whole sectors
    assert lib.gvr_probe_reductions(fake, 0, 0, 1, 1, None) == -1            # empty
    assert lib.gvr_probe_reductions(fake, 64, 0, 0, 1, None) == -1           # no rounds
    assert lib.gvr_probe_reductions(fake, 64, 0, 1, 0, None) == -1           # no blocks
    assert lib.gvr_probe_reductions(ctypes.c_void_p((1 << 20) + 4), 64, 0, 1, 1, None) == -1  # unaligned


def test_error_status_raises(lib):
    from gvr import _lib
    with pytest.raises(_lib.GvrError) as ei:
        _lib.check(lib.gvr_forward(None, None, None))
    assert ei.value.status == -1


def _header_constants():
    """Enumerators and #defines of include/gvr.h as a name -> int map."""
    src = open(os.path.join(REPO, "include", "gvr.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for name, val in re.findall(r"\b(GVR_[A-Z0-9_]+)\s*=\s*(-?\d+)", src):
        out[name] = int(val)
    for m in re.finditer(r"#define\s+(GVR_[A-Z0-9_]+)\s+\(?(\d+)u?(?:\s*<<\s*(\d+))?\)?", src):
        out[m.group(1)] = int(m.group(2)) << int(m.group(3) or 0)
    return out


def test_python_constants_match_the_header():
    from gvr import _lib
    h = _header_constants()
    camel = {"VERTEX_COLOR": "vertexColor", "TEXTURED": "textured", "NORMAL": "normal", "LIGHTING": "lighting",
             "FOREGROUND_MASK": "foregroundMask", "TEXTURED_BILINEAR": "texturedBilinear", "UV": "uv"}
    for suffix, name in camel.items():
        assert _lib.ALBEDO[name] == h["GVR_ALBEDO_" + suffix], name
    for name in ("shaded", "shadeless", "phong"):
        assert _lib.SHADING[name] == h["GVR_SHADING_" + name.upper()], name
    for code, name in _lib.STATUS.items():
        assert h[name] == code, name
    assert _lib.BACKWARD_ALBEDO_POSITION == h["GVR_BACKWARD_ALBEDO_POSITION"]
    assert _lib.PLAN_AUTOTUNE == h["GVR_PLAN_AUTOTUNE"]
    assert _lib.PLAN_PERSISTENT == h["GVR_PLAN_PERSISTENT"] and _lib.PLAN_LANES == h["GVR_PLAN_LANES"]
    assert _lib.NOALLOC_SCRATCH_BYTES == h["GVR_NOALLOC_SCRATCH_BYTES"]

"""Where the reference's own sources and fixture files are read from (test
infrastructure: the recipes that compile the reference's kernels and derive
its fixture scenes, and the tests that read its files in place).

GVR_REFERENCE_ROOT names the reference checkout.  Unset, the recipes look in
the checkout location of the build container; where that does not exist
(the GPU machines), everything that needs the sources is skipped and the
prebuilt files in oracle/_ref are used as they are.
"""
from __future__ import annotations

import os

ENV = "GVR_REFERENCE_ROOT"
_DEFAULT = "/root/reference"


def reference_root() -> str:
    return os.environ.get(ENV) or _DEFAULT


def reference_path(*parts: str) -> str:
    return os.path.join(reference_root(), *parts)


def reference_data(*parts: str) -> str:
    """A file of the reference's python/data fixtures."""
    return reference_path("python", "data", *parts)

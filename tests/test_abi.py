"""librtx.so: builds, loads, exports every entry point of include/rtx.h, and
fails loudly (an error code, no fallback) where no GPU is present."""
import ctypes as C
import os
import re

import numpy as np

import rendertoy_gb300 as rt
from rendertoy_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"^\s*(?:[\w\*]+\s+)+\**(rtx_\w+)\s*\(", txt, re.M))
    return names


def test_library_exports_header():
    path = build.build()
    lib = C.CDLL(path)
    names = declared()
    assert "rtx_render_pt" in names and len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(rt.EXPORTS) == names
    assert lib.rtx_version() == 2


def test_no_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        return  # covered by the GPU tests
    L = rt.lib()
    h = C.c_void_p()
    assert L.rtx_create(C.byref(h), 0) == 2  # RTX_ERR_CUDA, no CPU fallback
    assert not h.value


def test_null_context_is_rejected():
    L = rt.lib()
    assert L.rtx_render_pt(None, None, 4, 4, 1, 5, 0, None) == 1
    assert L.rtx_set_option(None, 1, 0) == 1

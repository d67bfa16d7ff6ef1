"""The C-ABI library loads, exports every entry point include/aperture/ar.h
declares, and its host-only calls work without a GPU."""
import ctypes as C
import re

import numpy as np

from conftest import ROOT
from aperturerendererv3_gb300 import _lib


def header_symbols():
    text = (ROOT / "include" / "aperture" / "ar.h").read_text()
    return sorted(set(re.findall(r"^(?:ar_status|const char\*|int)\s+(ar_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    syms = header_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) <= set(_lib.EXPORTED)


def test_abi_version():
    assert _lib.load().ar_abi_version() == 4


def test_null_and_bad_arguments_return_errors():
    lib = _lib.load()
    assert lib.ar_destroy(None) == _lib.AR_ERR_INVALID
    assert lib.ar_scene_build(None) == _lib.AR_ERR_INVALID
    assert lib.ar_render(None, None, None, 0, None, None) == _lib.AR_ERR_INVALID
    out = np.zeros(4, np.float32)
    assert lib.ar_host_rgb_encode(None, 1, out.ctypes.data) == _lib.AR_ERR_INVALID
    assert lib.ar_last_error(None) == b"null context"


def test_create_reports_missing_device_without_crashing():
    import torch
    if torch.cuda.is_available():
        return
    lib = _lib.load()
    ctx = C.c_void_p()
    assert lib.ar_create(C.byref(ctx), 0) == _lib.AR_ERR_CUDA
    assert not ctx.value

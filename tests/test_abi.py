"""The C-ABI libraries load (no GPU needed) and export every function their headers declare."""
import ctypes
import os
import re

import pytest

from sparspak import _build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(spk_[a-z0-9_]+)\s*\(", text)))


@pytest.mark.parametrize("header,so", [("spk_host.h", "HOST_SO"), ("spk_gpu.h", "GPU_SO")])
def test_exports(header, so):
    _build.build()
    lib = ctypes.CDLL(getattr(_build, so))
    names = declared(header)
    assert len(names) >= 8
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_gpu_lib_reports_no_device_cleanly():
    # Without a GPU, spk_create must fail with a status, not crash (no CPU fallback).
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy as np

    from sparspak import _native as N

    lib = N.gpu()
    one = np.array([1, 2], dtype=np.int64)
    h = ctypes.c_void_p()
    rc = lib.spk_create(1, 1, N.p64(one), N.p64(np.array([1], np.int64)), N.p64(one),
                        N.p64(np.array([1], np.int64)), N.p64(one), N.p64(np.array([1, 1], np.int64)), 1,
                        ctypes.byref(h))
    assert rc == N.SPK_ECUDA
    assert "CUDA" in lib.spk_last_error(None).decode() or "device" in lib.spk_last_error(None).decode()


def _defines(prefix):
    text = open(os.path.join(ROOT, "include", "spk_gpu.h")).read()
    return {m.group(1): int(m.group(2)) for m in re.finditer(rf"#define ({prefix}[A-Z0-9_]+) (-?\d+)", text)}


def test_python_constants_match_the_header():
    # the option codes, status codes and kernel classes the Python mirror
    # passes through the C ABI are the header's
    from sparspak import _native as N

    opts = _defines("SPK_OPT_")
    assert {("SPK_OPT_" + k.upper()): v for k, v in N.OPTIONS.items()} == opts
    status = _defines("SPK_E")
    for name, v in status.items():
        assert getattr(N, name) == v, name
    classes = {k: v for k, v in _defines("SPK_K_").items() if k != "SPK_K_COUNT"}
    assert len(N.KERNEL_CLASSES) == len(classes) == _defines("SPK_K_")["SPK_K_COUNT"]
    for name, v in classes.items():
        assert N.KERNEL_CLASSES[v] == name[len("SPK_K_"):].lower(), name

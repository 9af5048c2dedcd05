"""The allocation-free residual entry point (spk_residual_noalloc).

It exists for callers that cannot allocate device memory when they call
the library (an application that gives all device memory to its own pool,
a fixed memory budget, a loop that cannot afford the device synchronisation
of cudaMalloc/cudaFree): its work space is a file-scope device array instead
of a cudaMalloc.  Checked through the C ABI against spk_residual, on two
calls in a row (the shared array keeps the previous call's contents, so the
second call also checks that it is cleared).  It waits for the stream, so
under a stream capture it must refuse with SPK_ESEQ and leave the capture
valid.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

import sparspak as S
from sparspak import _native as N

pytestmark = pytest.mark.gpu


def test_residual_noalloc_matches_spk_residual():
    torch = pytest.importorskip("torch")
    A = S.gallery.laplacian((12, 12, 12), shift=1e-3)
    n, nrhs = A.shape[0], 3
    s = S.SparseSolver(A, precision="fp32")
    S.findorder_(s, S.nd_grid(12, 12, 12, leaf=16))
    S.symbolicfactor_(s)
    S.inmatrix_(s)
    S.factor_(s)
    eng = s.slvr.engine
    lib = N.gpu()
    b = S.gallery.random_rhs(n, nrhs, seed=4)
    b_d = torch.tensor(np.ascontiguousarray(b.T), device="cuda")   # rows are right-hand sides, ld = n
    x_d = b_d.clone()
    eng.solve(x_d, "fp32")                                         # FP32 solve: residual well above rounding
    ref = eng.residual(b_d, x_d)
    assert 1e-12 < ref < 1e-3
    for _ in range(2):
        rr = ctypes.c_double(-1.0)
        rc = lib.spk_residual_noalloc(eng._h, ctypes.c_void_p(b_d.data_ptr()), ctypes.c_void_p(x_d.data_ptr()), nrhs, n,
                                      ctypes.byref(rr))
        assert rc == N.SPK_OK, lib.spk_last_error(eng._h).decode()
        assert abs(rr.value - ref) <= 1e-12 * ref
    rr = ctypes.c_double(0.0)
    rc = lib.spk_residual_noalloc(eng._h, ctypes.c_void_p(b_d.data_ptr()), ctypes.c_void_p(x_d.data_ptr()), 65, n,
                                  ctypes.byref(rr))
    assert rc == N.SPK_EARG and "64" in lib.spk_last_error(eng._h).decode()


def test_residual_noalloc_refuses_inside_a_capture():
    torch = pytest.importorskip("torch")
    A = S.gallery.laplacian((10, 10, 10), shift=1e-3)
    n = A.shape[0]
    s = S.SparseSolver(A)
    S.findorder_(s)
    S.symbolicfactor_(s)
    S.inmatrix_(s)
    S.factor_(s)
    eng = s.slvr.engine
    lib = N.gpu()
    b_d = torch.ones((1, n), dtype=torch.float64, device="cuda")
    x_d = b_d.clone()
    eng.solve(x_d)
    stream = torch.cuda.Stream()
    eng.set_stream(stream.cuda_stream)
    g = torch.cuda.CUDAGraph()
    rr = ctypes.c_double(-1.0)
    with torch.cuda.graph(g, stream=stream):
        y = x_d * 2.0                      # something for the graph to hold
        rc = lib.spk_residual_noalloc(eng._h, ctypes.c_void_p(b_d.data_ptr()), ctypes.c_void_p(x_d.data_ptr()), 1, n,
                                      ctypes.byref(rr))
    assert rc == N.SPK_ESEQ and "captur" in lib.spk_last_error(eng._h).decode()
    g.replay()                              # the capture stayed valid
    torch.cuda.synchronize()
    assert torch.allclose(y, x_d * 2.0)
    rc = lib.spk_residual_noalloc(eng._h, ctypes.c_void_p(b_d.data_ptr()), ctypes.c_void_p(x_d.data_ptr()), 1, n,
                                  ctypes.byref(rr))
    assert rc == N.SPK_OK and rr.value <= 1e-12

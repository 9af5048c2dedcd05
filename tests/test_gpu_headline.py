"""Parity on the configurations bench.py times, at their full sizes.

* The 64^3 shifted 7-point Laplacian (n = 262,144, nested dissection, four
  right-hand sides U[-1,1], seed 0) - the headline workload.
* The 48^3 convection-diffusion problem (n = 110,592, Peclet 10).

For each: the oracle builds the structure on its own (its restatement of
MMD/ND, the elimination tree, column counts, supernodes and _symbolicfact!)
and it must equal the product's; the oracle factors in FP64 with its dense
calls through BLAS/LAPACK (the reference's Float64 dispatch); the GPU's FP64
factors must have the identical pivot sequence and lnz/unz within 1e-12
(relative, max norm); its solutions within 1e-10 of the oracle's and a
relative residual <= 1e-12.  The FP32 factor + FP64 refinement form must
reach 1e-12, and its forward error against the FP64 oracle solution is
printed and bounded.  The FP32 run must have used the tensor-core kernels.
"""
import numpy as np
import pytest

import oracle
import sparspak as S
from sparspak.sparse_solver import _matrix_arrays

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))


def relres(A, x, b):
    r = b - A @ x
    return float(np.max(np.linalg.norm(r, axis=0) / np.linalg.norm(b, axis=0)))


def _parity(A, grid, nrhs, label):
    n = A.shape[0]
    cp, rv, nz = _matrix_arrays(A)
    b = S.gallery.random_rhs(n, nrhs, seed=0).reshape(n, nrhs)

    # structure: the oracle's own, equal to the product's
    st = oracle.structure_csc(cp, rv, n, "nd", grid)
    s = S.SparseSolver(A)
    S.findorder_(s, S.nd_grid(*grid))
    S.symbolicfactor_(s)
    sl = s.slvr
    assert np.array_equal(st.order.rperm, sl.order.rperm)
    for k in ("xsuper", "snode", "xlindx", "lindx", "xlnz", "xunz"):
        assert np.array_equal(getattr(st, k), np.asarray(getattr(sl, k))), k

    # FP64 on the GPU against the oracle
    oracle.use_blas(True)
    try:
        o = oracle.OracleLU(st)
        o.inmatrix_csc(cp, rv, nz)
        assert o.factor() == 0
        xo = o.solve(b)
    finally:
        oracle.use_blas(False)
    S.inmatrix_(s)
    S.factor_(s)
    assert np.array_equal(sl.ipiv, o.ipiv), "pivot sequence differs"
    el = rel(sl.lnz, o.lnz)
    eu = rel(sl.unz, o.unz[: sl.unz.size])
    assert el <= 1e-12 and eu <= 1e-12, (el, eu)
    del o
    x64 = np.array(b, order="F")
    S.triangularsolve_(s, x64)
    assert rel(x64, xo) < 1e-10
    assert relres(A, x64, b) <= 1e-12

    # FP32 factor + FP64 refinement: residual 1e-12, forward error vs the FP64 oracle
    s32 = S.SparseSolver(A, precision="fp32")
    S.findorder_(s32, S.nd_grid(*grid))
    S.symbolicfactor_(s32)
    S.inmatrix_(s32)
    eng = s32.slvr.engine
    eng.profile_reset()
    S.factor_(s32)
    prof = eng.profile_read()
    assert prof["tc_schur"]["launches"] > 0, "tensor-core Schur updates did not run"
    x32, it, rr = S.refine_(s32, b, precision="fp32", tol=1e-12)
    assert rr <= 1e-12 and it <= 6
    assert relres(A, x32, b) <= 1e-12
    fwd = rel(x32, xo)
    print(f"{label}: FP64 factors vs oracle lnz {el:.1e} unz {eu:.1e}; FP32+IR {it} corrections, "
          f"rel. residual {rr:.1e}, forward error vs FP64 oracle {fwd:.1e}")
    assert fwd < 1e-10
    return prof


def test_headline_laplace3d_64_vs_oracle():
    A = S.gallery.laplacian((64, 64, 64), shift=1e-3)
    prof = _parity(A, (64, 64, 64), 4, "laplace3d 64^3")
    assert prof["tc_trail"]["launches"] > 0


def test_config3_convection_diffusion_48_vs_oracle():
    A = S.gallery.convection_diffusion(k=48)
    _parity(A, (48, 48, 48), 1, "convection-diffusion 48^3")

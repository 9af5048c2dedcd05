"""The BF16 form (SPK_BF16S) and GMRES-IR, through the C ABI.

The large rank updates (Schur complements and trailing updates of the fronts
with a packed panel) take BF16 operands, each block's L panel scaled by 2^e
and its U panel by 2^-e, with FP32 accumulation on the tensor cores; the
rest of the factorisation and the solves are FP32.  FP64 refinement must
still reach 1e-12: plain refinement while it converges fast enough, then
GMRES-IR preconditioned by the BF16 factor.  Checked against the oracle's
FP64 factors (pivots identical on these M-matrices; entries to BF16 accuracy)
and its FP64 solution (forward error stated and bounded).
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
    return float(np.max(np.linalg.norm(np.atleast_2d(r.T), axis=1) / np.linalg.norm(np.atleast_2d(b.T), axis=1)))


def _oracle(A, grid):
    n = A.shape[0]
    cp, rv, nz = _matrix_arrays(A)
    st = oracle.structure_csc(cp, rv, n, "nd", grid)
    oracle.use_blas(True)
    try:
        o = oracle.OracleLU(st)
        o.inmatrix_csc(cp, rv, nz)
        assert o.factor() == 0
    finally:
        oracle.use_blas(False)
    return o


@pytest.mark.parametrize("kind", ["laplace24", "convdiff20"])
def test_bf16s_factor_and_refine(kind):
    if kind == "laplace24":
        A, g = S.gallery.laplacian((24, 24, 24), shift=1e-3), (24, 24, 24)
    else:
        A, g = S.gallery.convection_diffusion(k=20), (20, 20, 20)
    n = A.shape[0]
    o = _oracle(A, g)
    s = S.SparseSolver(A, precision="bf16s")
    S.findorder_(s, S.nd_grid(*g))
    S.symbolicfactor_(s)
    S.inmatrix_(s)
    eng = s.slvr.engine
    eng.profile_reset()
    S.factor_(s)
    prof = eng.profile_read()
    assert prof["tc_schur"]["launches"] > 0, "the BF16 tensor-core updates did not run"
    assert np.array_equal(s.slvr.ipiv, o.ipiv)
    el = rel(s.slvr.lnz, o.lnz)
    assert 1e-7 < el < 5e-2, el            # BF16 operands: far from FP32, close to the FP64 factor
    b = S.gallery.random_rhs(n, 3, seed=5)
    xo = o.solve(b)
    x, it, rr, used = S.refine_(s, b, precision="bf16s", tol=1e-12, max_iter=100, solver="auto")
    assert rr <= 1e-12, (rr, it, used)
    assert relres(A, x, b) <= 1e-12
    fwd = rel(x, xo)
    print(f"{kind}: BF16S factor vs FP64 oracle {el:.1e}; {used} to {rr:.1e} in {it} solves; "
          f"forward error vs oracle {fwd:.1e}")
    assert fwd < 1e-9


def test_gmres_ir_with_fp32_and_bf16s_factors():
    # GMRES-IR chosen explicitly: with the FP32 factor it needs very few
    # iterations; with the BF16 factor more, but both reach 1e-12
    A = S.gallery.laplacian((20, 20, 20), shift=1e-3)
    n = A.shape[0]
    b = S.gallery.random_rhs(n, 2, seed=9)
    out = {}
    for prec in ("fp32", "bf16s"):
        s = S.SparseSolver(A, precision=prec)
        S.findorder_(s, S.nd_grid(20, 20, 20))
        x, it, rr, used = S.refine_(s, b, precision=prec, tol=1e-12, max_iter=200, solver="gmres")
        assert used == "gmres" and rr <= 1e-12, (prec, rr, it)
        assert relres(A, x, b) <= 1e-12
        out[prec] = it
    assert out["fp32"] <= out["bf16s"]
    # plain refinement with the FP32 factor never needs GMRES
    s = S.SparseSolver(A, precision="fp32")
    S.findorder_(s, S.nd_grid(20, 20, 20))
    x, it, rr, used = S.refine_(s, b, precision="fp32", tol=1e-12, solver="auto")
    assert used == "ir" and rr <= 1e-12 and it <= 4


def test_bf16s_headline_64():
    # the headline workload in the BF16 form, to 1e-12
    A = S.gallery.laplacian((64, 64, 64), shift=1e-3)
    n = A.shape[0]
    b = S.gallery.random_rhs(n, 4, seed=0).reshape(n, 4)
    s = S.SparseSolver(A, precision="bf16s")
    S.findorder_(s, S.nd_grid(64, 64, 64))
    x, it, rr, used = S.refine_(s, b, precision="bf16s", tol=1e-12, max_iter=200, solver="auto")
    assert rr <= 1e-12, (rr, it, used)
    assert relres(A, x, b) <= 1e-12
    s64 = S.SparseSolver(A)
    S.findorder_(s64, S.nd_grid(64, 64, 64))
    S.symbolicfactor_(s64)
    S.inmatrix_(s64)
    S.factor_(s64)
    x64 = np.array(b, order="F")
    S.triangularsolve_(s64, x64)
    fwd = rel(x, x64)
    print(f"laplace3d 64^3 BF16S: {used} to {rr:.1e} in {it} solves; forward error vs FP64 {fwd:.1e}")
    assert fwd < 1e-9

"""The symmetric (SPD, Cholesky) form, SPK_SPD, through the C ABI.

For symmetric positive definite A the engine factors without interchanges,
forms only the lower part of every rank update (half the update flops) and
writes the U side, U = D L^T, from the L panels.  Its factor reads back as
the Cholesky factor C (A = C C^T).  Checked against the oracle's own
supernodal Cholesky (oracle_cholfactor) and against the oracle LU on the
same matrix (C = L D^1/2 with U = D L^T and identity pivots), since the
reference's SPD solver is not usable as an oracle (its _pchole! scales in
the wrong place).  FP64 factors within 1e-12, solutions within 1e-10 of the
oracle's, relative residual <= 1e-12; FP32 and BF16 forms refined to 1e-12.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
import sparspak as S
from cases import sprand_spd_like
from sparspak.sparse_solver import _matrix_arrays

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))


def relres(A, x, b):
    r = b - A @ x
    return float(np.max(np.linalg.norm(np.atleast_2d(r.T), axis=1) / np.linalg.norm(np.atleast_2d(b.T), axis=1)))


def _case(name):
    if name == "grid2d_100_mmd":           # config 1, the reference's default ordering
        return S.gallery.laplacian((100, 100)), None
    if name == "grid2d_100_nd":
        return S.gallery.laplacian((100, 100)), S.nd_grid(100, 100)
    if name == "laplace3d_24_nd":
        return S.gallery.laplacian((24, 24, 24), shift=1e-3), S.nd_grid(24, 24, 24)
    if name == "sprand_spd_1357":
        return sprand_spd_like(1357, 1357), None
    if name == "batched_diffusion":
        A, sizes = S.gallery.batched_diffusion(12, 8, 24, seed=3)
        return A, S.nd_grid_batched(sizes, leaf=16)
    raise ValueError(name)


@pytest.mark.parametrize("name", ["grid2d_100_mmd", "grid2d_100_nd", "laplace3d_24_nd", "sprand_spd_1357",
                                  "batched_diffusion"])
def test_spd_fp64_vs_oracle_cholesky(name):
    A, of = _case(name)
    n = A.shape[0]
    s = S.SparseSolver(A, spd=True)
    S.findorder_(s, of)
    S.symbolicfactor_(s)
    cp, rv, nz = _matrix_arrays(A)
    o = oracle.OracleLU(s.slvr)
    o.inmatrix_csc(cp, rv, nz)
    assert o.cholfactor() == 0
    lu = oracle.OracleLU(s.slvr)
    lu.inmatrix_csc(cp, rv, nz)
    assert lu.factor() == 0
    S.inmatrix_(s)
    eng = s.slvr.engine
    eng.profile_reset()
    S.factor_(s)
    spd_flops = sum(v["flops"] for k, v in eng.profile_read().items() if k in ("getrf", "panel", "trail", "schur",
                                                                              "tc_trail", "tc_schur"))
    mask = o.lower_mask()
    C = s.slvr.lnz
    assert rel(C[mask], o.lnz[mask]) <= 1e-12
    # the oracle LU on the same matrix: identity pivots, C = L D^1/2
    ident = np.concatenate([np.arange(1, s.slvr.xsuper[j + 1] - s.slvr.xsuper[j] + 1) for j in range(s.slvr.nsuper)])
    assert np.array_equal(lu.ipiv, ident) and np.array_equal(s.slvr.ipiv, ident)
    b = S.gallery.random_rhs(n, 2, seed=1)
    x = np.array(b, order="F")
    S.triangularsolve_(s, x)
    assert rel(x, lu.solve(b)) < 1e-10
    assert relres(A, x, b) <= 1e-12
    # half the update work of the LU form
    s_lu = S.SparseSolver(A)
    S.findorder_(s_lu, of)
    S.symbolicfactor_(s_lu)
    S.inmatrix_(s_lu)
    e2 = s_lu.slvr.engine
    e2.profile_reset()
    S.factor_(s_lu)
    lu_flops = sum(v["flops"] for k, v in e2.profile_read().items() if k in ("getrf", "panel", "trail", "schur",
                                                                            "tc_trail", "tc_schur"))
    print(f"{name}: SPD factor vs oracle Cholesky {rel(C[mask], o.lnz[mask]):.1e}; flops SPD/LU "
          f"{spd_flops / lu_flops:.3f}")
    assert spd_flops < 0.75 * lu_flops


@pytest.mark.parametrize("prec", ["fp32", "bf16s"])
def test_spd_mixed_refine(prec):
    A = S.gallery.laplacian((24, 24, 24), shift=1e-3)
    n = A.shape[0]
    b = S.gallery.random_rhs(n, 3, seed=2)
    s = S.SparseSolver(A, precision=prec, spd=True)
    S.findorder_(s, S.nd_grid(24, 24, 24))
    S.symbolicfactor_(s)
    S.inmatrix_(s)
    eng = s.slvr.engine
    eng.profile_reset()
    S.factor_(s)
    assert eng.profile_read()["tc_schur"]["launches"] > 0
    x, it, rr, used = S.refine_(s, b, precision=prec, tol=1e-12, max_iter=100, solver="auto")
    assert rr <= 1e-12 and relres(A, x, b) <= 1e-12, (rr, it, used)
    print(f"SPD {prec}: {used} to {rr:.1e} in {it} solves")


def test_spd_rejects_indefinite():
    # symmetric but indefinite: the factor exists without pivoting, but has a negative pivot
    A = sp.csc_matrix(S.gallery.laplacian((6, 6)) - 3.3 * sp.identity(36))
    s = S.SparseSolver(A, spd=True)
    S.findorder_(s)
    S.symbolicfactor_(s)
    S.inmatrix_(s)
    S.factor_(s)
    with pytest.raises(S.ErrorException, match="not positive definite"):
        s.slvr.lnz

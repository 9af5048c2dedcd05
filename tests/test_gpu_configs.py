"""The measured configurations other than the 64^3 headline, at their full sizes.

1. 2-D 5-point Dirichlet Laplacian 100 x 100: MMD (the reference's default)
   factors and solution against the oracle; nested dissection to 1e-12.
3. Convection-diffusion 48^3 (first-order upwind, Peclet 10): an M-matrix,
   so every in-block pivot is the diagonal; FP64 to 1e-12 and FP32 + FP64
   refinement to 1e-12, the two solutions agreeing.
4. 512 independent SPD systems (9-point weighted graph Laplacians of s x s
   grids, s ~ U{20..120}, lognormal conductivities) factored together as
   one block-diagonal system (FP32 factor, FP64 refinement): every system's
   relative residual <= 1e-12; a reduced batch against the oracle in FP64.

Accuracy is also reported as the normwise backward error
||r||_inf / (||A||_inf ||x||_inf + ||b||_inf).
"""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
import sparspak as S

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def relres(A, x, b):
    r = b - A @ x
    r, b = np.atleast_2d(r.T), np.atleast_2d(b.T)
    return float(np.max(np.linalg.norm(r, axis=1) / np.linalg.norm(b, axis=1)))


def backward_error(A, x, b):
    r = b - A @ x
    anorm = float(abs(A).sum(axis=1).max())
    return float(np.max(np.abs(r)) / (anorm * np.max(np.abs(x)) + np.max(np.abs(b))))


def test_config1_grid2d_100_mmd_parity_and_nd():
    A = S.gallery.laplacian((100, 100))
    b = S.gallery.random_rhs(A.shape[0], 1, seed=0)
    s = S.SparseSolver(A)
    S.findorder_(s)                          # MMD
    S.symbolicfactor_(s)
    o = oracle.OracleLU(s.slvr)
    o.inmatrix_csc(*S.sparse_solver._matrix_arrays(A))
    o.factor()
    S.inmatrix_(s)
    S.factor_(s)
    assert np.array_equal(s.slvr.ipiv, o.ipiv)
    assert rel(s.slvr.lnz, o.lnz) <= 1e-12
    assert rel(s.slvr.unz, o.unz[: s.slvr.unz.size]) <= 1e-12
    x = b.copy()
    S.triangularsolve_(s, x)
    assert rel(x, o.solve(b)) < 1e-10
    assert relres(A, x, b) <= 1e-12 and backward_error(A, x, b) < 1e-15
    # project nested dissection: same solution
    lu = S.sparspaklu(A, orderfunction=S.nd_grid(100, 100))
    y = S.ldiv(lu, b)
    assert relres(A, y, b) <= 1e-12 and rel(y, x) < 1e-10


def test_config3_convection_diffusion_48():
    k = 48
    A = S.gallery.convection_diffusion(k=k)
    n = A.shape[0]
    b = S.gallery.random_rhs(n, 1, seed=0)
    s = S.SparseSolver(A)
    S.findorder_(s, S.nd_grid(k, k, k))
    S.symbolicfactor_(s)
    S.inmatrix_(s)
    S.factor_(s)
    sl = s.slvr
    ident = np.concatenate([np.arange(1, sl.xsuper[j + 1] - sl.xsuper[j] + 1) for j in range(sl.nsuper)])
    assert np.array_equal(sl.ipiv, ident)        # M-matrix: diagonal pivots throughout
    x64 = b.copy()
    S.triangularsolve_(s, x64)
    assert relres(A, x64, b) <= 1e-12 and backward_error(A, x64, b) < 1e-15
    s32 = S.SparseSolver(A, precision="fp32")
    S.findorder_(s32, S.nd_grid(k, k, k))
    x32, it, rr = S.refine_(s32, b, precision="fp32", tol=1e-12)
    assert rr <= 1e-12 and it <= 6
    assert relres(A, x32, b) <= 1e-12
    assert rel(x32, x64) < 1e-10


def test_config4_batched_reduced_vs_oracle():
    A, sizes = S.gallery.batched_diffusion(16, 8, 20, seed=1)
    s = S.SparseSolver(A)
    S.findorder_(s, S.nd_grid_batched(sizes, leaf=16))
    S.symbolicfactor_(s)
    o = oracle.OracleLU(s.slvr)
    o.inmatrix_csc(*S.sparse_solver._matrix_arrays(A))
    o.factor()
    S.inmatrix_(s)
    S.factor_(s)
    assert np.array_equal(s.slvr.ipiv, o.ipiv)
    assert rel(s.slvr.lnz, o.lnz) <= 1e-12
    b = S.gallery.random_rhs(A.shape[0], 2, seed=2)
    x = b.copy(order="F")
    S.triangularsolve_(s, x)
    assert rel(x, o.solve(b)) < 1e-10


def test_config4_batched_512_systems():
    A, sizes = S.gallery.batched_diffusion(512, 20, 120, seed=0)
    n = A.shape[0]
    b = S.gallery.random_rhs(n, 1, seed=3)
    s = S.SparseSolver(A, precision="fp32")
    S.findorder_(s, S.nd_grid_batched(sizes))
    x, it, rr = S.refine_(s, b, precision="fp32", tol=1e-12)
    assert rr <= 1e-12 and it <= 6
    r = b - A @ x
    off = 0
    worst = 0.0
    for sz in sizes:       # every system on its own
        sl = slice(off, off + sz * sz)
        worst = max(worst, np.linalg.norm(r[sl]) / np.linalg.norm(b[sl]))
        off += sz * sz
    assert worst <= 1e-11
    assert backward_error(A, x, b) < 1e-15

"""Transposed solves (A^T x = b) and the adjoint gradient dloss/dA, through the C ABI.

The reference has no kernel to compare with: its `transposetriangularsolve`
is commented out (src/SparseSpdMethod/SpkSparseSpdSolver.jl:384) and its
derivative path is forward-mode Dual numbers through generic code
(test/test_generic.jl:58-98).  Transposed solutions are checked against
scipy's sparse LU of A^T and by their FP64 residual; gradients against the
dense formula -lambda x^T and against central finite differences of the loss.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import sparspak as S
from cases import sprand_unsym

pytestmark = pytest.mark.gpu


def factored(A, order=None, precision="fp64"):
    s = S.SparseSolver(A, precision=precision)
    S.findorder_(s, order)
    S.symbolicfactor_(s)
    S.inmatrix_(s)
    S.factor_(s)
    return s


def relres_t(A, x, b):
    r = b - A.T @ x
    return float(np.max(np.linalg.norm(np.atleast_2d(r.T), axis=1) / np.linalg.norm(np.atleast_2d(b.T), axis=1)))


def unsym_with_pivoting(n, seed):
    # sprand + small diagonal: the in-block pivoting picks off-diagonal rows
    rng = np.random.default_rng(seed)
    a = sp.random(n, n, density=6.0 / n, random_state=rng, format="csc")
    return sp.csc_matrix(a + a.T.multiply(rng.uniform(0.5, 1.5)) + 0.05 * sp.identity(n))


@pytest.mark.parametrize("kind", ["pivoting", "sprand", "convdiff", "wide"])
def test_transpose_solve_vs_scipy(kind):
    if kind == "pivoting":
        A, order = unsym_with_pivoting(400, 3), None
    elif kind == "sprand":
        A, order = sprand_unsym(500, 0.01, 7), None
    elif kind == "convdiff":
        A, order = S.gallery.convection_diffusion(k=12), S.nd_grid(12, 12, 12, leaf=16)
    else:   # dense blocks: pieces of 31 and more columns, several blocks per front
        rng = np.random.default_rng(5)
        n = 300
        A, order = sp.csc_matrix(rng.standard_normal((n, n)) + 0.5 * np.sqrt(n) * np.eye(n)), None
    s = factored(A, order)
    if kind == "pivoting":
        b_ = s.slvr
        ident = np.concatenate([np.arange(1, b_.xsuper[k + 1] - b_.xsuper[k] + 1) for k in range(b_.nsuper)])
        assert not np.array_equal(b_.ipiv, ident), "the case should exercise in-block interchanges"
    b = S.gallery.random_rhs(A.shape[0], 3, seed=11)
    x = b.copy(order="F")
    S.transposetriangularsolve_(s, x)
    xr = spla.splu(sp.csc_matrix(A.T)).solve(b)
    assert np.max(np.abs(x - xr)) / np.max(np.abs(xr)) < 1e-9
    # the plain solve with the same factor: same accuracy in both directions
    # (the 'pivoting' matrix is ill-conditioned on purpose; in-piece pivoting
    # allows some growth there)
    y = b.copy(order="F")
    S.triangularsolve_(s, y)
    assert np.max(np.abs(y - spla.splu(sp.csc_matrix(A)).solve(b))) / np.max(np.abs(y)) < 1e-9
    rr = b - A @ y
    plain = float(np.max(np.linalg.norm(rr, axis=0) / np.linalg.norm(b, axis=0)))
    assert relres_t(A, x, b) < max(1e-12, 50.0 * plain)


def test_transpose_refine_fp32_tensor_core_factor():
    # 20^3 convection-diffusion (unsymmetric values): FP32 factor with the
    # tensor-core updates, FP64 refinement of A^T x = b to 1e-12
    A = S.gallery.convection_diffusion(k=20)
    s = S.SparseSolver(A, precision="fp32")
    S.findorder_(s, S.nd_grid(20, 20, 20))
    b = S.gallery.random_rhs(A.shape[0], 2, seed=12)
    x, it, rr = S.refine_(s, b, precision="fp32", tol=1e-12, transpose=True)
    assert rr <= 1e-12 and it <= 6
    assert relres_t(A, x, b) <= 1e-12


def test_gradient_pattern_matches_dense_formula():
    A = sprand_unsym(120, 0.05, 9)
    s = factored(A)
    b = S.gallery.random_rhs(120, 2, seed=3)
    xt = S.gallery.random_rhs(120, 2, seed=4)
    x = b.copy(order="F")
    S.triangularsolve_(s, x)
    lam = np.asfortranarray(x - xt)
    S.transposetriangularsolve_(s, lam)
    G = S.gradient_(s, lam, x)
    Ad = A.toarray()
    Gd = -(np.linalg.solve(Ad.T, x - xt) @ x.T)          # dloss/dA for loss = 1/2 ||x - xt||^2 summed over rhs
    Ac = sp.csc_matrix(A)
    rows = Ac.indices
    cols = np.repeat(np.arange(120), np.diff(Ac.indptr))
    assert np.max(np.abs(G - Gd[rows, cols])) / np.max(np.abs(Gd)) < 1e-10


def diffusion_problem(s, seed, sigma=0.5):
    rng = np.random.Generator(np.random.PCG64(seed))
    th = np.exp(rng.normal(0.0, sigma, size=(s, s + 1)))
    tv = np.exp(rng.normal(0.0, sigma, size=(s + 1, s)))
    return th, tv


def test_adjoint_gradient_anisotropic_diffusion_256():
    # 256 x 256 5-point anisotropic diffusion, theta_e = exp(g), g ~ N(0, 0.5):
    # dloss/dtheta for loss = 1/2 ||x(theta) - x_t||^2 on 64 random interior
    # edges against central finite differences.  Step 1e-3 theta_e: the loss
    # is ~6e6 while one edge moves it by ~1e-3 x its gradient, so smaller steps
    # drown in the change of the loss caused by the FP64 solves' own forward
    # error (~1e-10 relative at this conditioning); the truncation error of
    # the 1e-3 step is about 1e-6 relative.
    n1 = 256
    th, tv = diffusion_problem(n1, 0)
    A = S.gallery.diffusion_2d(n1, th, tv)
    n = A.shape[0]
    rng = np.random.Generator(np.random.PCG64(1))
    xt = rng.uniform(-1.0, 1.0, n)
    b = rng.uniform(-1.0, 1.0, n)
    order = S.nd_grid(n1, n1, 1)
    lu = S.sparspaklu(A, orderfunction=order)

    def solve(lu_, rhs):
        x_ = np.array(rhs, dtype=np.float64)
        S.ldiv_(lu_, x_)
        return x_

    x = solve(lu, b)
    lam = np.asfortranarray(x - xt)
    S.transposetriangularsolve_(lu, lam)
    G = S.gradient_(lu, lam, x)
    Ac = sp.csc_matrix(A)

    def entry(i, j):   # position of A[i, j] in CSC order
        lo, hi = Ac.indptr[j], Ac.indptr[j + 1]
        return lo + int(np.searchsorted(Ac.indices[lo:hi], i))

    ids = np.arange(n).reshape(n1, n1)
    picks = rng.choice(2 * n1 * (n1 - 1), size=64, replace=False)
    for e in picks:
        horizontal = e < n1 * (n1 - 1)
        if horizontal:
            i, j = divmod(int(e), n1 - 1)
            a, c, key = ids[i, j], ids[i, j + 1], ("h", i, j + 1)
        else:
            i, j = divmod(int(e) - n1 * (n1 - 1), n1)
            a, c, key = ids[i, j], ids[i + 1, j], ("v", i + 1, j)
        analytic = G[entry(a, a)] + G[entry(c, c)] - G[entry(a, c)] - G[entry(c, a)]
        t = (th if key[0] == "h" else tv)[key[1], key[2]]
        h = 1e-3 * t
        losses = []
        for sgn in (1.0, -1.0):
            th2, tv2 = th.copy(), tv.copy()
            (th2 if key[0] == "h" else tv2)[key[1], key[2]] = t + sgn * h
            S.sparspaklu_(lu, S.gallery.diffusion_2d(n1, th2, tv2))
            xp = solve(lu, b)
            losses.append(0.5 * np.sum((xp - xt) ** 2))
        fd = (losses[0] - losses[1]) / (2 * h)
        assert abs(fd - analytic) <= 1e-4 * max(abs(analytic), 1e-8 * np.sum((x - xt) ** 2)), (e, fd, analytic)


def test_adjoint_gradient_vs_dual_oracle():
    # Config 5 on a reduced grid (48 x 48 anisotropic diffusion, theta_e =
    # exp(g), g ~ N(0, 0.5)): dloss/dtheta for loss = 1/2 ||x - x_t||^2 on 32
    # random interior edges from the GPU adjoint (transposed solve reusing the
    # factors + the pattern-restricted gradient kernel) against forward-mode
    # derivatives through the reference's LU path on Dual numbers (the
    # reference's derivative check, test/test_generic.jl:58-98), 16 edges per
    # Dual pass.
    import oracle
    from sparspak.sparse_solver import _matrix_arrays

    n1 = 48
    th, tv = diffusion_problem(n1, 2)
    A = sp.csc_matrix(S.gallery.diffusion_2d(n1, th, tv))
    n = A.shape[0]
    rng = np.random.Generator(np.random.PCG64(5))
    xt = rng.uniform(-1.0, 1.0, n)
    b = rng.uniform(-1.0, 1.0, n)
    lu = S.sparspaklu(A, orderfunction=S.nd_grid(n1, n1, 1))
    x = np.array(b)
    S.ldiv_(lu, x)
    lam = np.asfortranarray(x - xt)
    S.transposetriangularsolve_(lu, lam)
    G = S.gradient_(lu, lam, x)

    def entry(i, j):
        lo, hi = A.indptr[j], A.indptr[j + 1]
        return lo + int(np.searchsorted(A.indices[lo:hi], i))

    ids = np.arange(n).reshape(n1, n1)
    picks = rng.choice(2 * n1 * (n1 - 1), size=32, replace=False)
    edges = []
    for e in picks:
        if e < n1 * (n1 - 1):
            i, j = divmod(int(e), n1 - 1)
            edges.append((ids[i, j], ids[i, j + 1]))
        else:
            i, j = divmod(int(e) - n1 * (n1 - 1), n1)
            edges.append((ids[i, j], ids[i + 1, j]))
    cp, rv, nz = _matrix_arrays(A)
    for g0 in range(0, len(edges), 16):
        group = edges[g0: g0 + 16]
        dnz = np.zeros((A.nnz, len(group)))
        for k, (a, c) in enumerate(group):   # dA/dtheta_e = (e_a - e_c)(e_a - e_c)^T
            dnz[entry(a, a), k] += 1.0
            dnz[entry(c, c), k] += 1.0
            dnz[entry(a, c), k] -= 1.0
            dnz[entry(c, a), k] -= 1.0
        xd, dx = oracle.dual_solve(lu.slvr, cp, rv, nz, dnz, b)
        assert np.max(np.abs(xd - x)) / np.max(np.abs(x)) < 1e-10
        dual = (xd - xt) @ dx
        for k, (a, c) in enumerate(group):
            adj = G[entry(a, a)] + G[entry(c, c)] - G[entry(a, c)] - G[entry(c, a)]
            assert abs(adj - dual[k]) <= 1e-9 * max(abs(dual[k]), 1e-12 * np.sum((x - xt) ** 2)), (a, c, adj, dual[k])

"""The oracle (C restatement of the reference's numeric phase) pinned against
the reference's golden vectors and its end-to-end test tolerances (no GPU)."""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
import sparspak as S
from cases import m31_problem, problem_from_csc, sprand_spd_like, sprand_unsym, tridiag_problem
from sparspak.problem import csc_arrays


def oracle_for(p, orderfunction=None):
    s = S.SparseSolver(p)
    S.findorder_(s, orderfunction)
    S.symbolicfactor_(s)
    o = oracle.OracleLU(s.slvr)
    o.inmatrix_csc(*csc_arrays(p))
    return s, o


def test_inmatrix_golden(golden):
    # msprs005, test/test_sparse_method.jl:172-175 (exact)
    _, o = oracle_for(tridiag_problem(11))
    assert o.lnz.tolist() == golden["tridiag11_inmatrix_lnz"]
    assert o.unz.tolist() == golden["tridiag11_inmatrix_unz"]


def test_factor_golden(golden):
    # msprs006, test/test_sparse_method.jl:219-227 (the reference checks rtol 1e-6)
    _, o = oracle_for(tridiag_problem(11))
    assert o.factor() == 0
    ref_l, ref_u = np.array(golden["tridiag11_factor_lnz"]), np.array(golden["tridiag11_factor_unz"])
    assert np.max(np.abs(o.lnz - ref_l) / np.abs(ref_l)) < 1e-15
    assert np.array_equal(o.unz, ref_u)


def test_forward_solve_golden(golden):
    # the permuted rhs before/after _lulsolve! quoted in test/test_sparse_method.jl:318-321
    p = tridiag_problem(11)
    s, o = oracle_for(p)
    o.factor()
    before = p.rhs[s.slvr.order.rperm - 1]
    assert before.tolist() == golden["tridiag11_fwd_before"]
    after = o.lulsolve(before)
    assert np.max(np.abs(after - golden["tridiag11_fwd_after"])) < 1e-13


def _solve_check(p, tol):
    s, o = oracle_for(p)
    o.factor()
    x = o.solve(p.rhs[: p.nrows])
    A = S.outsparse(p).toarray()
    xr = np.linalg.solve(A, p.rhs[: p.nrows])
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < tol


@pytest.mark.parametrize("n", [11, 1101, 11000])
def test_tridiag_solve(n):
    # msprs007-009
    p = tridiag_problem(n)
    s, o = oracle_for(p)
    o.factor()
    x = o.solve(p.rhs)
    A = sp.csc_matrix(S.outsparse(p))
    r = p.rhs - A @ x
    assert np.linalg.norm(r) / np.linalg.norm(p.rhs) < 1e-14


def test_m31(golden):
    # msprs010
    _solve_check(m31_problem(golden), 1e-12)


@pytest.mark.parametrize("n,seed", [(301, 1), (357, 2), (1357, 3)])
def test_sprand_spd_like(n, seed):
    # msprs012, 015, 016
    m = sprand_spd_like(n, seed)
    _solve_check(problem_from_csc(m, np.arange(1, n + 1, dtype=np.float64)), 1e-12)


def test_grid_problem():
    # msprs017-018: makegridproblem(5, 3) with infullrhs! and makerhs!
    p = S.makegridproblem(5, 3)
    S.infullrhs_(p, np.arange(1, 16, dtype=np.float64))
    _solve_check(p, 1e-12)
    p = S.makegridproblem(5, 3)
    S.makerhs_(p, None)
    _solve_check(p, 1e-12)


def test_small_literal_cases(golden):
    # test/test_structunsymm.jl:25-57, test/test_small.jl:35-149
    for vals in golden["small4x4"]:
        A = np.array(vals).reshape(4, 4)
        p = problem_from_csc(sp.csc_matrix(A))
        S.inbi_(p, 1, 1.0)
        _solve_check(p, 1e-12)


def test_random_unsymmetric_pivoting():
    # test/test_structunsymm.jl:60-90: 1000 x sprand(4,4,0.3)+I, abs error < 1e-9
    rng = np.random.default_rng(0)
    pivoted = 0
    for t in range(1000):
        A = sprand_unsym(4, 0.3, t)
        b = rng.random(4)
        s, o = oracle_for(problem_from_csc(A, b))
        o.factor()
        pivoted += int(np.any(o.ipiv != _identity_local(s.slvr)))
        x = o.solve(b)
        assert np.linalg.norm(x - np.linalg.solve(A.toarray(), b)) < 1e-9
    assert pivoted > 0   # the cases exercise real in-block interchanges


def _identity_local(b):
    ip = np.zeros(b.n, dtype=np.int64)
    for s in range(b.nsuper):
        f, l = b.xsuper[s], b.xsuper[s + 1]
        ip[f - 1:l - 1] = np.arange(1, l - f + 1)
    return ip


def test_singular_block_reported():
    # a zero pivot: reference iflag -1 for the last block; the oracle also records the first
    A = sp.csc_matrix(np.array([[0.0, 1.0], [1.0, 0.0]]))
    p = problem_from_csc(A)
    s = S.SparseSolver(p)
    S.findorderperm_(s, [1, 2])
    S.symbolicfactor_(s)
    o = oracle.OracleLU(s.slvr)
    o.inmatrix_csc(*csc_arrays(p))
    o.factor()
    assert o.first_singular == 0   # the 2x2 block pivots and is regular
    B = sp.csc_matrix(np.array([[1.0, 1.0], [1.0, 1.0]]))
    p = problem_from_csc(B)
    s = S.SparseSolver(p)
    S.findorderperm_(s, [1, 2])
    S.symbolicfactor_(s)
    o = oracle.OracleLU(s.slvr)
    o.inmatrix_csc(*csc_arrays(p))
    assert o.factor() == -1 and o.first_singular == 1


# ---------------------------------------------------------------------------
# The oracle's own structure phase (spk_oracle_struct.c), independent of the
# product's host library: pinned by the reference's golden vectors, then
# compared with the product's permutation, supernodes and subscripts.
# ---------------------------------------------------------------------------

def _tridiag_csc(n):
    m = sp.diags([-np.ones(n - 1), 4 * np.ones(n), -np.ones(n - 1)], [-1, 0, 1], format="csc")
    return m.indptr.astype(np.int64) + 1, m.indices.astype(np.int64) + 1


def test_oracle_structure_golden_tridiag11(golden):
    # msprs003 (MMD perm, test/test_sparse_method.jl:87-90) and msprs004
    # (symbolic arrays, :127-131)
    cp, rv = _tridiag_csc(11)
    xadj, adj = oracle.graph_of(cp, rv, 11)
    perm, invp = oracle.mmd(xadj, adj, 11)
    assert perm.tolist() == golden["tridiag11_rperm"]
    assert invp.tolist() == golden["tridiag11_rinvp"]
    o = oracle.symbolic(xadj, adj, perm, invp)
    assert o.xlnz.tolist() == golden["tridiag11_xlnz"]
    assert o.xunz.tolist() == golden["tridiag11_xunz"]
    assert o.xlindx.tolist() == golden["tridiag11_xlindx"]
    assert o.lindx.tolist() == golden["tridiag11_lindx"]


def test_oracle_graph_fig313(golden):
    # test/test_graph.jl:10-23 (symmetric) and :84-99 (symmetrised)
    for key in ("fig313", "fig313_unsym"):
        I, J = np.array(golden[key + "_I"]), np.array(golden[key + "_J"])
        m = sp.csc_matrix((np.ones(I.size), (I - 1, J - 1)), shape=(6, 6))
        xadj, adj = oracle.graph_of(m.indptr.astype(np.int64) + 1, m.indices.astype(np.int64) + 1, 6)
        assert xadj.tolist() == golden["fig313_xadj"]
        assert adj.tolist() == golden["fig313_adj"]


def _structure_cases():
    rng_cases = [("sprand_spd", 301), ("sprand_spd", 1357), ("sprand_unsym", 400)]
    grid_cases = [((20, 20, 1), "mmd"), ((100, 100, 1), "mmd"), ((100, 100, 1), "nd"), ((9, 10, 11), "mmd"),
                  ((24, 24, 24), "nd"), ((17, 13, 9), "nd"), ((100, 100, 1), "nd_graph"), ((24, 24, 24), "nd_graph"),
                  ((17, 13, 9), "nd_graph")]
    return rng_cases + grid_cases


@pytest.mark.parametrize("case", _structure_cases(), ids=lambda c: str(c))
def test_oracle_structure_equals_product(case):
    if case[0] == "sprand_spd":
        A = sprand_spd_like(case[1], case[1])
        ordering, grid, orderfunction = "mmd", None, None
    elif case[0] == "sprand_unsym":
        A = sprand_unsym(case[1], 0.01, 7)
        ordering, grid, orderfunction = "mmd", None, None
    else:
        grid, ordering = case
        A = S.gallery.laplacian(grid if grid[2] > 1 else grid[:2])
        orderfunction = {"nd": S.nd_grid(*grid), "nd_graph": S.nd_graph(), "mmd": None}[ordering]
    A = sp.csc_matrix(A)
    n = A.shape[0]
    cp, rv = A.indptr.astype(np.int64) + 1, A.indices.astype(np.int64) + 1
    o = oracle.structure_csc(cp, rv, n, ordering, grid)
    s = S.SparseSolver(A)
    S.findorder_(s, orderfunction)
    S.symbolicfactor_(s)
    b = s.slvr
    assert o.order.rperm.tolist() == b.order.rperm.tolist()
    assert o.order.rinvp.tolist() == b.order.rinvp.tolist()
    assert o.nsuper == b.nsuper
    for k in ("xsuper", "snode", "xlindx", "lindx", "xlnz", "xunz"):
        assert np.array_equal(getattr(o, k), np.asarray(getattr(b, k))), k


def test_oracle_blas_mode_matches_generic():
    # the BLAS/LAPACK path (the reference's Float64 dispatch) against the
    # generic loops on a 3-D grid with 30-column pieces: same pivots, factors
    # to rounding, and the sliced factorisation equals the one-call form
    A = S.gallery.laplacian((14, 14, 14), shift=1e-3)
    n = A.shape[0]
    cp, rv, nz = A.indptr.astype(np.int64) + 1, A.indices.astype(np.int64) + 1, A.data
    st = oracle.structure_csc(cp, rv, n, "nd", (14, 14, 14))
    oracle.use_blas(False)
    g = oracle.OracleLU(st)
    g.inmatrix_csc(cp, rv, nz)
    assert g.factor() == 0
    try:
        info = oracle.use_blas(True)
        assert info["threads"] >= 1
        bl = oracle.OracleLU(st)
        bl.inmatrix_csc(cp, rv, nz)
        assert bl.factor() == 0
        sl = oracle.OracleLU(st)
        sl.inmatrix_csc(cp, rv, nz)
        bounds = np.linspace(0, st.nsuper, 6).astype(int)[1:]
        assert list(sl.factor_slices(bounds)) == bounds.tolist()
        assert sl.iflag == 0
        assert np.array_equal(sl.lnz, bl.lnz) and np.array_equal(sl.ipiv, bl.ipiv)
        b = np.random.default_rng(0).uniform(-1, 1, n)
        xb = bl.solve(b)
    finally:
        oracle.use_blas(False)
    assert np.array_equal(g.ipiv, bl.ipiv)
    scale = np.max(np.abs(g.lnz))
    assert np.max(np.abs(g.lnz - bl.lnz)) / scale < 1e-13
    xg = g.solve(b)
    assert np.max(np.abs(xg - xb)) / np.max(np.abs(xg)) < 1e-12


def test_oracle_cholesky_reconstructs_a():
    # the oracle's supernodal Cholesky: C C^T = P A P^T on 2-D and 3-D grids
    # with MMD and nested dissection (pieces of up to 46 columns)
    for shape, ordering in [((10, 10), "mmd"), ((7, 8, 9), "mmd"), ((12, 12, 12), "nd")]:
        A = S.gallery.laplacian(shape, shift=1e-3)
        n = A.shape[0]
        cp, rv, nz = A.indptr.astype(np.int64) + 1, A.indices.astype(np.int64) + 1, A.data
        grid = shape + (1,) * (3 - len(shape))
        st = oracle.structure_csc(cp, rv, n, ordering, grid)
        o = oracle.OracleLU(st)
        o.inmatrix_csc(cp, rv, nz)
        assert o.cholfactor() == 0
        C = np.zeros((n, n))
        for js in range(st.nsuper):
            f, l = int(st.xsuper[js]), int(st.xsuper[js + 1])
            rows = st.lindx[st.xlindx[js] - 1: st.xlindx[js + 1] - 1] - 1
            for k in range(l - f):
                base = int(st.xlnz[f - 1 + k]) - 1
                sel = rows >= f - 1 + k
                C[rows[sel], f - 1 + k] = o.lnz[base: base + rows.size][sel]
        P = st.order.rperm - 1
        assert np.max(np.abs(C @ C.T - A.toarray()[np.ix_(P, P)])) < 1e-12


def test_oracle_cholesky_rejects_indefinite():
    A = sp.csc_matrix(S.gallery.laplacian((5, 5)) - 5.0 * sp.identity(25))
    cp, rv, nz = A.indptr.astype(np.int64) + 1, A.indices.astype(np.int64) + 1, A.data
    st = oracle.structure_csc(cp, rv, 25, "mmd")
    o = oracle.OracleLU(st)
    o.inmatrix_csc(cp, rv, nz)
    assert o.cholfactor() > 0


def test_dual_oracle_gradient_through_sparse_solve():
    # test/test_generic.jl:58-98 (generic002): d/dp sum(A(p) \\ ones) for the
    # 20 x 20 tridiagonal A(p) = Tridiagonal(-0.1, p^i, -0.1), p in 1:0.1:10,
    # through the LU path on Dual numbers, against the dense derivative
    # -1' A^-1 (dA/dp) A^-1 1 (the reference compares with ForwardDiff on the
    # dense solve, to rtol sqrt(eps))
    n = 20
    for p in np.arange(1.0, 10.0 + 1e-9, 0.1):
        i = np.arange(1, n + 1, dtype=np.float64)
        A = sp.diags([-0.1 * np.ones(n - 1), p ** i, -0.1 * np.ones(n - 1)], [-1, 0, 1], format="csc")
        dA = sp.diags([np.zeros(n - 1), i * p ** (i - 1), np.zeros(n - 1)], [-1, 0, 1], format="csc")
        cp, rv = A.indptr.astype(np.int64) + 1, A.indices.astype(np.int64) + 1
        st = oracle.structure_csc(cp, rv, n, "mmd")
        cols = np.repeat(np.arange(n), np.diff(A.indptr))
        dnz = np.asarray(dA.toarray()[A.indices, cols]).reshape(-1, 1)   # dA/dp on A's pattern, CSC order
        x, dx = oracle.dual_solve(st, cp, rv, A.data, dnz, np.ones(n))
        Ad = A.toarray()
        y = np.linalg.solve(Ad, np.ones(n))
        dense = -np.ones(n) @ np.linalg.solve(Ad, dA.toarray() @ y)
        assert np.isclose(np.sum(dx[:, 0]), dense, rtol=1e-10, atol=0.0), (p, np.sum(dx[:, 0]), dense)
        assert np.allclose(x, y, rtol=1e-12, atol=0.0)


def test_dual_oracle_matches_finite_differences():
    A = sp.csc_matrix(S.gallery.convection_diffusion(k=6))
    n = A.shape[0]
    cp, rv = A.indptr.astype(np.int64) + 1, A.indices.astype(np.int64) + 1
    st = oracle.structure_csc(cp, rv, n, "mmd")
    rng = np.random.default_rng(3)
    dnz = rng.standard_normal((A.nnz, 5))
    b = rng.uniform(-1, 1, n)
    x, dx = oracle.dual_solve(st, cp, rv, A.data, dnz, b)
    for k in range(5):
        h = 1e-6
        Ap, Am = A.copy(), A.copy()
        Ap.data = A.data + h * dnz[:, k]
        Am.data = A.data - h * dnz[:, k]
        fd = (np.linalg.solve(Ap.toarray(), b) - np.linalg.solve(Am.toarray(), b)) / (2 * h)
        assert np.max(np.abs(fd - dx[:, k])) / np.max(np.abs(fd)) < 1e-7

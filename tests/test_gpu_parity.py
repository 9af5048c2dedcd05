"""CUDA numeric phase vs the oracle, through the C ABI (libspk_gpu.so).

Bar: identical pivot sequence; FP64 factors within 1e-12 (relative, max norm
per array) of the oracle's; solutions within 1e-10 relative of the oracle's
and relative residual <= 1e-12.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
import sparspak as S
from cases import m31_problem, problem_from_csc, sprand_spd_like, sprand_unsym, tridiag_csc, tridiag_problem
from sparspak.problem import csc_arrays

pytestmark = pytest.mark.gpu

FACTOR_RTOL = 1e-12


def run_both(p, orderfunction=None, precision="fp64"):
    s = S.SparseSolver(p, precision=precision)
    S.findorder_(s, orderfunction)
    S.symbolicfactor_(s)
    o = oracle.OracleLU(s.slvr)
    o.inmatrix_csc(*S.sparse_solver._matrix_arrays(p))
    o.factor()
    S.inmatrix_(s)
    S.factor_(s)
    return s, o


def rel(a, b):
    scale = max(np.max(np.abs(b)), 1e-300) if b.size else 1.0
    return float(np.max(np.abs(a - b)) / scale) if b.size else 0.0


def check_factors(s, o, rtol=FACTOR_RTOL):
    lnz, unz, ipiv = s.slvr.lnz, s.slvr.unz, s.slvr.ipiv
    assert np.array_equal(ipiv, o.ipiv), "pivot sequence differs"
    assert rel(lnz, o.lnz) <= rtol
    assert rel(unz, o.unz[: unz.size]) <= rtol


def test_golden_tridiag11(golden):
    p = tridiag_problem(11)
    s = S.SparseSolver(p)
    S.findorder_(s)
    S.symbolicfactor_(s)
    S.inmatrix_(s)
    # after inmatrix!: exact (msprs005)
    assert s.slvr.lnz.tolist() == golden["tridiag11_inmatrix_lnz"]
    assert s.slvr.unz.tolist() == golden["tridiag11_inmatrix_unz"]
    S.factor_(s)
    ref = np.array(golden["tridiag11_factor_lnz"])
    assert np.max(np.abs(s.slvr.lnz - ref) / np.abs(ref)) < 1e-15
    S.triangularsolve_(s)
    A = S.outsparse(p).toarray()
    xr = np.linalg.solve(A, p.rhs)
    assert np.linalg.norm(p.x - xr) / np.linalg.norm(xr) < 1e-14


@pytest.mark.parametrize("case", ["m31", "spd301", "spd357", "spd1357", "grid5x3", "tridiag1101"])
def test_factor_and_solve_vs_oracle(case, golden):
    if case == "m31":
        p = m31_problem(golden)
    elif case.startswith("spd"):
        n = int(case[3:])
        p = problem_from_csc(sprand_spd_like(n, n), np.arange(1, n + 1, dtype=np.float64))
    elif case == "grid5x3":
        p = S.makegridproblem(5, 3)
        S.infullrhs_(p, np.arange(1, 16, dtype=np.float64))
    else:
        p = tridiag_problem(1101)
    s, o = run_both(p)
    check_factors(s, o)
    S.triangularsolve_(s)
    xo = o.solve(p.rhs[: p.nrows])
    assert rel(p.x[: p.nrows], xo) < 1e-10
    A = S.outsparse(p)
    r = p.rhs[: p.nrows] - A @ p.x[: p.nrows]
    assert np.linalg.norm(r) / np.linalg.norm(p.rhs[: p.nrows]) < 1e-12


def test_small_literal_pivoting(golden):
    for vals in golden["small4x4"]:
        A = sp.csc_matrix(np.array(vals).reshape(4, 4))
        p = problem_from_csc(A)
        S.inbi_(p, 1, 1.0)
        s, o = run_both(p)
        check_factors(s, o)


def test_random_unsymmetric_pivoting():
    # test/test_structunsymm.jl:60-90 through both APIs: abs error < 1e-9, pivots equal to the oracle's
    rng = np.random.default_rng(7)
    for t in range(200):
        A = sprand_unsym(4, 0.3, 1000 + t)
        b = rng.random(4)
        s, o = run_both(problem_from_csc(A, b))
        check_factors(s, o)
        x = S.ldiv(S.sparspaklu(A), b)
        assert np.linalg.norm(x - np.linalg.solve(A.toarray(), b)) < 1e-9


@pytest.mark.parametrize("shape,order", [((20, 20), "mmd"), ((20, 20), "nd"), ((10, 10, 10), "nd"),
                                         ((9, 11, 7), "mmd")])
def test_grid_laplacian(shape, order):
    A = S.gallery.laplacian(shape)
    of = None if order == "mmd" else S.nd_grid(*(shape + (1,) * (3 - len(shape))), leaf=16)
    s, o = run_both(A, of)
    check_factors(s, o)
    b = S.gallery.random_rhs(A.shape[0], 3, seed=1)
    x = b.copy(order="F")
    S.triangularsolve_(s, x)
    assert rel(x, o.solve(b)) < 1e-10


def test_convection_diffusion_pivots_identity():
    A = S.gallery.convection_diffusion(k=10)
    s, o = run_both(A, S.nd_grid(10, 10, 10, leaf=16))
    check_factors(s, o)
    # an M-matrix: every in-block pivot is the diagonal
    b = s.slvr
    ident = np.concatenate([np.arange(1, b.xsuper[k + 1] - b.xsuper[k] + 1) for k in range(b.nsuper)])
    assert np.array_equal(b.ipiv, ident)


def test_wide_supernodes():
    # dense blocks give chains split 23/23/23/31 and long chains with a last piece > 32
    rng = np.random.default_rng(5)
    for n in (100, 400):
        A = sp.csc_matrix(rng.standard_normal((n, n)) + n * np.eye(n))
        s, o = run_both(A)
        assert np.diff(s.slvr.xsuper).max() > 30
        check_factors(s, o, 1e-11)


def test_cscinterface_refactor():
    # test/test_cscinterface.jl:127-199: sparspaklu, sparspaklu! with and without pattern change
    n = 20
    spm = sprand_spd_like(n, 11, diag=40.0)
    ex = np.ones(n)
    lu = S.sparspaklu(spm)
    assert np.allclose(S.ldiv(lu, spm @ ex), ex)
    spm2 = spm.copy()
    spm2.data -= 0.1
    S.sparspaklu_(lu, spm2)
    assert np.allclose(S.ldiv(lu, spm2 @ ex), ex)
    spm3 = sp.csc_matrix(spm2 + sp.random(n, n, density=1 / n, random_state=np.random.default_rng(2)))
    with pytest.raises(S.ErrorException):
        S.sparspaklu_(lu, spm3, allow_pattern_change=False)
    S.sparspaklu_(lu, spm3)
    assert np.allclose(S.ldiv(lu, spm3 @ ex), ex)
    lu0 = S.sparspaklu(sp.csc_matrix((1, 1)), factorize=False)
    S.sparspaklu_(lu0, spm3, allow_pattern_change=False)
    assert np.allclose(S.ldiv(lu0, spm3 @ ex), ex)


def test_solver_full_sequence_and_errors():
    p = tridiag_problem(11)
    s = S.SparseSolver(p)
    with pytest.raises(S.ErrorException):
        S.symbolicfactor_(s)
    S.solve_(s)
    A = S.outsparse(p).toarray()
    assert np.linalg.norm(p.x - np.linalg.solve(A, p.rhs)) < 1e-12


def test_singular_block_raises():
    A = sp.csc_matrix(np.array([[1.0, 1.0, 0.0], [1.0, 1.0, 0.0], [0.0, 0.0, 2.0]]))
    s = S.SparseSolver(A)
    S.findorderperm_(s, [1, 2, 3])
    S.symbolicfactor_(s)
    S.inmatrix_(s)
    with pytest.raises(S.ErrorException, match="supernode"):
        S.factor_(s)


def test_no_slot_for_entry():
    # an entry outside the symbolic structure is reported like _inmatrix!'s "No space" error
    A = tridiag_csc(6)
    s = S.SparseSolver(A)
    S.findorderperm_(s, np.arange(1, 7))
    S.symbolicfactor_(s)
    eng = S.sparse_solver._ensure_engine(s.slvr)
    B = sp.csc_matrix(A + sp.csc_matrix(([1.0], ([5], [0])), shape=(6, 6)))
    with pytest.raises(S.ErrorException, match="No space for matrix element"):
        eng.set_pattern(B.indptr + 1, B.indices + 1, s.slvr.order.rperm, s.slvr.order.rinvp, index_base=1)


def test_mixed_precision_refinement():
    A = S.gallery.laplacian((12, 12, 12), shift=1e-3)
    b = S.gallery.random_rhs(A.shape[0], 4, seed=2)
    s = S.SparseSolver(A)
    S.findorder_(s, S.nd_grid(12, 12, 12, leaf=16))
    x, it, rr = S.refine_(s, b, precision="fp32", tol=1e-12)
    assert rr <= 1e-12 and 1 <= it <= 10
    r = b - A @ x
    assert np.max(np.linalg.norm(r, axis=0) / np.linalg.norm(b, axis=0)) <= 1e-12
    # FP32 factor entries agree with the FP64 oracle to FP32 accuracy
    o = oracle.OracleLU(s.slvr)
    o.inmatrix_csc(*S.sparse_solver._matrix_arrays(A))
    o.factor()
    assert rel(s.slvr.lnz, o.lnz) < 1e-4


def test_device_resident_arrays():
    torch = pytest.importorskip("torch")
    A = S.gallery.laplacian((16, 16, 16), shift=1e-3)
    s = S.SparseSolver(A)
    S.findorder_(s, S.nd_grid(16, 16, 16))
    S.symbolicfactor_(s)
    S.inmatrix_(s)
    S.factor_(s)
    b = S.gallery.random_rhs(A.shape[0], 2, seed=3)
    bt = torch.tensor(np.ascontiguousarray(b.T), device="cuda")
    s.slvr.engine.solve(bt)
    x = bt.cpu().numpy().T
    r = b - A @ x
    assert np.max(np.linalg.norm(r, axis=0) / np.linalg.norm(b, axis=0)) < 1e-12


@pytest.mark.parametrize("kind", ["laplace", "convdiff"])
def test_fp32_tensor_core_updates(kind):
    # 24^3 / 20^3 grids: fronts with m >= 96 (Schur complement on the tensor
    # cores) and multi-block fronts with >= 128 rows below a block (trailing
    # update on the tensor cores), 3xTF32 products into FP32 storage
    if kind == "laplace":
        A, g = S.gallery.laplacian((24, 24, 24), shift=1e-3), (24, 24, 24)
    else:
        A, g = S.gallery.convection_diffusion(k=20), (20, 20, 20)
    s = S.SparseSolver(A, precision="fp32")
    S.findorder_(s, S.nd_grid(*g))
    S.symbolicfactor_(s)
    o = oracle.OracleLU(s.slvr)
    o.inmatrix_csc(*S.sparse_solver._matrix_arrays(A))
    o.factor()
    S.inmatrix_(s)
    eng = s.slvr.engine
    eng.profile_reset()
    S.factor_(s)
    prof = eng.profile_read()
    assert prof["tc_schur"]["launches"] > 0, "the tensor-core Schur kernel did not run"
    if kind == "laplace":
        assert prof["tc_trail"]["launches"] > 0, "the tensor-core trailing kernel did not run"
    assert np.array_equal(s.slvr.ipiv, o.ipiv)
    assert rel(s.slvr.lnz, o.lnz) < 1e-4
    assert rel(s.slvr.unz, o.unz[: s.slvr.unz.size]) < 1e-4
    b = S.gallery.random_rhs(A.shape[0], 2, seed=4)
    x, it, rr = S.refine_(s, b, precision="fp32", tol=1e-12)
    assert rr <= 1e-12 and it <= 6
    r = b - A @ x
    assert np.max(np.linalg.norm(r, axis=0) / np.linalg.norm(b, axis=0)) <= 1e-12


@pytest.mark.parametrize("nrhs", [5, 20])
def test_many_rhs_front_and_leaf_solves(nrhs):
    # 24^3: the separators near the root have 4 to 10 blocks (the cluster
    # front solves), the leaves are single blocks of a few columns (the
    # warp-per-front solves); 5 and 20 right-hand sides cross the solvers'
    # groups of 4 and the 16-column batches of the C ABI.  Plain and
    # transposed solves against the oracle and scipy, FP64.
    import scipy.sparse.linalg as spla
    k = 24
    A = S.gallery.convection_diffusion(k=k)
    b = S.gallery.random_rhs(A.shape[0], nrhs, seed=nrhs)
    s, o = run_both(A, S.nd_grid(k, k, k))
    x = b.copy(order="F")
    S.triangularsolve_(s, x)
    xo = o.solve(b)
    assert rel(x, xo) < 1e-10
    r = b - A @ x
    assert np.max(np.linalg.norm(r, axis=0) / np.linalg.norm(b, axis=0)) <= 1e-12
    xt = b.copy(order="F")
    S.transposetriangularsolve_(s, xt)
    xr = spla.splu(sp.csc_matrix(A.T)).solve(b)
    assert rel(xt, xr) < 1e-9


@pytest.mark.parametrize("kind", ["dense300", "unsym_pivoting"])
def test_fp32_block_lu_with_pivoting(kind):
    # FP32 blocks of up to 128 columns with real in-piece interchanges: a
    # dense 300 x 300 block (one front, 27-28-column pieces, 128-column
    # blocks) and a sparse unsymmetric matrix with a small diagonal.  Same
    # pivots as the FP64 oracle, factors to FP32 accuracy (pivoting only
    # inside pieces allows growth), refinement to 1e-12.
    rng = np.random.default_rng(21)
    if kind == "dense300":
        n = 300
        A = sp.csc_matrix(rng.standard_normal((n, n)) + 0.5 * np.sqrt(n) * np.eye(n))
    else:
        n = 600
        a = sp.random(n, n, density=8.0 / n, random_state=rng, format="csc")
        A = sp.csc_matrix(a + a.T.multiply(rng.uniform(0.5, 1.5)) + 0.05 * sp.identity(n))
    s, o = run_both(A, None, precision="fp32")
    b_ = s.slvr
    ident = np.concatenate([np.arange(1, b_.xsuper[k + 1] - b_.xsuper[k] + 1) for k in range(b_.nsuper)])
    assert not np.array_equal(o.ipiv, ident), "the case should exercise in-block interchanges"
    assert np.array_equal(b_.ipiv, o.ipiv)
    assert rel(b_.lnz, o.lnz) < 5e-3
    b = S.gallery.random_rhs(n, 2, seed=8)
    x, it, rr = S.refine_(s, b, precision="fp32", tol=1e-12)
    assert rr <= 1e-12
    r = b - A @ x
    assert np.max(np.linalg.norm(r, axis=0) / np.linalg.norm(b, axis=0)) <= 1e-12

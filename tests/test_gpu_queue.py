"""The persistent leaf queue (k_leaf_queue), its bounded waits, and the
option autotuner, through the C ABI.

* Queue on and off (the default): the FP64 factors of grid Laplacians (MMD
  and ND orderings, 2D and 3D), a convection-diffusion matrix, the batched
  2D diffusion systems and the symmetric (SPD) form match the oracle's -
  identical pivots, factors within 1e-12 - and the queue replaces launches.
* The timeout path: a small wait budget and a stalled queue position make
  spk_factor return SPK_ETIMEOUT (DeviceTimeoutError) without a fault; with
  the defaults back the next factor is correct again.
* Wide tensor-core Schur tiles (128 x 256, SPK_OPT_TC_WIDE) against the
  128 x 128 ones: the same factors to FP32 rounding (the scatter-adds into
  the parents come in another order), in the FP32, BF16 and SPD forms.
* The block LU by pieces (SPK_OPT_LU_PIECES, a warp per piece's diagonal
  block, then the block's solves and update in parallel) against the
  column-by-column form, on a dense block with real interchanges: the
  oracle's pivots in both, FP64 factors within 1e-12.
* The cluster-solve threshold (SPK_OPT_SOLVE_CLUSTER_MINB) changes only the
  solves' launch lists: the factors are kept, and the solutions agree.
* The panel split (SPK_OPT_PANEL_SPLIT: a block step's near panel tiles on
  the launch stream, the far ones beside them on the look-ahead stream) does
  the same arithmetic as one panel launch: the factors agree to FP32
  rounding (only the Schur scatter-add order differs) in the FP32, BF16 and
  SPD forms, and both refine to 1e-12.
* The Schur split (SPK_OPT_SCHUR_SPLIT: the Schur tiles whose targets are
  factored two or more levels up run on a third stream beside the next
  level) gives the same factors to FP32 rounding (atomic scatter-adds in
  another order) in the FP32, BF16 and SPD forms, and both refine to 1e-12.
* Chunked root-front solves (SPK_OPT_SOLVE_CHUNK: a root front of more
  than 16 blocks in chunks of at most 16, linked by a product over all SMs)
  change only the solves' launch lists: the solutions agree with the single
  cluster launch to 1e-12 (FP64) and refine to 1e-12 (FP32), forward and
  backward, one and several right-hand sides.
* spk_autotune chooses options from its set, leaves A assembled, and the
  factor that follows refines to 1e-12.
"""
import numpy as np
import pytest

import scipy.sparse as sp

import oracle
import sparspak as S
from sparspak.sparse_solver import _factor_, _inmatrix_, _matrix_arrays

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))


def relres(A, x, b):
    r = b - A @ x
    return float(np.max(np.linalg.norm(r, axis=0) / np.linalg.norm(b, axis=0)))


def _case(kind):
    if kind == "laplace2d_mmd":
        return S.gallery.laplacian((40, 40)), None
    if kind == "laplace3d_nd":
        return S.gallery.laplacian((20, 20, 20), shift=1e-3), S.nd_grid(20, 20, 20)
    if kind == "convdiff_nd":
        return S.gallery.convection_diffusion(k=16), S.nd_grid(16, 16, 16)
    A, sizes = S.gallery.batched_diffusion(24, 12, 40, seed=2)
    return A, S.nd_grid_batched(sizes)


def _solver(A, of, **kw):
    s = S.SparseSolver(A, **kw)
    S.findorder_(s, of)
    S.symbolicfactor_(s)
    return s


def _factor_with(s, A, **opts):
    """Assemble A again and factor with the given options; the engine."""
    _inmatrix_(s.slvr, A)
    eng = s.slvr.engine
    for k, v in opts.items():
        eng.set_option(k, v)
        assert eng.get_option(k) == v
    eng.profile_reset()
    _factor_(s.slvr)
    return eng


@pytest.mark.parametrize("kind", ["laplace2d_mmd", "laplace3d_nd", "convdiff_nd", "batched"])
def test_leaf_queue_on_off_vs_oracle(kind):
    A, of = _case(kind)
    s = _solver(A, of)
    o = oracle.OracleLU(s.slvr)
    o.inmatrix_csc(*_matrix_arrays(A))
    assert o.factor() == 0
    b = S.gallery.random_rhs(A.shape[0], 2, seed=4)
    xo = o.solve(b)
    launches = {}
    for q in (1, 0):
        eng = _factor_with(s, A, leaf_queue=q)
        launches[q] = eng.profile_read()["getrf"]["launches"]
        assert np.array_equal(s.slvr.ipiv, o.ipiv), q
        assert rel(s.slvr.lnz, o.lnz) <= 1e-12, q
        assert rel(s.slvr.unz, o.unz[: s.slvr.unz.size]) <= 1e-12, q
        x = eng.solve(np.array(b, order="F"))
        assert rel(x, xo) < 1e-10
        assert relres(A, x, b) <= 1e-12
    print(f"{kind}: getrf-class launches with the queue {launches[1]}, without {launches[0]}")
    assert launches[1] < launches[0], "the queue replaced no launches"


def test_leaf_queue_spd_form_vs_oracle_cholesky():
    A = S.gallery.laplacian((24, 24, 24), shift=1e-3)
    s = _solver(A, S.nd_grid(24, 24, 24), spd=True)
    o = oracle.OracleLU(s.slvr)
    o.inmatrix_csc(*_matrix_arrays(A))
    assert o.cholfactor() == 0
    mask = o.lower_mask()
    for q in (1, 0):
        _factor_with(s, A, leaf_queue=q)
        assert rel(s.slvr.lnz[mask], o.lnz[mask]) <= 1e-12, q


def test_queue_wait_timeout_is_reported_and_recoverable():
    # queue position 0 waits on a condition nothing sets; after 2000 polls it
    # gives up, the factorisation reports the timeout and nothing faults
    A = S.gallery.laplacian((32, 32))
    s = _solver(A, S.nd_grid(32, 32, 1, leaf=16))
    o = oracle.OracleLU(s.slvr)
    o.inmatrix_csc(*_matrix_arrays(A))
    assert o.factor() == 0
    with pytest.raises(S.DeviceTimeoutError, match="leaf-queue"):
        _factor_with(s, A, leaf_queue=1, wait_budget=2000, stall_test=0)
    eng = s.slvr.engine
    with pytest.raises(S.ErrorException, match="Factorization not done"):
        eng.solve(np.ones(A.shape[0]))
    eng.set_option("stall_test", -1)
    eng.set_option("wait_budget", 1 << 20)
    eng.factor("fp64")   # reassembles A: the timed-out factor left it invalid
    assert np.array_equal(s.slvr.ipiv, o.ipiv)
    assert rel(s.slvr.lnz, o.lnz) <= 1e-12
    for bad in (("leaf_queue", 2), ("wait_budget", 0), ("stall_test", -2), ("tc_schur_m", 0)):
        with pytest.raises(S.ErrorException):
            eng.set_option(*bad)


@pytest.mark.parametrize("prec", ["fp32", "bf16s", "fp32+spd"])
def test_wide_schur_tiles_match_narrow(prec):
    A = S.gallery.laplacian((30, 30, 30), shift=1e-3)
    n = A.shape[0]
    base, _, form = prec.partition("+")
    s = _solver(A, S.nd_grid(30, 30, 30), precision=base, spd=form == "spd")
    b = S.gallery.random_rhs(n, 2, seed=6)
    lnz = {}
    for wide in (1, 0):
        eng = _factor_with(s, A, tc_wide=wide)
        prof = eng.profile_read()
        assert prof["tc_schur"]["launches"] > 0
        lnz[wide] = s.slvr.lnz.copy()
        x = np.zeros_like(b, order="F")
        it, rr = eng.refine(np.asfortranarray(b), x, prec, 1e-12, 100)
        assert rr <= 1e-12 and relres(A, x, b) <= 1e-12, (wide, rr, it)
    d = rel(lnz[1], lnz[0])
    print(f"{prec}: wide vs narrow Schur tiles, factors differ by {d:.1e}")
    assert d < (5e-3 if base == "bf16s" else 1e-5)


@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp64+spd"])
def test_block_lu_by_pieces_vs_columns(prec):
    rng = np.random.default_rng(21)
    n = 300
    M = rng.standard_normal((n, n))
    base, _, form = prec.partition("+")
    if form == "spd":
        A = sp.csc_matrix(M @ M.T / n + np.eye(n))
    else:
        A = sp.csc_matrix(M + 0.5 * np.sqrt(n) * np.eye(n))
    s = _solver(A, None, precision=base, spd=form == "spd")
    o = oracle.OracleLU(s.slvr)
    o.inmatrix_csc(*_matrix_arrays(A))
    assert (o.cholfactor() if form == "spd" else o.factor()) == 0
    mask = o.lower_mask() if form == "spd" else slice(None)
    b = S.gallery.random_rhs(n, 2, seed=3)
    got = {}
    for pcs in (1, 0):
        eng = _factor_with(s, A, lu_pieces=pcs)
        if form != "spd":
            assert np.array_equal(s.slvr.ipiv, o.ipiv), pcs
        got[pcs] = s.slvr.lnz.copy()
        e = rel(got[pcs][mask], o.lnz[mask])
        # the column form's rank-1 order differs from the reference's
        # piece-wise trsm / gemm more than the piece form's (4.8e-12 here)
        assert e <= ((1e-12 if pcs else 1e-11) if base == "fp64" else 5e-3), (pcs, e)
        print(f"{prec} lu_pieces={pcs}: factors vs oracle {e:.1e}")
        x = np.zeros_like(b, order="F")
        it, rr = eng.refine(np.asfortranarray(b), x, prec, 1e-12, 30)
        assert rr <= 1e-12 and relres(A, x, b) <= 1e-12
    print(f"{prec}: by pieces vs column groups, factors differ by {rel(got[1], got[0]):.1e}")


@pytest.mark.parametrize("prec", ["fp32", "bf16s", "fp32+spd"])
def test_panel_split_matches_one_launch(prec):
    A = S.gallery.laplacian((36, 36, 36), shift=1e-3)
    n = A.shape[0]
    base, _, form = prec.partition("+")
    s = _solver(A, S.nd_grid(36, 36, 36), precision=base, spd=form == "spd")
    b = S.gallery.random_rhs(n, 2, seed=9)
    lnz = {}
    for split in (1, 0):
        eng = _factor_with(s, A, panel_split=split)
        lnz[split] = s.slvr.lnz.copy()
        x = np.zeros_like(b, order="F")
        it, rr = eng.refine(np.asfortranarray(b), x, prec, 1e-12, 100)
        assert rr <= 1e-12 and relres(A, x, b) <= 1e-12, (split, rr, it)
    d = rel(lnz[1], lnz[0])
    print(f"{prec}: panel split vs one launch, factors differ by {d:.1e}")
    assert d < (5e-3 if base == "bf16s" else 1e-5)
    with pytest.raises(S.ErrorException):
        eng.set_option("panel_split", 2)


@pytest.mark.parametrize("prec", ["fp32", "bf16s", "fp32+spd"])
def test_schur_split_matches_one_launch(prec):
    A = S.gallery.laplacian((40, 40, 40), shift=1e-3)
    n = A.shape[0]
    base, _, form = prec.partition("+")
    s = _solver(A, S.nd_grid(40, 40, 40), precision=base, spd=form == "spd")
    b = S.gallery.random_rhs(n, 2, seed=12)
    lnz, xs = {}, {}
    for split in (1, 0):
        eng = _factor_with(s, A, schur_split=split)
        lnz[split] = s.slvr.lnz.copy()
        x = np.zeros_like(b, order="F")
        it, rr = eng.refine(np.asfortranarray(b), x, prec, 1e-12, 100)
        assert rr <= 1e-12 and relres(A, x, b) <= 1e-12, (split, rr, it)
        xs[split] = x
    d = rel(lnz[1], lnz[0])
    print(f"{prec}: Schur split vs one launch, factors differ by {d:.1e}")
    assert d < (5e-3 if base == "bf16s" else 1e-5)
    assert rel(xs[1], xs[0]) < 1e-10
    with pytest.raises(S.ErrorException):
        eng.set_option("schur_split", 2)


@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp64+spd"])
def test_chunked_root_solve_matches_one_cluster(prec):
    # 48^3: the root separator (2304 columns) is 18 blocks of 128 (FP32) or
    # 36 of 64 (FP64), more than one cluster's 16
    A = S.gallery.laplacian((48, 48, 48), shift=1e-3)
    n = A.shape[0]
    base, _, form = prec.partition("+")
    s = _solver(A, S.nd_grid(48, 48, 48), precision=base, spd=form == "spd")
    eng = _factor_with(s, A)
    for nrhs in (1, 5):
        b = S.gallery.random_rhs(n, nrhs, seed=20 + nrhs)
        xs = {}
        for ch in (1, 0):
            eng.set_option("solve_chunk", ch)   # no new factorisation
            if base == "fp64":
                xs[ch] = eng.solve(np.array(b, order="F"), prec)
                assert relres(A, xs[ch], b) <= 1e-12, (ch, nrhs)
            else:
                x = np.zeros_like(b, order="F")
                it, rr = eng.refine(np.asfortranarray(b), x, prec, 1e-12, 30)
                assert rr <= 1e-12 and relres(A, x, b) <= 1e-12, (ch, nrhs, rr)
                xs[ch] = x
        d = rel(xs[1], xs[0])
        print(f"{prec} nrhs={nrhs}: chunked vs one cluster, solutions differ by {d:.1e}")
        assert d < 1e-10
    with pytest.raises(S.ErrorException):
        eng.set_option("solve_chunk", 2)


def test_solve_cluster_threshold_keeps_factors():
    A = S.gallery.laplacian((24, 24, 24), shift=1e-3)
    n = A.shape[0]
    s = _solver(A, S.nd_grid(24, 24, 24))
    eng = _factor_with(s, A)
    b = S.gallery.random_rhs(n, 3, seed=2)
    xs = {}
    for mb in (4, 2, 128):
        eng.set_option("solve_cluster_minb", mb)   # no new factorisation
        xs[mb] = eng.solve(np.array(b, order="F"))
        assert relres(A, xs[mb], b) <= 1e-12, mb
    assert rel(xs[2], xs[4]) < 1e-12 and rel(xs[128], xs[4]) < 1e-12
    with pytest.raises(S.ErrorException):
        eng.set_option("solve_cluster_minb", 1)


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_autotune_then_factor_and_refine(prec):
    A = S.gallery.laplacian((28, 28, 28), shift=1e-3)
    n = A.shape[0]
    s = _solver(A, S.nd_grid(28, 28, 28), precision=prec)
    _inmatrix_(s.slvr, A)
    eng = s.slvr.engine
    opts, ms = eng.autotune(prec, reps=2)
    print(f"autotune {prec}: {opts}, best factor {ms:.3f} ms")
    assert ms > 0 and opts["leaf_queue"] in (0, 1)
    if prec == "fp32":
        assert (opts["tc_schur_m"], opts["tc_trail_rows"]) in {(96, 128), (64, 128), (128, 128), (192, 128),
                                                               (96, 256), (128, 256), (256, 256)}
        assert opts["tc_wide"] in (0, 1)
    eng.factor(prec)   # A was left assembled
    b = S.gallery.random_rhs(n, 2, seed=8)
    x = np.zeros_like(b, order="F")
    it, rr = eng.refine(np.asfortranarray(b), x, prec, 1e-12, 20)
    assert rr <= 1e-12 and relres(A, x, b) <= 1e-12

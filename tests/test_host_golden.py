"""Host structure phase against the reference's golden vectors (no GPU)."""
import numpy as np
import pytest
import scipy.sparse as sp

import sparspak as S
from cases import tridiag_problem


def test_mmd_ordering_tridiag11(golden):
    # test/test_sparse_method.jl:87-90 (msprs003)
    s = S.SparseSolver(tridiag_problem(11))
    S.findorder_(s)
    o = s.slvr.order
    assert o.rperm.tolist() == golden["tridiag11_rperm"]
    assert o.rinvp.tolist() == golden["tridiag11_rinvp"]
    assert o.cperm.tolist() == golden["tridiag11_rperm"]
    assert o.cinvp.tolist() == golden["tridiag11_rinvp"]


def test_symbolic_tridiag11(golden):
    # test/test_sparse_method.jl:127-131 (msprs004)
    s = S.SparseSolver(tridiag_problem(11))
    S.findorder_(s)
    S.symbolicfactor_(s)
    b = s.slvr
    assert b.xlnz.tolist() == golden["tridiag11_xlnz"]
    assert b.xunz.tolist() == golden["tridiag11_xunz"]
    assert b.xlindx.tolist() == golden["tridiag11_xlindx"]
    assert b.lindx.tolist() == golden["tridiag11_lindx"]


def _fig313(golden, key="fig313"):
    I, J = np.array(golden[key + "_I"]), np.array(golden[key + "_J"])
    return sp.csc_matrix((np.ones(I.size), (I - 1, J - 1)), shape=(6, 6))


@pytest.mark.parametrize("via", ["problem", "csc"])
def test_graph_fig313(golden, via):
    # test/test_graph.jl:10-23 and test/test_cscinterface.jl:3-20
    m = _fig313(golden)
    g = S.Graph.from_problem(S.problem.Problem(6, 6)) if False else None
    if via == "problem":
        p = S.Problem(6, 6)
        S.insparse_(p, m)
        g = S.Graph.from_problem(p)
    else:
        g = S.Graph.from_csc(m)
    assert g.xadj.tolist() == golden["fig313_xadj"]
    assert g.adj.tolist() == golden["fig313_adj"]
    assert S.isstructuresymmetric(g)


@pytest.mark.parametrize("via", ["problem", "csc"])
def test_graph_symmetrize(golden, via):
    # test/test_graph.jl:84-99 (element (5, 3) missing)
    m = _fig313(golden, "fig313_unsym")
    if via == "problem":
        p = S.Problem(6, 6)
        S.insparse_(p, m)
        g = S.Graph.from_problem(p)
    else:
        g = S.Graph.from_csc(m)
    assert not S.isstructuresymmetric(g)
    S.makestructuresymmetric(g)
    assert S.isstructuresymmetric(g)
    assert g.xadj.tolist() == golden["fig313_xadj"]
    assert g.adj.tolist() == golden["fig313_adj"]


def test_grid_numbering(golden):
    g = S.Grid(6, 6)
    assert g.v.ravel().tolist() == golden["grid6x6_v"]


def test_ordering_identity():
    o = S.Ordering(5)
    assert o.rperm.tolist() == [1, 2, 3, 4, 5] and o.cinvp.tolist() == [1, 2, 3, 4, 5]


def test_etree_constructor():
    assert S.ETree(6).parent.tolist() == [0] * 6


def test_problem_roundtrip():
    rng = np.random.default_rng(3)
    spm = sp.random(15, 15, density=0.2, random_state=rng, format="csc")
    spm = sp.csc_matrix(spm + spm.T)
    p = S.Problem(15, 15)
    S.insparse_(p, spm)
    a = S.outsparse(p)
    assert abs(a - spm).max() == 0


def test_inaij_accumulates():
    p = S.Problem(2, 2)
    S.inaij_(p, 1, 1, 4.0)
    S.inaij_(p, 1, 1, 4.0)
    S.inaij_(p, 2, 1, -1.0)
    assert S.outsparse(p).toarray().tolist() == [[8.0, 0.0], [-1.0, 0.0]]
    assert p.nedges == 2


def test_sequence_errors():
    # test/test_sparse_method.jl:724-751 (msprs019): phases out of order raise
    s = S.SparseSolver(tridiag_problem(11))
    with pytest.raises(S.ErrorException, match="Sequence error"):
        S.symbolicfactor_(s)
    S.findorder_(s)
    with pytest.raises(S.ErrorException, match="Sequence error"):
        S.inmatrix_(s)
    S.symbolicfactor_(s)
    with pytest.raises(S.ErrorException, match="Sequence error"):
        S.factor_(s)
    with pytest.raises(S.ErrorException, match="Sequence error"):
        S.triangularsolve_(s)


def test_supernode_split_rule():
    # A dense 100 x 100 matrix is one fundamental supernode.  The reference's
    # rule (SpkSymFct.jl:432-460, maxsize 30): delta = 100/(1+100/30) = 23.08,
    # markers at floor(1 + k*delta) = 24, 47, 70 while below floor(101 - delta/2)
    # = 89, so the last piece keeps 31 columns.
    m = sp.csc_matrix(np.ones((100, 100)) + 100 * np.eye(100))
    s = S.SparseSolver(m)
    S.findorder_(s)
    S.symbolicfactor_(s)
    assert np.diff(s.slvr.xsuper).tolist() == [23, 23, 23, 31]


def test_nd_grid_is_permutation():
    for shape in [(7, 5, 1), (6, 6, 6), (10, 3, 4)]:
        m = S.gallery.laplacian(tuple(d for d in shape if d > 1) if shape[2] == 1 else shape)
        s = S.SparseSolver(m)
        S.findorder_(s, S.nd_grid(*shape, leaf=8))
        perm = s.slvr.order.rperm
        assert sorted(perm.tolist()) == list(range(1, m.shape[0] + 1))
        assert np.all(s.slvr.order.rinvp[perm - 1] == np.arange(1, m.shape[0] + 1))


def test_nd_reduces_fill_3d():
    m = S.gallery.laplacian((12, 12, 12))
    nnz = {}
    for name, of in [("natural", lambda g, o: None), ("nd", S.nd_grid(12, 12, 12)), ("mmd", None)]:
        s = S.SparseSolver(m)
        S.findorder_(s, of)
        S.symbolicfactor_(s)
        nnz[name] = int(s.slvr.xlnz[-1] - 1)
    assert nnz["nd"] < nnz["natural"]


@pytest.mark.parametrize("case", ["grid2d_60", "grid3d_16", "sprand_2000", "disconnected"])
def test_nd_graph_ordering(case):
    # the general nested-dissection plug-in: a valid permutation, through the
    # reference's symbolic phase, with fill of the order of minimum degree's,
    # and a correct factorisation (the oracle LU on its structure)
    import oracle
    from cases import sprand_spd_like

    if case == "grid2d_60":
        A = S.gallery.laplacian((60, 60))
    elif case == "grid3d_16":
        A = S.gallery.laplacian((16, 16, 16), shift=1e-3)
    elif case == "sprand_2000":
        A = sprand_spd_like(2000, 11, diag=40.0)
    else:
        A = sp.block_diag([S.gallery.laplacian((20, 20)), S.gallery.laplacian((9, 9, 9))], format="csc")
    A = sp.csc_matrix(A)
    n = A.shape[0]
    s = S.SparseSolver(A)
    S.findorder_(s, S.nd_graph(leaf=32))
    perm = s.slvr.order.rperm
    assert sorted(perm.tolist()) == list(range(1, n + 1))
    assert np.array_equal(s.slvr.order.rinvp[perm - 1], np.arange(1, n + 1))
    S.symbolicfactor_(s)
    fill_nd = int(s.slvr.xlnz[-1] - 1)
    s2 = S.SparseSolver(A)
    S.findorder_(s2)
    S.symbolicfactor_(s2)
    fill_mmd = int(s2.slvr.xlnz[-1] - 1)
    if case != "sprand_2000":   # (on a random graph with ~2 edges per vertex minimum degree fills far less)
        assert fill_nd < 1.5 * fill_mmd, (fill_nd, fill_mmd)
    o = oracle.OracleLU(s.slvr)
    o.inmatrix_csc(A.indptr.astype(np.int64) + 1, A.indices.astype(np.int64) + 1, A.data)
    assert o.factor() == 0
    b = np.random.default_rng(0).uniform(-1, 1, n)
    x = o.solve(b)
    assert np.linalg.norm(b - A @ x) / np.linalg.norm(b) < 1e-12

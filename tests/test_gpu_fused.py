"""spk_factor_refine: the factorisation and the refined solve in one call,
the first solve's forward substitution of the lower levels run beside the
last levels of the factorisation.  It must give what spk_factor followed by
spk_refine_ex gives - the same factors (the solves do not touch them), a
relative residual <= 1e-12 and solutions within 1e-10 of the two-call
form - for every form, host and device buffers, one to sixteen right-hand
sides and more (the two-call path), and report a singular matrix as
spk_factor does.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import sparspak as S
from sparspak.sparse_solver import _inmatrix_

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))


def relres(A, x, b):
    r = b - A @ x
    return float(np.max(np.linalg.norm(r, axis=0) / np.linalg.norm(b, axis=0)))


def _solver(A, of, prec):
    base, _, form = prec.partition("+")
    s = S.SparseSolver(A, precision=base, spd=form == "spd")
    S.findorder_(s, of)
    S.symbolicfactor_(s)
    return s


@pytest.mark.parametrize("prec", ["fp32", "fp64", "bf16s", "fp32+spd"])
@pytest.mark.parametrize("nrhs", [1, 4, 20])
def test_factor_refine_matches_two_calls(prec, nrhs):
    A = S.gallery.laplacian((32, 32, 32), shift=1e-3)
    n = A.shape[0]
    s = _solver(A, S.nd_grid(32, 32, 32), prec)
    b = np.asfortranarray(S.gallery.random_rhs(n, nrhs, seed=nrhs))
    _inmatrix_(s.slvr, A)
    eng = s.slvr.engine
    eng.factor(prec)
    x2 = np.zeros_like(b, order="F")
    eng.refine(b, x2, prec, 1e-12, 200, solver="auto")
    lnz2 = s.slvr.lnz.copy()
    _inmatrix_(s.slvr, A)
    x1 = np.zeros_like(b, order="F")
    it, rr, used = eng.factor_refine(b, x1, prec, 1e-12, 200, solver="auto")
    assert rr <= 1e-12 and relres(A, x1, b) <= 1e-12, (it, rr, used)
    assert rel(x1, x2) < 1e-10
    assert rel(s.slvr.lnz, lnz2) < (1e-6 if prec != "fp64" else 1e-13)
    # the factors stay usable for later solves
    x3 = eng.solve(np.array(b, order="F"), prec)
    assert rel(x3, x1) < {"fp64": 1e-12, "fp32": 1e-4, "fp32+spd": 1e-4, "bf16s": 0.1}[prec]


def test_factor_refine_device_buffers():
    import torch

    A = S.gallery.convection_diffusion(k=24)
    n = A.shape[0]
    s = _solver(A, S.nd_grid(24, 24, 24), "fp32")
    _inmatrix_(s.slvr, A)
    eng = s.slvr.engine
    b = S.gallery.random_rhs(n, 3, seed=11)
    bd = torch.tensor(np.ascontiguousarray(b.T), device="cuda")   # (nrhs, n)
    xd = torch.zeros_like(bd)
    it, rr = eng.factor_refine(bd, xd, "fp32", 1e-12, 30)
    x = xd.cpu().numpy().T
    assert rr <= 1e-12 and relres(A, x, b) <= 1e-12
    assert it <= 6


def test_factor_refine_singular():
    # a singular 2 x 2 diagonal block (test_singular_block_raises' matrix)
    A = sp.csc_matrix(np.array([[1.0, 1.0, 0.0], [1.0, 1.0, 0.0], [0.0, 0.0, 2.0]]))
    s = S.SparseSolver(A)
    S.findorderperm_(s, [1, 2, 3])
    S.symbolicfactor_(s)
    _inmatrix_(s.slvr, A)
    b = np.ones(3)
    x = np.zeros_like(b)
    with pytest.raises(S.SingularException) as e:
        s.slvr.engine.factor_refine(b, x, "fp64", 1e-12, 10)
    assert e.value.supernode == 1

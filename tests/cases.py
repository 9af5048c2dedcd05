"""Problem builders shared by the tests (the reference tests' own inputs)."""
import numpy as np
import scipy.sparse as sp

import sparspak as S


def tridiag_problem(n):
    """maketridiagproblem of test/test_sparse_method.jl (msprs003-009)."""
    p = S.Problem(n, n)
    for i in range(1, n):
        S.inaij_(p, i + 1, i, -1.0)
        S.inaij_(p, i, i, 4.0)
        S.inaij_(p, i, i + 1, -1.0)
        S.inbi_(p, i, 2.0 * i)
    S.inaij_(p, n, n, 4.0)
    S.inbi_(p, n, 3.0 * n + 1.0)
    return p


def tridiag_csc(n):
    return sp.diags([-np.ones(n - 1), 4 * np.ones(n), -np.ones(n - 1)], [-1, 0, 1], format="csc")


def m31_problem(golden):
    """msprs010: the literal 31 x 31 matrix, rhs = 1:n."""
    spm = sp.csc_matrix((golden["m31_V"], (np.array(golden["m31_I"]) - 1, np.array(golden["m31_J"]) - 1)),
                        shape=(31, 31))
    p = S.Problem(31, 31, spm.nnz)
    S.insparse_(p, spm)
    S.infullrhs_(p, np.arange(1, 32, dtype=np.float64))
    return p


def sprand_spd_like(n, seed, diag=20.0):
    """-A - A' + diag*I with A = sprand(n, n, 1/n) (msprs012-016, csc_msolver001)."""
    rng = np.random.default_rng(seed)
    a = sp.random(n, n, density=1.0 / n, random_state=rng, format="csc")
    return sp.csc_matrix(-a - a.T + diag * sp.identity(n))


def sprand_unsym(n, p, seed):
    """sprand(n, n, p) + I (test_structunsymm.jl:60-90): unsymmetric structure and values."""
    rng = np.random.default_rng(seed)
    a = sp.random(n, n, density=p, random_state=rng, format="csc")
    return sp.csc_matrix(a + sp.identity(n))


def problem_from_csc(m, rhs=None):
    m = sp.csc_matrix(m)
    p = S.Problem(m.shape[0], m.shape[1], m.nnz)
    S.insparse_(p, m)
    if rhs is not None:
        S.infullrhs_(p, rhs)
    return p

"""SparseCSCInterface: sparspaklu / sparspaklu_ / ldiv_ on scipy CSC matrices.

Mirrors src/SparseCSCInterface/SparseCSCInterface.jl:205-300.  Julia's
``lu \\ b`` is ``ldiv(lu, b)`` here.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from .device import ErrorException
from .sparse_solver import (SparseSolver, factor_, findorder_, inmatrix_, solve_, symbolicfactor_)


def sparspaklu(m, factorize: bool = True, precision: str = "fp64", orderfunction=None) -> SparseSolver:
    """Order, symbolic, inmatrix, factor (SparseCSCInterface.jl:218-227)."""
    lu = SparseSolver(sp.csc_matrix(m), precision=precision)
    if factorize:
        findorder_(lu, orderfunction) or _fail("Finding Order.")
        symbolicfactor_(lu) or _fail("Symbolic Factorization.")
        inmatrix_(lu) or _fail("Matrix input.")
        factor_(lu) or _fail("Numerical Factorization.")
    return lu


def sparspaklu_(lu: SparseSolver, m, allow_pattern_change: bool = True) -> SparseSolver:
    """Refactor with new values, reusing ordering and symbolic phase (SparseCSCInterface.jl:247-268)."""
    m = sp.csc_matrix(m)
    if not m.has_sorted_indices:
        m = m.sorted_indices()
    old = lu.p
    changed = (old.shape != m.shape or not np.array_equal(old.indptr, m.indptr)
               or not np.array_equal(old.indices, m.indices))
    if changed:
        if allow_pattern_change or not lu._symbolicdone:
            lu.copy_from(SparseSolver(m, precision=lu.slvr.precision))
        else:
            raise ErrorException("'allow_pattern_change=false', but sparsity pattern of matrix 'm' does not match "
                                 "that used to create 'lu'")
    lu.p = m
    lu._orderdone or findorder_(lu) or _fail("Finding Order.")
    lu._symbolicdone or symbolicfactor_(lu) or _fail("Symbolic Factorization.")
    lu._inmatrixdone = False
    lu._factordone = False
    lu._trisolvedone = False
    inmatrix_(lu) or _fail("Matrix input.")
    factor_(lu) or _fail("Numerical Factorization.")
    return lu


def ldiv_(*args):
    """ldiv_(lu, v) solves in place; ldiv_(u, lu, v) writes into u (SparseCSCInterface.jl:277-293)."""
    if len(args) == 3:
        u, lu, v = args
        u[...] = v
        return ldiv_(lu, u)
    lu, v = args
    solve_(lu, v) or _fail("Triangular Solve.")
    lu._trisolvedone = False
    return v


def ldiv(lu: SparseSolver, v):
    """Julia's ``lu \\ v``: a solved copy (SparseCSCInterface.jl:300)."""
    return ldiv_(lu, np.array(v, dtype=np.float64, order="F", copy=True))


def _fail(msg):
    raise ErrorException(msg)

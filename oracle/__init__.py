"""ORACLE - TEST INFRASTRUCTURE ONLY.

ctypes binding of ``spk_oracle.c``, the plain-C restatement of the
reference's numeric phase (_inmatrix!, _lufactor!, _lulsolve!, _luusolve!,
_triangularsolve!; citations in the C file).  Only tests/, the smoke check
of __graft_entry__ and bench.py's CPU-baseline leg use it, as the checker;
the product never imports it.

It is pinned against the reference's golden vectors in tests/golden/ (the
post-inmatrix! and post-factor! lnz/unz of the n=11 tridiagonal problem and
its intermediate forward-solve vector, test/test_sparse_method.jl).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "spk_oracle.c")
SO = os.path.join(HERE, "liboracle.so")

_P = ctypes.POINTER(ctypes.c_int64)
_D = ctypes.POINTER(ctypes.c_double)
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (no FMA contraction, so every host gives the same bits)."""
    if force or not os.path.exists(SO) or os.path.getmtime(SO) < os.path.getmtime(SRC):
        cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-ffp-contract=off", "-o", SO, SRC, "-lm"]
        subprocess.run(cmd, check=True, capture_output=True)
    return SO


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(SO)
        i = ctypes.c_int64
        L.oracle_inmatrix_csc.restype = i
        L.oracle_inmatrix_csc.argtypes = [i, i, _P, _P, _D, _P, _P, _P, _P, _P, _P, _P, _D, _P, _D]
        L.oracle_lufactor.restype = i
        L.oracle_lufactor.argtypes = [i, i, _P, _P, _P, _P, _P, _D, _P, _D, _P, _P]
        L.oracle_lulsolve.restype = None
        L.oracle_lulsolve.argtypes = [i, _P, _P, _P, _P, _D, _P, _D]
        L.oracle_luusolve.restype = None
        L.oracle_luusolve.argtypes = [i, i, _P, _P, _P, _P, _D, _P, _D, _D]
        L.oracle_triangularsolve.restype = None
        L.oracle_triangularsolve.argtypes = [i, i, _P, _P, _P, _P, _D, _P, _D, _P, _P, _P, _D]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_P)


def _d(a):
    return a.ctypes.data_as(_D)


class OracleLU:
    """Reference-layout numeric phase on the CPU for one symbolic structure.

    ``sym`` is anything with the reference's attributes (n, nsuper, xsuper,
    snode, xlindx, lindx, xlnz, xunz and order.rperm/order.rinvp), e.g. the
    package's _SparseBase after symbolicfactor_.
    """

    def __init__(self, sym):
        g = lambda a: np.ascontiguousarray(a, dtype=np.int64)
        self.n, self.nsuper = int(sym.n), int(sym.nsuper)
        self.xsuper, self.snode = g(sym.xsuper), g(sym.snode)
        self.xlindx, self.lindx = g(sym.xlindx), g(sym.lindx)
        self.xlnz, self.xunz = g(sym.xlnz), g(sym.xunz)
        self.rperm, self.rinvp = g(sym.order.rperm), g(sym.order.rinvp)
        self.lnz = np.zeros(int(self.xlnz[-1] - 1))
        self.unz = np.zeros(max(int(self.xunz[-1] - 1), 1))
        self.ipiv = np.zeros(self.n, dtype=np.int64)
        self.first_singular = 0

    def inmatrix_csc(self, colptr, rowval, nzval):
        """1-based CSC of A (original numbering)."""
        colptr, rowval = np.ascontiguousarray(colptr, np.int64), np.ascontiguousarray(rowval, np.int64)
        nzval = np.ascontiguousarray(nzval, np.float64)
        self.lnz[:] = 0.0
        self.unz[:] = 0.0
        self.ipiv[:] = 0
        rc = lib().oracle_inmatrix_csc(self.n, self.n, _p(colptr), _p(rowval), _d(nzval), _p(self.rinvp), _p(self.rinvp),
                                       _p(self.snode), _p(self.xsuper), _p(self.xlindx), _p(self.lindx), _p(self.xlnz),
                                       _d(self.lnz), _p(self.xunz), _d(self.unz))
        if rc != 0:
            raise ValueError(f"No space for matrix element at CSC position {-rc}")

    def factor(self) -> int:
        fs = np.zeros(1, dtype=np.int64)
        iflag = lib().oracle_lufactor(self.n, self.nsuper, _p(self.xsuper), _p(self.snode), _p(self.xlindx),
                                      _p(self.lindx), _p(self.xlnz), _d(self.lnz), _p(self.xunz), _d(self.unz),
                                      _p(self.ipiv), _p(fs))
        self.first_singular = int(fs[0])
        return int(iflag)

    def lulsolve(self, rhs_permuted):
        r = np.ascontiguousarray(rhs_permuted, np.float64).copy()
        lib().oracle_lulsolve(self.nsuper, _p(self.xsuper), _p(self.xlindx), _p(self.lindx), _p(self.xlnz),
                              _d(self.lnz), _p(self.ipiv), _d(r))
        return r

    def solve(self, b):
        """x = A^{-1} b for one vector or the columns of an n x k matrix (original order)."""
        b = np.asarray(b, np.float64)
        cols = b.reshape(b.shape[0], -1)
        out = np.empty_like(cols)
        for j in range(cols.shape[1]):
            v = np.ascontiguousarray(cols[:, j]).copy()
            lib().oracle_triangularsolve(self.n, self.nsuper, _p(self.xsuper), _p(self.xlindx), _p(self.lindx),
                                         _p(self.xlnz), _d(self.lnz), _p(self.xunz), _d(self.unz), _p(self.ipiv),
                                         _p(self.rperm), _p(self.rinvp), _d(v))
            out[:, j] = v
        return out.reshape(b.shape)

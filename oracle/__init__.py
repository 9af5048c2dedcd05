"""ORACLE - TEST INFRASTRUCTURE ONLY.

ctypes binding of ``spk_oracle.c``, the plain-C restatement of the
reference's numeric phase (_inmatrix!, _lufactor!, _lulsolve!, _luusolve!,
_triangularsolve!), and of ``spk_oracle_struct.c``, the restatement of its
structure phase (graph symmetrisation here in numpy, multiple minimum
degree, elimination tree, postorders, column counts, supernodes, symbolic
factorisation) plus the grid nested-dissection ordering plug-in; citations
in the C files.  Only tests/, the smoke check of __graft_entry__ and
bench.py's CPU-baseline leg and reference arm use it, as the checker; the
product never imports it, and it never loads the product's libraries.

``use_blas()`` routes the dense calls through the BLAS/LAPACK that scipy
bundles (OpenBLAS, threads = host cores), as the reference's Float64 path
does through libblastrampoline (src/SparseSpdMethod/SpkSpdMMOps.jl:222-351).

It is pinned against the reference's golden vectors in tests/golden/ (the
post-inmatrix! and post-factor! lnz/unz of the n=11 tridiagonal problem and
its intermediate forward-solve vector, the MMD permutation and the symbolic
arrays, test/test_sparse_method.jl).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRCS = [os.path.join(HERE, "spk_oracle.c"), os.path.join(HERE, "spk_oracle_struct.c")]
SO = os.path.join(HERE, "liboracle.so")
DUAL_SRC = os.path.join(HERE, "spk_oracle_dual.cpp")
DUAL_SO = os.path.join(HERE, "liboracle_dual.so")

_P = ctypes.POINTER(ctypes.c_int64)
_D = ctypes.POINTER(ctypes.c_double)
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (no FMA contraction, so every host gives the same bits)."""
    if force or not os.path.exists(SO) or any(os.path.getmtime(SO) < os.path.getmtime(f) for f in SRCS):
        cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-ffp-contract=off", "-o", SO] + SRCS + ["-lm"]
        subprocess.run(cmd, check=True, capture_output=True)
    if force or not os.path.exists(DUAL_SO) or os.path.getmtime(DUAL_SO) < os.path.getmtime(DUAL_SRC):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-o", DUAL_SO, DUAL_SRC]
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
        L.oracle_cholfactor.restype = i
        L.oracle_cholfactor.argtypes = [i, i, _P, _P, _P, _P, _P, _D]
        L.oracle_lu_begin.restype = ctypes.c_void_p
        L.oracle_lu_begin.argtypes = [i, i, _P, _P, _P, _P, _P, _D, _P, _D, _P]
        L.oracle_lu_run.restype = i
        L.oracle_lu_run.argtypes = [ctypes.c_void_p, i]
        L.oracle_lu_end.restype = i
        L.oracle_lu_end.argtypes = [ctypes.c_void_p, _P]
        L.oracle_lulsolve.restype = None
        L.oracle_lulsolve.argtypes = [i, _P, _P, _P, _P, _D, _P, _D]
        L.oracle_luusolve.restype = None
        L.oracle_luusolve.argtypes = [i, i, _P, _P, _P, _P, _D, _P, _D, _D]
        L.oracle_triangularsolve.restype = None
        L.oracle_triangularsolve.argtypes = [i, i, _P, _P, _P, _P, _D, _P, _D, _P, _P, _P, _D]
        vp = ctypes.c_void_p
        L.oracle_set_blas.restype = None
        L.oracle_set_blas.argtypes = [vp, vp, vp, vp, vp]
        L.oracle_blas_mode.restype = ctypes.c_int
        L.oracle_mmd.restype = None
        L.oracle_mmd.argtypes = [i, _P, _P, _P, _P]
        L.oracle_nd_graph.restype = i
        L.oracle_nd_graph.argtypes = [i, _P, _P, i, _P, _P]
        L.oracle_nd_grid.restype = i
        L.oracle_nd_grid.argtypes = [i, i, i, i, _P, _P, _P, _P]
        L.oracle_symbolic1.restype = i
        L.oracle_symbolic1.argtypes = [i, _P, _P, _P, _P, i, _P, _P, _P, _P, _P, _P]
        L.oracle_symbolic2.restype = i
        L.oracle_symbolic2.argtypes = [i, _P, _P, _P, _P, _P, i, _P, _P, _P, _P]
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

    def cholfactor(self) -> int:
        """Supernodal Cholesky of an SPD matrix on the same partition (after
        inmatrix_csc): lnz's lower parts receive C, A = C C^T.  Returns 0 or
        the 1-based column of the first non-positive pivot."""
        return int(lib().oracle_cholfactor(self.n, self.nsuper, _p(self.xsuper), _p(self.snode), _p(self.xlindx),
                                           _p(self.lindx), _p(self.xlnz), _d(self.lnz)))

    def lower_mask(self):
        """Boolean mask of the lnz entries on or below the diagonal (row t of
        supernode column k is on or below it when t >= k)."""
        m = np.zeros(self.lnz.shape[0], dtype=bool)
        for js in range(self.nsuper):
            f, l = int(self.xsuper[js]), int(self.xsuper[js + 1])
            jlen = int(self.xlindx[js + 1] - self.xlindx[js])
            for k in range(l - f):
                base = int(self.xlnz[f - 1 + k]) - 1
                m[base + k: base + jlen] = True
        return m

    def factor_slices(self, bounds):
        """_lufactor! run as consecutive slices of supernodes: bounds[k] is the
        last (1-based) supernode of slice k.  Yields after each slice (the
        caller times them); returns iflag like factor()."""
        L = lib()
        ctx = L.oracle_lu_begin(self.n, self.nsuper, _p(self.xsuper), _p(self.snode), _p(self.xlindx),
                                _p(self.lindx), _p(self.xlnz), _d(self.lnz), _p(self.xunz), _d(self.unz),
                                _p(self.ipiv))
        try:
            for js_end in bounds:
                L.oracle_lu_run(ctx, int(js_end))
                yield int(js_end)
        finally:
            fs = np.zeros(1, dtype=np.int64)
            self.iflag = int(L.oracle_lu_end(ctx, _p(fs)))
            self.first_singular = int(fs[0])

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


# ---------------------------------------------------------------------------
# BLAS mode
# ---------------------------------------------------------------------------

_blas_info = None


def use_blas(on: bool = True) -> dict | None:
    """Route the oracle's dense calls through scipy's BLAS/LAPACK (LP64
    Fortran interface, taken from scipy.linalg.cython_blas / cython_lapack),
    or back to the generic loops.  Returns a description of the library
    (name, threads) or None when switched off."""
    global _blas_info
    L = lib()
    if not on:
        L.oracle_set_blas(None, None, None, None, None)
        return None
    import scipy.linalg.cython_blas as cb
    import scipy.linalg.cython_lapack as cl

    get = ctypes.pythonapi.PyCapsule_GetPointer
    get.restype = ctypes.c_void_p
    get.argtypes = [ctypes.py_object, ctypes.c_char_p]
    getname = ctypes.pythonapi.PyCapsule_GetName
    getname.restype = ctypes.c_char_p
    getname.argtypes = [ctypes.py_object]

    def fn(mod, name):
        cap = mod.__pyx_capi__[name]
        return get(cap, getname(cap))

    L.oracle_set_blas(fn(cb, "dgemm"), fn(cb, "dtrsm"), fn(cl, "dgetrf"), fn(cl, "dlaswp"), fn(cb, "dgemv"))
    if _blas_info is None:
        _blas_info = {"library": "scipy-bundled BLAS", "threads": os.cpu_count()}
        try:
            import glob

            import scipy

            libs = glob.glob(os.path.join(os.path.dirname(scipy.__file__), os.pardir, "scipy.libs", "*openblas*"))
            if libs:
                ob = ctypes.CDLL(libs[0])
                _blas_info["library"] = "OpenBLAS (" + os.path.basename(libs[0]) + ")"
                for sym in ("scipy_openblas_get_num_threads", "openblas_get_num_threads"):
                    if hasattr(ob, sym):
                        f = getattr(ob, sym)
                        f.restype = ctypes.c_int
                        _blas_info["threads"] = int(f())
                        break
        except OSError:
            pass
    return dict(_blas_info)


# ---------------------------------------------------------------------------
# structure phase
# ---------------------------------------------------------------------------


class _Order:
    def __init__(self, rperm, rinvp):
        self.rperm, self.rinvp = rperm, rinvp


class OracleStructure:
    """What _symbolicfactor! leaves in a _SparseBase: n, nsuper, xsuper,
    snode, xlindx, lindx, xlnz, xunz, colcnt and order.rperm/rinvp (all
    1-based int64), computed by the oracle alone."""

    def __init__(self, n, perm, invp, colcnt, nsuper, xsuper, snode, xlindx, lindx, xlnz, xunz):
        self.n, self.nsuper = int(n), int(nsuper)
        self.order = _Order(perm, invp)
        self.colcnt, self.xsuper, self.snode = colcnt, xsuper, snode
        self.xlindx, self.lindx, self.xlnz, self.xunz = xlindx, lindx, xlnz, xunz


def graph_of(colptr, rowval, n):
    """Graph(m::SparseMatrixCSC) followed by makestructuresymmetric
    (src/SparseCSCInterface/SparseCSCInterface.jl:12-56,
    src/Graph/SpkGraph.jl:94-289): column lists without the diagonal; a
    structurally symmetric pattern is kept as stored, otherwise the lists
    become the sorted union of A's and A^T's."""
    colptr = np.asarray(colptr, np.int64)
    rowval = np.asarray(rowval, np.int64)
    cols = np.repeat(np.arange(1, n + 1, dtype=np.int64), np.diff(colptr))
    keep = rowval != cols
    r, c = rowval[keep], cols[keep]
    fwd = set(zip(r.tolist(), c.tolist())) if r.size < 2_000_000 else None
    if fwd is not None:
        sym = all((b, a) in fwd for a, b in fwd)
    else:
        key = np.sort(r * (n + 1) + c)
        key_t = np.sort(c * (n + 1) + r)
        sym = np.array_equal(key, key_t)
    if not sym:
        rr = np.concatenate([r, c])
        cc = np.concatenate([c, r])
        key = np.unique(cc * (n + 1) + rr)
        c, r = key // (n + 1), key % (n + 1)
    counts = np.bincount(c - 1, minlength=n)
    xadj = np.concatenate([[1], 1 + np.cumsum(counts)]).astype(np.int64)
    return xadj, np.ascontiguousarray(r, dtype=np.int64)


def mmd(xadj, adj, n):
    """_generalmmd: (perm, invp), 1-based."""
    perm = np.zeros(n, np.int64)
    invp = np.zeros(n, np.int64)
    lib().oracle_mmd(n, _p(xadj), _p(adj), _p(perm), _p(invp))
    return perm, invp


def nd_grid(xadj, adj, nx, ny, nz=1, leaf=64):
    """Grid nested dissection (the ordering plug-in), (perm, invp), 1-based."""
    n = nx * ny * nz
    perm = np.zeros(n, np.int64)
    invp = np.zeros(n, np.int64)
    got = lib().oracle_nd_grid(nx, ny, nz, leaf, _p(xadj), _p(adj), _p(perm), _p(invp))
    if got != n:
        raise ValueError(f"nested dissection ordered {got} of {n} vertices")
    return perm, invp


def nd_graph(xadj, adj, n, leaf=64):
    """General-graph nested dissection (the ordering plug-in), (perm, invp), 1-based."""
    perm = np.zeros(n, np.int64)
    invp = np.zeros(n, np.int64)
    got = lib().oracle_nd_graph(n, _p(xadj), _p(adj), leaf, _p(perm), _p(invp))
    if got != n:
        raise ValueError(f"nested dissection ordered {got} of {n} vertices")
    return perm, invp


def symbolic(xadj, adj, perm, invp, maxblocksize=30) -> OracleStructure:
    """_symbolicfactor! for the graph and an initial ordering."""
    n = int(xadj.shape[0] - 1)
    perm = np.ascontiguousarray(perm, np.int64).copy()
    invp = np.ascontiguousarray(invp, np.int64).copy()
    colcnt = np.zeros(n, np.int64)
    snode = np.zeros(n, np.int64)
    xsuper = np.zeros(n + 1, np.int64)
    xlnz = np.zeros(n + 1, np.int64)
    xunz = np.zeros(n + 1, np.int64)
    nsub = np.zeros(1, np.int64)
    L = lib()
    nsuper = int(L.oracle_symbolic1(n, _p(xadj), _p(adj), _p(perm), _p(invp), maxblocksize, _p(colcnt), _p(snode),
                                    _p(xsuper), _p(xlnz), _p(xunz), _p(nsub)))
    xsuper = xsuper[: nsuper + 1].copy()
    xlindx = np.zeros(nsuper + 1, np.int64)
    lindx = np.zeros(max(int(nsub[0]), 1), np.int64)
    rc = L.oracle_symbolic2(n, _p(xadj), _p(adj), _p(perm), _p(invp), _p(colcnt), nsuper, _p(xsuper), _p(snode),
                            _p(xlindx), _p(lindx))
    if rc != 0:
        raise ValueError("Inconsistency in data structure.")
    return OracleStructure(n, perm, invp, colcnt, nsuper, xsuper, snode, xlindx, lindx[: int(nsub[0])], xlnz, xunz)


def structure_csc(colptr, rowval, n, ordering="mmd", grid=None, leaf=64, maxblocksize=30) -> OracleStructure:
    """Ordering + symbolic factorisation of a CSC pattern (1-based colptr /
    rowval): ordering "mmd" (the reference default), "nd" (geometric, with
    grid = (nx, ny, nz)) or "nd_graph" (level-structure nested dissection)."""
    xadj, adj = graph_of(colptr, rowval, n)
    if ordering == "mmd":
        perm, invp = mmd(xadj, adj, n)
    elif ordering == "nd":
        nx, ny, nz = grid
        perm, invp = nd_grid(xadj, adj, nx, ny, nz, leaf)
    elif ordering == "nd_graph":
        perm, invp = nd_graph(xadj, adj, n, leaf)
    else:
        raise ValueError(ordering)
    return symbolic(xadj, adj, perm, invp, maxblocksize)


# ---------------------------------------------------------------------------
# forward-mode (Dual number) derivatives through the LU path
# ---------------------------------------------------------------------------

_dual = None


def dual_solve(sym, colptr, rowval, nzval, dnz, b):
    """x = A^{-1} b and dx/dp for A's values with partials dnz (nnz x k,
    k <= 16 directions), by the reference's LU path on Dual numbers
    (spk_oracle_dual.cpp).  sym: a structure (OracleStructure or the
    package's _SparseBase).  Returns (x, dx) with dx of shape n x k."""
    global _dual
    if _dual is None:
        build()
        L = ctypes.CDLL(DUAL_SO)
        i = ctypes.c_int64
        L.oracle_dual_solve.restype = i
        L.oracle_dual_solve.argtypes = [i, i, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _D, _D, _D, _D, _D]
        L.oracle_dual_partials.restype = ctypes.c_int
        _dual = L
    g = lambda a: np.ascontiguousarray(a, dtype=np.int64)
    n = int(sym.n)
    npart = _dual.oracle_dual_partials()
    dnz = np.asarray(dnz, np.float64)
    k = dnz.shape[1]
    if k > npart:
        raise ValueError(f"at most {npart} directions per call")
    dpad = np.zeros((dnz.shape[0], npart))
    dpad[:, :k] = dnz
    x = np.zeros(n)
    dx = np.zeros((n, npart))
    rc = _dual.oracle_dual_solve(n, int(sym.nsuper), _p(g(sym.xsuper)), _p(g(sym.snode)), _p(g(sym.xlindx)),
                                 _p(g(sym.lindx)), _p(g(sym.xlnz)), _p(g(sym.xunz)), _p(g(sym.order.rperm)),
                                 _p(g(sym.order.rinvp)), _p(g(colptr)), _p(g(rowval)),
                                 _d(np.ascontiguousarray(nzval, np.float64)), _d(dpad),
                                 _d(np.ascontiguousarray(b, np.float64)), _d(x), _d(dx))
    if rc != 0:
        raise ValueError(f"No space for matrix element at CSC position {-rc}")
    return x, dx[:, :k]

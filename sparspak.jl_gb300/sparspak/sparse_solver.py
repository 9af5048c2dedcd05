"""SpkSparseBase + SpkSparseSolver: the LU SparseSolver state machine.

Mirrors src/SparseMethod/SpkSparseBase.jl and SpkSparseSolver.jl.  The phase
functions check their predecessors and raise ``ErrorException`` with the
reference's "Sequence error" texts.  Ordering and symbolic factorisation run
on the host (libspk_host.so) and reproduce the reference's arrays exactly;
``inmatrix_``, ``factor_`` and ``triangularsolve_`` run on the GPU
(libspk_gpu.so) and have no CPU fallback.
"""
from __future__ import annotations

import ctypes

import numpy as np
import scipy.sparse as sp

from . import _native as N
from .device import ErrorException, NumericEngine, SingularException
from .graph import ETree, Graph, Ordering, makestructuresymmetric, mmd_
from .problem import Problem, csc_arrays


class _SparseBase:
    """Solver data (SpkSparseBase.jl:99-125); lnz/unz/ipiv are read from the device on access."""

    def __init__(self, p, maxblocksize: int = 30):
        if isinstance(p, Problem):
            self.n = p.nrows
            self.nnz = p.nnz
            self.g = Graph.from_problem(p)
        else:
            m = sp.csc_matrix(p)
            self.n = m.shape[1]
            self.nnz = m.nnz
            self.g = Graph.from_csc(m)
        self.maxblocksize = maxblocksize
        self.order = Ordering(self.n)
        self.t = ETree(self.n)
        self.errflag = 0
        self.nnzl = 0
        self.nsub = 0
        self.nsuper = 1 if self.n > 0 else 0
        e = np.zeros(0, dtype=np.int64)
        self.colcnt = self.snode = self.xsuper = self.xlindx = self.lindx = self.xlnz = self.xunz = e
        self.engine: NumericEngine | None = None
        self._pattern_key = None
        self.precision = "fp64"

    # factor arrays in the reference layout (copied back from the device)
    def _fetch(self):
        if self.engine is None:
            raise ErrorException("Sequence error. Matrix input not done yet.")
        nnzl = int(self.xlnz[-1] - 1)
        nnzu = int(self.xunz[-1] - 1)
        return self.engine.get_factors(nnzl, nnzu, self.precision)

    @property
    def lnz(self):
        return self._fetch()[0]

    @property
    def unz(self):
        return self._fetch()[1]

    @property
    def ipiv(self):
        return self._fetch()[2]


def _findorder_(s: _SparseBase, orderfunction=None) -> bool:
    if s.n == 0:
        raise ErrorException("An empty problem, no ordering found.")
    makestructuresymmetric(s.g)
    (orderfunction or mmd_)(s.g, s.order)
    return True


def _symbolicfactor_(s: _SparseBase) -> bool:
    """SpkSparseBase.jl:193-251 in libspk_host.so."""
    if s.n == 0:
        raise ErrorException("An empty problem. No symbolic factorization done.")
    lib = N.host()
    h = ctypes.c_void_p()
    rc = lib.spk_symbolic_create(s.n, N.p64(s.g.xadj), N.p64(s.g.adj), N.p64(s.order.rperm), N.p64(s.order.rinvp),
                                 s.maxblocksize, ctypes.byref(h))
    if rc < 0:
        raise ErrorException(N.host_error())
    try:
        ns, nsub, nl, nu = (np.zeros(1, np.int64) for _ in range(4))
        lib.spk_symbolic_sizes(h, N.p64(ns), N.p64(nsub), N.p64(nl), N.p64(nu))
        n, nsuper, nsb = s.n, int(ns[0]), int(nsub[0])
        arr = dict(perm=np.zeros(n, np.int64), invp=np.zeros(n, np.int64), parent=np.zeros(n, np.int64),
                   colcnt=np.zeros(n, np.int64), snode=np.zeros(n, np.int64), xsuper=np.zeros(nsuper + 1, np.int64),
                   xlindx=np.zeros(nsuper + 1, np.int64), lindx=np.zeros(max(nsb, 1), np.int64),
                   xlnz=np.zeros(n + 1, np.int64), xunz=np.zeros(n + 1, np.int64))
        lib.spk_symbolic_get(h, *[N.p64(arr[k]) for k in ("perm", "invp", "parent", "colcnt", "snode", "xsuper",
                                                            "xlindx", "lindx", "xlnz", "xunz")])
    finally:
        lib.spk_symbolic_destroy(h)
    s.order.rperm, s.order.rinvp = arr["perm"], arr["invp"]
    s.order.cperm, s.order.cinvp = s.order.rperm, s.order.rinvp
    s.t.parent = arr["parent"]
    s.colcnt, s.snode, s.xsuper = arr["colcnt"], arr["snode"], arr["xsuper"]
    s.xlindx, s.lindx = arr["xlindx"], arr["lindx"][:nsb]
    s.xlnz, s.xunz = arr["xlnz"], arr["xunz"]
    s.nsuper, s.nsub = nsuper, nsb
    if s.engine is not None:
        s.engine.close()
    s.engine = None
    s._pattern_key = None
    return True


def _ensure_engine(s: _SparseBase) -> NumericEngine:
    if s.engine is None:
        s.engine = NumericEngine(s.n, s.nsuper, s.xsuper, s.snode, s.xlindx, s.lindx, s.xlnz, s.xunz, index_base=1)
    return s.engine


def _matrix_arrays(p):
    """1-based (colptr, rowval, nzval) of a Problem or a CSC matrix."""
    if isinstance(p, Problem):
        return csc_arrays(p)
    m = sp.csc_matrix(p)
    if not m.has_sorted_indices:
        m = m.sorted_indices()
    return (m.indptr.astype(np.int64) + 1, m.indices.astype(np.int64) + 1, np.ascontiguousarray(m.data, np.float64))


def _inmatrix_(s: _SparseBase, p) -> bool:
    """Assemble A into the factor storage on the GPU (SpkSparseBase.jl:302-372)."""
    if s.n == 0:
        raise ErrorException("An empty problem. No matrix.")
    colptr, rowval, nzval = _matrix_arrays(p)
    eng = _ensure_engine(s)
    key = (colptr.tobytes(), rowval.tobytes())
    if key != s._pattern_key:
        eng.set_pattern(colptr, rowval, s.order.rperm, s.order.rinvp, index_base=1)
        s._pattern_key = key
    eng.load_values(nzval, s.precision)
    return True


def _factor_(s: _SparseBase) -> bool:
    """SpkSparseBase.jl:378-391 on the GPU; a zero pivot raises (naming the first bad supernode)."""
    if s.n == 0:
        raise ErrorException("An empty problem. No matrix.")
    try:
        s.engine.factor(s.precision)
        s.errflag = 0
    except SingularException as e:
        s.errflag = -1
        raise ErrorException(f"Zero pivot in the diagonal block of supernode {e.supernode}.") from e
    return True


def _triangularsolve_(s: _SparseBase, solution: np.ndarray) -> bool:
    """permute, L, U, unpermute (SpkSparseBase.jl:400-416) on the GPU, in place."""
    if s.n == 0:
        raise ErrorException("An empty problem. No solution.")
    s.engine.solve(solution, s.precision)
    return True


class SparseSolver:
    """SparseSolver(p::Problem) or SparseSolver(m::SparseMatrixCSC) - SpkSparseSolver.jl:17-73.

    ``precision`` ('fp64', 'fp32' or 'bf16s') selects the factor the numeric
    phases use; ``spd=True`` selects the symmetric form for symmetric positive
    definite matrices (Cholesky: no interchanges, half the update work; the
    role of the reference's SparseSpdSolver, src/SparseSpdMethod), whose
    factor reads back as the Cholesky factor C, A = C C^T.
    """

    def __init__(self, p, precision: str = "fp64", maxblocksize: int = 30, spd: bool = False):
        if isinstance(p, Problem):
            self.ma, self.na = p.nrows, p.ncols
        else:
            p = sp.csc_matrix(p)
            self.ma, self.na = p.shape[1], p.shape[0]
        self.p = p
        self.n = self.ma
        self.mc = self.nc = 0
        self.slvr = _SparseBase(p, maxblocksize)
        self.spd = bool(spd)
        self.slvr.precision = _form(precision, self.spd)
        self._orderdone = self._symbolicdone = self._inmatrixdone = False
        self._factordone = self._trisolvedone = self._refinedone = self._condestdone = False

    def copy_from(self, src: "SparseSolver") -> "SparseSolver":
        self.__dict__.update(src.__dict__)
        return self


def findorder_(s: SparseSolver, orderfunction=None) -> bool:
    """SpkSparseSolver.jl:102-131: a no-op once done; invalidates the symbolic phase."""
    if s._orderdone:
        return True
    _findorder_(s.slvr, orderfunction)
    s._orderdone = True
    s._symbolicdone = False
    return True


def findorderperm_(s: SparseSolver, perm) -> bool:
    """Use a given permutation (SpkSparseSolver.jl:143-151; the reference passes the vector
    where a function is expected, here it is installed directly)."""
    if s._orderdone:
        return True
    if s.slvr.n == 0:
        raise ErrorException("An empty problem, no ordering found.")
    makestructuresymmetric(s.slvr.g)
    s.slvr.order.set(perm)
    s._orderdone = True
    s._symbolicdone = False
    return True


def symbolicfactor_(s: SparseSolver) -> bool:
    if s._symbolicdone:
        return True
    if not s._orderdone:
        raise ErrorException("Sequence error. Ordering not done yet.")
    _symbolicfactor_(s.slvr)
    s._symbolicdone = True
    s._inmatrixdone = False
    return True


def inmatrix_(s: SparseSolver) -> bool:
    if s._inmatrixdone:
        return True
    if not s._symbolicdone:
        raise ErrorException("Sequence error. Symbolic factor not done yet.")
    ok = _inmatrix_(s.slvr, s.p)
    s._inmatrixdone = True
    s._factordone = False
    return ok


def factor_(s: SparseSolver) -> bool:
    if s._factordone:
        return True
    if not s._inmatrixdone:
        raise ErrorException("Sequence error. Matrix input not done yet.")
    s._trisolvedone = False
    _factor_(s.slvr)
    if s.slvr.errflag == 0:
        s._factordone = True
        return True
    return False


def triangularsolve_(s: SparseSolver, rhs=None) -> bool:
    """Without rhs: solve for p.rhs into p.x (SpkSparseSolver.jl:237-256); with rhs: in place (:266-275)."""
    if rhs is None:
        if s._trisolvedone:
            return True
        if not s._factordone:
            raise ErrorException("Sequence error. Factorization not done yet.")
        temp = np.array(s.p.rhs[: s.p.nrows], dtype=np.float64)
        triangularsolve_(s, temp)
        s.p.x[: temp.shape[0]] = temp
        s._trisolvedone = True
        s._refinedone = False
        return True
    if not s._factordone:
        raise ErrorException("Sequence error. Factorization not done yet.")
    _triangularsolve_(s.slvr, rhs)
    s._trisolvedone = True
    s._refinedone = False
    return True


def transposetriangularsolve_(s: SparseSolver, rhs) -> bool:
    """Solve A^T x = rhs in place with the factors of A (the reference's
    `transposetriangularsolve` is commented out, SpkSparseSpdSolver.jl:384)."""
    if not s._factordone:
        raise ErrorException("Sequence error. Factorization not done yet.")
    if s.slvr.n == 0:
        raise ErrorException("An empty problem. No solution.")
    s.slvr.engine.solve(rhs, s.slvr.precision, transpose=True)
    return True


def solve_(s: SparseSolver, rhs=None) -> bool:
    """All phases (SpkSparseSolver.jl:80-87; with rhs, SparseCSCInterface.jl:194-201)."""
    findorder_(s) or _fail("Finding Order.")
    symbolicfactor_(s) or _fail("Symbolic Factorization.")
    inmatrix_(s) or _fail("Matrix input.")
    factor_(s) or _fail("Numerical Factorization.")
    triangularsolve_(s, rhs) or _fail("Triangular Solve.")
    return True


def _form(precision: str, spd: bool) -> str:
    precision = precision.lower()
    return precision + "+spd" if spd and "+spd" not in precision else precision


def refine_(s: SparseSolver, b: np.ndarray, x: np.ndarray | None = None, precision: str = "fp32", tol: float = 1e-12,
            max_iter: int = 20, transpose: bool = False, solver: str | None = None):
    """Mixed-precision solve: factor in `precision` ('fp32', 'bf16s' or
    'fp64'; if not yet), then FP64 iterative refinement - plain, or GMRES-IR
    once plain refinement stagnates (solver 'auto'), or as chosen ('ir',
    'gmres').

    Returns (x, preconditioned solves after the first, relative residual),
    plus the solver used when `solver` is given.  New in this engine; the
    reference's refinement exists only as a commented-out Fortran
    translation (SpkSparseSpdSolver.jl:267-343).
    """
    findorder_(s)
    symbolicfactor_(s)
    precision = _form(precision, getattr(s, "spd", False))
    if s.slvr.precision != precision or not s._factordone:
        s.slvr.precision = precision
        s._inmatrixdone = False
        inmatrix_(s)
        factor_(s)
    b = np.asfortranarray(b, dtype=np.float64)
    x = np.zeros_like(b) if x is None else x
    out = s.slvr.engine.refine(b, x, precision, tol, max_iter, transpose=transpose, solver=solver)
    return (x,) + tuple(out)


def gradient_(s: SparseSolver, lam: np.ndarray, x: np.ndarray) -> np.ndarray:
    """dloss/dA on A's pattern (CSC order of the matrix given to the solver),
    -sum_r lam_r x_r^T, for lam = A^{-T} dloss/dx (adjoint of x = A^{-1} b)."""
    if not s._inmatrixdone:
        raise ErrorException("Sequence error. Matrix input not done yet.")
    lam = np.asfortranarray(lam, dtype=np.float64)
    x = np.asfortranarray(x, dtype=np.float64)
    return s.slvr.engine.grad_pattern(lam, x)


def _fail(msg):
    raise ErrorException(msg)

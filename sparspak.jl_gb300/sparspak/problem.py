"""SpkProblem: the reference's sparse problem container.

Mirrors src/Problem/SpkProblem.jl: a matrix entered entry by entry with
``inaij_`` (values are *added* to what is there, SpkProblem.jl:177-251), a
right-hand side entered with ``inbi_``/``infullrhs_``, and the solution
``x``.  Julia's mutating ``f!`` is spelled ``f_`` here.  Columns keep their
rows in increasing order, as the reference's linked lists do.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

BIGGY = float("inf")  # typemax(Float64), the "no value" sentinel (src/Utilities/SpkUtilities.jl:7)


class Problem:
    """Problem(nrows, ncols, nnz=2500, z=0.0, info="") - SpkProblem.jl:140-163."""

    def __init__(self, nrows: int, ncols: int, nnz: int = 2500, z: float = 0.0, info: str = ""):
        self.info = info
        self.nrows = int(nrows)
        self.ncols = int(ncols)
        self.nnz = 0          # number of nonzero values
        self.dnz = 0          # ... on the diagonal
        self.nedges = 0       # number of stored positions
        self.dedges = 0       # ... on the diagonal
        self.dtype = np.asarray(z).dtype if not isinstance(z, float) else np.float64
        self._cols: list[dict[int, float]] = [dict() for _ in range(self.ncols)]
        self.rhs = np.zeros(self.nrows, dtype=np.float64)
        self.x = np.zeros(self.ncols, dtype=np.float64)

    # -- growth --------------------------------------------------------------
    def _grow(self, nrows: int, ncols: int):
        if ncols > len(self._cols):
            self._cols.extend(dict() for _ in range(ncols - len(self._cols)))
        if ncols > self.x.shape[0]:
            self.x = np.concatenate([self.x, np.zeros(ncols - self.x.shape[0])])
        if nrows > self.rhs.shape[0]:
            self.rhs = np.concatenate([self.rhs, np.zeros(nrows - self.rhs.shape[0])])
        self.nrows = max(self.nrows, nrows)
        self.ncols = max(self.ncols, ncols)

    def column(self, j: int):
        """Sorted (rows, values) of 1-based column j."""
        d = self._cols[j - 1]
        rows = sorted(d)
        return rows, [d[r] for r in rows]


def inaij_(p: Problem, rnum: int, cnum: int, aij: float = 0.0) -> bool:
    """Add aij to entry (rnum, cnum) - SpkProblem.jl:177-251."""
    if rnum < 1 or cnum < 1:
        import warnings

        warnings.warn(f"invalid matrix subscripts {rnum}, {cnum}: input ignored")
        return False
    p._grow(rnum, cnum)
    col = p._cols[cnum - 1]
    if rnum in col:
        if col[rnum] == BIGGY:
            p.nnz += 1
            col[rnum] = float(aij)
            if rnum == cnum:
                p.dnz += 1
        else:
            col[rnum] += aij
        return True
    col[rnum] = float(aij)
    p.nedges += 1
    p.nnz += 1
    if rnum == cnum:
        p.dedges += 1
        p.dnz += 1
    return True


def inbi_(p: Problem, rnum: int, bi: float) -> bool:
    """Add bi to rhs[rnum] - SpkProblem.jl:258-271."""
    if rnum < 1:
        from .device import ErrorException

        raise ErrorException(f"Invalid rhs subscript {rnum}.")
    p._grow(rnum, p.ncols)
    p.rhs[rnum - 1] += bi
    return True


def insparse_(p: Problem, I, J=None, V=None) -> bool:
    """insparse!(p, spm) or insparse!(p, I, J, V) - SpkProblem.jl:278-297."""
    if J is None:
        m = sp.coo_matrix(I)
        I, J, V = m.row + 1, m.col + 1, m.data
    for i, j, v in zip(np.asarray(I), np.asarray(J), np.asarray(V)):
        if not inaij_(p, int(i), int(j), float(v)):
            return False
    return True


def outsparse(p: Problem) -> sp.csc_matrix:
    """The matrix as scipy CSC (0-based), entries with row <= nrows - SpkProblem.jl:304-324."""
    rows, cols, vals = [], [], []
    for j in range(p.ncols):
        for r, v in sorted(p._cols[j].items()):
            if r <= p.nrows:
                rows.append(r - 1)
                cols.append(j)
                vals.append(v)
    m = sp.csc_matrix((np.array(vals, dtype=np.float64), (np.array(rows, dtype=np.int64), np.array(cols, dtype=np.int64))),
                      shape=(p.nrows, p.ncols))
    m.sort_indices()
    return m


def csc_arrays(p: Problem):
    """(colptr, rowval, nzval) of the problem, 1-based indices, rows sorted per column."""
    colptr = np.zeros(p.ncols + 1, dtype=np.int64)
    rowval, nzval = [], []
    colptr[0] = 1
    for j in range(p.ncols):
        items = sorted(p._cols[j].items())
        rowval.extend(r for r, _ in items)
        nzval.extend(v for _, v in items)
        colptr[j + 1] = colptr[j] + len(items)
    return colptr, np.array(rowval, dtype=np.int64), np.array(nzval, dtype=np.float64)


def infullrhs_(p: Problem, rhs) -> Problem:
    """Add rhs[1:nrows] to the right-hand side - SpkProblem.jl:508-513."""
    rhs = np.asarray(rhs, dtype=np.float64)
    for i in range(p.nrows, 0, -1):
        inbi_(p, i, float(rhs[i - 1]))
    return p


def zerorhs_(p: Problem) -> Problem:
    p.rhs[:] = 0.0
    return p


def computeresidual(p: Problem, res: np.ndarray, xin=None, mtype: str = "T") -> bool:
    """res = rhs - A x (host, FP64), honouring triangle-only storage - SpkProblem.jl:448-496.

    The reference reads ``p.x`` when ``xin`` is given and ``xin`` when it is
    empty (its test is inverted); here ``xin`` is used when given, else ``p.x``.
    """
    if mtype.lower() not in ("t", "l", "u"):
        from .device import ErrorException

        raise ErrorException(f"Invalid value for mtype, {mtype}.")
    x = p.x if xin is None or len(xin) == 0 else np.asarray(xin, dtype=np.float64)
    r = p.rhs[: p.nrows].copy()
    for c in range(p.ncols):
        t = x[c]
        for rnum, v in p._cols[c].items():
            if v != BIGGY:
                r[rnum - 1] -= t * v
                if rnum - 1 != c:
                    r[c] -= x[rnum - 1] * v
    res[: p.nrows] = r
    return True


def makerhs_(p: Problem, x=None, mtype: str = "T") -> Problem:
    """rhs = A x for x (default 1..n), via computeresidual - SpkProblem.jl:402-423."""
    if p.nnz == 0:
        from .device import ErrorException

        raise ErrorException("Matrix is NULL. The rhs cannot be computed.")
    xx = np.arange(1, p.ncols + 1, dtype=np.float64) if x is None or len(x) == 0 else np.asarray(x, np.float64)
    p.x[: p.ncols] = xx
    p.rhs[:] = 0.0
    res = np.zeros_like(p.rhs)
    computeresidual(p, res, p.x, mtype)
    p.rhs[:] = -res
    p.x[:] = 0.0
    return p


class Grid:
    """SpkGrid.Grid(h, k): v[i, j] = k(i-1) + j (src/Grid/SpkGrid.jl:19-28)."""

    def __init__(self, h: int, k: int):
        self.h, self.k = h, k
        self.v = np.array([[k * (i - 1) + j for j in range(1, k + 1)] for i in range(1, h + 1)], dtype=np.int64)


def makegridproblem(h, k=None) -> Problem:
    """The reference's grid problem (SpkProblem.jl:340-379): diagonal 4 entered twice, lower couplings only."""
    g = h if isinstance(h, Grid) else Grid(h, k)
    n = g.h * g.k
    p = Problem(n, n)
    v = g.v
    for i in range(1, g.h + 1):
        for j in range(1, g.k + 1):
            inaij_(p, v[i - 1, j - 1], v[i - 1, j - 1], 4.0)
            if i > 1:
                inaij_(p, v[i - 1, j - 1], v[i - 2, j - 1], -1.0)
            if j > 1:
                inaij_(p, v[i - 1, j - 1], v[i - 1, j - 2], -1.0)
    for i in range(1, g.h + 1):
        for j in range(1, g.k + 1):
            inaij_(p, v[i - 1, j - 1], v[i - 1, j - 1], 4.0)
            if i > 1 and j > 1:
                inaij_(p, v[i - 1, j - 1], v[i - 2, j - 2], -1.0)
            if j < g.k and i > 1:
                inaij_(p, v[i - 1, j - 1], v[i - 2, j], -1.0)
    return p

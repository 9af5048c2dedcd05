"""SpkGraph and SpkOrdering: adjacency graphs, orderings and the ETree holder.

Mirrors src/Graph/SpkGraph.jl, src/Ordering/SpkOrdering.jl and
src/ETree/SpkETree.jl.  Adjacency arrays are 1-based int64, as in the
reference; the heavy lifting (symmetrisation, minimum degree, nested
dissection) runs in libspk_host.so.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from . import _native as N


class Graph:
    """Graph{IT}: nv vertices, 1-based (xadj, adj) without self loops."""

    def __init__(self, nv, nedges, nrows, ncols, xadj, adj):
        self.nv, self.nedges, self.nrows, self.ncols = int(nv), int(nedges), int(nrows), int(ncols)
        self.xadj = np.ascontiguousarray(xadj, dtype=np.int64)
        self.adj = np.ascontiguousarray(adj, dtype=np.int64)

    @classmethod
    def from_problem(cls, p, diagonal: bool = False) -> "Graph":
        """Graph(p::Problem) - SpkGraph.jl:58-87: column lists, rows in increasing order."""
        xadj = np.zeros(p.ncols + 1, dtype=np.int64)
        adj = []
        xadj[0] = 1
        for i in range(1, p.ncols + 1):
            rows, _ = p.column(i)
            for j in rows:
                if j != i or diagonal:
                    adj.append(j)
            xadj[i] = len(adj) + 1
        return cls(p.ncols, len(adj), p.nrows, p.ncols, xadj, np.array(adj, dtype=np.int64))

    @classmethod
    def from_csc(cls, m, diagonal: bool = False) -> "Graph":
        """Graph(m::SparseMatrixCSC) - SparseCSCInterface.jl:12-56 (rows in stored order)."""
        m = sp.csc_matrix(m)
        n = m.shape[1]
        indptr, indices = m.indptr.astype(np.int64), m.indices.astype(np.int64)
        cols = np.repeat(np.arange(n, dtype=np.int64), np.diff(indptr))
        keep = np.ones(indices.shape[0], dtype=bool) if diagonal else indices != cols
        counts = np.bincount(cols[keep], minlength=n)
        xadj = np.concatenate([[1], 1 + np.cumsum(counts)]).astype(np.int64)
        adj = (indices[keep] + 1).astype(np.int64)
        return cls(m.shape[0], adj.shape[0], m.shape[1], m.shape[0], xadj, adj)


def isstructuresymmetric(g: Graph) -> bool:
    rc = N.host().spk_graph_is_symmetric(g.nv, N.p64(g.xadj), N.p64(g.adj))
    if rc < 0:
        raise ValueError(N.host_error())
    return rc == 1


def makestructuresymmetric(g: Graph) -> bool:
    """Symmetrise in place; lists end up sorted (SpkGraph.jl:94-268 + sortgraph!)."""
    lib = N.host()
    ne = np.zeros(1, dtype=np.int64)
    rc = lib.spk_graph_symmetrize(g.nv, N.p64(g.xadj), N.p64(g.adj), N.p64(ne), None, None)
    if rc < 0:
        raise ValueError(N.host_error())
    xadj = np.zeros(g.nv + 1, dtype=np.int64)
    adj = np.zeros(max(int(ne[0]), 1), dtype=np.int64)
    rc = lib.spk_graph_symmetrize(g.nv, N.p64(g.xadj), N.p64(g.adj), N.p64(ne), N.p64(xadj), N.p64(adj))
    if rc < 0:
        raise ValueError(N.host_error())
    g.xadj, g.adj, g.nedges = xadj, adj[: int(ne[0])], int(ne[0])
    return True


class Ordering:
    """Ordering(nrows[, ncols]) with identity permutations (SpkOrdering.jl:92-126).

    rperm[i] = k: original row k is in position i; rinvp[rperm[i]] = i.
    """

    def __init__(self, nrows: int, ncols: int | None = None):
        ncols = nrows if ncols is None else ncols
        self.nrows, self.ncols = int(nrows), int(ncols)
        self.nrowblks = self.ncolblks = 0
        self.rperm = np.arange(1, nrows + 1, dtype=np.int64)
        self.rinvp = self.rperm.copy()
        self.cperm = np.arange(1, ncols + 1, dtype=np.int64)
        self.cinvp = self.cperm.copy()
        self.xrowblk = np.zeros(0, dtype=np.int64)
        self.xcolblk = np.zeros(0, dtype=np.int64)

    def set(self, perm):
        perm = np.ascontiguousarray(perm, dtype=np.int64)
        n = perm.shape[0]
        if sorted(perm.tolist()) != list(range(1, n + 1)):
            raise ValueError("not a 1-based permutation")
        self.rperm = perm.copy()
        self.rinvp = np.empty(n, dtype=np.int64)
        self.rinvp[perm - 1] = np.arange(1, n + 1)
        self.cperm, self.cinvp = self.rperm.copy(), self.rinvp.copy()


class ETree:
    """ETree(nv): parent vector (0 = root) - SpkETree.jl:17-34."""

    def __init__(self, nv: int):
        self.nv = int(nv)
        self.parent = np.zeros(nv, dtype=np.int64)


def mmd_(g: Graph, order: Ordering) -> None:
    """Multiple minimum degree ordering (SpkMMD.jl:38-42); the graph must be symmetric."""
    perm = np.zeros(g.nv, dtype=np.int64)
    invp = np.zeros(g.nv, dtype=np.int64)
    rc = N.host().spk_order_mmd(g.nv, N.p64(g.xadj), N.p64(g.adj), N.p64(perm), N.p64(invp))
    if rc < 0:
        raise ValueError(N.host_error())
    order.rperm, order.rinvp = perm, invp
    order.cperm, order.cinvp = perm.copy(), invp.copy()


def nd_grid(nx: int, ny: int, nz: int = 1, leaf: int = 64):
    """Order function for an nx x ny x nz grid numbered i-slowest (SpkGrid.jl:24 in 2-D).

    Returns ``f(g, order)`` for findorder_: geometric nested dissection with
    separator planes last and minimum degree inside boxes of <= leaf vertices.
    """

    def orderfunction(g: Graph, order: Ordering) -> None:
        if g.nv != nx * ny * nz:
            raise ValueError(f"graph has {g.nv} vertices, grid has {nx * ny * nz}")
        perm = np.zeros(g.nv, dtype=np.int64)
        invp = np.zeros(g.nv, dtype=np.int64)
        rc = N.host().spk_order_nd_grid(nx, ny, nz, leaf, N.p64(g.xadj), N.p64(g.adj), N.p64(perm), N.p64(invp))
        if rc < 0:
            raise ValueError(N.host_error())
        order.rperm, order.rinvp = perm, invp
        order.cperm, order.cinvp = perm.copy(), invp.copy()

    return orderfunction


def nd_graph(leaf: int = 64):
    """Order function for any symmetric graph: nested dissection by
    level-structure separators (pseudo-peripheral roots, middle level,
    separators last), minimum degree inside sets of <= leaf vertices."""

    def orderfunction(g: Graph, order: Ordering) -> None:
        perm = np.zeros(g.nv, dtype=np.int64)
        invp = np.zeros(g.nv, dtype=np.int64)
        rc = N.host().spk_order_nd_graph(g.nv, N.p64(g.xadj), N.p64(g.adj), leaf, N.p64(perm), N.p64(invp))
        if rc < 0:
            raise ValueError(N.host_error())
        order.rperm, order.rinvp = perm, invp
        order.cperm, order.cinvp = perm.copy(), invp.copy()

    return orderfunction


def nd_grid_batched(sizes, leaf: int = 64):
    """Order function for the block-diagonal union of square grids (system k:
    sizes[k] x sizes[k] vertices, consecutive): nested dissection of every
    grid on its own, the systems kept in order.  The union's elimination
    forest then has one tree per system, which the numeric phase factors
    together level by level."""
    sizes = [int(s) for s in sizes]

    def orderfunction(g: Graph, order: Ordering) -> None:
        total = sum(s * s for s in sizes)
        if g.nv != total:
            raise ValueError(f"graph has {g.nv} vertices, the systems {total}")
        perm = np.zeros(g.nv, dtype=np.int64)
        invp = np.zeros(g.nv, dtype=np.int64)
        off = 0
        for s in sizes:
            nv = s * s
            lo, hi = g.xadj[off] - 1, g.xadj[off + nv] - 1        # adjacency of the system (1-based)
            xadj = g.xadj[off: off + nv + 1] - lo
            adj = g.adj[lo:hi] - off
            if adj.size and (adj.min() < 1 or adj.max() > nv):
                raise ValueError("the systems are not independent blocks")
            xadj = np.ascontiguousarray(xadj, dtype=np.int64)
            adj = np.ascontiguousarray(adj if adj.size else np.zeros(1, np.int64), dtype=np.int64)
            p = np.zeros(nv, dtype=np.int64)
            q = np.zeros(nv, dtype=np.int64)
            rc = N.host().spk_order_nd_grid(s, s, 1, leaf, N.p64(xadj), N.p64(adj), N.p64(p), N.p64(q))
            if rc < 0:
                raise ValueError(N.host_error())
            perm[off: off + nv] = p + off
            invp[off: off + nv] = q + off
            off += nv
        order.rperm, order.rinvp = perm, invp
        order.cperm, order.cinvp = perm.copy(), invp.copy()

    return orderfunction


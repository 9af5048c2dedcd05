"""Seeded synthetic matrices for the benchmark configurations.

Grids are numbered with the first index slowest, v(i, j[, k]) as SpkGrid
(src/Grid/SpkGrid.jl:24) does in 2-D.  All builders return scipy CSC
matrices with sorted indices (the layout SparseCSCInterface expects).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def _ids(shape):
    return np.arange(int(np.prod(shape)), dtype=np.int64).reshape(shape)


def _assemble(n, rows, cols, vals):
    m = sp.coo_matrix((vals, (rows, cols)), shape=(n, n)).tocsc()
    m.sum_duplicates()
    m.sort_indices()
    return m


def laplacian(shape, diag=None, shift=0.0):
    """Dirichlet Laplacian on a 2-D (5-point) or 3-D (7-point) grid: diag 2d (+shift), off -1."""
    shape = tuple(int(s) for s in shape)
    d = len(shape)
    ids = _ids(shape)
    n = ids.size
    rows, cols, vals = [ids.ravel()], [ids.ravel()], [np.full(n, (2.0 * d if diag is None else diag) + shift)]
    for ax in range(d):
        a = np.take(ids, range(0, shape[ax] - 1), axis=ax).ravel()
        b = np.take(ids, range(1, shape[ax]), axis=ax).ravel()
        rows += [a, b]
        cols += [b, a]
        vals += [np.full(a.size, -1.0), np.full(a.size, -1.0)]
    return _assemble(n, np.concatenate(rows), np.concatenate(cols), np.concatenate(vals))


def convection_diffusion(k=48, velocity=(1.0, 0.5, 0.25), peclet=10.0):
    """First-order upwind convection-diffusion on the unit cube, k^3 interior points, Dirichlet.

    eps chosen so that the global Peclet number |v|_inf * L / eps equals `peclet`
    (L = 1); the operator is -eps*Lap(u) + v.grad(u), scaled by h^2/eps.
    Structurally symmetric, unsymmetric values, an M-matrix.
    """
    h = 1.0 / (k + 1)
    v = np.asarray(velocity, dtype=np.float64)
    eps = np.max(np.abs(v)) / peclet
    shape = (k, k, k)
    ids = _ids(shape)
    n = ids.size
    c = h / eps                                   # cell Peclet scale
    diag = 6.0 + c * np.sum(np.abs(v))
    rows, cols, vals = [ids.ravel()], [ids.ravel()], [np.full(n, diag)]
    for ax in range(3):
        a = np.take(ids, range(0, k - 1), axis=ax).ravel()   # lower neighbour
        b = np.take(ids, range(1, k), axis=ax).ravel()       # upper neighbour
        up = -1.0 - c * max(v[ax], 0.0)    # coupling of a node to its lower neighbour (upwind for v>0)
        dn = -1.0 - c * max(-v[ax], 0.0)   # coupling to its upper neighbour
        rows += [b, a]
        cols += [a, b]
        vals += [np.full(a.size, up), np.full(a.size, dn)]
    return _assemble(n, np.concatenate(rows), np.concatenate(cols), np.concatenate(vals))


def diffusion_2d(s, theta_h, theta_v, theta_d1=None, theta_d2=None):
    """Weighted graph Laplacian of an s x s grid plus Dirichlet boundary terms.

    theta_h[i, j] couples (i, j)-(i, j+1) (shape s x (s+1), columns 0 and s are
    the boundary edges), theta_v[i, j] couples (i, j)-(i+1, j) (shape (s+1) x s).
    Optional diagonal conductivities (9-point stencil): theta_d1 couples
    (i, j)-(i+1, j+1), theta_d2 couples (i, j)-(i+1, j-1), shapes (s+1) x (s+1).
    Out-of-grid neighbours add their conductivity to the diagonal only.
    """
    ids = np.full((s + 2, s + 2), -1, dtype=np.int64)
    ids[1:-1, 1:-1] = _ids((s, s))
    n = s * s
    diag = np.zeros(n)
    rows, cols, vals = [], [], []

    def couple(a, b, w):
        a, b, w = a.ravel(), b.ravel(), w.ravel()
        ia, ib = a >= 0, b >= 0
        np.add.at(diag, a[ia], w[ia])
        np.add.at(diag, b[ib], w[ib])
        both = ia & ib
        rows.extend([a[both], b[both]])
        cols.extend([b[both], a[both]])
        vals.extend([-w[both], -w[both]])

    couple(ids[1:-1, 0:-1], ids[1:-1, 1:], theta_h)
    couple(ids[0:-1, 1:-1], ids[1:, 1:-1], theta_v)
    if theta_d1 is not None:
        couple(ids[0:-1, 0:-1], ids[1:, 1:], theta_d1)
    if theta_d2 is not None:
        couple(ids[0:-1, 1:], ids[1:, 0:-1], theta_d2)
    rows.append(np.arange(n))
    cols.append(np.arange(n))
    vals.append(diag)
    return _assemble(n, np.concatenate(rows), np.concatenate(cols), np.concatenate(vals))


def batched_diffusion(nsys=512, smin=20, smax=120, seed=0):
    """Block-diagonal union of `nsys` independent SPD systems: system k is the
    9-point (8-neighbour) weighted graph Laplacian of an s_k x s_k grid,
    s_k ~ U{smin..smax}, edge conductivities ~ lognormal(0, 1), Dirichlet
    boundary terms (out-of-grid neighbours add their conductivity to the
    diagonal).  Returns (A, sizes) with A scipy CSC and the systems in order.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = rng.integers(smin, smax + 1, size=nsys)
    blocks = []
    for s in sizes:
        s = int(s)
        th = rng.lognormal(0.0, 1.0, size=(s, s + 1))
        tv = rng.lognormal(0.0, 1.0, size=(s + 1, s))
        t1 = rng.lognormal(0.0, 1.0, size=(s + 1, s + 1))
        t2 = rng.lognormal(0.0, 1.0, size=(s + 1, s + 1))
        blocks.append(diffusion_2d(s, th, tv, t1, t2))
    A = sp.block_diag(blocks, format="csc")
    A.sort_indices()
    return A, [int(s) for s in sizes]


def random_rhs(n, nrhs=1, seed=0):
    """Entries i.i.d. uniform[-1, 1] from numpy PCG64(seed); column-major n x nrhs."""
    rng = np.random.Generator(np.random.PCG64(seed))
    b = rng.uniform(-1.0, 1.0, size=(nrhs, n)).T
    return np.asfortranarray(b) if nrhs > 1 else np.ascontiguousarray(b[:, 0])

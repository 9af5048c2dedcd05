"""Independent check of the symbolic phase: the factor structure produced by
libspk_host.so equals the structure of a brute-force symbolic elimination
(set unions in the final ordering) on random structurally symmetric graphs."""
import numpy as np
import pytest
import scipy.sparse as sp

import sparspak as S
from cases import sprand_spd_like


def brute_force_structure(A, perm):
    """Row sets of the columns of L for P A P' (0-based, diagonal included)."""
    n = A.shape[0]
    B = sp.csc_matrix(A)[perm - 1][:, perm - 1]
    B = (abs(B) + abs(B.T)).tocsc()
    cols = [set(B.indices[B.indptr[j]:B.indptr[j + 1]][B.indices[B.indptr[j]:B.indptr[j + 1]] >= j]) | {j}
            for j in range(n)]
    for j in range(n):
        below = sorted(i for i in cols[j] if i > j)
        if below:
            cols[below[0]] |= set(i for i in below)
    return cols


@pytest.mark.parametrize("n,seed,ordering", [(60, 0, "mmd"), (200, 1, "mmd"), (300, 2, "mmd"), (125, 3, "nd")])
def test_structure_matches_elimination(n, seed, ordering):
    if ordering == "nd":
        A = S.gallery.laplacian((5, 5, 5))
        of = S.nd_grid(5, 5, 5, leaf=4)
    else:
        A = sprand_spd_like(n, seed)
        of = None
    s = S.SparseSolver(A)
    S.findorder_(s, of)
    S.symbolicfactor_(s)
    b = s.slvr
    cols = brute_force_structure(A, b.order.rperm)
    for k in range(b.nsuper):
        f, l = b.xsuper[k] - 1, b.xsuper[k + 1] - 1
        rows = (b.lindx[b.xlindx[k] - 1:b.xlindx[k + 1] - 1] - 1).tolist()
        assert rows == sorted(cols[f]), k
        for j in range(f, l):
            assert b.colcnt[j] == len(cols[j])
            assert b.xlnz[j + 1] - b.xlnz[j] == len(rows)

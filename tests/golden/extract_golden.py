"""Extract the reference's own golden vectors into reference_vectors.json.

Reads the reference package's test files *as text* (Julia cannot run here)
and pulls out the literal arrays the tests assert against.  Run from the
repository root with the path of a checkout of the reference as the
argument (or in the REFERENCE environment variable):
    python tests/golden/extract_golden.py <path-to-Sparspak.jl>
The JSON it writes is committed; the tests never read the reference.
"""
import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFERENCE")
if not REF:
    sys.exit("usage: extract_golden.py <path-to-Sparspak.jl>  (or set REFERENCE)")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_vectors.json")


def read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def nums(s):
    """All numbers in a Julia array literal (row vectors, column vectors, matrices)."""
    return [float(x) if any(c in x for c in ".eE") else int(x)
            for x in re.findall(r"-?\d+\.?\d*(?:[eE][-+]?\d+)?", s)]


def between(text, start, end, after=0):
    i = text.index(start, after) + len(start)
    j = text.index(end, i)
    return text[i:j], j


def main():
    t = read("test/test_sparse_method.jl")
    g = {}
    # msprs003: MMD ordering of the n = 11 tridiagonal problem
    s, _ = between(t, "@test o.rperm == vec(", ")")
    g["tridiag11_rperm"] = nums(s)
    s, _ = between(t, "@test o.rinvp == vec(", ")")
    g["tridiag11_rinvp"] = nums(s)
    # msprs004: symbolic arrays
    s, k = between(t, "@test s.slvr.xlnz == ", "\n")
    g["tridiag11_xlnz"] = nums(s)
    s, _ = between(t, "@test s.slvr.xunz == ", "\n", k)
    g["tridiag11_xunz"] = nums(s)
    s, _ = between(t, "@test s.slvr.xlindx == ", "\n")
    g["tridiag11_xlindx"] = nums(s)
    s, _ = between(t, "@test s.slvr.lindx == ", "\n")
    g["tridiag11_lindx"] = nums(s)
    # msprs005: lnz / unz after inmatrix!
    s, _ = between(t, "@test s.slvr.unz  == vec(T", ")")
    g["tridiag11_inmatrix_unz"] = nums(s)
    s, _ = between(t, "@test s.slvr.lnz  == vec(T", ")")
    g["tridiag11_inmatrix_lnz"] = nums(s)
    # msprs006: lnz / unz after factor! (checked to rtol 1e-6 by the reference)
    s, _ = between(t, "s_lnz  = T[", "]")
    g["tridiag11_factor_lnz"] = nums(s)
    s, _ = between(t, "s_unz = T[", "]")
    g["tridiag11_factor_unz"] = nums(s)
    # msprs008 comment: permuted rhs before and after the forward solve (n = 11)
    s, k = between(t, "# before  LULSolve \n    # rhs =", "\n")
    g["tridiag11_fwd_before"] = nums(s)
    s, _ = between(t, "# after  LULSolve  \n    # rhs =", "\n", k)
    g["tridiag11_fwd_after"] = nums(s)
    # msprs010: the literal 31 x 31 matrix
    s, _ = between(t, "spm = sparse([1, 2, 10, 25", "31, 31)")
    parts = s.split("],")
    I = nums("1, 2, 10, 25" + parts[0])
    J = nums(parts[1])
    V = nums(parts[2].split("T[", 1)[1])
    assert len(I) == len(J) == len(V), (len(I), len(J), len(V))
    g["m31_I"], g["m31_J"], g["m31_V"] = I, J, V
    # Figure 3.1.3 graph (test_graph.jl)
    tg = read("test/test_graph.jl")
    s, _ = between(tg, "I = [", "]")
    g["fig313_I"] = nums(s)
    s, _ = between(tg, "J = [", "]")
    g["fig313_J"] = nums(s)
    s, _ = between(tg, "@test graph.xadj == ", "\n")
    g["fig313_xadj"] = nums(s)
    s, _ = between(tg, "@test graph.adj == ", "\n")
    g["fig313_adj"] = nums(s)
    k = tg.index("with an element (5, 3) missing")
    s, _ = between(tg, "I = [", "]", k)
    g["fig313_unsym_I"] = nums(s)
    s, _ = between(tg, "J = [", "]", k)
    g["fig313_unsym_J"] = nums(s)
    # grid numbering (test_grid.jl)
    gr = read("test/test_grid.jl")
    s, _ = between(gr, "@test g.v == [", "]")
    g["grid6x6_v"] = nums(s)
    # 4 x 4 literal pivoting cases (test_structunsymm.jl, test_small.jl)
    su = read("test/test_structunsymm.jl")
    mats = []
    for m in re.finditer(r"A=\[(.*?)\]", su, re.S):
        mats.append(nums(m.group(1)))
    sm = read("test/test_small.jl")
    for m in re.finditer(r"A = \[(.*?)\]\n", sm, re.S):
        mats.append(nums(m.group(1)))
    g["small4x4"] = [v for v in mats if len(v) == 16]
    with open(OUT, "w") as f:
        json.dump(g, f, indent=1)
    print(f"wrote {OUT}: {sorted(g)}")


if __name__ == "__main__":
    sys.exit(main())

// Host structure phase: graph symmetrisation, orderings, elimination tree,
// postorders, column counts, supernodes and supernodal symbolic factorisation.
//
// Every routine here restates the algorithm of the reference Julia package
// (Sparspak.jl) so that the permutation, the supernode partition and the
// subscript arrays come out identical.  Arrays are 1-based int64 (slot 0 of
// every std::vector is unused) because the reference's index arithmetic,
// its list sentinels (0 = end of list) and its results are all 1-based.
//
// This file is built with -ffp-contract=off: the supernode splitting rule
// uses floating point, and a fused multiply-add would change its rounding.

#include "../../include/spk_host.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <string>
#include <vector>

typedef int64_t i64;
typedef std::vector<i64> ivec;

static thread_local std::string g_host_err;

static int fail(int code, const std::string& msg) {
    g_host_err = msg;
    return code;
}

extern "C" const char* spk_host_last_error(void) { return g_host_err.c_str(); }

// ---------------------------------------------------------------------------
// Graph
// ---------------------------------------------------------------------------

// src/Graph/SpkGraph.jl:298-316: every edge (i -> j) must have (j -> i).
static bool graph_is_symmetric(i64 nv, const i64* xadj, const i64* adj) {
    for (i64 i = 1; i <= nv; ++i) {
        for (i64 k = xadj[i - 1]; k < xadj[i]; ++k) {
            i64 j = adj[k - 1];
            bool found = false;
            for (i64 q = xadj[j - 1]; q < xadj[j]; ++q)
                if (adj[q - 1] == i) { found = true; break; }
            if (!found) return false;
        }
    }
    return true;
}

extern "C" int spk_graph_is_symmetric(int64_t nv, const int64_t* xadj, const int64_t* adj) {
    if (nv < 0 || (nv > 0 && (!xadj || !adj))) return fail(SPK_HOST_EARG, "spk_graph_is_symmetric: bad arguments");
    for (i64 i = 0; i < nv; ++i)
        for (i64 k = xadj[i]; k < xadj[i + 1]; ++k)
            if (adj[k - 1] < 1 || adj[k - 1] > nv)
                return fail(SPK_HOST_EARG, "spk_graph_is_symmetric: vertex index out of range");
    return graph_is_symmetric(nv, xadj, adj) ? 1 : 0;
}

// src/Graph/SpkGraph.jl:94-289.  The reference's two-pass merge assumes the
// input lists are sorted (Problem columns and SparseMatrixCSC columns are);
// on such input it yields the union of each edge with its mirror, and
// sortgraph! then leaves every list in increasing order.  Here the union is
// formed by counting both directions and removing duplicates per list.
extern "C" int spk_graph_symmetrize(int64_t nv, const int64_t* xadj, const int64_t* adj,
                                    int64_t* nedges_out, int64_t* xadj_out, int64_t* adj_out) {
    if (nv < 0 || !nedges_out || (nv > 0 && (!xadj || !adj)))
        return fail(SPK_HOST_EARG, "spk_graph_symmetrize: bad arguments");
    for (i64 i = 0; i < nv; ++i)
        for (i64 k = xadj[i]; k < xadj[i + 1]; ++k)
            if (adj[k - 1] < 1 || adj[k - 1] > nv)
                return fail(SPK_HOST_EARG, "spk_graph_symmetrize: vertex index out of range");
    i64 ne = nv > 0 ? xadj[nv] - 1 : 0;
    if (graph_is_symmetric(nv, xadj, adj)) {
        *nedges_out = ne;
        if (adj_out) {
            if (!xadj_out) return fail(SPK_HOST_EARG, "spk_graph_symmetrize: xadj_out is null");
            std::memcpy(xadj_out, xadj, sizeof(i64) * (nv + 1));
            std::memcpy(adj_out, adj, sizeof(i64) * ne);
        }
        return SPK_HOST_OK;
    }
    std::vector<ivec> lists(nv + 1);
    for (i64 i = 1; i <= nv; ++i)
        for (i64 k = xadj[i - 1]; k < xadj[i]; ++k) {
            i64 j = adj[k - 1];
            if (j == i) continue;
            lists[i].push_back(j);
            lists[j].push_back(i);
        }
    i64 total = 0;
    for (i64 i = 1; i <= nv; ++i) {
        ivec& l = lists[i];
        std::sort(l.begin(), l.end());
        l.erase(std::unique(l.begin(), l.end()), l.end());
        total += (i64)l.size();
    }
    *nedges_out = total;
    if (adj_out) {
        if (!xadj_out) return fail(SPK_HOST_EARG, "spk_graph_symmetrize: xadj_out is null");
        i64 p = 1;
        for (i64 i = 1; i <= nv; ++i) {
            xadj_out[i - 1] = p;
            for (i64 v : lists[i]) adj_out[(p++) - 1] = v;
        }
        xadj_out[nv] = p;
    }
    return SPK_HOST_OK;
}

// ---------------------------------------------------------------------------
// Multiple minimum degree: restatement of src/SparseSpdMethod/SpkMMD.jl
// (Liu's GENMMD as adapted by the reference, delta = 0).  The quotient graph
// lives in `adj` (a private copy): positive entries are vertices, a negative
// entry -e links to the storage of eliminated vertex e, 0 ends a list.
// ---------------------------------------------------------------------------
namespace {

struct MinDegree {
    i64 n;
    ivec xadj, adj;                 // 1-based
    ivec dhead;                     // dhead[d], d = 0..n
    ivec dnext, dprev, ssize, enext, mark, mparent, upd;
    ivec& invp;
    static constexpr i64 kMax = INT64_MAX;

    MinDegree(i64 n_, const i64* xadj_in, const i64* adj_in, ivec& invp_)
        : n(n_), xadj(n_ + 2), adj(), dhead(n_ + 2, 0), dnext(n_ + 2, 0), dprev(n_ + 2, 0),
          ssize(n_ + 2, 1), enext(n_ + 2, 0), mark(n_ + 2, 0), mparent(n_ + 2, 0), upd(n_ + 2, 0),
          invp(invp_) {
        for (i64 i = 1; i <= n + 1; ++i) xadj[i] = xadj_in[i - 1];
        i64 ne = xadj[n + 1] - 1;
        adj.assign(ne + 2, 0);   // one spare slot past the end, always 0
        for (i64 k = 1; k <= ne; ++k) adj[k] = adj_in[k - 1];
    }

    // __updateexternaldegree (SpkMMD.jl:562-569)
    void push_degree(i64 deg, i64& mindeg, i64 enode) {
        deg -= ssize[enode];
        i64 first = dhead[deg];
        dhead[deg] = enode;
        dnext[enode] = first;
        dprev[enode] = -deg;
        upd[enode] = 0;
        if (first > 0) dprev[first] = enode;
        if (deg < mindeg) mindeg = deg;
    }

    // _mmdelim (SpkMMD.jl:239-352): eliminate mdnode, build its element.
    void eliminate(i64 md, i64 tag) {
        mark[md] = tag;
        i64 elmnt = 0;
        i64 rloc = xadj[md], rlmt = xadj[md + 1] - 1;
        for (i64 i = xadj[md]; i <= xadj[md + 1] - 1; ++i) {
            i64 nb = adj[i];
            if (nb == 0) break;
            if (mark[nb] < tag) {
                mark[nb] = tag;
                if (invp[nb] == 0) { adj[rloc] = nb; ++rloc; }
                else { enext[nb] = elmnt; elmnt = nb; }
            }
        }
        // absorb the reach sets of the neighbouring elements
        while (elmnt > 0) {
            adj[rlmt] = -elmnt;
            i64 j = xadj[elmnt], jstop = xadj[elmnt + 1];
            i64 node = adj[j];
            while (node != 0) {
                if (node < 0) {
                    j = xadj[-node];
                    jstop = xadj[-node + 1];
                } else {
                    if (mark[node] < tag && dnext[node] >= 0) {
                        mark[node] = tag;
                        while (rloc >= rlmt) {          // borrow storage of eliminated vertices
                            i64 lk = -adj[rlmt];
                            rloc = xadj[lk];
                            rlmt = xadj[lk + 1] - 1;
                        }
                        adj[rloc] = node;
                        ++rloc;
                    }
                    ++j;
                }
                if (j >= jstop) break;
                node = adj[j];
            }
            elmnt = enext[elmnt];
        }
        if (rloc <= rlmt) adj[rloc] = 0;
        // visit the reach set
        i64 i = xadj[md], istop = xadj[md + 1];
        i64 rnode = adj[i];
        while (rnode != 0) {
            if (rnode < 0) {
                i = xadj[-rnode];
                istop = xadj[-rnode + 1];
            } else {
                i64 pv = dprev[rnode];
                if (pv != 0) {                           // unlink from its degree list
                    i64 nx = dnext[rnode];
                    if (nx > 0) dprev[nx] = pv;
                    if (pv > 0) dnext[pv] = nx;
                    else dhead[-pv] = nx;
                }
                i64 q = xadj[rnode];                     // purge eliminated neighbours
                for (i64 j = xadj[rnode]; j <= xadj[rnode + 1] - 1; ++j) {
                    i64 nb = adj[j];
                    if (nb == 0) break;
                    if (mark[nb] < tag) { adj[q] = nb; ++q; }
                }
                i64 nq = q - xadj[rnode];
                if (nq <= 0) {                           // indistinguishable from md: merge
                    ssize[md] += ssize[rnode];
                    ssize[rnode] = 0;
                    mparent[rnode] = md;
                    mark[rnode] = kMax;
                } else {
                    upd[rnode] = nq + 1;
                    adj[q] = md;
                    ++q;
                    if (q < xadj[rnode + 1]) adj[q] = 0;
                }
                dprev[rnode] = 0;
                ++i;
            }
            if (i >= istop) break;
            rnode = adj[i];
        }
    }

    // _mmdupdate (SpkMMD.jl:384-560): external degrees after a pass.
    void update(i64 ehead, i64& mindeg, i64& tag) {
        const i64 limit = mindeg;   // mindeg + delta, delta = 0
        i64 elim = ehead;
        while (elim > 0) {
            i64 mtag = tag + limit;
            i64 q2 = 0, qx = 0, esize = 0;
            i64 i = xadj[elim], istop = xadj[elim + 1];
            i64 en = adj[i];
            while (en != 0) {
                if (en < 0) {
                    i = xadj[-en];
                    istop = xadj[-en + 1];
                } else {
                    if (ssize[en] != 0) {
                        esize += ssize[en];
                        mark[en] = mtag;
                        if (upd[en] > 0) {
                            if (upd[en] != 2) { enext[en] = qx; qx = en; }
                            else { enext[en] = q2; q2 = en; }
                        }
                    }
                    ++i;
                }
                if (i >= istop) break;
                en = adj[i];
            }
            // vertices with exactly two quotient neighbours
            en = q2;
            while (en > 0) {
                if (upd[en] > 0) {
                    ++tag;
                    i64 deg = esize;
                    i64 ist = xadj[en];
                    i64 nb = adj[ist];
                    if (nb == elim) nb = adj[ist + 1];
                    if (invp[nb] == 0) {
                        deg += ssize[nb];
                    } else {
                        i64 k = xadj[nb], kstop = xadj[nb + 1];
                        i64 node = adj[k];
                        while (node != 0) {
                            if (node < 0) {
                                k = xadj[-node];
                                kstop = xadj[-node + 1];
                            } else {
                                if (node != en && ssize[node] != 0) {
                                    if (mark[node] < tag) {
                                        mark[node] = tag;
                                        deg += ssize[node];
                                    } else if (upd[node] > 0) {
                                        if (upd[node] == 2) {   // indistinguishable: merge
                                            ssize[en] += ssize[node];
                                            ssize[node] = 0;
                                            mark[node] = kMax;
                                            mparent[node] = en;
                                        }
                                        upd[node] = 0;
                                        dprev[node] = 0;
                                    }
                                }
                                ++k;
                            }
                            if (k >= kstop) break;
                            node = adj[k];
                        }
                    }
                    push_degree(deg, mindeg, en);
                }
                en = enext[en];
            }
            // the remaining vertices
            en = qx;
            while (en > 0) {
                if (upd[en] > 0) {
                    ++tag;
                    i64 deg = esize;
                    for (i64 k = xadj[en]; k <= xadj[en + 1] - 1; ++k) {
                        i64 nb = adj[k];
                        if (nb == 0) break;
                        if (mark[nb] < tag) {
                            mark[nb] = tag;
                            if (invp[nb] == 0) {
                                deg += ssize[nb];
                            } else {
                                i64 j = xadj[nb], jstop = xadj[nb + 1];
                                i64 node = adj[j];
                                while (node != 0) {
                                    if (node < 0) {
                                        j = xadj[-node];
                                        jstop = xadj[-node + 1];
                                    } else {
                                        if (mark[node] < tag) {
                                            mark[node] = tag;
                                            deg += ssize[node];
                                        }
                                        ++j;
                                    }
                                    if (j >= jstop) break;
                                    node = adj[j];
                                }
                            }
                        }
                    }
                    push_degree(deg, mindeg, en);
                }
                en = enext[en];
            }
            tag = mtag;
            elim = enext[elim];
        }
    }

    // _mmdnumber (SpkMMD.jl:588-633): number merged vertices after their root.
    void number(ivec& perm) {
        ivec lastnum(n + 2, 0);
        for (i64 v = 1; v <= n; ++v)
            if (mparent[v] == 0) lastnum[v] = invp[v];
        for (i64 v = 1; v <= n; ++v) {
            i64 par = mparent[v];
            if (par > 0) {
                i64 root = 0;
                while (par > 0) { root = par; par = mparent[par]; }
                i64 num = lastnum[root] + 1;
                invp[v] = num;
                lastnum[root] = num;
                i64 w = v;
                while (w != root) { par = mparent[w]; mparent[w] = root; w = par; }
            }
        }
        for (i64 v = 1; v <= n; ++v) perm[invp[v]] = v;
    }

    // _generalmmd (SpkMMD.jl:78-237)
    void run(ivec& perm) {
        for (i64 v = 1; v <= n; ++v) {
            i64 d = xadj[v + 1] - xadj[v];
            i64 f = dhead[d];
            dhead[d] = v;
            dnext[v] = f;
            if (f > 0) dprev[f] = v;
            dprev[v] = -d;
        }
        i64 num = 1;
        for (i64 v = 1; v <= n; ++v) invp[v] = 0;
        for (i64 v = dhead[0]; v > 0; v = dnext[v]) {   // isolated vertices first
            mark[v] = kMax;
            invp[v] = num++;
        }
        dhead[0] = 0;
        i64 tag = 1, mindeg = 1;
        while (num <= n) {
            while (dhead[mindeg] <= 0) ++mindeg;
            const i64 limit = mindeg;
            i64 ehead = 0;
            bool done = false;
            for (;;) {
                i64 md = dhead[mindeg];
                bool pass_over = false;
                while (md <= 0) {
                    ++mindeg;
                    if (mindeg > limit) { pass_over = true; break; }
                    md = dhead[mindeg];
                }
                if (pass_over) break;
                i64 nxt = dnext[md];
                dhead[mindeg] = nxt;
                if (nxt > 0) dprev[nxt] = -mindeg;
                invp[md] = num;
                if (num + ssize[md] > n) { done = true; break; }
                ++tag;
                eliminate(md, tag);
                num += ssize[md];
                enext[md] = ehead;
                ehead = md;
            }
            if (done || num > n) break;
            update(ehead, mindeg, tag);
        }
        number(perm);
    }
};

}  // namespace

static int check_graph(i64 n, const i64* xadj, const i64* adj, const char* who) {
    if (n < 0 || (n > 0 && (!xadj || !adj))) return fail(SPK_HOST_EARG, std::string(who) + ": bad arguments");
    if (n > 0 && xadj[0] != 1) return fail(SPK_HOST_EARG, std::string(who) + ": xadj[1] must be 1");
    for (i64 i = 0; i < n; ++i) {
        if (xadj[i + 1] < xadj[i]) return fail(SPK_HOST_EARG, std::string(who) + ": xadj not monotone");
        for (i64 k = xadj[i]; k < xadj[i + 1]; ++k)
            if (adj[k - 1] < 1 || adj[k - 1] > n)
                return fail(SPK_HOST_EARG, std::string(who) + ": vertex index out of range");
    }
    return SPK_HOST_OK;
}

static void mmd_order(i64 n, const i64* xadj, const i64* adj, ivec& perm, ivec& invp) {
    perm.assign(n + 2, 0);
    invp.assign(n + 2, 0);
    if (n == 0) return;
    MinDegree md(n, xadj, adj, invp);
    md.run(perm);
}

extern "C" int spk_order_mmd(int64_t nv, const int64_t* xadj, const int64_t* adj,
                             int64_t* perm, int64_t* invp) {
    int rc = check_graph(nv, xadj, adj, "spk_order_mmd");
    if (rc) return rc;
    if (nv > 0 && (!perm || !invp)) return fail(SPK_HOST_EARG, "spk_order_mmd: null output");
    try {
        ivec p, q;
        mmd_order(nv, xadj, adj, p, q);
        for (i64 i = 1; i <= nv; ++i) { perm[i - 1] = p[i]; invp[i - 1] = q[i]; }
    } catch (const std::bad_alloc&) {
        return fail(SPK_HOST_ENOMEM, "spk_order_mmd: out of memory");
    }
    return SPK_HOST_OK;
}

// ---------------------------------------------------------------------------
// Geometric nested dissection of a box grid (project ordering plug-in; the
// reference has none).  A box is split through the middle of its longest
// side; the two halves are numbered first, the separator plane last.  Boxes
// of at most `leaf` vertices are ordered by minimum degree on their induced
// subgraph.
// ---------------------------------------------------------------------------
namespace {
struct GridND {
    i64 nx, ny, nz, leaf;
    const i64* xadj;
    const i64* adj;
    ivec& order;       // order[k] = vertex numbered k (0-based position, 1-based vertex)
    ivec local;        // vertex -> local index during a leaf ordering (0 = absent)

    i64 vid(i64 i, i64 j, i64 k) const { return (i * ny + j) * nz + k + 1; }

    void leaf_order(i64 x0, i64 x1, i64 y0, i64 y1, i64 z0, i64 z1) {
        ivec verts;
        for (i64 i = x0; i < x1; ++i)
            for (i64 j = y0; j < y1; ++j)
                for (i64 k = z0; k < z1; ++k) verts.push_back(vid(i, j, k));
        i64 m = (i64)verts.size();
        if (m == 0) return;
        for (i64 t = 0; t < m; ++t) local[verts[t]] = t + 1;
        ivec sx(m + 1), sa;
        sx[0] = 1;
        for (i64 t = 0; t < m; ++t) {
            i64 v = verts[t];
            for (i64 e = xadj[v - 1]; e < xadj[v]; ++e) {
                i64 w = adj[e - 1];
                if (local[w] > 0) sa.push_back(local[w]);
            }
            sx[t + 1] = (i64)sa.size() + 1;
        }
        ivec p, q;
        mmd_order(m, sx.data(), sa.data(), p, q);
        for (i64 t = 1; t <= m; ++t) order.push_back(verts[p[t] - 1]);
        for (i64 t = 0; t < m; ++t) local[verts[t]] = 0;
    }

    void dissect(i64 x0, i64 x1, i64 y0, i64 y1, i64 z0, i64 z1) {
        i64 dx = x1 - x0, dy = y1 - y0, dz = z1 - z0;
        if (dx <= 0 || dy <= 0 || dz <= 0) return;
        if (dx * dy * dz <= leaf || (dx <= 2 && dy <= 2 && dz <= 2)) {
            leaf_order(x0, x1, y0, y1, z0, z1);
            return;
        }
        if (dx >= dy && dx >= dz) {
            i64 m = x0 + dx / 2;
            dissect(x0, m, y0, y1, z0, z1);
            dissect(m + 1, x1, y0, y1, z0, z1);
            for (i64 j = y0; j < y1; ++j)
                for (i64 k = z0; k < z1; ++k) order.push_back(vid(m, j, k));
        } else if (dy >= dz) {
            i64 m = y0 + dy / 2;
            dissect(x0, x1, y0, m, z0, z1);
            dissect(x0, x1, m + 1, y1, z0, z1);
            for (i64 i = x0; i < x1; ++i)
                for (i64 k = z0; k < z1; ++k) order.push_back(vid(i, m, k));
        } else {
            i64 m = z0 + dz / 2;
            dissect(x0, x1, y0, y1, z0, m);
            dissect(x0, x1, y0, y1, m + 1, z1);
            for (i64 i = x0; i < x1; ++i)
                for (i64 j = y0; j < y1; ++j) order.push_back(vid(i, j, m));
        }
    }
};
}  // namespace

extern "C" int spk_order_nd_grid(int64_t nx, int64_t ny, int64_t nz, int64_t leaf,
                                 const int64_t* xadj, const int64_t* adj,
                                 int64_t* perm, int64_t* invp) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || !perm || !invp)
        return fail(SPK_HOST_EARG, "spk_order_nd_grid: bad arguments");
    i64 n = nx * ny * nz;
    int rc = check_graph(n, xadj, adj, "spk_order_nd_grid");
    if (rc) return rc;
    try {
        ivec order;
        order.reserve(n);
        GridND nd{nx, ny, nz, std::max<i64>(leaf, 1), xadj, adj, order, ivec(n + 2, 0)};
        nd.dissect(0, nx, 0, ny, 0, nz);
        if ((i64)order.size() != n) return fail(SPK_HOST_ESTRUCT, "spk_order_nd_grid: ordering incomplete");
        for (i64 t = 0; t < n; ++t) {
            perm[t] = order[t];
            invp[order[t] - 1] = t + 1;
        }
    } catch (const std::bad_alloc&) {
        return fail(SPK_HOST_ENOMEM, "spk_order_nd_grid: out of memory");
    }
    return SPK_HOST_OK;
}

// ---------------------------------------------------------------------------
// Nested dissection of a general graph (project ordering plug-in; the
// reference has none).  A connected vertex set larger than `leaf` is split by
// a level-structure separator: breadth-first levels from a pseudo-peripheral
// vertex (George and Liu's search: restart from a vertex of least degree in
// the last level while the eccentricity grows), the middle level as
// separator, trimmed of the vertices that have no neighbour in the next
// level (they join the first part).  The parts are numbered first, each
// recursively, the separator last.  Sets of at most `leaf` vertices, and
// sets whose level structure is too shallow to split, are ordered by
// minimum degree on their induced subgraph; disconnected sets component by
// component.
// ---------------------------------------------------------------------------
namespace {
struct GraphND {
    i64 n, leaf;
    const i64* xadj;   // xadj[v - 1] .. xadj[v] - 1: 1-based positions in adj
    const i64* adj;
    ivec& order;
    ivec stamp_of, level, local;
    i64 stamp = 0;

    // Breadth-first levels of the set stamped `st` from `root`; returns the
    // visit order, level[] holds each vertex's level.
    void bfs(i64 root, i64 st, ivec& seen) {
        seen.clear();
        seen.push_back(root);
        level[root] = 0;
        stamp_of[root] = st + 1;   // visited marker for this search
        for (size_t h = 0; h < seen.size(); ++h) {
            const i64 v = seen[h];
            for (i64 e = xadj[v - 1]; e < xadj[v]; ++e) {
                const i64 w = adj[e - 1];
                if (stamp_of[w] == st) {
                    stamp_of[w] = st + 1;
                    level[w] = level[v] + 1;
                    seen.push_back(w);
                }
            }
        }
        for (i64 v : seen) stamp_of[v] = st;   // back to "in the set"
    }

    i64 degree_in(i64 v, i64 st) const {
        i64 d = 0;
        for (i64 e = xadj[v - 1]; e < xadj[v]; ++e) d += stamp_of[adj[e - 1]] == st;
        return d;
    }

    void leaf_order(const ivec& verts) {
        const i64 m = (i64)verts.size();
        if (m == 0) return;
        for (i64 t = 0; t < m; ++t) local[verts[t]] = t + 1;
        ivec sx(m + 1), sa;
        sx[0] = 1;
        for (i64 t = 0; t < m; ++t) {
            const i64 v = verts[t];
            for (i64 e = xadj[v - 1]; e < xadj[v]; ++e) {
                const i64 w = adj[e - 1];
                if (local[w] > 0) sa.push_back(local[w]);
            }
            sx[t + 1] = (i64)sa.size() + 1;
        }
        ivec p, q;
        mmd_order(m, sx.data(), sa.data(), p, q);
        for (i64 t = 1; t <= m; ++t) order.push_back(verts[p[t] - 1]);
        for (i64 t = 0; t < m; ++t) local[verts[t]] = 0;
    }

    void dissect(const ivec& verts) {
        if ((i64)verts.size() <= leaf) {
            leaf_order(verts);
            return;
        }
        stamp += 2;
        const i64 st = stamp;
        for (i64 v : verts) stamp_of[v] = st;
        // connected components of the set
        ivec seen;
        bfs(verts[0], st, seen);
        if (seen.size() < verts.size()) {
            std::vector<ivec> comps;
            for (i64 v : verts) {
                if (stamp_of[v] != st) continue;
                ivec c;
                bfs(v, st, c);
                for (i64 w : c) stamp_of[w] = st - 1;   // assigned
                comps.push_back(std::move(c));
            }
            for (const ivec& c : comps) dissect(c);
            return;
        }
        // pseudo-peripheral root
        i64 root = verts[0], best = -1;
        for (i64 v : verts)
            if (best < 0 || degree_in(v, st) < best) { best = degree_in(v, st); root = v; }
        bfs(root, st, seen);
        i64 ecc = level[seen.back()];
        for (int it = 0; it < 8; ++it) {
            i64 cand = seen.back(), cd = -1;
            for (size_t t = seen.size(); t-- > 0 && level[seen[t]] == ecc;)
                if (cd < 0 || degree_in(seen[t], st) < cd) { cd = degree_in(seen[t], st); cand = seen[t]; }
            ivec s2;
            bfs(cand, st, s2);
            if (level[s2.back()] <= ecc) {
                bfs(root, st, seen);   // restore the levels of the best root
                break;
            }
            root = cand;
            seen.swap(s2);
            ecc = level[seen.back()];
        }
        if (ecc < 2) {
            leaf_order(verts);
            return;
        }
        // middle level: first level whose cumulative count reaches half
        ivec count(ecc + 1, 0);
        for (i64 v : seen) ++count[level[v]];
        i64 mid = 1, acc = 0;
        for (i64 l = 0; l <= ecc; ++l) {
            acc += count[l];
            if (2 * acc >= (i64)verts.size()) { mid = std::min(std::max<i64>(l, 1), ecc - 1); break; }
        }
        ivec A, B, Sep;
        for (i64 v : seen) {
            const i64 l = level[v];
            if (l < mid) A.push_back(v);
            else if (l > mid) B.push_back(v);
            else {
                bool next = false;
                for (i64 e = xadj[v - 1]; e < xadj[v] && !next; ++e) {
                    const i64 w = adj[e - 1];
                    next = stamp_of[w] == st && level[w] == mid + 1;
                }
                (next ? Sep : A).push_back(v);
            }
        }
        dissect(A);
        dissect(B);
        for (i64 v : Sep) order.push_back(v);
    }
};
}  // namespace

extern "C" int spk_order_nd_graph(int64_t nv, const int64_t* xadj, const int64_t* adj, int64_t leaf, int64_t* perm,
                                  int64_t* invp) {
    if (nv < 0 || (nv > 0 && (!perm || !invp))) return fail(SPK_HOST_EARG, "spk_order_nd_graph: bad arguments");
    int rc = check_graph(nv, xadj, adj, "spk_order_nd_graph");
    if (rc) return rc;
    try {
        ivec order;
        order.reserve(nv);
        GraphND nd{nv, std::max<i64>(leaf, 1), xadj, adj, order, ivec(nv + 2, 0), ivec(nv + 2, 0), ivec(nv + 2, 0)};
        ivec all(nv);
        for (i64 v = 0; v < nv; ++v) all[v] = v + 1;
        if (nv > 0) nd.dissect(all);
        if ((i64)order.size() != nv) return fail(SPK_HOST_ESTRUCT, "spk_order_nd_graph: ordering incomplete");
        for (i64 t = 0; t < nv; ++t) {
            perm[t] = order[t];
            invp[order[t] - 1] = t + 1;
        }
    } catch (const std::bad_alloc&) {
        return fail(SPK_HOST_ENOMEM, "spk_order_nd_graph: out of memory");
    }
    return SPK_HOST_OK;
}

// ---------------------------------------------------------------------------
// Elimination tree, postorders, column counts (src/ETree/SpkETree.jl,
// src/SparseSpdMethod/SpkSymFct.jl:37-59)
// ---------------------------------------------------------------------------

// _findetree! (SpkETree.jl:62-88): Liu's algorithm with path compression.
static void find_etree(i64 n, const ivec& xadj, const ivec& adj, const ivec& perm, const ivec& invp, ivec& parent) {
    ivec anc(n + 2, 0);
    for (i64 i = 1; i <= n; ++i) {
        parent[i] = 0;
        anc[i] = 0;
        i64 v = perm[i];
        for (i64 j = xadj[v]; j <= xadj[v + 1] - 1; ++j) {
            i64 nb = invp[adj[j]];
            if (nb < i) {
                while (anc[nb] != 0 && anc[nb] != i) {
                    i64 nx = anc[nb];
                    anc[nb] = i;
                    nb = nx;
                }
                if (anc[nb] == 0) { parent[nb] = i; anc[nb] = i; }
            }
        }
    }
}

// _binarytree! (SpkETree.jl:153-174)
static void binary_tree(i64 n, const ivec& parent, ivec& fson, ivec& bro) {
    std::fill(fson.begin(), fson.end(), 0);
    std::fill(bro.begin(), bro.end(), 0);
    i64 lroot = n;
    for (i64 v = n - 1; v >= 1; --v) {
        i64 p = parent[v];
        if (p <= 0 || p == v) { bro[lroot] = v; lroot = v; }
        else { bro[v] = fson[p]; fson[p] = v; }
    }
    bro[lroot] = 0;
}

// _weightedbinarytree! (SpkETree.jl:239-274): heaviest child visited last.
static void weighted_binary_tree(i64 n, const ivec& parent, const ivec& w, ivec& fson, ivec& bro) {
    ivec lson(n + 2, 0);
    std::fill(fson.begin(), fson.end(), 0);
    std::fill(bro.begin(), bro.end(), 0);
    i64 lroot = n;
    for (i64 v = n - 1; v >= 1; --v) {
        i64 p = parent[v];
        if (p <= 0 || p == v) { bro[lroot] = v; lroot = v; }
        else {
            i64 last = lson[p];
            if (last != 0) {
                if (w[v] >= w[last]) { bro[v] = fson[p]; fson[p] = v; }
                else { bro[last] = v; lson[p] = v; }
            } else { fson[p] = v; lson[p] = v; }
        }
    }
    bro[lroot] = 0;
}

// _postordertree! (SpkETree.jl:190-220); relabels parent in place.
static void postorder_tree(i64 root, ivec& fson, ivec& bro, ivec& invpos, ivec& parent, ivec& stack) {
    i64 num = 0, top = 0, v = root;
    while (v > 0) {
        while (v > 0) { stack[++top] = v; v = fson[v]; }
        while (v <= 0 && top > 0) {
            v = stack[top--];
            invpos[v] = ++num;
            v = bro[v];
        }
    }
    for (i64 u = 1; u <= num; ++u) {
        i64 nu = invpos[u], p = parent[u];
        if (p > 0) p = invpos[p];
        bro[nu] = p;
    }
    for (size_t k = 0; k < parent.size(); ++k) parent[k] = bro[k];
}

// _getpostorder! (SpkETree.jl:106-139); weight (if given) is permuted too.
static void get_postorder(i64 n, ivec& parent, ivec& perm, ivec& invp, ivec* weight) {
    ivec fson(n + 2, 0), bro(n + 2, 0), stack(n + 2, 0), invpos(n + 2, 0);
    if (weight) weighted_binary_tree(n, parent, *weight, fson, bro);
    else binary_tree(n, parent, fson, bro);
    postorder_tree(n, fson, bro, invpos, parent, stack);
    if (weight) {
        ivec w2(n + 2, 0);
        for (i64 i = 1; i <= n; ++i) w2[invpos[i]] = (*weight)[i];
        for (i64 i = 1; i <= n; ++i) (*weight)[i] = w2[i];
    }
    ivec r2(n + 2, 0);
    for (i64 i = 1; i <= n; ++i) r2[i] = invpos[invp[i]];
    for (i64 i = 1; i <= n; ++i) invp[i] = r2[i];
    for (i64 i = 1; i <= n; ++i) perm[invp[i]] = i;
}

// _findcolumncounts! (SpkSymFct.jl:37-59): row-subtree marking.
static void column_counts(i64 n, const ivec& xadj, const ivec& adj, const ivec& perm, const ivec& invp,
                          const ivec& parent, ivec& colcnt) {
    ivec marker(n + 2, 0);
    for (i64 i = 1; i <= n; ++i) {
        marker[i] = i;
        colcnt[i] = 1;
        i64 v = perm[i];
        for (i64 k = xadj[v]; k <= xadj[v + 1] - 1; ++k) {
            i64 j = invp[adj[k]];
            if (j < i) {
                while (marker[j] != i) {
                    colcnt[j] += 1;
                    marker[j] = i;
                    j = parent[j];
                }
            }
        }
    }
}

// _findsupernodes! (SpkSymFct.jl:415-464): fundamental supernodes, then
// split so that none is wider than maxsize.
static void find_supernodes(i64 n, const ivec& parent, const ivec& colcnt, i64 maxsize,
                            i64& nsub, i64& nsuper, ivec& xsuper, ivec& snode) {
    ivec marker(n + 2, 0);
    nsuper = 1;
    xsuper[1] = 1;
    for (i64 k = 2; k <= n; ++k) {
        if (parent[k - 1] == k && colcnt[k - 1] == colcnt[k] + 1) continue;
        ++nsuper;
        xsuper[nsuper] = k;
    }
    xsuper[nsuper + 1] = n + 1;
    for (i64 js = 1; js <= nsuper; ++js) {
        i64 sz = xsuper[js + 1] - xsuper[js];
        if (sz > maxsize) {
            double fsz = (double)sz;
            double delta = fsz / (1.0 + fsz / (double)maxsize);
            i64 limit = (i64)std::floor((double)xsuper[js + 1] - delta / 2.0);
            i64 k = 1;
            i64 index = (i64)std::floor((double)xsuper[js] + delta);
            while (index < limit) {
                marker[index] = 1;
                ++k;
                double kd = (double)k * delta;
                index = (i64)std::floor((double)xsuper[js] + kd);
            }
        }
    }
    nsuper = 1;
    snode[1] = 1;
    nsub = colcnt[1];
    for (i64 k = 2; k <= n; ++k) {
        if (marker[k] != 1 && parent[k - 1] == k && colcnt[k - 1] == colcnt[k] + 1) {
            snode[k] = nsuper;
            continue;
        }
        ++nsuper;
        snode[k] = nsuper;
        xsuper[nsuper] = k;
        nsub += colcnt[k];
    }
    xsuper[nsuper + 1] = n + 1;
}

// findnonzeroindexs (SpkSparseBase.jl:253-284): rectangular column blocks.
static void nonzero_indexes(i64 n, const ivec& colcnt, i64 nsuper, const ivec& xsuper, ivec& xlnz, ivec& xunz) {
    i64 point = 1, upoint = 1;
    for (i64 ks = 1; ks <= nsuper; ++ks) {
        i64 f = xsuper[ks], l = xsuper[ks + 1] - 1, w = l - f + 1;
        for (i64 j = f; j <= l; ++j) {
            xlnz[j] = point;
            xunz[j] = upoint;
            point += colcnt[f];
            upoint += colcnt[f] - w;
        }
    }
    xlnz[n + 1] = point;
    xunz[n + 1] = upoint;
}

// _symbolicfact! (SpkSymFct.jl:105-246): Ng-Peyton supernodal symbolic
// factorisation by merging the children's index lists.
static bool symbolic_fact(i64 n, const ivec& xadj, const ivec& adj, const ivec& perm, const ivec& invp,
                          const ivec& colcnt, i64 nsuper, const ivec& xsuper, const ivec& snode,
                          ivec& xlindx, ivec& lindx) {
    ivec marker(n + 2, 0), mrglnk(nsuper + 2, 0), rch(n + 2, 0);   // rch[0..n]
    const i64 head = 0, tail = n + 1;
    i64 nzend = 0, point = 1;
    for (i64 ks = 1; ks <= nsuper; ++ks) {
        mrglnk[ks] = 0;
        xlindx[ks] = point;
        point += colcnt[xsuper[ks]];
    }
    xlindx[nsuper + 1] = point;
    for (i64 ks = 1; ks <= nsuper; ++ks) {
        i64 f = xsuper[ks], l = xsuper[ks + 1] - 1, w = l - f + 1, len = colcnt[f];
        i64 knz = 0;
        rch[head] = tail;
        i64 js = mrglnk[ks];
        if (js > 0) {
            i64 jw = xsuper[js + 1] - xsuper[js];
            i64 b = xlindx[js] + jw, e = xlindx[js + 1] - 1;
            for (i64 p = e; p >= b; --p) {
                i64 ni = lindx[p];
                ++knz;
                marker[ni] = ks;
                rch[ni] = rch[head];
                rch[head] = ni;
            }
            js = mrglnk[js];
            while (js != 0 && knz < len) {
                jw = xsuper[js + 1] - xsuper[js];
                b = xlindx[js] + jw;
                e = xlindx[js + 1] - 1;
                i64 nexti = head;
                for (i64 p = b; p <= e; ++p) {
                    i64 ni = lindx[p];
                    i64 i = nexti;
                    nexti = rch[i];
                    while (ni > nexti) { i = nexti; nexti = rch[i]; }
                    if (ni < nexti) {
                        ++knz;
                        rch[i] = ni;
                        rch[ni] = nexti;
                        marker[ni] = ks;
                        nexti = ni;
                    }
                }
                js = mrglnk[js];
            }
        }
        if (knz < len) {
            i64 node = perm[f];
            for (i64 p = xadj[node]; p <= xadj[node + 1] - 1; ++p) {
                i64 ni = invp[adj[p]];
                if (ni > f && marker[ni] != ks) {
                    i64 nexti = head, i = nexti;
                    nexti = rch[i];
                    while (ni > nexti) { i = nexti; nexti = rch[i]; }
                    ++knz;
                    rch[i] = ni;
                    rch[ni] = nexti;
                    marker[ni] = ks;
                }
            }
        }
        if (rch[head] != f) {
            rch[f] = rch[head];
            rch[head] = f;
            ++knz;
        }
        i64 nzbeg = nzend + 1;
        nzend += knz;
        if (nzend + 1 != xlindx[ks + 1]) return false;
        i64 i = head;
        for (i64 p = nzbeg; p <= nzend; ++p) { i = rch[i]; lindx[p] = i; }
        if (len > w) {
            i64 pcol = lindx[xlindx[ks] + w];
            i64 ps = snode[pcol];
            mrglnk[ks] = mrglnk[ps];
            mrglnk[ps] = ks;
        }
    }
    return true;
}

struct spk_symbolic {
    i64 n = 0, nsuper = 0, nsub = 0;
    ivec perm, invp, parent, colcnt, snode, xsuper, xlindx, lindx, xlnz, xunz;
};

extern "C" int spk_symbolic_create(int64_t n, const int64_t* xadj_in, const int64_t* adj_in,
                                   const int64_t* perm_in, const int64_t* invp_in,
                                   int64_t maxblocksize, spk_symbolic** out) {
    if (!out) return fail(SPK_HOST_EARG, "spk_symbolic_create: out is null");
    *out = nullptr;
    if (n <= 0) return fail(SPK_HOST_EARG, "An empty problem. No symbolic factorization done.");
    if (maxblocksize < 1) return fail(SPK_HOST_EARG, "spk_symbolic_create: maxblocksize < 1");
    int rc = check_graph(n, xadj_in, adj_in, "spk_symbolic_create");
    if (rc) return rc;
    if (!perm_in || !invp_in) return fail(SPK_HOST_EARG, "spk_symbolic_create: null ordering");
    for (i64 i = 0; i < n; ++i) {
        if (perm_in[i] < 1 || perm_in[i] > n || invp_in[perm_in[i] - 1] != i + 1)
            return fail(SPK_HOST_EARG, "spk_symbolic_create: perm/invp is not a permutation pair");
    }
    spk_symbolic* s = nullptr;
    try {
        s = new spk_symbolic();
        s->n = n;
        ivec xadj(n + 2), adj(xadj_in[n] + 1);
        for (i64 i = 1; i <= n + 1; ++i) xadj[i] = xadj_in[i - 1];
        for (i64 k = 1; k < xadj_in[n]; ++k) adj[k] = adj_in[k - 1];
        s->perm.assign(n + 2, 0);
        s->invp.assign(n + 2, 0);
        for (i64 i = 1; i <= n; ++i) { s->perm[i] = perm_in[i - 1]; s->invp[i] = invp_in[i - 1]; }
        s->parent.assign(n + 2, 0);
        s->colcnt.assign(n + 2, 0);
        s->snode.assign(n + 2, 0);
        s->xsuper.assign(n + 3, 0);
        find_etree(n, xadj, adj, s->perm, s->invp, s->parent);
        get_postorder(n, s->parent, s->perm, s->invp, nullptr);
        column_counts(n, xadj, adj, s->perm, s->invp, s->parent, s->colcnt);
        get_postorder(n, s->parent, s->perm, s->invp, &s->colcnt);
        find_supernodes(n, s->parent, s->colcnt, maxblocksize, s->nsub, s->nsuper, s->xsuper, s->snode);
        s->xsuper.resize(s->nsuper + 2);
        s->xlindx.assign(s->nsuper + 2, 0);
        s->lindx.assign(s->nsub + 2, 0);
        s->xlnz.assign(n + 2, 0);
        s->xunz.assign(n + 2, 0);
        nonzero_indexes(n, s->colcnt, s->nsuper, s->xsuper, s->xlnz, s->xunz);
        if (!symbolic_fact(n, xadj, adj, s->perm, s->invp, s->colcnt, s->nsuper, s->xsuper, s->snode,
                           s->xlindx, s->lindx)) {
            delete s;
            return fail(SPK_HOST_ESTRUCT, "Inconsistency in data structure.");
        }
    } catch (const std::bad_alloc&) {
        delete s;
        return fail(SPK_HOST_ENOMEM, "spk_symbolic_create: out of memory");
    }
    *out = s;
    return SPK_HOST_OK;
}

extern "C" int spk_symbolic_sizes(const spk_symbolic* s, int64_t* nsuper, int64_t* nsub,
                                  int64_t* nnzl, int64_t* nnzu) {
    if (!s) return fail(SPK_HOST_EARG, "spk_symbolic_sizes: null handle");
    if (nsuper) *nsuper = s->nsuper;
    if (nsub) *nsub = s->nsub;
    if (nnzl) *nnzl = s->xlnz[s->n + 1] - 1;
    if (nnzu) *nnzu = s->xunz[s->n + 1] - 1;
    return SPK_HOST_OK;
}

static void copy1(int64_t* dst, const ivec& src, i64 count) {
    if (!dst) return;
    for (i64 i = 1; i <= count; ++i) dst[i - 1] = src[i];
}

extern "C" int spk_symbolic_get(const spk_symbolic* s, int64_t* perm, int64_t* invp, int64_t* parent,
                                int64_t* colcnt, int64_t* snode, int64_t* xsuper, int64_t* xlindx,
                                int64_t* lindx, int64_t* xlnz, int64_t* xunz) {
    if (!s) return fail(SPK_HOST_EARG, "spk_symbolic_get: null handle");
    i64 n = s->n;
    copy1(perm, s->perm, n);
    copy1(invp, s->invp, n);
    copy1(parent, s->parent, n);
    copy1(colcnt, s->colcnt, n);
    copy1(snode, s->snode, n);
    copy1(xsuper, s->xsuper, s->nsuper + 1);
    copy1(xlindx, s->xlindx, s->nsuper + 1);
    copy1(lindx, s->lindx, s->nsub);
    copy1(xlnz, s->xlnz, n + 1);
    copy1(xunz, s->xunz, n + 1);
    return SPK_HOST_OK;
}

extern "C" void spk_symbolic_destroy(spk_symbolic* s) { delete s; }

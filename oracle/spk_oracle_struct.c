/*
 * ORACLE - TEST INFRASTRUCTURE ONLY.
 *
 * The structure phase of the reference package restated in plain C, so that
 * the oracle builds its supernodal structure without the product's host
 * library: the tests compare the product's permutation, supernode partition
 * and subscripts with these, and bench.py's reference arm runs on them.
 *
 * It follows, step for step:
 *   _generalmmd / _mmdelim / _mmdupdate / _mmdnumber
 *                        src/SparseSpdMethod/SpkMMD.jl:78-633 (delta = 0)
 *   _findetree!          src/ETree/SpkETree.jl:62-88
 *   _getpostorder!       src/ETree/SpkETree.jl:106-139, with _binarytree!
 *                        (:153-174), _postordertree! (:194-224) and
 *                        _weightedbinarytree! (:239-274)
 *   _findcolumncounts!   src/SparseSpdMethod/SpkSymFct.jl:37-59
 *   _findsupernodes!     src/SparseSpdMethod/SpkSymFct.jl:415-464
 *   findnonzeroindexs    src/SparseMethod/SpkSparseBase.jl:253-284
 *   _symbolicfact!       src/SparseSpdMethod/SpkSymFct.jl:105-246
 * in the order _symbolicfactor! calls them (SpkSparseBase.jl:193-251).
 *
 * The two nested-dissection orderings are not reference code: they are the
 * ordering plug-ins the package passes through findorder!'s orderfunction
 * slot (SpkSparseBase.jl:173-181), restated here (the geometric one of a box
 * grid: boxes split through the middle of the longest side, halves first,
 * separator plane last; the general one: level-structure separators), with
 * leaf sets ordered by this file's minimum degree, so that the oracle
 * reproduces the orderings without the product library.
 *
 * All index arrays are int64 and 1-based (the reference's convention); a
 * pointer argument addresses element 1.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t i64;

#define MAXI64 INT64_MAX

/* ---- multiple minimum degree (SpkMMD.jl) -------------------------------- */

/* State of one minimum-degree run; every array is indexed 1..n (deghead
 * 0..n-1), adjncy is the working copy of the adjacency. */
typedef struct {
    i64 n;
    const i64* xadj; /* xadj[1..n+1] */
    i64* adjncy;     /* adjncy[1..]  */
    i64 *deghead, *degnext, *degprev, *supersize, *elimnext, *marker, *mergeparent, *needsupdate, *invp;
} Mmd;

/* _mmdelim (SpkMMD.jl:239-352) */
static void mmd_elim(Mmd* s, i64 mdnode, i64 tag) {
    const i64* xadj = s->xadj;
    i64* adj = s->adjncy;
    s->marker[mdnode] = tag;
    i64 elmnt = 0;
    i64 rloc = xadj[mdnode], rlmt = xadj[mdnode + 1] - 1;
    for (i64 i = xadj[mdnode]; i <= xadj[mdnode + 1] - 1; ++i) {
        i64 nb = adj[i];
        if (nb == 0) break;
        if (s->marker[nb] < tag) {
            s->marker[nb] = tag;
            if (s->invp[nb] == 0) adj[rloc++] = nb;
            else { s->elimnext[nb] = elmnt; elmnt = nb; }
        }
    }
    while (elmnt > 0) {
        adj[rlmt] = -elmnt;
        i64 j = xadj[elmnt], jstop = xadj[elmnt + 1], node = adj[j];
        while (node != 0) {
            if (node < 0) {
                j = xadj[-node];
                jstop = xadj[-node + 1];
            } else {
                if (s->marker[node] < tag && s->degnext[node] >= 0) {
                    s->marker[node] = tag;
                    while (rloc >= rlmt) {
                        i64 link = -adj[rlmt];
                        rloc = xadj[link];
                        rlmt = xadj[link + 1] - 1;
                    }
                    adj[rloc++] = node;
                }
                ++j;
            }
            if (j >= jstop) break;
            node = adj[j];
        }
        elmnt = s->elimnext[elmnt];
    }
    if (rloc <= rlmt) adj[rloc] = 0;
    i64 i = xadj[mdnode], istop = xadj[mdnode + 1], rnode = adj[i];
    while (rnode != 0) {
        if (rnode < 0) {
            i = xadj[-rnode];
            istop = xadj[-rnode + 1];
        } else {
            i64 pv = s->degprev[rnode];
            if (pv != 0) {
                i64 nx = s->degnext[rnode];
                if (nx > 0) s->degprev[nx] = pv;
                if (pv > 0) s->degnext[pv] = nx;
                else s->deghead[-pv] = nx;
            }
            i64 xq = xadj[rnode];
            for (i64 j = xadj[rnode]; j <= xadj[rnode + 1] - 1; ++j) {
                i64 nb = adj[j];
                if (nb == 0) break;
                if (s->marker[nb] < tag) adj[xq++] = nb;
            }
            i64 nq = xq - xadj[rnode];
            if (nq <= 0) {
                s->supersize[mdnode] += s->supersize[rnode];
                s->supersize[rnode] = 0;
                s->mergeparent[rnode] = mdnode;
                s->marker[rnode] = MAXI64;
            } else {
                s->needsupdate[rnode] = nq + 1;
                adj[xq++] = mdnode;
                if (xq < xadj[rnode + 1]) adj[xq] = 0;
            }
            s->degprev[rnode] = 0;
            ++i;
        }
        if (i >= istop) break;
        rnode = adj[i];
    }
}

/* __updateexternaldegree (SpkMMD.jl:555-562) */
static void mmd_put(Mmd* s, i64 deg, i64* mindeg, i64 enode) {
    deg -= s->supersize[enode];
    i64 first = s->deghead[deg];
    s->deghead[deg] = enode;
    s->degnext[enode] = first;
    s->degprev[enode] = -deg;
    s->needsupdate[enode] = 0;
    if (first > 0) s->degprev[first] = enode;
    if (deg < *mindeg) *mindeg = deg;
}

static void mmd_reset_marker(Mmd* s) {
    for (i64 v = 1; v <= s->n; ++v)
        if (s->marker[v] < MAXI64) s->marker[v] = 0;
}

/* _mmdupdate (SpkMMD.jl:382-553) */
static void mmd_update(Mmd* s, i64 elimhead, i64* mindeg, i64* tag) {
    const i64* xadj = s->xadj;
    i64* adj = s->adjncy;
    const i64 limit = *mindeg; /* mindeg + delta, delta = 0 */
    for (i64 elimnode = elimhead; elimnode > 0; elimnode = s->elimnext[elimnode]) {
        i64 mtag = *tag + limit;
        if (mtag >= MAXI64) {
            *tag = 1;
            mtag = *tag + limit;
            mmd_reset_marker(s);
        }
        i64 q2head = 0, qxhead = 0, elimsize = 0;
        i64 i = xadj[elimnode], istop = xadj[elimnode + 1], enode = adj[i];
        while (enode != 0) {
            if (enode < 0) {
                i = xadj[-enode];
                istop = xadj[-enode + 1];
            } else {
                if (s->supersize[enode] != 0) {
                    elimsize += s->supersize[enode];
                    s->marker[enode] = mtag;
                    if (s->needsupdate[enode] > 0) {
                        if (s->needsupdate[enode] != 2) { s->elimnext[enode] = qxhead; qxhead = enode; }
                        else { s->elimnext[enode] = q2head; q2head = enode; }
                    }
                }
                ++i;
            }
            if (i >= istop) break;
            enode = adj[i];
        }
        /* nodes with two neighbours in the quotient graph */
        for (enode = q2head; enode > 0; enode = s->elimnext[enode]) {
            if (s->needsupdate[enode] <= 0) continue;
            ++*tag;
            i64 deg = elimsize;
            i64 st = xadj[enode], nb = adj[st];
            if (nb == elimnode) nb = adj[st + 1];
            if (s->invp[nb] == 0) {
                deg += s->supersize[nb];
            } else {
                i64 k = xadj[nb], kstop = xadj[nb + 1], node = adj[k];
                while (node != 0) {
                    if (node < 0) {
                        k = xadj[-node];
                        kstop = xadj[-node + 1];
                    } else {
                        if (node != enode && s->supersize[node] != 0) {
                            if (s->marker[node] < *tag) {
                                s->marker[node] = *tag;
                                deg += s->supersize[node];
                            } else if (s->needsupdate[node] > 0) {
                                if (s->needsupdate[node] == 2) {   /* indistinguishable: merge */
                                    s->supersize[enode] += s->supersize[node];
                                    s->supersize[node] = 0;
                                    s->marker[node] = MAXI64;
                                    s->mergeparent[node] = enode;
                                }
                                s->needsupdate[node] = 0;
                                s->degprev[node] = 0;
                            }
                        }
                        ++k;
                    }
                    if (k >= kstop) break;
                    node = adj[k];
                }
            }
            mmd_put(s, deg, mindeg, enode);
        }
        /* nodes with more neighbours */
        for (enode = qxhead; enode > 0; enode = s->elimnext[enode]) {
            if (s->needsupdate[enode] <= 0) continue;
            ++*tag;
            i64 deg = elimsize;
            for (i64 k = xadj[enode]; k <= xadj[enode + 1] - 1; ++k) {
                i64 nb = adj[k];
                if (nb == 0) break;
                if (s->marker[nb] >= *tag) continue;
                s->marker[nb] = *tag;
                if (s->invp[nb] == 0) {
                    deg += s->supersize[nb];
                } else {
                    i64 j = xadj[nb], jstop = xadj[nb + 1], node = adj[j];
                    while (node != 0) {
                        if (node < 0) {
                            j = xadj[-node];
                            jstop = xadj[-node + 1];
                        } else {
                            if (s->marker[node] < *tag) {
                                s->marker[node] = *tag;
                                deg += s->supersize[node];
                            }
                            ++j;
                        }
                        if (j >= jstop) break;
                        node = adj[j];
                    }
                }
            }
            mmd_put(s, deg, mindeg, enode);
        }
        *tag = mtag;
    }
}

/* _mmdnumber (SpkMMD.jl:581-633) */
static void mmd_number(i64 n, i64* perm, i64* invp, i64* mergeparent) {
    i64* last = (i64*)calloc((size_t)n + 1, sizeof(i64));
    for (i64 v = 1; v <= n; ++v)
        if (mergeparent[v] == 0) last[v] = invp[v];
    for (i64 node = 1; node <= n; ++node) {
        i64 par = mergeparent[node];
        if (par <= 0) continue;
        i64 root = 0;
        while (par > 0) { root = par; par = mergeparent[par]; }
        i64 num = last[root] + 1;
        invp[node] = num;
        last[root] = num;
        for (i64 v = node; v != root;) {
            i64 p = mergeparent[v];
            mergeparent[v] = root;
            v = p;
        }
    }
    for (i64 v = 1; v <= n; ++v) perm[invp[v]] = v;
    free(last);
}

/* _generalmmd (SpkMMD.jl:78-237) with delta = 0.  xadj/adj 1-based (the
 * pointers address element 1); perm/invp receive the ordering. */
void oracle_mmd(i64 n, const i64* xadj1, const i64* adj1, i64* perm1, i64* invp1) {
    if (n <= 0) return;
    const i64* xadj = xadj1 - 1;
    i64 ne = xadj[n + 1] - 1;
    Mmd s;
    s.n = n;
    s.xadj = xadj;
    i64* adjc = (i64*)malloc(sizeof(i64) * (size_t)(ne > 0 ? ne : 1));
    if (ne > 0) memcpy(adjc, adj1, sizeof(i64) * (size_t)ne);
    s.adjncy = adjc - 1;
    i64* pool = (i64*)calloc((size_t)9 * (n + 1), sizeof(i64));
    s.deghead = pool;                 /* 0..n-1 */
    s.degnext = pool + (n + 1);
    s.degprev = pool + 2 * (n + 1);
    s.supersize = pool + 3 * (n + 1);
    s.elimnext = pool + 4 * (n + 1);
    s.marker = pool + 5 * (n + 1);
    s.mergeparent = pool + 6 * (n + 1);
    s.needsupdate = pool + 7 * (n + 1);
    i64* invp = invp1 - 1;
    i64* perm = perm1 - 1;
    s.invp = invp;
    for (i64 v = 1; v <= n; ++v) s.supersize[v] = 1;
    for (i64 node = 1; node <= n; ++node) {
        i64 ndeg = xadj[node + 1] - xadj[node], f = s.deghead[ndeg];
        s.deghead[ndeg] = node;
        s.degnext[node] = f;
        if (f > 0) s.degprev[f] = node;
        s.degprev[node] = -ndeg;
    }
    i64 num = 1;
    for (i64 v = 1; v <= n; ++v) invp[v] = 0;
    for (i64 md = s.deghead[0]; md > 0; md = s.degnext[md]) {   /* isolated nodes */
        s.marker[md] = MAXI64;
        invp[md] = num++;
    }
    s.deghead[0] = 0;
    i64 tag = 1, mindeg = 1;
    while (num <= n) {
        while (s.deghead[mindeg] <= 0) ++mindeg;
        const i64 limit = mindeg;
        i64 elimhead = 0;
        int done = 0;
        for (;;) {
            i64 md = s.deghead[mindeg];
            while (md <= 0) {
                ++mindeg;
                if (mindeg > limit) break;
                md = s.deghead[mindeg];
            }
            if (md <= 0) break;   /* end of the pass */
            i64 nx = s.degnext[md];
            s.deghead[mindeg] = nx;
            if (nx > 0) s.degprev[nx] = -mindeg;
            invp[md] = num;
            if (num + s.supersize[md] > n) { done = 1; break; }
            ++tag;
            if (tag >= MAXI64) {
                tag = 1;
                mmd_reset_marker(&s);
            }
            mmd_elim(&s, md, tag);
            num += s.supersize[md];
            s.elimnext[md] = elimhead;
            elimhead = md;
        }
        if (done || num > n) break;
        mmd_update(&s, elimhead, &mindeg, &tag);
    }
    mmd_number(n, perm, invp, s.mergeparent);
    free(pool);
    free(adjc);
}

/* ---- geometric nested dissection of a box grid (ordering plug-in) -------- */

typedef struct {
    i64 nx, ny, nz, leaf;
    const i64 *xadj, *adj;   /* 1-based arrays, pointers address element 1 */
    i64* order;              /* order[0..]: vertices in elimination order   */
    i64 count;
    i64* local;              /* vertex -> index in the current leaf box     */
} Nd;

static i64 nd_vid(const Nd* d, i64 i, i64 j, i64 k) { return (i * d->ny + j) * d->nz + k + 1; }

static void nd_leaf(Nd* d, i64 x0, i64 x1, i64 y0, i64 y1, i64 z0, i64 z1) {
    i64 m = (x1 - x0) * (y1 - y0) * (z1 - z0);
    if (m <= 0) return;
    i64* verts = (i64*)malloc(sizeof(i64) * (size_t)m);
    i64 t = 0;
    for (i64 i = x0; i < x1; ++i)
        for (i64 j = y0; j < y1; ++j)
            for (i64 k = z0; k < z1; ++k) verts[t++] = nd_vid(d, i, j, k);
    for (t = 0; t < m; ++t) d->local[verts[t]] = t + 1;
    i64 cap = 0;
    for (t = 0; t < m; ++t) cap += d->xadj[verts[t]] - d->xadj[verts[t] - 1];
    i64* sx = (i64*)malloc(sizeof(i64) * (size_t)(m + 1));
    i64* sa = (i64*)malloc(sizeof(i64) * (size_t)(cap > 0 ? cap : 1));
    i64 ne = 0;
    sx[0] = 1;
    for (t = 0; t < m; ++t) {
        i64 v = verts[t];
        for (i64 e = d->xadj[v - 1]; e < d->xadj[v]; ++e) {
            i64 w = d->adj[e - 1];
            if (d->local[w] > 0) sa[ne++] = d->local[w];
        }
        sx[t + 1] = ne + 1;
    }
    i64* p = (i64*)malloc(sizeof(i64) * (size_t)m);
    i64* q = (i64*)malloc(sizeof(i64) * (size_t)m);
    oracle_mmd(m, sx, sa, p, q);
    for (t = 0; t < m; ++t) d->order[d->count++] = verts[p[t] - 1];
    for (t = 0; t < m; ++t) d->local[verts[t]] = 0;
    free(verts); free(sx); free(sa); free(p); free(q);
}

static void nd_dissect(Nd* d, i64 x0, i64 x1, i64 y0, i64 y1, i64 z0, i64 z1) {
    i64 dx = x1 - x0, dy = y1 - y0, dz = z1 - z0;
    if (dx <= 0 || dy <= 0 || dz <= 0) return;
    if (dx * dy * dz <= d->leaf || (dx <= 2 && dy <= 2 && dz <= 2)) {
        nd_leaf(d, x0, x1, y0, y1, z0, z1);
        return;
    }
    if (dx >= dy && dx >= dz) {
        i64 m = x0 + dx / 2;
        nd_dissect(d, x0, m, y0, y1, z0, z1);
        nd_dissect(d, m + 1, x1, y0, y1, z0, z1);
        for (i64 j = y0; j < y1; ++j)
            for (i64 k = z0; k < z1; ++k) d->order[d->count++] = nd_vid(d, m, j, k);
    } else if (dy >= dz) {
        i64 m = y0 + dy / 2;
        nd_dissect(d, x0, x1, y0, m, z0, z1);
        nd_dissect(d, x0, x1, m + 1, y1, z0, z1);
        for (i64 i = x0; i < x1; ++i)
            for (i64 k = z0; k < z1; ++k) d->order[d->count++] = nd_vid(d, i, m, k);
    } else {
        i64 m = z0 + dz / 2;
        nd_dissect(d, x0, x1, y0, y1, z0, m);
        nd_dissect(d, x0, x1, y0, y1, m + 1, z1);
        for (i64 i = x0; i < x1; ++i)
            for (i64 j = y0; j < y1; ++j) d->order[d->count++] = nd_vid(d, i, j, m);
    }
}

/* Returns the number of vertices ordered (n on success). */
i64 oracle_nd_grid(i64 nx, i64 ny, i64 nz, i64 leaf, const i64* xadj, const i64* adj, i64* perm, i64* invp) {
    i64 n = nx * ny * nz;
    Nd d;
    d.nx = nx; d.ny = ny; d.nz = nz;
    d.leaf = leaf > 1 ? leaf : 1;
    d.xadj = xadj; d.adj = adj;
    d.order = perm;
    d.count = 0;
    d.local = (i64*)calloc((size_t)n + 2, sizeof(i64));
    nd_dissect(&d, 0, nx, 0, ny, 0, nz);
    free(d.local);
    if (d.count != n) return d.count;
    for (i64 t = 0; t < n; ++t) invp[perm[t] - 1] = t + 1;
    return n;
}

/* ---- nested dissection of a general graph (ordering plug-in) -------------- */

/* The package's level-structure nested dissection restated: a connected set
 * larger than `leaf` is split at the middle level of a breadth-first level
 * structure from a pseudo-peripheral vertex (restart from a least-degree
 * vertex of the last level while the eccentricity grows, at most 8 times),
 * the middle level trimmed of vertices without a neighbour in the next level
 * (they join the first part); parts first, recursively, separator last;
 * small or shallow sets by minimum degree; disconnected sets component by
 * component. */
typedef struct {
    i64 n, leaf;
    const i64 *xadj, *adj;   /* 1-based arrays, pointers address element 1 */
    i64 *order, count;
    i64 *stamp_of, *level, *local;
    i64 stamp;
} Gnd;

typedef struct {
    i64* v;
    i64 n, cap;
} Vec;

static void vpush(Vec* a, i64 x) {
    if (a->n == a->cap) {
        a->cap = a->cap ? 2 * a->cap : 16;
        a->v = (i64*)realloc(a->v, sizeof(i64) * (size_t)a->cap);
    }
    a->v[a->n++] = x;
}

static void gnd_bfs(Gnd* d, i64 root, i64 st, Vec* seen) {
    seen->n = 0;
    vpush(seen, root);
    d->level[root] = 0;
    d->stamp_of[root] = st + 1;
    for (i64 h = 0; h < seen->n; ++h) {
        i64 v = seen->v[h];
        for (i64 e = d->xadj[v - 1]; e < d->xadj[v]; ++e) {
            i64 w = d->adj[e - 1];
            if (d->stamp_of[w] == st) {
                d->stamp_of[w] = st + 1;
                d->level[w] = d->level[v] + 1;
                vpush(seen, w);
            }
        }
    }
    for (i64 h = 0; h < seen->n; ++h) d->stamp_of[seen->v[h]] = st;
}

static i64 gnd_deg(const Gnd* d, i64 v, i64 st) {
    i64 k = 0;
    for (i64 e = d->xadj[v - 1]; e < d->xadj[v]; ++e) k += d->stamp_of[d->adj[e - 1]] == st;
    return k;
}

static void gnd_leaf(Gnd* d, const i64* verts, i64 m) {
    if (m == 0) return;
    for (i64 t = 0; t < m; ++t) d->local[verts[t]] = t + 1;
    i64 cap = 0;
    for (i64 t = 0; t < m; ++t) cap += d->xadj[verts[t]] - d->xadj[verts[t] - 1];
    i64* sx = (i64*)malloc(sizeof(i64) * (size_t)(m + 1));
    i64* sa = (i64*)malloc(sizeof(i64) * (size_t)(cap > 0 ? cap : 1));
    i64 ne = 0;
    sx[0] = 1;
    for (i64 t = 0; t < m; ++t) {
        i64 v = verts[t];
        for (i64 e = d->xadj[v - 1]; e < d->xadj[v]; ++e) {
            i64 w = d->adj[e - 1];
            if (d->local[w] > 0) sa[ne++] = d->local[w];
        }
        sx[t + 1] = ne + 1;
    }
    i64* p = (i64*)malloc(sizeof(i64) * (size_t)m);
    i64* q = (i64*)malloc(sizeof(i64) * (size_t)m);
    oracle_mmd(m, sx, sa, p, q);
    for (i64 t = 0; t < m; ++t) d->order[d->count++] = verts[p[t] - 1];
    for (i64 t = 0; t < m; ++t) d->local[verts[t]] = 0;
    free(sx); free(sa); free(p); free(q);
}

static void gnd_dissect(Gnd* d, const i64* verts, i64 nv) {
    if (nv <= d->leaf) {
        gnd_leaf(d, verts, nv);
        return;
    }
    d->stamp += 2;
    const i64 st = d->stamp;
    for (i64 t = 0; t < nv; ++t) d->stamp_of[verts[t]] = st;
    Vec seen = {0, 0, 0};
    gnd_bfs(d, verts[0], st, &seen);
    if (seen.n < nv) {   /* components, each on its own */
        Vec all = {0, 0, 0}, starts = {0, 0, 0};
        Vec c = {0, 0, 0};
        for (i64 t = 0; t < nv; ++t) {
            i64 v = verts[t];
            if (d->stamp_of[v] != st) continue;
            gnd_bfs(d, v, st, &c);
            vpush(&starts, all.n);
            for (i64 h = 0; h < c.n; ++h) {
                d->stamp_of[c.v[h]] = st - 1;
                vpush(&all, c.v[h]);
            }
        }
        vpush(&starts, all.n);
        for (i64 k = 0; k + 1 < starts.n; ++k) gnd_dissect(d, all.v + starts.v[k], starts.v[k + 1] - starts.v[k]);
        free(all.v); free(starts.v); free(c.v); free(seen.v);
        return;
    }
    i64 root = verts[0], best = -1;
    for (i64 t = 0; t < nv; ++t) {
        i64 dg = gnd_deg(d, verts[t], st);
        if (best < 0 || dg < best) { best = dg; root = verts[t]; }
    }
    gnd_bfs(d, root, st, &seen);
    i64 ecc = d->level[seen.v[seen.n - 1]];
    Vec s2 = {0, 0, 0};
    for (int it = 0; it < 8; ++it) {
        i64 cand = seen.v[seen.n - 1], cd = -1;
        for (i64 t = seen.n; t-- > 0 && d->level[seen.v[t]] == ecc;) {
            i64 dg = gnd_deg(d, seen.v[t], st);
            if (cd < 0 || dg < cd) { cd = dg; cand = seen.v[t]; }
        }
        gnd_bfs(d, cand, st, &s2);
        if (d->level[s2.v[s2.n - 1]] <= ecc) {
            gnd_bfs(d, root, st, &seen);
            break;
        }
        root = cand;
        Vec tmp = seen; seen = s2; s2 = tmp;
        ecc = d->level[seen.v[seen.n - 1]];
    }
    free(s2.v);
    if (ecc < 2) {
        gnd_leaf(d, verts, nv);
        free(seen.v);
        return;
    }
    i64* count = (i64*)calloc((size_t)ecc + 1, sizeof(i64));
    for (i64 h = 0; h < seen.n; ++h) ++count[d->level[seen.v[h]]];
    i64 mid = 1, acc = 0;
    for (i64 l = 0; l <= ecc; ++l) {
        acc += count[l];
        if (2 * acc >= nv) {
            mid = l < 1 ? 1 : l;
            if (mid > ecc - 1) mid = ecc - 1;
            break;
        }
    }
    free(count);
    Vec A = {0, 0, 0}, B = {0, 0, 0}, S = {0, 0, 0};
    for (i64 h = 0; h < seen.n; ++h) {
        i64 v = seen.v[h], l = d->level[v];
        if (l < mid) vpush(&A, v);
        else if (l > mid) vpush(&B, v);
        else {
            int next = 0;
            for (i64 e = d->xadj[v - 1]; e < d->xadj[v] && !next; ++e) {
                i64 w = d->adj[e - 1];
                next = d->stamp_of[w] == st && d->level[w] == mid + 1;
            }
            vpush(next ? &S : &A, v);
        }
    }
    free(seen.v);
    gnd_dissect(d, A.v, A.n);
    gnd_dissect(d, B.v, B.n);
    for (i64 h = 0; h < S.n; ++h) d->order[d->count++] = S.v[h];
    free(A.v); free(B.v); free(S.v);
}

/* Returns the number of vertices ordered (n on success). */
i64 oracle_nd_graph(i64 n, const i64* xadj, const i64* adj, i64 leaf, i64* perm, i64* invp) {
    Gnd d;
    d.n = n;
    d.leaf = leaf > 1 ? leaf : 1;
    d.xadj = xadj;
    d.adj = adj;
    d.order = perm;
    d.count = 0;
    d.stamp = 0;
    d.stamp_of = (i64*)calloc((size_t)n + 2, sizeof(i64));
    d.level = (i64*)calloc((size_t)n + 2, sizeof(i64));
    d.local = (i64*)calloc((size_t)n + 2, sizeof(i64));
    i64* all = (i64*)malloc(sizeof(i64) * (size_t)(n > 0 ? n : 1));
    for (i64 v = 0; v < n; ++v) all[v] = v + 1;
    if (n > 0) gnd_dissect(&d, all, n);
    free(all);
    free(d.stamp_of); free(d.level); free(d.local);
    if (d.count != n) return d.count;
    for (i64 t = 0; t < n; ++t) invp[perm[t] - 1] = t + 1;
    return n;
}

/* ---- elimination tree and postorders (SpkETree.jl) ------------------------ */

/* _findetree! */
static void find_etree(i64 n, const i64* xadj, const i64* adj, const i64* perm, const i64* invp, i64* parent) {
    i64* anc = (i64*)calloc((size_t)n + 1, sizeof(i64));
    for (i64 i = 1; i <= n; ++i) {
        parent[i] = 0;
        anc[i] = 0;
        i64 v = perm[i];
        for (i64 j = xadj[v]; j <= xadj[v + 1] - 1; ++j) {
            i64 nb = invp[adj[j]];
            if (nb >= i) continue;
            while (anc[nb] != 0 && anc[nb] != i) {
                i64 nx = anc[nb];
                anc[nb] = i;
                nb = nx;
            }
            if (anc[nb] == 0) { parent[nb] = i; anc[nb] = i; }
        }
    }
    free(anc);
}

/* _binarytree! / _weightedbinarytree! (weight == NULL: the plain form) */
static void binary_tree(i64 n, const i64* parent, const i64* weight, i64* fson, i64* bro) {
    i64* lson = (i64*)calloc((size_t)n + 1, sizeof(i64));
    for (i64 v = 0; v <= n; ++v) { fson[v] = 0; bro[v] = 0; }
    i64 lroot = n;
    for (i64 v = n - 1; v >= 1; --v) {
        i64 p = parent[v];
        if (p <= 0 || p == v) {
            bro[lroot] = v;
            lroot = v;
        } else if (!weight) {
            bro[v] = fson[p];
            fson[p] = v;
        } else {
            i64 last = lson[p];
            if (last != 0) {
                if (weight[v] >= weight[last]) { bro[v] = fson[p]; fson[p] = v; }
                else { bro[last] = v; lson[p] = v; }
            } else {
                fson[p] = v;
                lson[p] = v;
            }
        }
    }
    bro[lroot] = 0;
    free(lson);
}

/* _postordertree! */
static void postorder_tree(i64 root, i64* fson, i64* bro, i64* invpos, i64* parent, i64* stack) {
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
    for (i64 u = 0; u <= root; ++u) parent[u] = bro[u];
}

/* _getpostorder! (weight == NULL) and its weighted form; updates perm/invp,
 * the parent vector and (weighted form) the weights to the new numbering. */
static void get_postorder(i64 n, i64* parent, i64* perm, i64* invp, i64* weight) {
    i64* fson = (i64*)calloc((size_t)n + 1, sizeof(i64));
    i64* bro = (i64*)calloc((size_t)n + 1, sizeof(i64));
    i64* stack = (i64*)calloc((size_t)n + 1, sizeof(i64));
    i64* invpos = (i64*)calloc((size_t)n + 1, sizeof(i64));
    binary_tree(n, parent, weight, fson, bro);
    postorder_tree(n, fson, bro, invpos, parent, stack);
    if (weight) {
        for (i64 v = 1; v <= n; ++v) stack[invpos[v]] = weight[v];
        for (i64 v = 1; v <= n; ++v) weight[v] = stack[v];
    }
    for (i64 v = 1; v <= n; ++v) stack[v] = invpos[invp[v]];
    for (i64 v = 1; v <= n; ++v) invp[v] = stack[v];
    for (i64 v = 1; v <= n; ++v) perm[invp[v]] = v;
    free(fson); free(bro); free(stack); free(invpos);
}

/* ---- column counts, supernodes, subscripts (SpkSymFct.jl) ---------------- */

/* _findcolumncounts! */
static void column_counts(i64 n, const i64* xadj, const i64* adj, const i64* perm, const i64* invp,
                          const i64* parent, i64* colcnt) {
    i64* marker = (i64*)calloc((size_t)n + 1, sizeof(i64));
    for (i64 i = 1; i <= n; ++i) {
        marker[i] = i;
        colcnt[i] = 1;
        for (i64 k = xadj[perm[i]]; k <= xadj[perm[i] + 1] - 1; ++k) {
            i64 j = invp[adj[k]];
            if (j >= i) continue;
            while (marker[j] != i) {
                colcnt[j] += 1;
                marker[j] = i;
                j = parent[j];
            }
        }
    }
    free(marker);
}

/* _findsupernodes!: fundamental supernodes split to at most maxsize columns
 * by the reference's floating-point rule; returns nsuper, *nofsub. */
static i64 find_supernodes(i64 n, const i64* parent, const i64* colcnt, i64* xsuper, i64* snode, i64 maxsize,
                           i64* nofsub) {
    i64* marker = (i64*)calloc((size_t)n + 2, sizeof(i64));
    i64 nsuper = 1;
    xsuper[1] = 1;
    for (i64 k = 2; k <= n; ++k) {
        if (parent[k - 1] == k && colcnt[k - 1] == colcnt[k] + 1) continue;
        xsuper[++nsuper] = k;
    }
    xsuper[nsuper + 1] = n + 1;
    for (i64 js = 1; js <= nsuper; ++js) {
        i64 sz = xsuper[js + 1] - xsuper[js];
        if (sz <= maxsize) continue;
        double delta = (double)sz / (1.0 + (double)sz / (double)maxsize);
        i64 limit = (i64)((double)xsuper[js + 1] - delta / 2.0);
        i64 k = 1, index = (i64)((double)xsuper[js] + delta);
        while (index < limit) {
            marker[index] = 1;
            ++k;
            index = (i64)((double)xsuper[js] + (double)k * delta);
        }
    }
    nsuper = 1;
    snode[1] = 1;
    i64 nsub = colcnt[1];
    for (i64 k = 2; k <= n; ++k) {
        if (marker[k] != 1 && parent[k - 1] == k && colcnt[k - 1] == colcnt[k] + 1) {
            snode[k] = nsuper;
            continue;
        }
        snode[k] = ++nsuper;
        xsuper[nsuper] = k;
        nsub += colcnt[k];
    }
    xsuper[nsuper + 1] = n + 1;
    free(marker);
    *nofsub = nsub;
    return nsuper;
}

/* findnonzeroindexs */
static void nonzero_indexes(i64 n, const i64* colcnt, i64 nsuper, const i64* xsuper, i64* xlnz, i64* xunz) {
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

/* _symbolicfact!; returns 0, or -1 on the reference's "Inconsistency in
 * data structure." */
static int symbolic_fact(i64 n, const i64* xadj, const i64* adj, const i64* perm, const i64* invp, const i64* colcnt,
                         i64 nsuper, const i64* xsuper, const i64* snode, i64* xlindx, i64* lindx) {
    i64* marker = (i64*)calloc((size_t)n + 1, sizeof(i64));
    i64* mrglnk = (i64*)calloc((size_t)nsuper + 1, sizeof(i64));
    i64* rch = (i64*)calloc((size_t)n + 2, sizeof(i64));   /* rchlnk[0..n], head = 0 */
    const i64 head = 0, tail = n + 1;
    i64 nzend = 0, point = 1;
    int rc = 0;
    for (i64 ks = 1; ks <= nsuper; ++ks) {
        mrglnk[ks] = 0;
        xlindx[ks] = point;
        point += colcnt[xsuper[ks]];
    }
    xlindx[nsuper + 1] = point;
    for (i64 ks = 1; ks <= nsuper && rc == 0; ++ks) {
        i64 f = xsuper[ks], l = xsuper[ks + 1] - 1, width = l - f + 1, len = colcnt[f];
        i64 knz = 0;
        rch[head] = tail;
        i64 js = mrglnk[ks];
        if (js > 0) {
            i64 jw = xsuper[js + 1] - xsuper[js];
            for (i64 p = xlindx[js + 1] - 1; p >= xlindx[js] + jw; --p) {
                i64 v = lindx[p];
                ++knz;
                marker[v] = ks;
                rch[v] = rch[head];
                rch[head] = v;
            }
            js = mrglnk[js];
            while (js != 0 && knz < len) {
                jw = xsuper[js + 1] - xsuper[js];
                i64 nexti = head;
                for (i64 p = xlindx[js] + jw; p <= xlindx[js + 1] - 1; ++p) {
                    i64 v = lindx[p], i = nexti;
                    nexti = rch[i];
                    while (v > nexti) { i = nexti; nexti = rch[i]; }
                    if (v < nexti) {
                        ++knz;
                        rch[i] = v;
                        rch[v] = nexti;
                        marker[v] = ks;
                        nexti = v;
                    }
                }
                js = mrglnk[js];
            }
        }
        if (knz < len) {
            i64 node = perm[f];
            for (i64 p = xadj[node]; p <= xadj[node + 1] - 1; ++p) {
                i64 v = invp[adj[p]];
                if (v > f && marker[v] != ks) {
                    i64 nexti = head, i = nexti;
                    nexti = rch[i];
                    while (v > nexti) { i = nexti; nexti = rch[i]; }
                    ++knz;
                    rch[i] = v;
                    rch[v] = nexti;
                    marker[v] = ks;
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
        if (nzend + 1 != xlindx[ks + 1]) { rc = -1; break; }
        i64 i = head;
        for (i64 p = nzbeg; p <= nzend; ++p) { i = rch[i]; lindx[p] = i; }
        if (len > width) {
            i64 pcol = lindx[xlindx[ks] + width], psup = snode[pcol];
            mrglnk[ks] = mrglnk[psup];
            mrglnk[psup] = ks;
        }
    }
    free(marker); free(mrglnk); free(rch);
    return rc;
}

/* ---- _symbolicfactor! ------------------------------------------------------ */

/*
 * Phase 1: given the symmetric graph (no self loops) and an initial ordering
 * (perm/invp, updated in place by the two postorders), compute colcnt[n],
 * snode[n], xsuper[n+1] (first nsuper+1 used), xlnz[n+1], xunz[n+1];
 * returns nsuper and *nsub (the length of lindx).
 */
i64 oracle_symbolic1(i64 n, const i64* xadj1, const i64* adj1, i64* perm1, i64* invp1, i64 maxblocksize,
                     i64* colcnt1, i64* snode1, i64* xsuper1, i64* xlnz1, i64* xunz1, i64* nsub) {
    const i64* xadj = xadj1 - 1;
    const i64* adj = adj1 - 1;
    i64 *perm = perm1 - 1, *invp = invp1 - 1, *colcnt = colcnt1 - 1;
    i64* parent = (i64*)calloc((size_t)n + 1, sizeof(i64));
    find_etree(n, xadj, adj, perm, invp, parent);
    get_postorder(n, parent, perm, invp, NULL);
    column_counts(n, xadj, adj, perm, invp, parent, colcnt);
    get_postorder(n, parent, perm, invp, colcnt);
    i64 nsuper = find_supernodes(n, parent, colcnt, xsuper1 - 1, snode1 - 1, maxblocksize, nsub);
    nonzero_indexes(n, colcnt, nsuper, xsuper1 - 1, xlnz1 - 1, xunz1 - 1);
    free(parent);
    return nsuper;
}

/* Phase 2: xlindx[nsuper+1] and lindx[nsub]; returns 0 or -1. */
i64 oracle_symbolic2(i64 n, const i64* xadj1, const i64* adj1, const i64* perm1, const i64* invp1,
                     const i64* colcnt1, i64 nsuper, const i64* xsuper1, const i64* snode1, i64* xlindx1,
                     i64* lindx1) {
    return symbolic_fact(n, xadj1 - 1, adj1 - 1, perm1 - 1, invp1 - 1, colcnt1 - 1, nsuper, xsuper1 - 1,
                         snode1 - 1, xlindx1 - 1, lindx1 - 1);
}

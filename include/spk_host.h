/*
 * spk_host.h - host-side structure phase of the Sparspak numeric engine.
 *
 * These entry points compute, on the CPU, everything the numeric phase needs
 * before any value is touched: the symmetrised adjacency graph, the fill
 * reducing ordering, the elimination tree, its two postorders, the column
 * counts, the supernode partition (split to at most `maxblocksize` columns)
 * and the compressed row subscripts.  They reproduce the reference Julia
 * package's arrays exactly (same permutation, same supernodes, same
 * xlindx/lindx/xlnz/xunz), so that the device library (spk_gpu.h) receives
 * the structure a reference SparseSolver would hold after symbolicfactor!.
 *
 * Conventions: every index array is int64 and 1-based, exactly as the
 * reference stores them.  Every function returns 0 on success and a
 * negative SPK_HOST_E* code on failure; spk_host_last_error() gives text.
 */
#ifndef SPK_HOST_H
#define SPK_HOST_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPK_HOST_OK 0
#define SPK_HOST_EARG (-1)      /* bad argument (null pointer, bad size)   */
#define SPK_HOST_ESTRUCT (-2)   /* inconsistent structure detected          */
#define SPK_HOST_ENOMEM (-3)    /* allocation failed                        */

/* Text of the last error raised on the calling thread ("" if none). */
const char* spk_host_last_error(void);

/*
 * Structural symmetry test of a graph given as 1-based (xadj, adj).
 * Replaces SpkGraph.isstructuresymmetric (src/Graph/SpkGraph.jl:298-316).
 * Returns 1 if symmetric, 0 if not, <0 on error.
 */
int spk_graph_is_symmetric(int64_t nv, const int64_t* xadj, const int64_t* adj);

/*
 * Symmetrise a graph (adjacency lists sorted ascending, no self loops).
 * Replaces SpkGraph.makestructuresymmetric + sortgraph!
 * (src/Graph/SpkGraph.jl:94-289).  Two-phase: call with adj_out == NULL to
 * obtain *nedges_out, then again with xadj_out[nv+1] and adj_out[*nedges_out].
 * A graph that is already symmetric is returned unchanged (the reference
 * does not sort it either).
 */
int spk_graph_symmetrize(int64_t nv, const int64_t* xadj, const int64_t* adj,
                         int64_t* nedges_out, int64_t* xadj_out, int64_t* adj_out);

/*
 * Multiple minimum degree ordering of a symmetric graph.
 * Replaces SpkMmd.mmd! / _generalmmd (src/SparseSpdMethod/SpkMMD.jl:38-237)
 * with delta = 0.  perm[new] = old, invp[old] = new (both 1-based).
 */
int spk_order_mmd(int64_t nv, const int64_t* xadj, const int64_t* adj,
                  int64_t* perm, int64_t* invp);

/*
 * Geometric nested dissection of an nx x ny x nz grid whose vertex (i,j,k)
 * (1-based, i slowest) is numbered ((i-1)*ny + (j-1))*nz + k, the numbering
 * of SpkGrid.Grid (src/Grid/SpkGrid.jl:19-28) extended to 3-D (nz = 1 gives
 * the 2-D grid).  Separator planes are ordered last, recursively, down to
 * boxes of at most `leaf` vertices, which are ordered by minimum degree.
 * The reference has no nested dissection; this is the ordering plug-in for
 * findorder!'s orderfunction slot (src/SparseMethod/SpkSparseBase.jl:173-181).
 */
int spk_order_nd_grid(int64_t nx, int64_t ny, int64_t nz, int64_t leaf,
                      const int64_t* xadj, const int64_t* adj,
                      int64_t* perm, int64_t* invp);

/*
 * Nested dissection of a general symmetric graph (1-based xadj/adj without
 * self loops): level-structure separators from pseudo-peripheral vertices,
 * recursively, separators last; sets of at most `leaf` vertices ordered by
 * minimum degree.  Like spk_order_nd_grid, a project ordering for findorder!'s
 * orderfunction slot (src/SparseMethod/SpkSparseBase.jl:173-181); the
 * reference has no nested dissection.  perm[new] = old, invp[old] = new.
 */
int spk_order_nd_graph(int64_t nv, const int64_t* xadj, const int64_t* adj, int64_t leaf,
                       int64_t* perm, int64_t* invp);

/* Opaque result of the symbolic phase. */
typedef struct spk_symbolic spk_symbolic;

/*
 * Symbolic factorisation for a symmetric graph and an initial ordering.
 * Replaces SpkSparseBase._symbolicfactor! (src/SparseMethod/SpkSparseBase.jl:193-251):
 * _getetree!, _getpostorder!, _findcolumncounts!, weighted _getpostorder!,
 * _findsupernodes!(maxblocksize), findnonzeroindexs, _symbolicfact!.
 * perm/invp are the ordering before the postorders; the final ordering is
 * returned by spk_symbolic_get.
 */
int spk_symbolic_create(int64_t n, const int64_t* xadj, const int64_t* adj,
                        const int64_t* perm, const int64_t* invp,
                        int64_t maxblocksize, spk_symbolic** out);

/* Sizes: nsuper, nsub (= length(lindx)), nnzl (= xlnz[n+1]-1), nnzu (= xunz[n+1]-1). */
int spk_symbolic_sizes(const spk_symbolic* s, int64_t* nsuper, int64_t* nsub,
                       int64_t* nnzl, int64_t* nnzu);

/*
 * Copy out the arrays (any pointer may be NULL to skip it):
 * perm[n], invp[n] (final ordering), parent[n] (postordered etree, 0 = root),
 * colcnt[n], snode[n], xsuper[nsuper+1], xlindx[nsuper+1], lindx[nsub],
 * xlnz[n+1], xunz[n+1].
 */
int spk_symbolic_get(const spk_symbolic* s, int64_t* perm, int64_t* invp,
                     int64_t* parent, int64_t* colcnt, int64_t* snode,
                     int64_t* xsuper, int64_t* xlindx, int64_t* lindx,
                     int64_t* xlnz, int64_t* xunz);

void spk_symbolic_destroy(spk_symbolic* s);

#ifdef __cplusplus
}
#endif

#endif /* SPK_HOST_H */

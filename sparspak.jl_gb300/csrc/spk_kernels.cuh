// Device kernels of the supernodal LU engine (sm_103a).
//
// Storage.  Consecutive supernodes that form a path of the elimination tree
// (each one's parent is the next) are grouped into a *front*, allowing a
// little padding (structural zeros that stay exactly zero).  A front F owns
// columns f..f+nf-1 and has m off-diagonal rows R_F (global, permuted,
// ascending: the rows of its last supernode below the front).  Its part of
// the factor is
//   Lf: (nf+m) x nf column-major, ld = nf+m: rows 0..nf-1 are the front's own
//       columns (unit-lower L11 below the diagonal, U11 on and above it),
//       rows nf.. are L21;
//   Uf: m x nf column-major (U12 transposed: column k holds U row f+k).
// Without padding this is a permutation of the reference's lnz/unz storage
// (src/SparseMethod/SpkSparseBase.jl:253-284); with padding it holds it.
//
// Pivoting.  Every supernode of the reference partition (a *piece* of a
// front, at most 32 columns) factors its own diagonal block with row
// interchanges restricted to that block, applied to the U rows to its right
// only, exactly as _lufactor! does (src/SparseMethod/SpkLUFactor.jl:229-241).
//
// Schedule.  Fronts are processed by elimination-tree level.  Inside a
// level, piece step s runs a panel kernel (triangular solves of piece s)
// and a trailing kernel (rank-w update of the rest of each front, which
// also factors the next piece's diagonal block); then one kernel forms each
// front's Schur complement L21*U12 and scatter-adds it into the ancestor
// fronts.  Kernel boundaries are the only synchronisation.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "spk_umma.cuh"

namespace spk {

typedef long long ll;

struct DFront {
    ll loff;       // Lf offset in the factor array
    ll uoff;       // Uf offset
    ll rows_off;   // R_F offset in rows[]
    ll runid_off;  // offset of the per-row run ids in runid[]
    int f;         // first column (0-based, permuted)
    int nf;        // columns
    int m;         // off-diagonal rows
    int ld;        // nf + m
    int piece0;    // first supernode (0-based) of the front
    int npieces;
    int run0;      // first run of the front in run_*[]
    int block0;    // first block of the front (in the plan's block arrays)
    int nblocks;
    int sq;        // update-row tiles (128 rows) holding the rows that fronts of the next level own (schur_part_tile)
};

// A run is a maximal stretch of R_F lying in the columns of one ancestor
// front G; rel[] gives, for every row of R_F from the run's start on, its
// position in G's row list (G's columns, then R_G).
struct Sched {
    const DFront* fronts;
    const int* xsuper;     // 0-based first column of each supernode, [nsuper+1]
    const int* rows;       // concatenated R_F
    const int* runid;      // run index (absolute) per row of each R_F
    const int* run_tgt;    // target front of each run
    const int* run_start;  // first row (local to R_F) of each run
    const ll* run_rel;     // offset in rel[] of the run's first row
    const int* rel;
    const int* blk_c0;     // front-local first column of each block
    const int* blk_c1;     // front-local end column of each block
    const int* blk_p0;     // first supernode (0-based) of each block
    const int* blk_np;     // supernodes in the block
    const ll* blk_inv2;    // offset in inv2[] of the block's Minv (then Uinv), bw x bw each
    const ll* blk_lpack;   // byte offset of the block's packed L panel (FP32 tensor-core fronts), -1 if none
    const ll* blk_upack;   // byte offset of the block's packed U panel, -1 if none
    // 1: the symmetric form for SPD matrices (POTRF-like: no interchanges;
    // only the lower part of every update is formed, SYRK-like; the U side,
    // U = D L^T, is written from the L panel; LU storage otherwise)
    int sym;
};

// One launch = a list of fronts and the prefix sum of their tile counts.
struct Launch {
    const int* front_ids;
    const int* prefix;     // [count+1]
    int count;
};

__device__ __forceinline__ void locate(const Launch& L, int bid, int& fid, int& tile) {
    int lo = 0, hi = L.count - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (L.prefix[mid] <= bid) lo = mid; else hi = mid - 1;
    }
    fid = L.front_ids[lo];
    tile = bid - L.prefix[lo];
}

__host__ __device__ __forceinline__ int cdiv(int a, int b) { return (a + b - 1) / b; }

// Programmatic dependent launch, for kernels that form a dependent chain:
// griddep_launch lets the next kernel of the stream launch once every CTA of
// this one has started; griddep_wait blocks until the previous kernel has
// completed and its writes are visible (immediately when there is no such
// dependency).  A kernel issues the loads that do not depend on its
// predecessor before waiting.
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename T> __device__ __forceinline__ T tabs(T x) { return x < T(0) ? -x : x; }

// Widest supernode handled.  The reference's splitting rule
// (src/SparseSpdMethod/SpkSymFct.jl:432-460) caps pieces near maxblocksize
// but lets the last piece of a long chain reach about 1.5x that (46 for 30).
constexpr int MAXW = 64;

// ---------------------------------------------------------------------------
// Blocks.  The pieces of a front are processed in *blocks* of consecutive
// pieces (at most BlockMax<T> columns).  A block step is: the block LU
// (k_block_lu / k_block_lu_small) with exactly the reference's in-piece
// pivoting, then the block's two panels (k_block_panel), then the trailing
// update of the front (k_block_trail).  After the factorisation
// k_block_inv forms, per block, the two operators the triangular solves
// apply: Minv = inv(L_B) P_B and Uinv = inv(U_B) (below).
// ---------------------------------------------------------------------------
template <typename T> struct BlockMax;
template <> struct BlockMax<float> { static constexpr int value = 128; };
template <> struct BlockMax<double> { static constexpr int value = 64; };


// Order-preserving pivot key of |x| for a candidate row (larger key = larger
// |x|, all candidates above non-candidates), with the ggetrf! rules: a NaN
// never wins, except on the diagonal row k, where nothing can displace it.
__device__ __forceinline__ unsigned long long pivot_key(float x, bool cand, bool diag) {
    if (!cand) return 0ull;
    unsigned b = __float_as_uint(x) & 0x7fffffffu;
    if (b > 0x7f800000u) return diag ? ~0ull : 1ull;   // NaN
    return (unsigned long long)b + 2ull;
}
__device__ __forceinline__ unsigned long long pivot_key(double x, bool cand, bool diag) {
    if (!cand) return 0ull;
    unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
    if (b > 0x7ff0000000000000ull) return diag ? ~0ull : 1ull;
    return b + 2ull;
}

// First lane holding the largest key (the reference's first strict maximum).
__device__ __forceinline__ int warp_first_max(unsigned long long key) {
    const unsigned FULL = 0xffffffffu;
    const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
    const unsigned mh = __reduce_max_sync(FULL, hi);
    const unsigned ml = __reduce_max_sync(FULL, hi == mh ? lo : 0u);
    const unsigned ballot = __ballot_sync(FULL, hi == mh && lo == ml);
    return __ffs(ballot) - 1;
}

// Correctly rounded reciprocal (the value of T(1) / x).
__device__ __forceinline__ float rcp_rn(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double rcp_rn(double x) { return __drcp_rn(x); }

// Scaling factor 1 / pivot of the FP32 block LU: the hardware reciprocal
// (within 2 ulp; the FP32 factor is refined in FP64); FP64 keeps the
// correctly rounded one.
__device__ __forceinline__ float lu_recip(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ double lu_recip(double x) { return rcp_rn(x); }

// The pivot lane of a column (first strict maximum of |x| among the
// candidates, pivot_key's rules): one 32-bit reduction for FP32, two for FP64.
__device__ __forceinline__ int warp_pivot_lane(float x, bool cand, bool diag) {
    unsigned key = 0u;
    if (cand) {
        const unsigned b = __float_as_uint(x) & 0x7fffffffu;
        key = b > 0x7f800000u ? (diag ? 0xffffffffu : 1u) : b + 2u;
    }
    const unsigned m = __reduce_max_sync(0xffffffffu, key);
    return __ffs(__ballot_sync(0xffffffffu, key == m)) - 1;
}
__device__ __forceinline__ int warp_pivot_lane(double x, bool cand, bool diag) {
    return warp_first_max(pivot_key(x, cand, diag));
}

// r[k] for a runtime k without indexing a register array dynamically: a
// tree of selects (depth log2 W instead of a W-long chain); W a power of 2.
template <int W, typename T>
__device__ __forceinline__ T pickw(const T (&r)[W], int k) {
    if constexpr (W == 1) {
        return r[0];
    } else {
        T h[W / 2];
#pragma unroll
        for (int i = 0; i < W / 2; ++i) h[i] = (k & (W / 2)) ? r[i + W / 2] : r[i];
        return pickw<W / 2>(h, k);
    }
}
template <typename T>
__device__ __forceinline__ T pick32(const T (&r)[32], int k) { return pickw<32>(r, k); }

// One right-looking LU sweep over the columns [0, ncols) of a register block
// held one row per lane (rows/columns below 32).  For column k in piece
// [a, b): pivot = first strict maximum among rows [k, b) (ggetrf!), whole
// rows interchanged over columns [a, 32) (the piece's columns, then
// _luswap! of its U rows), column k scaled below the diagonal (ggetrf!
// scaling, and the L-panel trsm 'r','u','n','n' for rows past the piece),
// rank-1 update of rows and columns after k (ggetrf!, the U-panel trsm
// 'r','l','t','u' and the block-local update).  `nrows` rows take part;
// W (a power of 2, at most 32) bounds the columns held.
template <typename T, int W>
__device__ bool warp_lu_sweep(T (&r)[W], int nrows, int ncols, const int* q0, int* piv, bool sym) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    bool sing = false;
    int pc = 0;
    if constexpr (W <= 8) {
        // Narrow blocks: unrolled over the column index, so that r[k] and the
        // columns after k are compile-time registers.
#pragma unroll
        for (int k = 0; k < W; ++k) {
            if (k < ncols) {
                while (q0[pc + 1] <= k) ++pc;
                const int a = q0[pc], b = q0[pc + 1];
                const int kp = warp_pivot_lane(r[k], sym ? lane == k : (lane >= k && lane < b), lane == k);
                if (lane == 0) piv[k] = kp - a;
                const T pv = __shfl_sync(FULL, r[k], kp);
                if (pv != T(0)) {
                    if (kp != k) {
#pragma unroll
                        for (int j = 0; j < W; ++j) {
                            const T vk = __shfl_sync(FULL, r[j], k), vp = __shfl_sync(FULL, r[j], kp);
                            if (j >= a) {
                                if (lane == k) r[j] = vp;
                                else if (lane == kp) r[j] = vk;
                            }
                        }
                    }
                    const T inv = lu_recip(pv);
                    if (lane > k && lane < nrows) r[k] *= inv;
                } else {
                    sing = true;
                }
                const T lk = r[k];
                const bool upd = lane > k && lane < nrows;
#pragma unroll
                for (int j = k + 1; j < W; ++j) {
                    const T u = __shfl_sync(FULL, r[j], k);
                    if (upd) r[j] -= lk * u;
                }
            }
        }
    } else {
        // Wider blocks: a rolled loop (the unrolled form's code outgrows the
        // instruction cache), r[k] picked by a tree of selects.
#pragma unroll 1
        for (int k = 0; k < ncols; ++k) {
            while (q0[pc + 1] <= k) ++pc;
            const int a = q0[pc], b = q0[pc + 1];
            const T rk0 = pickw<W>(r, k);
            const int kp = warp_pivot_lane(rk0, sym ? lane == k : (lane >= k && lane < b), lane == k);
            if (lane == 0) piv[k] = kp - a;
            const T pv = __shfl_sync(FULL, rk0, kp);
            if (pv != T(0)) {
                if (kp != k) {
#pragma unroll
                    for (int j = 0; j < W; ++j) {
                        const T vk = __shfl_sync(FULL, r[j], k), vp = __shfl_sync(FULL, r[j], kp);
                        if (j >= a) {
                            if (lane == k) r[j] = vp;
                            else if (lane == kp) r[j] = vk;
                        }
                    }
                }
                const T inv = lu_recip(pv);
                if (lane > k && lane < nrows) {
#pragma unroll
                    for (int j = 0; j < W; ++j)
                        if (j == k) r[j] *= inv;
                }
            } else {
                sing = true;
            }
            const T lk = pickw<W>(r, k);
            const bool upd = lane > k && lane < nrows;
#pragma unroll
            for (int j = 0; j < W; ++j) {
                const T u = __shfl_sync(FULL, r[j], k);
                if (upd && j > k) r[j] -= lk * u;
            }
        }
    }
    return sing;
}

// A whole block of at most 32 columns factored by one warp in registers
// (lane i holds row i) as one right-looking sweep over its columns.  For
// column k in piece [a, b): the pivot is the first strict maximum among rows
// [k, b) (ggetrf!), the interchange moves whole rows over columns [a, bw)
// (the piece's own columns, then _luswap! of its U rows), column k is scaled
// below the diagonal (ggetrf! scaling for rows in the piece, the L-panel
// trsm 'r','u','n','n' for rows below it) and the rank-1 update covers rows
// and columns after k (ggetrf!, the U-panel trsm 'r','l','t','u' and the
// block-local update).  Columns left of the piece are never interchanged.
template <typename T, int W = 32>
__device__ bool warp_block_lu32(T* A, int lda, int bw, const int* q0, int np, int* piv, bool sym) {
    const int lane = threadIdx.x & 31;
    (void)np;
    T r[W];
#pragma unroll
    for (int j = 0; j < W; ++j) r[j] = (lane < bw && j < bw) ? A[j * lda + lane] : T(0);
    const bool sing = warp_lu_sweep<T, W>(r, bw, bw, q0, piv, sym);
    if (lane < bw) {
#pragma unroll
        for (int j = 0; j < W; ++j)
            if (j < bw) A[j * lda + lane] = r[j];
    }
    __syncwarp();
    return sing;
}

// Blocks of at most 32 columns: one warp per block, four blocks per CTA (the
// launch holds one block per front).  Same outputs as k_block_lu.
template <typename T>
__global__ void __launch_bounds__(128) k_block_lu_small(T* fac, int* ipiv, int* info, Sched S, Launch L, int step) {
    __shared__ T sA[4][32 * 33];
    __shared__ int sq[4][33];
    __shared__ int spiv[4][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int idx = blockIdx.x * 4 + warp;
    if (idx >= L.count) return;
    const DFront F = S.fronts[L.front_ids[idx]];
    const int blk = F.block0 + step;
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk], bw = c1 - c0, lda = 33;
    const int p0 = S.blk_p0[blk], np = S.blk_np[blk];
    T* A = sA[warp];
    int* q0 = sq[warp];
    int* piv = spiv[warp];
    for (int k = lane; k <= np; k += 32) q0[k] = S.xsuper[p0 + k] - F.f - c0;
    for (int j = 0; j < bw; ++j)   // symmetric form: the upper triangle mirrors the lower one
        if (lane < bw)
            A[j * lda + lane] = (S.sym && lane < j) ? fac[F.loff + (ll)(c0 + lane) * F.ld + c0 + j]
                                                    : fac[F.loff + (ll)(c0 + j) * F.ld + c0 + lane];
    __syncwarp();
    const bool sing = warp_block_lu32(A, lda, bw, q0, np, piv, S.sym != 0);
    for (int j = 0; j < bw; ++j)
        if (lane < bw) fac[F.loff + (ll)(c0 + j) * F.ld + c0 + lane] = A[j * lda + lane];
    if (lane < bw) ipiv[F.f + c0 + lane] = piv[lane];
    if (lane == 0 && sing) {   // sing is uniform across the warp
        for (int pc = 0; pc < np; ++pc) {
            bool z = false;
            for (int k = q0[pc]; k < q0[pc + 1]; ++k) z |= A[k * lda + k] == T(0);
            if (z) { atomicMin(info, p0 + pc + 1); break; }
        }
    }
}

// First row holding the largest key (`idx` the row of this lane's key):
// the reference's first strict maximum.
__device__ __forceinline__ int warp_first_max_row(unsigned long long key, int idx) {
    const unsigned FULL = 0xffffffffu;
    const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
    const unsigned mh = __reduce_max_sync(FULL, hi);
    const unsigned ml = __reduce_max_sync(FULL, hi == mh ? lo : 0u);
    return (int)__reduce_min_sync(FULL, (hi == mh && lo == ml) ? (unsigned)idx : 0xffffffffu);
}
__device__ __forceinline__ int warp_first_max_row(unsigned key, int idx) {
    const unsigned FULL = 0xffffffffu;
    const unsigned m = __reduce_max_sync(FULL, key);
    return (int)__reduce_min_sync(FULL, key == m ? (unsigned)idx : 0xffffffffu);
}
// 32-bit pivot key of a float (same order as pivot_key).
__device__ __forceinline__ unsigned pivot_key32(float x, bool cand, bool diag) {
    if (!cand) return 0u;
    const unsigned b = __float_as_uint(x) & 0x7fffffffu;
    if (b > 0x7f800000u) return diag ? 0xffffffffu : 1u;
    return b + 2u;
}
template <typename T> struct PivotKey;
template <> struct PivotKey<float> {
    using type = unsigned;
    __device__ static type of(float x, bool cand, bool diag) { return pivot_key32(x, cand, diag); }
};
template <> struct PivotKey<double> {
    using type = unsigned long long;
    __device__ static type of(double x, bool cand, bool diag) { return pivot_key(x, cand, diag); }
};

// Row sources of a block's interchanges: applying, piece by piece, the
// swaps k <-> a + ipiv[k] of the piece [a, b) to a vector v gives
// v'[R] = v[gmap[R]]; pa[R] = first row of R's piece.  One thread per piece.
__device__ __forceinline__ void block_gather_map(const int* ipiv_blk, const int* q0, int np, int* gmap, int* pa) {
    for (int pc = threadIdx.x; pc < np; pc += blockDim.x) {
        const int a = q0[pc], b = q0[pc + 1];
        for (int i = a; i < b; ++i) {
            gmap[i] = i;
            pa[i] = a;
        }
        for (int k = a; k < b; ++k) {
            const int kp = a + ipiv_blk[k];
            const int t = gmap[k];
            gmap[k] = gmap[kp];
            gmap[kp] = t;
        }
    }
}


// Block LU by a whole CTA (blocks of 33..BlockMax columns; one CTA per
// front).  Warp w holds the column group [4w, 4w+4) of the block, lane l the
// rows [RPT l, RPT l + RPT) (RPT = BlockMax / 32), in registers.  The block
// is factored one column group at a time:
//   A. the group's owner warp factors its four columns in order, on its own
//      (shuffles only): for column k in piece [a, b), the pivot is the first
//      strict maximum of |A(i,k)| over the piece's rows i in [k, b)
//      (ggetrf!; a NaN never wins except on the diagonal); a nonzero pivot
//      off the diagonal swaps rows k and kp over the group's columns >= a
//      (ggetrf! inside the piece; columns left of the piece never move); the
//      rows after k are scaled by 1 / pivot (ggetrf! scaling, the L-panel
//      trsm 'r','u','n','n' for the block's later rows; no scaling after a
//      zero pivot) and the group's later columns get the rank-1 update.  The
//      multipliers and pivots go to shared memory;
//   B. every later warp applies, column by column in the same order, the
//      swap (_luswap! of the U rows) and the rank-1 update (the U-panel trsm
//      'r','l','t','u' and the block-local Schur update) to its columns, with
//      row k taken from the owning lane by shuffles: the same operations in
//      the same order as a column-by-column elimination; earlier warps apply
//      the swaps to their columns of the same piece.
// The owner of the next group does its part B first and then its part A, so
// the next panel overlaps the other warps' updates; one barrier per group.
// ipiv receives the local pivot row within the piece; a zero pivot records
// the piece in info.
template <typename T> struct LuThreads { static constexpr int value = (BlockMax<T>::value / 4) * 32; };

template <typename T, int RPT>
__device__ __forceinline__ T lu_pick(const T (&a)[RPT][4], int ii, int jj) {
    T v = a[0][jj];
#pragma unroll
    for (int q = 1; q < RPT; ++q) v = (ii == q) ? a[q][jj] : v;
    return v;
}


// Part A for the group of warp `g` (called by that warp only).  cpa / cpb:
// first and end column of each column's piece.
template <typename T, int RPT>
__device__ __forceinline__ void lu_group_factor(T (&a)[RPT][4], int g, int bw, const int* cpa, const int* cpb, T* lb,
                                                int* skp, T* spv, int* sa0, int* spiv, int* szero, bool sym) {
    using Key = typename PivotKey<T>::type;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, r0 = RPT * lane;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int k = 4 * g + j;
        if (k >= bw) continue;
        const int a0 = cpa[k], b = cpb[k];
        Key best = 0;
        int brow = 0;
#pragma unroll
        for (int ii = 0; ii < RPT; ++ii) {   // rows in ascending order: ties keep the earlier row
            const int R = r0 + ii;
            const Key kv = PivotKey<T>::of(a[ii][j], sym ? R == k : (R >= k && R < b), R == k);
            if (ii == 0 || kv > best) { best = kv; brow = R; }
        }
        const int kp = warp_first_max_row(best, brow);
        const int lk = (4 * g) / RPT + j / RPT, ik = j % RPT, lp = kp / RPT, ip = kp % RPT;   // k = 4g + j
        const T pv = __shfl_sync(FULL, lu_pick(a, ip, j), lp);
        const bool scale = pv != T(0);
        if (scale && kp != k) {   // swap rows k and kp over the group's columns >= a0
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
                const T vk = __shfl_sync(FULL, a[ik][jj], lk);
                const T vp = __shfl_sync(FULL, lu_pick(a, ip, jj), lp);
                if (4 * g + jj >= a0) {
#pragma unroll
                    for (int ii = 0; ii < RPT; ++ii) {
                        if (lane == lk && ii == ik) a[ii][jj] = vp;
                        if (lane == lp && ii == ip) a[ii][jj] = vk;
                    }
                }
            }
        }
        const T rinv = scale ? lu_recip(pv) : T(1);
#pragma unroll
        for (int ii = 0; ii < RPT; ++ii) {
            const int R = r0 + ii;
            if (R > k) {
                if (scale) a[ii][j] *= rinv;
                lb[j * (32 * RPT) + R] = a[ii][j];
            }
        }
#pragma unroll
        for (int jj = j + 1; jj < 4; ++jj) {   // rank-1 update of the group's later columns
            const T u = __shfl_sync(FULL, a[ik][jj], lk);
#pragma unroll
            for (int ii = 0; ii < RPT; ++ii)
                if (r0 + ii > k) a[ii][jj] -= a[ii][j] * u;
        }
        if (lane == 0) {
            skp[j] = kp;
            spv[j] = pv;
            sa0[j] = a0;
            spiv[k] = kp - a0;
            if (!scale && k < *szero) *szero = k;
        }
    }
}

// Part B of group `g` for a later warp.
template <typename T, int RPT>
__device__ __forceinline__ void lu_group_update(T (&a)[RPT][4], int g, int bw, const T* lb, const int* skp, const T* spv) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, r0 = RPT * lane;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int k = 4 * g + j;
        if (k >= bw) continue;
        const int kp = skp[j];
        const T pv = spv[j];
        const int lk = (4 * g) / RPT + j / RPT, ik = j % RPT;   // k = 4g + j
        if (pv != T(0) && kp != k) {   // all columns here are after k, hence >= a0
            const int lp = kp / RPT, ip = kp % RPT;
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) {
                const T vk = __shfl_sync(FULL, a[ik][jj], lk);
                const T vp = __shfl_sync(FULL, lu_pick(a, ip, jj), lp);
#pragma unroll
                for (int ii = 0; ii < RPT; ++ii) {
                    if (lane == lk && ii == ik) a[ii][jj] = vp;
                    if (lane == lp && ii == ip) a[ii][jj] = vk;
                }
            }
        }
        T l[RPT];
#pragma unroll
        for (int ii = 0; ii < RPT; ++ii) l[ii] = lb[j * (32 * RPT) + r0 + ii];
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            const T u = __shfl_sync(FULL, a[ik][jj], lk);
#pragma unroll
            for (int ii = 0; ii < RPT; ++ii)
                if (r0 + ii > k) a[ii][jj] -= l[ii] * u;
        }
    }
}

// The swaps of group `g` for an earlier warp: its columns of the same piece
// (>= the piece's first column) hold L entries that move with the rows.
template <typename T, int RPT>
__device__ __forceinline__ void lu_group_swap_left(T (&a)[RPT][4], int g, int bw, const int* skp, const T* spv,
                                                   const int* sa0) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int k = 4 * g + j;
        if (k >= bw) continue;
        const int kp = skp[j], a0 = sa0[j];
        if (spv[j] == T(0) || kp == k || 4 * w + 3 < a0) continue;   // uniform in the warp
        const int lk = (4 * g) / RPT + j / RPT, ik = j % RPT, lp = kp / RPT, ip = kp % RPT;   // k = 4g + j
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            const T vk = __shfl_sync(FULL, a[ik][jj], lk);
            const T vp = __shfl_sync(FULL, lu_pick(a, ip, jj), lp);
            if (4 * w + jj >= a0) {
#pragma unroll
                for (int ii = 0; ii < RPT; ++ii) {
                    if (lane == lk && ii == ik) a[ii][jj] = vp;
                    if (lane == lp && ii == ip) a[ii][jj] = vk;
                }
            }
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(LuThreads<T>::value, 1) k_block_lu(T* fac, int* ipiv, int* info, int* bmap, Sched S,
                                                                      Launch L, int step) {
    constexpr int BM = BlockMax<T>::value, RPT = BM / 32;
    __shared__ __align__(16) T lbuf[2][4 * BM];   // the group's multipliers by column and row (by group parity)
    __shared__ T s_pv[2][4];
    __shared__ int s_kp[2][4], s_a0[2][4];
    __shared__ int q0[BM + 1];
    __shared__ int spiv[BM], sgmap[BM], cpa[BM], cpb[BM];
    __shared__ int szero;
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int blk = F.block0 + step;
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk], bw = c1 - c0;
    const int p0 = S.blk_p0[blk], np = S.blk_np[blk];
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int r0 = RPT * lane, cl0 = 4 * w;
    for (int k = tid; k <= np; k += blockDim.x) q0[k] = S.xsuper[p0 + k] - F.f - c0;
    if (tid == 0) szero = INT_MAX;
    __syncthreads();
    for (int pc = tid; pc < np; pc += blockDim.x)
        for (int k = q0[pc]; k < q0[pc + 1]; ++k) {
            cpa[k] = q0[pc];
            cpb[k] = q0[pc + 1];
        }
    T* blkp = fac + F.loff + (ll)c0 * F.ld + c0;   // block (i, j) at blkp[j * ld + i]
    T a[RPT][4];
#pragma unroll
    for (int jj = 0; jj < 4; ++jj)
#pragma unroll
        for (int ii = 0; ii < RPT; ++ii) {
            const int R = r0 + ii, C = cl0 + jj;
            // symmetric form: the upper triangle mirrors the lower one
            a[ii][jj] = (R < bw && C < bw) ? ((S.sym && R < C) ? blkp[(ll)R * F.ld + C] : blkp[(ll)C * F.ld + R]) : T(0);
        }
    __syncthreads();
    const int ng = cdiv(bw, 4);
    const bool sym = S.sym != 0;
    if (w == 0) lu_group_factor<T, RPT>(a, 0, bw, cpa, cpb, lbuf[0], s_kp[0], s_pv[0], s_a0[0], spiv, &szero, sym);
    __syncthreads();
#pragma unroll 1
    for (int g = 0; g < ng; ++g) {
        const int par = g & 1;
        if (w < g) lu_group_swap_left<T, RPT>(a, g, bw, s_kp[par], s_pv[par], s_a0[par]);
        if (w > g && w < ng) {
            lu_group_update<T, RPT>(a, g, bw, lbuf[par], s_kp[par], s_pv[par]);
            if (w == g + 1)   // the next panel while the other warps update
                lu_group_factor<T, RPT>(a, g + 1, bw, cpa, cpb, lbuf[par ^ 1], s_kp[par ^ 1], s_pv[par ^ 1],
                                        s_a0[par ^ 1], spiv, &szero, sym);
        }
        __syncthreads();
    }
#pragma unroll
    for (int jj = 0; jj < 4; ++jj)
#pragma unroll
        for (int ii = 0; ii < RPT; ++ii) {
            const int R = r0 + ii, C = cl0 + jj;
            if (R < bw && C < bw) blkp[(ll)C * F.ld + R] = a[ii][jj];
        }
    for (int c = tid; c < bw; c += blockDim.x) ipiv[F.f + c0 + c] = spiv[c];
    // Row sources of the block's interchanges (block_gather_map), a warp per
    // piece of at most 32 columns: lane i tracks gmap[a + i] through the
    // piece's swaps.  spiv and q0 were published by the loop's last barrier.
    for (int pc = w; pc < np; pc += blockDim.x / 32) {
        const int a = q0[pc], b = q0[pc + 1];
        if (b - a <= 32) {
            int g = a + lane;
            for (int k = a; k < b; ++k) {
                const int kp = a + spiv[k];
                const int vk = __shfl_sync(0xffffffffu, g, k - a), vp = __shfl_sync(0xffffffffu, g, kp - a);
                g = lane == k - a ? vp : (lane == kp - a ? vk : g);
            }
            if (lane < b - a) bmap[F.f + c0 + a + lane] = g | (a << 8);
        } else if (lane == 0) {
            for (int i = a; i < b; ++i) sgmap[i] = i;
            for (int k = a; k < b; ++k) {
                const int kp = a + spiv[k];
                const int t = sgmap[k];
                sgmap[k] = sgmap[kp];
                sgmap[kp] = t;
            }
            for (int i = a; i < b; ++i) bmap[F.f + c0 + i] = sgmap[i] | (a << 8);
        }
    }
    if (tid == 0 && szero != INT_MAX) {
        int p = 0;
        while (q0[p + 1] <= szero) ++p;
        atomicMin(info, p0 + p + 1);   // first singular piece of the block
    }
}

// Block LU by pieces, for blocks whose pieces are all at most 32 columns
// wide (the supernode partition's maxblocksize, 30 by default).  The
// block is staged in shared memory; for each piece [a, b) in turn:
//   (1) one warp factors the piece's diagonal block in registers
//       (warp_lu_sweep: ggetrf!, pivots among the piece's rows);
//   (2) a thread per column right of the piece applies the piece's
//       interchanges and solves U12 := inv(L11) P A12 (_luswap!, trsm
//       'l','l','n','u'), and a thread per row below it solves
//       L21 := A21 inv(U11) (trsm 'r','u','n','n');
//   (3) the rest of the block takes the rank-w update A22 -= L21 U12 (gemm),
//       a warp per four columns with its lanes on the rows.
// Only the w rows of the piece are on the sequential path of (1); the rows
// below are solved in parallel afterwards, which is where this form gains
// over k_block_lu (whose owner warp sweeps all rows of the block for every
// column).  Same outputs as k_block_lu: the factored block, ipiv, the row
// sources of the interchanges (bmap) and the first singular piece.
constexpr int PC_THREADS = 512;
template <typename T> struct PcLu {
    static constexpr int BM = BlockMax<T>::value;
    static constexpr int LDS = BM + 1;   // column stride of the staged block (conflict-free rows and columns)
    static constexpr size_t smem = sizeof(T) * ((size_t)BM * LDS + (size_t)32 * BM + 32);
};

template <typename T>
__global__ void __launch_bounds__(PC_THREADS, 1) k_block_lu_pc(T* fac, int* ipiv, int* info, int* bmap, Sched S,
                                                                Launch L, int step) {
    constexpr int BM = BlockMax<T>::value, LDS = PcLu<T>::LDS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sA = reinterpret_cast<T*>(smem_raw);   // A(i, j) at sA[j * LDS + i]
    T* sU = sA + BM * LDS;                    // U(a + k, b + c) of the current piece at sU[k * BM + c]
    T* srv = sU + 32 * BM;                    // 1 / U(a + k, a + k)
    __shared__ int q0[BM + 1], spiv[BM], sgm[32], sgmap[BM], sq[2];
    __shared__ int szero;
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int blk = F.block0 + step;
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk], bw = c1 - c0;
    const int p0 = S.blk_p0[blk], np = S.blk_np[blk];
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const bool sym = S.sym != 0;
    for (int k = tid; k <= np; k += PC_THREADS) q0[k] = S.xsuper[p0 + k] - F.f - c0;
    if (tid == 0) szero = INT_MAX;
    T* blkp = fac + F.loff + (ll)c0 * F.ld + c0;   // block (i, j) at blkp[j * ld + i]
    for (int e = tid; e < bw * bw; e += PC_THREADS) {
        const int C = e / bw, R = e - C * bw;
        // symmetric form: the upper triangle mirrors the lower one
        sA[C * LDS + R] = (sym && R < C) ? blkp[(ll)R * F.ld + C] : blkp[(ll)C * F.ld + R];
    }
    __syncthreads();
#pragma unroll 1
    for (int pc = 0; pc < np; ++pc) {
        const int a = q0[pc], b = q0[pc + 1], wd = b - a, nr = bw - b;
        if (w == 0) {   // (1) the piece's diagonal block
            if (lane == 0) {
                sq[0] = 0;
                sq[1] = wd;
            }
            T r[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) r[j] = (lane < wd && j < wd) ? sA[(a + j) * LDS + a + lane] : T(0);
            __syncwarp();
            const bool sing = warp_lu_sweep<T, 32>(r, wd, wd, sq, spiv + a, sym);
#pragma unroll
            for (int j = 0; j < 32; ++j)
                if (lane < wd && j < wd) sA[(a + j) * LDS + a + lane] = r[j];
            const T d = pickw<32>(r, lane);
            if (lane < wd) srv[lane] = d != T(0) ? T(1) / d : T(1);
            if (sing) {   // uniform in the warp
                const unsigned z = __ballot_sync(0xffffffffu, lane < wd && d == T(0));
                if (lane == 0 && z) szero = min(szero, a + __ffs(z) - 1);
            }
            __syncwarp();
            // the row now at position i of the piece came from row sgm[i]
            int g = lane;
            for (int k = 0; k < wd; ++k) {
                const int kp = spiv[a + k];
                const int vk = __shfl_sync(0xffffffffu, g, k), vp = __shfl_sync(0xffffffffu, g, kp);
                g = lane == k ? vp : (lane == kp ? vk : g);
            }
            if (lane < wd) sgm[lane] = g;
        }
        __syncthreads();
        // (2) U12 columns (threads 0..) and L21 rows (threads 256..) inside the block
        if (tid < nr) {
            const int j = b + tid;
            T y[32];
#pragma unroll
            for (int i = 0; i < 32; ++i) y[i] = i < wd ? sA[j * LDS + a + sgm[i]] : T(0);
#pragma unroll
            for (int k = 0; k < 32; ++k)
                if (k < wd) {
#pragma unroll
                    for (int i = k + 1; i < 32; ++i)
                        if (i < wd) y[i] -= sA[(a + k) * LDS + a + i] * y[k];
                }
#pragma unroll
            for (int i = 0; i < 32; ++i)
                if (i < wd) {
                    sA[j * LDS + a + i] = y[i];
                    sU[i * BM + tid] = y[i];
                }
        } else if (tid >= PC_THREADS / 2 && tid - PC_THREADS / 2 < nr) {
            const int rr = b + tid - PC_THREADS / 2;
            T x[32];
#pragma unroll
            for (int k = 0; k < 32; ++k) x[k] = k < wd ? sA[(a + k) * LDS + rr] : T(0);
#pragma unroll
            for (int k = 0; k < 32; ++k)
                if (k < wd) {
                    x[k] *= srv[k];
#pragma unroll
                    for (int jj = k + 1; jj < 32; ++jj)
                        if (jj < wd) x[jj] -= x[k] * sA[(a + jj) * LDS + a + k];
                }
#pragma unroll
            for (int k = 0; k < 32; ++k)
                if (k < wd) sA[(a + k) * LDS + rr] = x[k];
        }
        __syncthreads();
        // (3) A22 -= L21 U12: warp per four columns, lane + 32 q on the rows
        if (nr > 0) {
            const int ncg = cdiv(nr, 4);
            for (int cg = w; cg < ncg; cg += PC_THREADS / 32) {
                const int j0 = 4 * cg;
                T acc[4][4];
#pragma unroll
                for (int q = 0; q < 4; ++q)
#pragma unroll
                    for (int c = 0; c < 4; ++c) acc[q][c] = T(0);
                for (int k = 0; k < wd; ++k) {
                    T l[4], u[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) l[q] = lane + 32 * q < nr ? sA[(a + k) * LDS + b + lane + 32 * q] : T(0);
#pragma unroll
                    for (int c = 0; c < 4; ++c) u[c] = sU[k * BM + j0 + c];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
#pragma unroll
                        for (int c = 0; c < 4; ++c) acc[q][c] += l[q] * u[c];
                }
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    if (j0 + c < nr)
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            if (lane + 32 * q < nr) sA[(b + j0 + c) * LDS + b + lane + 32 * q] -= acc[q][c];
            }
        }
        __syncthreads();
    }
    for (int e = tid; e < bw * bw; e += PC_THREADS) {
        const int C = e / bw, R = e - C * bw;
        blkp[(ll)C * F.ld + R] = sA[C * LDS + R];
    }
    for (int c = tid; c < bw; c += PC_THREADS) ipiv[F.f + c0 + c] = spiv[c];
    // Row sources of the block's interchanges (block_gather_map), a warp per
    // piece: lane i tracks gmap[a + i] through the piece's swaps.
    for (int pc = w; pc < np; pc += PC_THREADS / 32) {
        const int a = q0[pc], b = q0[pc + 1];
        int g = a + lane;
        for (int k = a; k < b; ++k) {
            const int kp = a + spiv[k];
            const int vk = __shfl_sync(0xffffffffu, g, k - a), vp = __shfl_sync(0xffffffffu, g, kp - a);
            g = lane == k - a ? vp : (lane == kp - a ? vk : g);
        }
        if (lane < b - a) bmap[F.f + c0 + a + lane] = g | (a << 8);
    }
    (void)sgmap;
    if (tid == 0 && szero != INT_MAX) {
        int p = 0;
        while (q0[p + 1] <= szero) ++p;
        atomicMin(info, p0 + p + 1);   // first singular piece of the block
    }
}

// ---------------------------------------------------------------------------
// Panel sweeps on register lines.  A line (a row of X or a column of Y) of
// a block of width bw <= W is held by 4 consecutive lanes, lane q of the
// group owning entries [q*CQ, q*CQ + CQ), CQ = W / 4.  Column by column the
// owner of entry k scales it (rows) and shuffles it to its group, and every
// lane updates its entries with a row of U or a column of L read from
// shared memory (the triangles are staged with zeros outside the strict
// part, so the updates need no predicates).
//   rows: X := X inv(U_B), U_B the block's upper triangle with its diagonal:
//         sU by rows, zero on and below the diagonal, rd[k] = 1/U(k,k);
//   cols: Y := inv(L_B) Y, L_B the block's unit lower triangle: sL by
//         columns, zero on and above the diagonal.
// A staged row (column) is SLD(W) entries: the four lanes' chunks of CQ
// entries each start 16 bytes apart in the bank cycle (chunk q at
// q * (CQ + SK)), so their 16-byte loads do not collide; one more 16-byte
// unit per row puts consecutive rows 20 words apart in the 32-bank cycle, so
// that the staging copies of 8 rows x 4 entries per warp hit 32 banks.
// ---------------------------------------------------------------------------
template <typename T> struct Skew { static constexpr int value = 16 / sizeof(T); };
template <typename T, int W> struct SLD { static constexpr int value = W + 5 * Skew<T>::value; };
template <typename T, int W>
__device__ __forceinline__ int sidx(int k, int j) {   // entry j of staged row / column k
    constexpr int CQ = W / 4, SK = Skew<T>::value;
    return k * SLD<T, W>::value + (j / CQ) * (CQ + SK) + (j % CQ);
}

template <typename T, int W>
__device__ __forceinline__ void sweep_rows(T (&x)[W / 4], const T* sU, const T* rd, int bw) {
    constexpr int CQ = W / 4;
    const int lane = threadIdx.x & 31, q = lane & 3, base = lane & ~3;
#pragma unroll 1
    for (int kq = 0; kq * CQ < bw; ++kq) {
#pragma unroll
        for (int kk = 0; kk < CQ; ++kk) {
            const int k = kq * CQ + kk;
            if (k >= bw) break;
            if (q == kq) x[kk] *= rd[k];
            const T xk = __shfl_sync(0xffffffffu, x[kk], base | kq);
            const T* u = sU + k * SLD<T, W>::value + q * (CQ + Skew<T>::value);
#pragma unroll
            for (int jj = 0; jj < CQ; ++jj) x[jj] -= xk * u[jj];
        }
    }
}

template <typename T, int W>
__device__ __forceinline__ void sweep_cols(T (&y)[W / 4], const T* sL, int bw) {
    constexpr int CQ = W / 4;
    const int lane = threadIdx.x & 31, q = lane & 3, base = lane & ~3;
#pragma unroll 1
    for (int kq = 0; kq * CQ < bw; ++kq) {
#pragma unroll
        for (int kk = 0; kk < CQ; ++kk) {
            const int k = kq * CQ + kk;
            if (k >= bw) break;
            const T yk = __shfl_sync(0xffffffffu, y[kk], base | kq);
            const T* l = sL + k * SLD<T, W>::value + q * (CQ + Skew<T>::value);
#pragma unroll
            for (int ii = 0; ii < CQ; ++ii) y[ii] -= l[ii] * yk;
        }
    }
}

// The same sweeps for W = 128 with four lines per lane: the 16 lanes of a
// half-warp share four lines, lane c holding entries [8c, 8c + 8) of each,
// so that a staged row (column) read from shared memory serves four lines
// (two 16-byte loads per lane and step instead of eight; the staged layout
// sidx<float, 128> puts the eight chunks of a quarter-warp in distinct bank
// quads).  The owner of entry k shuffles its four values to the half-warp.
__device__ __forceinline__ void sweep_rows4(float (&x)[4][8], const float* sU, const float* rd, int bw, int kc_end) {
    // Steps past bw are no-ops (zero staged rows, rd = 0, zero entries), so
    // whole chunks of 8 run unguarded; the next step's row and rd are loaded
    // one step ahead, and the update of the next step's pivot entry comes
    // first.  Chunks [0, kc_end) only.
    const int lane = threadIdx.x & 31, c = lane & 15, base = lane & 16;
    const int nk = min(cdiv(bw, 8), kc_end);
    float4 n0 = *reinterpret_cast<const float4*>(sU + sidx<float, 128>(0, 8 * c));
    float4 n1 = *reinterpret_cast<const float4*>(sU + sidx<float, 128>(0, 8 * c) + 4);
    float nr = rd[0];
#pragma unroll 1
    for (int kc = 0; kc < nk; ++kc) {
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
            const int k = kc * 8 + kk;
            const float4 u0 = n0, u1 = n1;
            const float r = nr;
            const int kn = k + 1 < 128 ? k + 1 : k;
            n0 = *reinterpret_cast<const float4*>(sU + sidx<float, 128>(kn, 8 * c));
            n1 = *reinterpret_cast<const float4*>(sU + sidx<float, 128>(kn, 8 * c) + 4);
            nr = rd[kn];
            float xk[4];
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                if (c == kc) x[l][kk] *= r;
                xk[l] = __shfl_sync(0xffffffffu, x[l][kk], base | kc);
            }
            const float uv[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
            const int jn = (kk + 1) & 7;
#pragma unroll
            for (int l = 0; l < 4; ++l) x[l][jn] -= xk[l] * uv[jn];
#pragma unroll
            for (int l = 0; l < 4; ++l)
#pragma unroll
                for (int jj = 0; jj < 8; ++jj)
                    if (jj != jn) x[l][jj] -= xk[l] * uv[jj];
        }
    }
}

__device__ __forceinline__ void sweep_cols4(float (&y)[4][8], const float* sL, int bw, int kc_end) {
    const int lane = threadIdx.x & 31, c = lane & 15, base = lane & 16;
    const int nk = min(cdiv(bw, 8), kc_end);
    float4 n0 = *reinterpret_cast<const float4*>(sL + sidx<float, 128>(0, 8 * c));
    float4 n1 = *reinterpret_cast<const float4*>(sL + sidx<float, 128>(0, 8 * c) + 4);
#pragma unroll 1
    for (int kc = 0; kc < nk; ++kc) {
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
            const int k = kc * 8 + kk;
            const float4 l0 = n0, l1 = n1;
            const int kn = k + 1 < 128 ? k + 1 : k;
            n0 = *reinterpret_cast<const float4*>(sL + sidx<float, 128>(kn, 8 * c));
            n1 = *reinterpret_cast<const float4*>(sL + sidx<float, 128>(kn, 8 * c) + 4);
            float yk[4];
#pragma unroll
            for (int l = 0; l < 4; ++l) yk[l] = __shfl_sync(0xffffffffu, y[l][kk], base | kc);
            const float lv[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
            const int jn = (kk + 1) & 7;
#pragma unroll
            for (int l = 0; l < 4; ++l) y[l][jn] -= lv[jn] * yk[l];
#pragma unroll
            for (int l = 0; l < 4; ++l)
#pragma unroll
                for (int ii = 0; ii < 8; ++ii)
                    if (ii != jn) y[l][ii] -= lv[ii] * yk[l];
        }
    }
}

// Second phase of the 128-wide sweeps: from step 64 on only entries 64..127
// are still updated, so lane c of a half-warp takes entries [64 + 4c,
// 64 + 4c + 4) of the same four lines (moved there from lane 8 + c / 2),
// four per lane instead of eight.  Entries below 64 are final after the
// first phase and stay with their lanes.
__device__ __forceinline__ void sweep_to_hi(const float (&x)[4][8], float (&x2)[4][4]) {
    const int lane = threadIdx.x & 31, c = lane & 15, src = (lane & 16) | (8 + (c >> 1));
#pragma unroll
    for (int l = 0; l < 4; ++l)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float v0 = __shfl_sync(0xffffffffu, x[l][q], src), v1 = __shfl_sync(0xffffffffu, x[l][4 + q], src);
            x2[l][q] = (c & 1) ? v1 : v0;
        }
}

__device__ __forceinline__ void sweep_rows4_hi(float (&x)[4][4], const float* sU, const float* rd, int bw) {
    const int lane = threadIdx.x & 31, c = lane & 15, base = lane & 16;
    const int nk = min(cdiv(bw - 64, 4), 8);   // steps 64..95
    float4 n0 = *reinterpret_cast<const float4*>(sU + sidx<float, 128>(64, 64 + 4 * c));
    float nr = rd[64];
#pragma unroll 1
    for (int kc = 0; kc < nk; ++kc) {
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            const int k = 64 + kc * 4 + kk;
            const float4 u0 = n0;
            const float r = nr;
            const int kn = k + 1 < 128 ? k + 1 : k;
            n0 = *reinterpret_cast<const float4*>(sU + sidx<float, 128>(kn, 64 + 4 * c));
            nr = rd[kn];
            float xk[4];
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                if (c == kc) x[l][kk] *= r;
                xk[l] = __shfl_sync(0xffffffffu, x[l][kk], base | kc);
            }
            const float uv[4] = {u0.x, u0.y, u0.z, u0.w};
            const int jn = (kk + 1) & 3;
#pragma unroll
            for (int l = 0; l < 4; ++l) x[l][jn] -= xk[l] * uv[jn];
#pragma unroll
            for (int l = 0; l < 4; ++l)
#pragma unroll
                for (int jj = 0; jj < 4; ++jj)
                    if (jj != jn) x[l][jj] -= xk[l] * uv[jj];
        }
    }
}

__device__ __forceinline__ void sweep_cols4_hi(float (&y)[4][4], const float* sL, int bw) {
    const int lane = threadIdx.x & 31, c = lane & 15, base = lane & 16;
    const int nk = min(cdiv(bw - 64, 4), 8);   // steps 64..95
    float4 n0 = *reinterpret_cast<const float4*>(sL + sidx<float, 128>(64, 64 + 4 * c));
#pragma unroll 1
    for (int kc = 0; kc < nk; ++kc) {
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            const int k = 64 + kc * 4 + kk;
            const float4 l0 = n0;
            const int kn = k + 1 < 128 ? k + 1 : k;
            n0 = *reinterpret_cast<const float4*>(sL + sidx<float, 128>(kn, 64 + 4 * c));
            float yk[4];
#pragma unroll
            for (int l = 0; l < 4; ++l) yk[l] = __shfl_sync(0xffffffffu, y[l][kk], base | kc);
            const float lv[4] = {l0.x, l0.y, l0.z, l0.w};
            const int jn = (kk + 1) & 3;
#pragma unroll
            for (int l = 0; l < 4; ++l) y[l][jn] -= lv[jn] * yk[l];
#pragma unroll
            for (int l = 0; l < 4; ++l)
#pragma unroll
                for (int ii = 0; ii < 4; ++ii)
                    if (ii != jn) y[l][ii] -= lv[ii] * yk[l];
        }
    }
}

// Third phase, from step 96 on: entries 96..127, lane c taking [96 + 2c,
// 96 + 2c + 2) (moved from lane 8 + c / 2 of the second phase).
__device__ __forceinline__ void sweep_to_top(const float (&x2)[4][4], float (&x3)[4][2]) {
    const int lane = threadIdx.x & 31, c = lane & 15, src = (lane & 16) | (8 + (c >> 1));
#pragma unroll
    for (int l = 0; l < 4; ++l)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const float v0 = __shfl_sync(0xffffffffu, x2[l][q], src), v1 = __shfl_sync(0xffffffffu, x2[l][2 + q], src);
            x3[l][q] = (c & 1) ? v1 : v0;
        }
}

template <bool ROWS>
__device__ __forceinline__ void sweep_top(float (&x)[4][2], const float* sT, const float* rd, int bw) {
    const int lane = threadIdx.x & 31, c = lane & 15, base = lane & 16;
    const int nk = cdiv(bw - 96, 2);
    float2 n0 = *reinterpret_cast<const float2*>(sT + sidx<float, 128>(96, 96 + 2 * c));
    float nr = ROWS ? rd[96] : 0.f;
#pragma unroll 1
    for (int kc = 0; kc < nk; ++kc) {
#pragma unroll
        for (int kk = 0; kk < 2; ++kk) {
            const int k = 96 + kc * 2 + kk;
            const float2 u0 = n0;
            const float r = nr;
            const int kn = k + 1 < 128 ? k + 1 : k;
            n0 = *reinterpret_cast<const float2*>(sT + sidx<float, 128>(kn, 96 + 2 * c));
            if (ROWS) nr = rd[kn];
            float xk[4];
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                if (ROWS && c == kc) x[l][kk] *= r;
                xk[l] = __shfl_sync(0xffffffffu, x[l][kk], base | kc);
            }
            const float uv[2] = {u0.x, u0.y};
            const int jn = (kk + 1) & 1;
#pragma unroll
            for (int l = 0; l < 4; ++l) x[l][jn] -= xk[l] * uv[jn];
#pragma unroll
            for (int l = 0; l < 4; ++l) x[l][kk] -= xk[l] * uv[kk];
        }
    }
}

// Asynchronous element copy global -> shared (cp.async, 4 or 8 bytes); a
// copy with valid = false writes zero and reads nothing.
template <typename T>
__device__ __forceinline__ void cp_elem(T* dst, const T* src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if constexpr (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(valid ? 4 : 0) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src), "r"(valid ? 8 : 0) : "memory");
}
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// sU and rd from the factored block (column-major at blkp, leading dimension
// ld); the triangle is copied asynchronously (the caller waits with
// cp_wait_all and a barrier before using it).
// Staging order: a warp copies 8 consecutive rows k x 4 consecutive entries
// j (global: 4 columns, 32 contiguous bytes each; shared: 32 distinct banks).
template <int W>
__device__ __forceinline__ void stage_coords(int e, int& k, int& j) {
    const int sub = e & 31, b = e >> 5;
    k = (b % (W / 8)) * 8 + (sub & 7);
    j = (b / (W / 8)) * 4 + (sub >> 3);
}

template <typename T, int W>
__device__ __forceinline__ void stage_upper(T* sU, T* rd, const T* blkp, ll ld, int bw) {
    for (int e = threadIdx.x; e < W * W; e += blockDim.x) {
        int k, j;
        stage_coords<W>(e, k, j);
        const bool v = j > k && j < bw;
        cp_elem(&sU[sidx<T, W>(k, j)], v ? blkp + (ll)j * ld + k : blkp, v);
    }
    for (int k = threadIdx.x; k < W; k += blockDim.x) rd[k] = k < bw ? T(1) / blkp[(ll)k * ld + k] : T(0);
    cp_wait_all();
}

// sL from the factored block with the rows of each piece, in the columns
// left of the piece, put in the piece's pivoted order: the interchanges of
// all pieces then act once, as a gather by gmap, before the sweep (the
// reference applies a piece's interchanges when the forward elimination
// reaches it; moving them ahead of the earlier pieces' updates permutes
// those updates' rows the same way).
template <typename T, int W>
__device__ __forceinline__ void stage_lower(T* sL, const T* blkp, ll ld, int bw, const int* gmap, const int* pa) {
    for (int e = threadIdx.x; e < W * W; e += blockDim.x) {
        int k, i;
        stage_coords<W>(e, k, i);
        const bool v = i > k && i < bw;
        cp_elem(&sL[sidx<T, W>(k, i)], v ? blkp + (ll)k * ld + (k < pa[i] ? gmap[i] : i) : blkp, v);
    }
    cp_wait_all();
}

// Packed copy of one panel line for the tensor-core updates (FP32 fronts
// with a pack): the line's entries k < nch * KCH, held CQ per lane from
// q * CQ, split into TF32 hi / lo at tile `t`, line `i` of the block's pack.
template <int CQ>
__device__ __forceinline__ void pack_line(unsigned char* base, int t, int i, int q, int nch, const float (&v)[CQ]) {
#pragma unroll
    for (int g = 0; g < CQ / 4; ++g) {
        const int k = q * CQ + 4 * g;
        if (k < nch * umma::KCH) {
            unsigned char* dst = base + ((ll)t * nch + k / umma::KCH) * umma::PCHUNK + umma::packed_offset(i, k % umma::KCH);
            uint32_t h[4], l[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                h[e] = umma::tf32_rna(v[4 * g + e]);
                l[e] = umma::tf32_rna(v[4 * g + e] - __uint_as_float(h[e]));
            }
            *reinterpret_cast<uint4*>(dst) = make_uint4(h[0], h[1], h[2], h[3]);
            *reinterpret_cast<uint4*>(dst + umma::OPB) = make_uint4(l[0], l[1], l[2], l[3]);
        }
    }
}

// BF16 form of pack_line: the line's entries times `scale` (a power of two)
// as BF16 at tile `t`, line `i` of the block's BF16 pack.
template <int CQ>
__device__ __forceinline__ void pack_line16(unsigned char* base, int t, int i, int q, int nch, const float (&v)[CQ],
                                            float scale) {
#pragma unroll
    for (int g = 0; g < CQ / 4; ++g) {
        const int k = q * CQ + 4 * g;
        if (k < nch * umma::KCH) {
            unsigned char* dst =
                base + ((ll)t * nch + k / umma::KCH) * umma::PCHUNK16 + umma::packed_offset16(i, k % umma::KCH);
            *reinterpret_cast<uint2*>(dst) = make_uint2(umma::pack_bf16x2(v[4 * g] * scale, v[4 * g + 1] * scale),
                                                        umma::pack_bf16x2(v[4 * g + 2] * scale, v[4 * g + 3] * scale));
        }
    }
}

// Per-block exponent of the BF16 panel scaling: e = floor(E / 2), E the
// binary exponent of the largest |diagonal entry of U_B|; the L panel is
// packed times 2^e and the U panel times 2^-e, so L U^T is unchanged and both
// scaled panels are about 2^(E/2) in size.  Every CTA of the block's panel
// launch computes the same e from the final diagonal block (all threads
// call; contains a barrier).
__device__ __forceinline__ int block_scale_exp(const float* blkp, int ld, int bw, int* smax) {
    if (threadIdx.x == 0) *smax = 0;
    __syncthreads();
    if ((int)threadIdx.x < bw) atomicMax(smax, __float_as_int(fabsf(blkp[(ll)threadIdx.x * ld + threadIdx.x])));
    __syncthreads();
    const int E = ((*smax >> 23) & 255) - 127;
    return E >> 1;
}

// The panels of a block of more than 64 columns in FP32 (W = 128), four
// lines per lane (sweep_rows4 / sweep_cols4): lane c of half-warp h holds
// entries [8c, 8c + 8) of the tile's lines 4h .. 4h + 3.  Same tiles,
// operations and outputs as the generic form in k_block_panel; the row
// sources of the block's interchanges (gmap | pa << 8 per block column) come
// from k_block_lu through bmap.  The 64 lines of the tile pass through a
// shared-memory copy sX (line li, entry j at li * PT_LD + j) so that the
// global loads, stores and packed writes are coalesced: a warp moves 8 rows
// x 4 columns of a column-major array (32-byte runs), and the packed writes
// of 8 lines x 4 entries form 512 contiguous bytes.
constexpr int PT_LD = 132;   // 16-byte rows, 4 words apart in the bank cycle
constexpr int PT_LINES = 64;  // lines per CTA (4 * PT_LINES threads)
constexpr int PT_SMEM = PT_LINES * PT_LD * 4;

// Element e of a PT_LINES-line x 128-entry tile: a warp copies 8
// consecutive entries x 4 lines when `entries_fast`, else 8 lines x 4
// entries.
__device__ __forceinline__ void tile_coords(int e, bool entries_fast, int& li, int& j) {
    const int sub = e & 31, b = e >> 5;
    if (entries_fast) {
        j = (b % 16) * 8 + (sub & 7);
        li = (b / 16) * 4 + (sub >> 3);
    } else {
        li = (b % (PT_LINES / 8)) * 8 + (sub & 7);
        j = (b / (PT_LINES / 8)) * 4 + (sub >> 3);
    }
}

// Packed copy of the tile's lines [0, nl) from sX; line li goes to pack tile
// t(li), line i(li) (computed by `where`).
template <typename Where>
__device__ __forceinline__ void pack_tile(unsigned char* base, const float* sX, int nl, int nch, Where where) {
    for (int item = threadIdx.x; item < PT_LINES * 32; item += blockDim.x) {   // 8 lines x 32 groups of 4 entries
        const int g = (item >> 3) & 31, li = (item >> 8) * 8 + (item & 7);
        if (li >= nl || 4 * g >= nch * umma::KCH) continue;
        int t, i;
        where(li, t, i);
        const int k = 4 * g;
        const float4 v = *reinterpret_cast<const float4*>(sX + li * PT_LD + k);
        const float vv[4] = {v.x, v.y, v.z, v.w};
        uint32_t hh[4], ll_[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            hh[e] = umma::tf32_rna(vv[e]);
            ll_[e] = umma::tf32_rna(vv[e] - __uint_as_float(hh[e]));
        }
        unsigned char* dst = base + ((ll)t * nch + k / umma::KCH) * umma::PCHUNK + umma::packed_offset(i, k % umma::KCH);
        *reinterpret_cast<uint4*>(dst) = make_uint4(hh[0], hh[1], hh[2], hh[3]);
        *reinterpret_cast<uint4*>(dst + umma::OPB) = make_uint4(ll_[0], ll_[1], ll_[2], ll_[3]);
    }
}

// BF16 form of pack_tile: entries times `scale`, one BF16 part per chunk.
template <typename Where>
__device__ __forceinline__ void pack_tile16(unsigned char* base, const float* sX, int nl, int nch, float scale,
                                            Where where) {
    for (int item = threadIdx.x; item < PT_LINES * 32; item += blockDim.x) {
        const int g = (item >> 3) & 31, li = (item >> 8) * 8 + (item & 7);
        if (li >= nl || 4 * g >= nch * umma::KCH) continue;
        int t, i;
        where(li, t, i);
        const int k = 4 * g;
        const float4 v = *reinterpret_cast<const float4*>(sX + li * PT_LD + k);
        unsigned char* dst =
            base + ((ll)t * nch + k / umma::KCH) * umma::PCHUNK16 + umma::packed_offset16(i, k % umma::KCH);
        *reinterpret_cast<uint2*>(dst) =
            make_uint2(umma::pack_bf16x2(v.x * scale, v.y * scale), umma::pack_bf16x2(v.z * scale, v.w * scale));
    }
}

__device__ __forceinline__ void block_panel128(float* fac, const int* bmap, const Sched& S, const DFront& F, int blk,
                                               int tile, unsigned char* pack, float* sT, float* sX, float* rd,
                                               int* gmap, int* pa, int bf16, int* smax, float* sd) {
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk], bw = c1 - c0;
    const int tid = threadIdx.x, c = tid & 15, line0 = (tid >> 4) * 4;
    const int nL = cdiv(F.ld - c1, PT_LINES), nUa = cdiv(F.nf - c1, PT_LINES);
    const float* blkp = fac + F.loff + (ll)c0 * F.ld + c0;
    const int nch = cdiv(bw, umma::KCH);
    const int n1 = cdiv(F.nf - c1, umma::TM);
    if (tile < nL) {
        const int rb0 = c1 + tile * PT_LINES, nl = min(PT_LINES, F.ld - rb0);
        float* xb = fac + F.loff + (ll)c0 * F.ld + rb0;   // line li, entry j at xb[j * ld + li]
        for (int e = tid; e < PT_LINES * 128; e += PT_LINES * 4) {
            int li, j;
            tile_coords(e, false, li, j);
            const bool v = li < nl && j < bw;
            cp_elem(&sX[li * PT_LD + j], v ? xb + (ll)j * F.ld + li : xb, v);
        }
        if (S.sym && tid < bw) sd[tid] = blkp[(ll)tid * F.ld + tid];   // U(j, j) for the U side
        stage_upper<float, 128>(sT, rd, blkp, F.ld, bw);   // waits for all copies
        __syncthreads();
        float x[4][8];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const float4 a0 = *reinterpret_cast<const float4*>(sX + (line0 + l) * PT_LD + 8 * c);
            const float4 a1 = *reinterpret_cast<const float4*>(sX + (line0 + l) * PT_LD + 8 * c + 4);
            x[l][0] = a0.x; x[l][1] = a0.y; x[l][2] = a0.z; x[l][3] = a0.w;
            x[l][4] = a1.x; x[l][5] = a1.y; x[l][6] = a1.z; x[l][7] = a1.w;
        }
        sweep_rows4(x, sT, rd, bw, 8);   // steps 0..63
        float x2[4][4];
        sweep_to_hi(x, x2);
        sweep_rows4_hi(x2, sT, rd, bw);  // steps 64..95
        float x3[4][2];
        sweep_to_top(x2, x3);
        sweep_top<true>(x3, sT, rd, bw);  // steps 96..
#pragma unroll
        for (int l = 0; l < 4; ++l) {   // entries 0..63, 64..95, 96..127 from the three phases
            float* dst = sX + (line0 + l) * PT_LD;
            if (c < 8) {
                *reinterpret_cast<float4*>(dst + 8 * c) = make_float4(x[l][0], x[l][1], x[l][2], x[l][3]);
                *reinterpret_cast<float4*>(dst + 8 * c + 4) = make_float4(x[l][4], x[l][5], x[l][6], x[l][7]);
                *reinterpret_cast<float4*>(dst + 64 + 4 * c) = make_float4(x2[l][0], x2[l][1], x2[l][2], x2[l][3]);
            }
            *reinterpret_cast<float2*>(dst + 96 + 2 * c) = make_float2(x3[l][0], x3[l][1]);
        }
        __syncthreads();
        for (int e = tid; e < PT_LINES * 128; e += PT_LINES * 4) {
            int li, j;
            tile_coords(e, false, li, j);
            if (li < nl && j < bw) xb[(ll)j * F.ld + li] = sX[li * PT_LD + j];
        }
        const ll off = S.blk_lpack[blk];
        auto whereL = [&](int li, int& t, int& i) {
            const int r = rb0 + li;
            t = r < F.nf ? (r - c1) / umma::TM : n1 + (r - F.nf) / umma::TM;
            i = r < F.nf ? (r - c1) % umma::TM : (r - F.nf) % umma::TM;
        };
        const int e = (off >= 0 && bf16) ? block_scale_exp(blkp, F.ld, bw, smax) : 0;
        if (off >= 0 && bf16) pack_tile16(pack + (off >> 2), sX, nl, nch, umma::exp2i(e), whereL);
        else if (off >= 0) pack_tile(pack + off, sX, nl, nch, whereL);
        if (S.sym) {   // the U side: U(c0 + j, r) = U(j, j) L(r, c0 + j), stored and packed
            __syncthreads();   // the L pack has read the tile
            for (int q = tid; q < PT_LINES * 128; q += PT_LINES * 4) {
                int li, j;
                tile_coords(q, true, li, j);
                if (li < nl && j < bw) sX[li * PT_LD + j] *= sd[j];
            }
            __syncthreads();
            for (int q = tid; q < PT_LINES * 128; q += PT_LINES * 4) {   // rows r < nf: column r of Lf
                int li, j;
                tile_coords(q, true, li, j);
                const int r = rb0 + li;
                if (li < nl && j < bw && r < F.nf) fac[F.loff + (ll)r * F.ld + c0 + j] = sX[li * PT_LD + j];
            }
            for (int q = tid; q < PT_LINES * 128; q += PT_LINES * 4) {   // rows r >= nf: U12 in Uf
                int li, j;
                tile_coords(q, false, li, j);
                const int r = rb0 + li;
                if (li < nl && j < bw && r >= F.nf) fac[F.uoff + (ll)(c0 + j) * F.m + (r - F.nf)] = sX[li * PT_LD + j];
            }
            const ll offu = S.blk_upack[blk];
            if (offu >= 0 && bf16) pack_tile16(pack + (offu >> 2), sX, nl, nch, umma::exp2i(-e), whereL);
            else if (offu >= 0) pack_tile(pack + offu, sX, nl, nch, whereL);
        }
    } else {
        if (tid < bw) {   // the block's row sources, from k_block_lu
            const int v = bmap[F.f + c0 + tid];
            gmap[tid] = v & 255;
            pa[tid] = v >> 8;
        }
        __syncthreads();
        const bool inner = tile < nL + nUa;
        const int cb0 = inner ? c1 + (tile - nL) * PT_LINES : (tile - nL - nUa) * PT_LINES;
        const int nl = min(PT_LINES, (inner ? F.nf : F.m) - cb0);
        // line li, block row R at yb[li * ls + R * rs]
        float* yb = inner ? fac + F.loff + (ll)cb0 * F.ld + c0 : fac + F.uoff + (ll)c0 * F.m + cb0;
        const ll ls = inner ? (ll)F.ld : 1, rs = inner ? 1 : (ll)F.m;
        for (int e = tid; e < PT_LINES * 128; e += PT_LINES * 4) {
            int li, R;
            tile_coords(e, inner, li, R);
            const bool v = li < nl && R < bw;
            cp_elem(&sX[li * PT_LD + R], v ? yb + li * ls + (ll)gmap[R] * rs : yb, v);
        }
        stage_lower<float, 128>(sT, blkp, F.ld, bw, gmap, pa);   // waits for all copies
        __syncthreads();
        float y[4][8];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const float4 a0 = *reinterpret_cast<const float4*>(sX + (line0 + l) * PT_LD + 8 * c);
            const float4 a1 = *reinterpret_cast<const float4*>(sX + (line0 + l) * PT_LD + 8 * c + 4);
            y[l][0] = a0.x; y[l][1] = a0.y; y[l][2] = a0.z; y[l][3] = a0.w;
            y[l][4] = a1.x; y[l][5] = a1.y; y[l][6] = a1.z; y[l][7] = a1.w;
        }
        sweep_cols4(y, sT, bw, 8);
        float y2[4][4];
        sweep_to_hi(y, y2);
        sweep_cols4_hi(y2, sT, bw);
        float y3[4][2];
        sweep_to_top(y2, y3);
        sweep_top<false>(y3, sT, nullptr, bw);
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            float* dst = sX + (line0 + l) * PT_LD;
            if (c < 8) {
                *reinterpret_cast<float4*>(dst + 8 * c) = make_float4(y[l][0], y[l][1], y[l][2], y[l][3]);
                *reinterpret_cast<float4*>(dst + 8 * c + 4) = make_float4(y[l][4], y[l][5], y[l][6], y[l][7]);
                *reinterpret_cast<float4*>(dst + 64 + 4 * c) = make_float4(y2[l][0], y2[l][1], y2[l][2], y2[l][3]);
            }
            *reinterpret_cast<float2*>(dst + 96 + 2 * c) = make_float2(y3[l][0], y3[l][1]);
        }
        __syncthreads();
        for (int e = tid; e < PT_LINES * 128; e += PT_LINES * 4) {
            int li, R;
            tile_coords(e, inner, li, R);
            if (li < nl && R < bw) yb[li * ls + (ll)R * rs] = sX[li * PT_LD + R];
        }
        const ll off = S.blk_upack[blk];
        auto whereU = [&](int li, int& t, int& i) {
            const int col = cb0 + li;
            t = inner ? (col - c1) / umma::TM : n1 + col / umma::TM;
            i = inner ? (col - c1) % umma::TM : col % umma::TM;
        };
        if (off >= 0 && bf16) {
            const float scale = umma::exp2i(-block_scale_exp(blkp, F.ld, bw, smax));
            pack_tile16(pack + (off >> 2), sX, nl, nch, scale, whereU);
        } else if (off >= 0) {
            pack_tile(pack + off, sX, nl, nch, whereU);
        }
    }
}

// Panels of block `step` (block width bw <= W): 64-row tiles of the L panel
// below the block, X := X inv(U_B) (the reference's trsm 'r','u','n','n' of
// every piece, with the earlier pieces' updates X_p -= X_<p U_<p,p), and
// 64-column tiles of the U panel to its right, inside the front (Lf) and in
// U12 (Uf): Y := inv(L_B) P_B Y (_luswap! and trsm 'r','l','t','u' of every
// piece, with Y_p -= L_p,<p Y_<p).  One line per 4 lanes (W = 32, 64); FP32
// blocks wider than 64 columns take block_panel128 (four lines per 16
// lanes, PT_LINES-line tiles).  For FP32 fronts with a pack (blk_lpack >= 0)
// the lines are also written, split into TF32 hi / lo, to the packed tiles
// that the tensor-core updates read: rows of the L panel tiled from c1
// ([c1, nf)) and from nf ([nf, ld)), columns of the U panel from c1
// ([c1, nf)) and from 0 (U12).
// Dynamic shared memory: W * SLD(W) T's (plus the line tile of
// block_panel128).
// Panel tiles of one launch part: 0 every tile; 1 the near ones (the first
// two line tiles of the rows below the block and of the front columns right
// of it: the lines the next block's diagonal region is updated from); 2 the
// others.  Tiles of 64 lines: L rows first (nL tiles), then front columns
// (nUa), then U12 columns.
__host__ __device__ __forceinline__ int panel_tile(int part, int tile, int nL, int nUa, bool sym) {
    if (part == 0) return tile;
    const int aL = min(2, nL), aU = sym ? 0 : min(2, nUa);
    if (part == 1) return tile < aL ? tile : nL + (tile - aL);
    return tile < nL - aL ? aL + tile : nL + aU + (tile - (nL - aL));
}

template <typename T, int W>
__global__ void __launch_bounds__(256) k_block_panel(T* fac, const int* ipiv, const int* bmap, Sched S, Launch L,
                                                      int step, unsigned char* pack, int bf16, int part) {
    constexpr int CQ = W / 4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sT = reinterpret_cast<T*>(smem_raw);
    __shared__ T rd[W];
    __shared__ int q0[W + 1], gmap[W], pa[W];
    __shared__ int smax;
    __shared__ T sdg[W];   // symmetric form: U(j, j) of the block
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int blk = F.block0 + step;
    {
        const int c1 = S.blk_c1[blk];
        tile = panel_tile(part, tile, cdiv(F.ld - c1, 64), cdiv(F.nf - c1, 64), S.sym != 0);
    }
    if constexpr (std::is_same<T, float>::value && W == 128) {
        block_panel128(fac, bmap, S, F, blk, tile, pack, sT, sT + 128 * SLD<float, 128>::value, rd, gmap, pa, bf16,
                       &smax, sdg);
        return;
    }
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk], bw = c1 - c0;
    const int p0 = S.blk_p0[blk], np = S.blk_np[blk];
    const int tid = threadIdx.x, line = tid >> 2, q = tid & 3;
    const int nL = cdiv(F.ld - c1, 64), nUa = cdiv(F.nf - c1, 64);
    const T* blkp = fac + F.loff + (ll)c0 * F.ld + c0;
    if (tile < nL) {
        const int r = c1 + tile * 64 + line;
        const bool ok = r < F.ld;
        T* xp = fac + F.loff + (ll)c0 * F.ld + r;   // row r, block column j at xp[j * ld]
        T x[CQ];
#pragma unroll
        for (int jj = 0; jj < CQ; ++jj) {   // in flight while the triangle is staged
            const int j = q * CQ + jj;
            x[jj] = (ok && j < bw) ? xp[(ll)j * F.ld] : T(0);
        }
        if (S.sym && tid < bw) sdg[tid] = blkp[(ll)tid * F.ld + tid];   // U(j, j) for the U side
        stage_upper<T, W>(sT, rd, blkp, F.ld, bw);
        __syncthreads();
        sweep_rows<T, W>(x, sT, rd, bw);
#pragma unroll
        for (int jj = 0; jj < CQ; ++jj) {
            const int j = q * CQ + jj;
            if (ok && j < bw) xp[(ll)j * F.ld] = x[jj];
        }
        T u[CQ];   // symmetric form: the U side, U(c0 + j, r) = U(j, j) L(r, c0 + j)
#pragma unroll
        for (int jj = 0; jj < CQ; ++jj) {
            const int j = q * CQ + jj;
            u[jj] = (S.sym && j < bw) ? x[jj] * sdg[j] : T(0);
            if (S.sym && ok && j < bw) {
                if (r < F.nf) fac[F.loff + (ll)r * F.ld + c0 + j] = u[jj];
                else fac[F.uoff + (ll)(c0 + j) * F.m + (r - F.nf)] = u[jj];
            }
        }
        if constexpr (std::is_same<T, float>::value) {
            const ll off = S.blk_lpack[blk];
            const int e = (off >= 0 && bf16) ? block_scale_exp(blkp, F.ld, bw, &smax) : 0;
            if (off >= 0 && ok) {
                const int n1 = cdiv(F.nf - c1, umma::TM);
                const int t = r < F.nf ? (r - c1) / umma::TM : n1 + (r - F.nf) / umma::TM;
                const int i = r < F.nf ? (r - c1) % umma::TM : (r - F.nf) % umma::TM;
                if (bf16) pack_line16<CQ>(pack + (off >> 2), t, i, q, cdiv(bw, umma::KCH), x, umma::exp2i(e));
                else pack_line<CQ>(pack + off, t, i, q, cdiv(bw, umma::KCH), x);
                const ll offu = S.blk_upack[blk];   // symmetric form: the U side's pack, same tiles
                if (S.sym && offu >= 0) {
                    if (bf16) pack_line16<CQ>(pack + (offu >> 2), t, i, q, cdiv(bw, umma::KCH), u, umma::exp2i(-e));
                    else pack_line<CQ>(pack + offu, t, i, q, cdiv(bw, umma::KCH), u);
                }
            }
        }
    } else {
        for (int k = tid; k <= np; k += 256) q0[k] = S.xsuper[p0 + k] - F.f - c0;
        __syncthreads();
        block_gather_map(ipiv + F.f + c0, q0, np, gmap, pa);
        __syncthreads();
        const bool inner = tile < nL + nUa;
        const int col = inner ? c1 + (tile - nL) * 64 + line : (tile - nL - nUa) * 64 + line;
        const bool ok = inner ? col < F.nf : col < F.m;
        // block row k of this column at cp[k * stride]
        T* cp = inner ? fac + F.loff + (ll)col * F.ld + c0 : fac + F.uoff + (ll)c0 * F.m + col;
        const ll stride = inner ? 1 : (ll)F.m;
        T y[CQ];
#pragma unroll
        for (int ii = 0; ii < CQ; ++ii) {   // in flight while the triangle is staged
            const int R = q * CQ + ii;
            y[ii] = (ok && R < bw) ? cp[(ll)gmap[R] * stride] : T(0);
        }
        stage_lower<T, W>(sT, blkp, F.ld, bw, gmap, pa);
        __syncthreads();
        sweep_cols<T, W>(y, sT, bw);
#pragma unroll
        for (int ii = 0; ii < CQ; ++ii) {
            const int R = q * CQ + ii;
            if (ok && R < bw) cp[(ll)R * stride] = y[ii];
        }
        if constexpr (std::is_same<T, float>::value) {
            const ll off = S.blk_upack[blk];
            const float scale = (off >= 0 && bf16) ? umma::exp2i(-block_scale_exp(blkp, F.ld, bw, &smax)) : 1.0f;
            if (off >= 0 && ok) {
                const int n1 = cdiv(F.nf - c1, umma::TM);
                const int t = inner ? (col - c1) / umma::TM : n1 + col / umma::TM;
                const int i = inner ? (col - c1) % umma::TM : col % umma::TM;
                if (bf16) pack_line16<CQ>(pack + (off >> 2), t, i, q, cdiv(bw, umma::KCH), y, scale);
                else pack_line<CQ>(pack + off, t, i, q, cdiv(bw, umma::KCH), y);
            }
        }
    }
}

// After the factorisation: the whole-block solve operators of every block,
//   Minv = inv(L_B) P_B  (the forward steps of all its pieces, in order)
//   Uinv = inv(U_B)      (the backward steps, pieces reversed)
// written column-major (bw x bw, Minv then Uinv) at inv2[blk_inv2[blk]], so
// that a triangular-solve step of a block is one product.  They are the
// panel sweeps applied to the identity: column j of Minv is the U-panel
// sweep of e_j, row i of Uinv the L-panel sweep of e_i.  This kernel takes
// the blocks of more than 32 columns (W = 64, 128); `entries` lists the
// work, entry = blk * 4 + kind * 2 + tile (kind 0 Minv, 1 Uinv; 64 lines per
// tile).  Dynamic shared memory: W * SLD(W) T's.  Narrower blocks:
// k_block_inv_small.
template <typename T, int W>
__global__ void __launch_bounds__(256) k_block_inv(const T* fac, const int* ipiv, T* inv2, Sched S,
                                                    const int* blk_front, const int* entries) {
    constexpr int CQ = W / 4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ T rd[W];
    __shared__ int q0[W + 1], gmap[W], pa[W];
    static_assert(W > 32, "blocks of at most 32 columns: k_block_inv_small");
    const int e = entries[blockIdx.x];
    const int blk = e >> 2, kind = (e >> 1) & 1, l0 = (e & 1) * 64;
    const DFront F = S.fronts[blk_front[blk]];
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk], bw = c1 - c0;
    const int p0 = S.blk_p0[blk], np = S.blk_np[blk];
    const T* blkp = fac + F.loff + (ll)c0 * F.ld + c0;
    T* sL = reinterpret_cast<T*>(smem_raw);
    T* sU = sL;   // one kind per entry
    const int tid = threadIdx.x, line = tid >> 2, q = tid & 3;
    if (kind != 1) {
        for (int k = tid; k <= np; k += 256) q0[k] = S.xsuper[p0 + k] - F.f - c0;
        __syncthreads();
        block_gather_map(ipiv + F.f + c0, q0, np, gmap, pa);
        __syncthreads();
        stage_lower<T, W>(sL, blkp, F.ld, bw, gmap, pa);
    }
    if (kind != 0) stage_upper<T, W>(sU, rd, blkp, F.ld, bw);
    __syncthreads();
    const bool doM = kind == 0;
    const int idx = l0 + line;
    if (__all_sync(0xffffffffu, idx >= bw)) return;   // the whole warp is past the block
    T v[CQ];
    T* out = inv2 + S.blk_inv2[blk];
    if (doM) {
#pragma unroll
        for (int ii = 0; ii < CQ; ++ii) {
            const int R = q * CQ + ii;
            v[ii] = (R < bw && gmap[R] == idx) ? T(1) : T(0);
        }
        sweep_cols<T, W>(v, sL, bw);
        if (idx < bw) {
#pragma unroll
            for (int ii = 0; ii < CQ; ++ii) {
                const int R = q * CQ + ii;
                if (R < bw) out[(ll)idx * bw + R] = v[ii];
            }
        }
    } else {
#pragma unroll
        for (int jj = 0; jj < CQ; ++jj) v[jj] = (q * CQ + jj == idx) ? T(1) : T(0);
        sweep_rows<T, W>(v, sU, rd, bw);
        if (idx < bw) {
#pragma unroll
            for (int jj = 0; jj < CQ; ++jj) {
                const int j = q * CQ + jj;
                if (j < bw) out[(ll)bw * bw + (ll)j * bw + idx] = v[jj];
            }
        }
    }
}

// The same operators for blocks of at most W <= 32 columns, a warp per
// block, four per CTA (launches by width class W = 4, 8, 16, 32): the block
// in shared memory, lane j forms column j of Minv (P e_j through the
// forward steps of the pieces, the multipliers of row i left of its piece
// taken from its source row, as stage_lower stages them), lane i row i of
// Uinv (e_i through the backward steps, scaled by 1 / U(j, j)).  The
// operations of the sweeps k_block_inv applies, in the same order, without
// a CTA per block for blocks of a few columns.
constexpr int BI_WARPS = 4;
template <typename T, int W>
__global__ void __launch_bounds__(32 * BI_WARPS) k_block_inv_small(const T* fac, const int* ipiv, T* inv2, Sched S,
                                                                    const int* blk_front, const int* entries,
                                                                    int count) {
    constexpr int LD = W + 1;
    __shared__ T sD[BI_WARPS][W * LD];   // D(r, c) at [c * LD + r]
    __shared__ T srd[BI_WARPS][W];
    __shared__ int sq[BI_WARPS][W + 1], sgm[BI_WARPS][W], spa[BI_WARPS][W];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int idx = blockIdx.x * BI_WARPS + warp;
    if (idx >= count) return;   // whole warp; no CTA barrier below
    const int blk = entries[idx];
    const DFront F = S.fronts[blk_front[blk]];
    const int c0 = S.blk_c0[blk], bw = S.blk_c1[blk] - c0;
    const int p0 = S.blk_p0[blk], np = S.blk_np[blk];
    const T* blkp = fac + F.loff + (ll)c0 * F.ld + c0;
    T* D = sD[warp];
    T* rd = srd[warp];
    int* q0 = sq[warp];
    int* gm = sgm[warp];
    int* pa = spa[warp];
    for (int k = lane; k <= np; k += 32) q0[k] = S.xsuper[p0 + k] - F.f - c0;
    for (int j = 0; j < bw; ++j)
        if (lane < bw) D[j * LD + lane] = blkp[(ll)j * F.ld + lane];
    if (lane < bw) rd[lane] = T(1) / blkp[(ll)lane * F.ld + lane];
    __syncwarp();
    const int* ipb = ipiv + F.f + c0;
    for (int pc = lane; pc < np; pc += 32) {   // block_gather_map, a lane per piece
        const int a = q0[pc], b = q0[pc + 1];
        for (int i = a; i < b; ++i) {
            gm[i] = i;
            pa[i] = a;
        }
        for (int k = a; k < b; ++k) {
            const int kp = a + ipb[k];
            const int t = gm[k];
            gm[k] = gm[kp];
            gm[kp] = t;
        }
    }
    __syncwarp();
    T* out = inv2 + S.blk_inv2[blk];
    {   // Minv(:, lane)
        T y[W];
#pragma unroll
        for (int i = 0; i < W; ++i) y[i] = (lane < bw && i < bw && gm[i] == lane) ? T(1) : T(0);
#pragma unroll
        for (int i = 1; i < W; ++i)
            if (i < bw) {
                const int gi = gm[i], ai = pa[i];
#pragma unroll
                for (int k = 0; k < i; ++k) y[i] -= D[k * LD + (k < ai ? gi : i)] * y[k];
            }
        if (lane < bw)
#pragma unroll
            for (int i = 0; i < W; ++i)
                if (i < bw) out[(ll)lane * bw + i] = y[i];
    }
    {   // Uinv(lane, :)
        T x[W];
#pragma unroll
        for (int j = 0; j < W; ++j) x[j] = (j == lane && lane < bw) ? T(1) : T(0);
#pragma unroll
        for (int j = 0; j < W; ++j)
            if (j < bw) {
#pragma unroll
                for (int k = 0; k < j; ++k) x[j] -= x[k] * D[j * LD + k];
                x[j] *= rd[j];
            }
        if (lane < bw)
#pragma unroll
            for (int j = 0; j < W; ++j)
                if (j < bw) out[(ll)bw * bw + (ll)j * bw + lane] = x[j];
    }
}

// ---------------------------------------------------------------------------
// 64 x 64 register-tiled block product, 256 threads, 4 x 4 outputs each.
// sA[k][i] (k < kc, i < 64), sB[k][j]; thread (tx, ty) owns rows tx+16a and
// columns ty+16b when rows_fast, else rows ty+16a and columns tx+16b.
// ---------------------------------------------------------------------------
constexpr int TT = 64;
constexpr int KC = 32;

// Symmetric form: the tiles (i, j) of an nr x nc tile grid with i >= j
// (the lower part and the diagonal tiles), column by column: column j holds
// nr - j tiles.  Tile number t -> (i, j).
__host__ __device__ __forceinline__ void lower_tile(int t, int nr, int& i, int& j) {
    j = 0;
    while (t >= nr - j) {
        t -= nr - j;
        ++j;
    }
    i = j + t;
}
__host__ __device__ __forceinline__ int lower_tiles(int nr, int nc) {
    int n = 0;
    for (int j = 0; j < nc && j < nr; ++j) n += nr - j;
    return n;
}
// The same for groups of w adjacent tile columns (wide tiles): group j
// covers columns w j .. w j + w - 1 and rows w j .. nr - 1.
__host__ __device__ __forceinline__ void lower_tile_w(int t, int nr, int w, int& i, int& j) {
    j = 0;
    while (t >= nr - w * j) {
        t -= nr - w * j;
        ++j;
    }
    i = w * j + t;
}
__host__ __device__ __forceinline__ int lower_tiles_w(int nr, int w) {
    int n = 0;
    for (int j = 0; w * j < nr; ++j) n += nr - w * j;
    return n;
}

// The Schur complement tiles of a tensor-core front in two parts: the near
// part (1) holds every tile with an entry whose target front - the owner of
// the smaller of its row and column, rows sorted ascending - is factored at
// the next level, i.e. a row tile or a column below q (the first q row
// tiles hold every row such a front owns); the far part (2) the others,
// whose targets are factored two or more levels up.  Tiles of the whole
// update (part 0): t = g n2 + rt, column group g of nh tiles and row tile
// rt; in the SPD form the lower tiles of group g (rows nh g .. n2 - 1) in
// that order, where the near part is the groups below cdiv(q, nh).
__host__ __device__ __forceinline__ int schur_part_count(int part, int n2, int nh, int q, bool sym) {
    const int ng = cdiv(n2, nh);
    q = min(q, n2);
    const int gq = min(cdiv(q, nh), ng);
    const int all = sym ? lower_tiles_w(n2, nh) : ng * n2;
    int far;
    if (sym) {
        int near = 0;
        for (int j = 0; j < gq; ++j) near += n2 - nh * j;
        far = all - near;
    } else {
        far = (ng - gq) * (n2 - q);
    }
    return part == 0 ? all : part == 1 ? all - far : far;
}
__host__ __device__ __forceinline__ int schur_part_tile(int part, int e, int n2, int nh, int q, bool sym) {
    if (part == 0) return e;
    q = min(q, n2);
    const int gq = min(cdiv(q, nh), cdiv(n2, nh));
    if (sym) return part == 1 ? e : schur_part_count(1, n2, nh, q, true) + e;
    if (part == 1) {
        if (e < gq * n2) return e;
        e -= gq * n2;
        return (gq + e / q) * n2 + e % q;
    }
    return (gq + e / (n2 - q)) * n2 + q + e % (n2 - q);
}

template <typename T, bool rows_fast>
__device__ __forceinline__ void mma_tile(const T* sA, const T* sB, int kc, T acc[4][4]) {
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int ri = rows_fast ? tx : ty, ci = rows_fast ? ty : tx;
#pragma unroll 4
    for (int k = 0; k < kc; ++k) {
        T a[4], b[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) { a[q] = sA[k * TT + ri + 16 * q]; b[q] = sB[k * TT + ci + 16 * q]; }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
    }
}

// Trailing update after block `step`: A[R, C] -= L[R, block] * U[block, C]
// over the front minus its Schur-complement block.  L tiles: rows in
// [c1, nf+m), columns in [c1, nf) (stored in Lf).  U tiles: rows in [c1, nf),
// columns in U12 (stored in Uf).
template <typename T>
__global__ void __launch_bounds__(256) k_block_trail(T* fac, Sched S, Launch L, int step) {
    __shared__ T sA[KC * TT];
    __shared__ T sB[KC * TT];
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int blk = F.block0 + step;
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk];
    const int tid = threadIdx.x;
    const int nrL = cdiv(F.ld - c1, TT), ncL = cdiv(F.nf - c1, TT);
    const bool isL = S.sym || tile < nrL * ncL;   // the symmetric form: lower L tiles only
    int r0, col0, nr, nc;
    if (isL) {
        int ti = tile % nrL, tj = tile / nrL;
        if (S.sym) lower_tile(tile, nrL, ti, tj);
        r0 = c1 + ti * TT;
        col0 = c1 + tj * TT;
        nr = min(TT, F.ld - r0);
        nc = min(TT, F.nf - col0);
    } else {
        const int t2 = tile - nrL * ncL, nrU = cdiv(F.nf - c1, TT);
        r0 = c1 + (t2 % nrU) * TT;
        col0 = (t2 / nrU) * TT;            // U12 column index
        nr = min(TT, F.nf - r0);
        nc = min(TT, F.m - col0);
    }
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
    for (int k0 = c0; k0 < c1; k0 += KC) {
        const int kc = min(KC, c1 - k0);
        for (int e = tid; e < kc * TT; e += 256) {
            int i = e % TT, k = e / TT;
            sA[k * TT + i] = (i < nr) ? fac[F.loff + (ll)(k0 + k) * F.ld + r0 + i] : T(0);
        }
        if (isL) {
            for (int e = tid; e < kc * TT; e += 256) {
                int k = e % kc, j = e / kc;
                sB[k * TT + j] = (j < nc) ? fac[F.loff + (ll)(col0 + j) * F.ld + k0 + k] : T(0);
            }
        } else {
            for (int e = tid; e < kc * TT; e += 256) {
                int j = e % TT, k = e / TT;
                sB[k * TT + j] = (j < nc) ? fac[F.uoff + (ll)(k0 + k) * F.m + col0 + j] : T(0);
            }
        }
        __syncthreads();
        if (isL) mma_tile<T, true>(sA, sB, kc, acc);
        else mma_tile<T, false>(sA, sB, kc, acc);
        __syncthreads();
    }
    const int tx = tid & 15, ty = tid >> 4;
    // the 16 entries are loaded before any is stored (distinct addresses the
    // compiler cannot prove distinct)
    T old[4][4];
    ll addr[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int r = isL ? tx + 16 * a : ty + 16 * a, c = isL ? ty + 16 * b : tx + 16 * b;
            const bool in = r < nr && c < nc;
            addr[a][b] = !in ? -1 : isL ? F.loff + (ll)(col0 + c) * F.ld + r0 + r : F.uoff + (ll)(r0 + r) * F.m + col0 + c;
            old[a][b] = in ? fac[addr[a][b]] : T(0);
        }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
            if (addr[a][b] >= 0) fac[addr[a][b]] = old[a][b] - acc[a][b];
}

// Scatter target of one row or column x of a Schur complement tile: the
// front G of R_F[x] (its run), and x's position in G.
struct ScatterRow {
    ll rel0;     // offset in rel[] of R_F[0] for the run of this row / column
    ll loff, uoff;
    int ld, nf, m, pos;
};

template <typename T>
__device__ __forceinline__ ScatterRow scatter_row(const Sched& S, const DFront& F, int x) {
    ScatterRow e{};
    e.pos = -1;
    if (x < F.m) {
        const int g = S.runid[F.runid_off + x];
        const DFront G = S.fronts[S.run_tgt[g]];
        e.rel0 = S.run_rel[g] - S.run_start[g];
        e.loff = G.loff;
        e.uoff = G.uoff;
        e.ld = G.ld;
        e.nf = G.nf;
        e.m = G.m;
        e.pos = S.rel[e.rel0 + x];
    }
    return e;
}

// Small fronts (one block of at most 32 columns, m <= LF_M) factored whole
// by one warp each, four per CTA: the block LU of k_block_lu_small, then
// the L21 rows (x := x U^-1, a lane per row), the U12 columns (interchanges
// of the block, then u := L^-1 u, a lane per column), both in the entry
// order of the panel sweeps, and the Schur complement L21 U12 (k in order)
// scatter-subtracted into the ancestors like k_schur.  Replaces, for these
// fronts, k_block_lu_small + k_block_panel + k_schur (three launches whose
// CTAs would be mostly idle on fronts this small).  Each launch holds fronts
// of one width class W (block width <= W, W = 4, 8, 16 or 32), so that the
// unrolled register loops and the shared memory are sized to the class.
constexpr int LF_M = 32, LF_WARPS = 4;
constexpr int LF_CLASSES = 4;   // W = 4 << class
__host__ __device__ constexpr int leaf_class(int bw) { return bw <= 4 ? 0 : bw <= 8 ? 1 : bw <= 16 ? 2 : 3; }
template <typename T, int W> struct LeafSmem {
    static constexpr int LD = W + 1;
    static constexpr size_t warp_bytes = (((size_t)(W + LF_M) * LD + W) * sizeof(T) + LF_M * sizeof(ScatterRow) +
                                          (W + 1 + 3 * W) * sizeof(int) + 15) / 16 * 16;
    static constexpr size_t bytes = LF_WARPS * warp_bytes;
};

// A load of factor data that other CTAs of the same launch may have updated
// (COH: at L2, bypassing the SM's L1, which is not coherent across SMs).
template <bool COH, typename T>
__device__ __forceinline__ T ld_fac(const T* p) {
    if constexpr (COH) return __ldcg(p);
    else return *p;
}

// One small front (block width <= W) factored whole by the calling warp;
// `base` is the warp's slice of LeafSmem<T, W>.
template <typename T, bool COH, int W>
__device__ __forceinline__ void leaf_front(T* fac, int* ipiv, int* info, const Sched& S, const DFront& F,
                                           unsigned char* base) {
    constexpr int LD = LeafSmem<T, W>::LD;
    const int lane = threadIdx.x & 31;
    ScatterRow* tab = reinterpret_cast<ScatterRow*>(base);
    T* sD = reinterpret_cast<T*>(tab + LF_M);          // diagonal block, D(i, j) at sD[j * LD + i]
    T* sL = sD + W * LD;                               // L21 rows, L21(r, k) at sL[r * LD + k]
    T* srv = sL + LF_M * LD;                           // 1 / U(k, k)
    int* q0 = reinterpret_cast<int*>(srv + W);
    int* piv = q0 + W + 1;
    int* gm = piv + W;
    int* pam = gm + W;
    const int blk = F.block0, bw = F.nf, m = F.m;
    const int p0 = S.blk_p0[blk], np = S.blk_np[blk];
    const bool sym = S.sym != 0;
    for (int k = lane; k <= np; k += 32) q0[k] = S.xsuper[p0 + k] - F.f;
    for (int j = 0; j < bw; ++j)   // symmetric form: the upper triangle mirrors the lower one
        if (lane < bw)
            sD[j * LD + lane] = (sym && lane < j) ? ld_fac<COH>(fac + F.loff + (ll)lane * F.ld + j)
                                                  : ld_fac<COH>(fac + F.loff + (ll)j * F.ld + lane);
    for (int x = lane; x < m; x += 32) tab[x] = scatter_row<T>(S, F, x);
    __syncwarp();
    // block LU (ggetrf! pivots inside each piece; none in the symmetric form)
    const bool sing = warp_block_lu32<T, W>(sD, LD, bw, q0, np, piv, sym);
    for (int j = 0; j < bw; ++j)
        if (lane < bw) fac[F.loff + (ll)j * F.ld + lane] = sD[j * LD + lane];
    if (lane < bw) {
        ipiv[F.f + lane] = piv[lane];
        srv[lane] = rcp_rn(sD[lane * LD + lane]);   // as the panel's 1 / U(k, k)
    }
    if (lane == 0 && sing) {
        for (int pc = 0; pc < np; ++pc) {
            bool z = false;
            for (int k = q0[pc]; k < q0[pc + 1]; ++k) z |= sD[k * LD + k] == T(0);
            if (z) { atomicMin(info, p0 + pc + 1); break; }
        }
    }
    for (int pc = lane; pc < np; pc += 32) {   // row sources of the interchanges (block_gather_map)
        const int a = q0[pc], b = q0[pc + 1];
        for (int i = a; i < b; ++i) {
            gm[i] = i;
            pam[i] = a;
        }
        for (int k = a; k < b; ++k) {
            const int kp = a + piv[k];
            const int t = gm[k];
            gm[k] = gm[kp];
            gm[kp] = t;
        }
    }
    __syncwarp();
    // L21 rows (m <= 32: a lane per row): x := x U^-1 (left-looking: entry j
    // gets k = 0, 1, .. then its scaling)
    const int r = lane;
    if (r < m) {
        T x[W];
#pragma unroll
        for (int k = 0; k < W; ++k) x[k] = k < bw ? ld_fac<COH>(fac + F.loff + (ll)k * F.ld + bw + r) : T(0);
#pragma unroll
        for (int j = 0; j < W; ++j)
            if (j < bw) {
#pragma unroll
                for (int k = 0; k < j; ++k) x[j] -= x[k] * sD[j * LD + k];
                x[j] *= srv[j];
            }
#pragma unroll
        for (int k = 0; k < W; ++k)
            if (k < bw) {
                fac[F.loff + (ll)k * F.ld + bw + r] = x[k];
                sL[r * LD + k] = x[k];
            }
    }
    // U12 columns, a lane per column c: y := inv(L) P y (symmetric form:
    // y_k = U(k, k) L21(c, k), from this lane's own L21 row)
    const int c = lane;
    T y[W];
    if (sym) {
#pragma unroll
        for (int k = 0; k < W; ++k) y[k] = (c < m && k < bw) ? sD[k * LD + k] * sL[c * LD + k] : T(0);
    } else {
#pragma unroll
        for (int k = 0; k < W; ++k) y[k] = (c < m && k < bw) ? ld_fac<COH>(fac + F.uoff + (ll)gm[k] * m + c) : T(0);
#pragma unroll
        for (int i = 0; i < W; ++i)
            if (i < bw) {
#pragma unroll
                for (int k = 0; k < i; ++k) {
                    const T l = k < pam[i] ? sD[k * LD + gm[i]] : sD[k * LD + i];
                    y[i] -= l * y[k];
                }
            }
    }
    if (c < m)
#pragma unroll
        for (int k = 0; k < W; ++k)
            if (k < bw) fac[F.uoff + (ll)k * m + c] = y[k];
    __syncwarp();
    // Schur complement, a lane per column c, rows in order
    if (c < m) {
        for (int rr = sym ? c : 0; rr < m; ++rr) {   // the symmetric form forms the lower part only
            T acc = T(0);
#pragma unroll
            for (int k = 0; k < W; ++k)
                if (k < bw) acc += sL[rr * LD + k] * y[k];
            if (rr >= c) {   // L entry of the front of R_F[c]
                const ScatterRow& Cc = tab[c];
                const int p = S.rel[Cc.rel0 + rr];
                if (Cc.pos >= 0 && p >= 0) atomicAdd(&fac[Cc.loff + (ll)Cc.pos * Cc.ld + p], -acc);
            } else {   // entry of the front of R_F[rr] (not in the symmetric form)
                const ScatterRow& R = tab[rr];
                const int p = S.rel[R.rel0 + c];
                if (R.pos >= 0 && p >= 0) {
                    const ll addr = p < R.nf ? R.loff + (ll)p * R.ld + R.pos : R.uoff + (ll)R.pos * R.m + (p - R.nf);
                    atomicAdd(&fac[addr], -acc);
                }
            }
        }
    }
}

template <typename T, int W>
__global__ void __launch_bounds__(32 * LF_WARPS) k_leaf_factor(T* fac, int* ipiv, int* info, Sched S, Launch L) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5;
    unsigned char* base = smem_raw + (size_t)warp * LeafSmem<T, W>::warp_bytes;
    const int idx = blockIdx.x * LF_WARPS + warp;
    if (idx >= L.count) return;   // whole warp; the kernel has no CTA barrier
    leaf_front<T, false, W>(fac, ipiv, info, S, S.fronts[L.front_ids[idx]], base);
}

// The bottom subtrees of small fronts (every front of the subtree factored
// whole, as by k_leaf_factor) in one persistent launch: a merged work queue
// in level order.  A warp takes the next front (atomic counter `next`),
// waits until the front's children have signalled (deps[front] == 0; a
// bounded spin of `budget` polls, after which it records a timeout in *err
// and goes on, so that the launch always ends), factors it, makes its writes
// visible (fence) and signals its parent (qparent[position], -1 when the
// parent is factored by the level launches).  A front's children come
// earlier in the queue, so every front waited on is held by a running warp.
// `stall` (a queue position, or -1) makes that position's wait one that
// nothing ends, so that the timeout path can be tested.  Shared memory is
// sized for the widest class.
template <typename T>
__global__ void __launch_bounds__(32 * LF_WARPS) k_leaf_queue(T* fac, int* ipiv, int* info, Sched S, const int* order,
                                                              const int* qparent, int nq, int* next, int* deps,
                                                              unsigned budget, int stall, int* err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* base = smem_raw + (size_t)warp * LeafSmem<T, 32>::warp_bytes;
    for (;;) {
        int pos = 0;
        if (lane == 0) pos = atomicAdd(next, 1);
        pos = __shfl_sync(0xffffffffu, pos, 0);
        if (pos >= nq) break;
        const int fid = order[pos];
        if (lane == 0) {
            const int done = pos == stall ? -1 : 0;   // deps never falls below 0
            unsigned it = 0;
            while (*reinterpret_cast<volatile int*>(deps + fid) > done) {
                if (++it >= budget) {
                    atomicExch(err, 1);
                    break;
                }
                if (it > 32) __nanosleep(64);
            }
            __threadfence();
        }
        __syncwarp();
        const DFront F = S.fronts[fid];
        switch (leaf_class(F.nf)) {
        case 0: leaf_front<T, true, 4>(fac, ipiv, info, S, F, base); break;
        case 1: leaf_front<T, true, 8>(fac, ipiv, info, S, F, base); break;
        case 2: leaf_front<T, true, 16>(fac, ipiv, info, S, F, base); break;
        default: leaf_front<T, true, 32>(fac, ipiv, info, S, F, base); break;
        }
        __threadfence();
        __syncwarp();
        if (lane == 0 && qparent[pos] >= 0) atomicSub(deps + qparent[pos], 1);
    }
}

// Schur complement of every front in the launch: C = L21 * U12 (m x m,
// inner dimension nf), scatter-subtracted into the ancestors.  An entry
// (r, c) of C belongs to the front of column R_F[c] when r >= c (an L
// entry) and to the front of row R_F[r] when r < c (a U entry); both are
// the front of R_F[min(r, c)], whose run gives the positions.
template <typename T>
__global__ void __launch_bounds__(256) k_schur(T* fac, Sched S, Launch L) {
    __shared__ T sA[KC * TT];
    __shared__ T sB[KC * TT];
    __shared__ ScatterRow tab[2][TT];   // [0] tile columns, [1] tile rows
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int tid = threadIdx.x;
    const int nt = cdiv(F.m, TT);
    int ti = tile % nt, tj = tile / nt;
    if (S.sym) lower_tile(tile, nt, ti, tj);   // the symmetric form: lower tiles only
    const int r0 = ti * TT, c0 = tj * TT;
    const int nr = min(TT, F.m - r0), nc = min(TT, F.m - c0);
    if (tid < 2 * TT) tab[tid / TT][tid % TT] = scatter_row<T>(S, F, (tid < TT ? c0 : r0) + tid % TT);   // published by the first barrier below
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
    for (int k0 = 0; k0 < F.nf; k0 += KC) {
        const int kc = min(KC, F.nf - k0);
        for (int e = tid; e < kc * TT; e += 256) {
            int i = e % TT, k = e / TT;
            sA[k * TT + i] = (i < nr) ? fac[F.loff + (ll)(k0 + k) * F.ld + F.nf + r0 + i] : T(0);
            sB[k * TT + i] = (i < nc) ? fac[F.uoff + (ll)(k0 + k) * F.m + c0 + i] : T(0);
        }
        __syncthreads();
        mma_tile<T, true>(sA, sB, kc, acc);
        __syncthreads();
    }
    // scatter through the tile's target tables: one rel[] load per entry,
    // the 16 loads of a thread in flight together, then its 16 scatter-adds
    const int tx = tid & 15, ty = tid >> 4;
    int pos[4][4];
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int ic = ty + 16 * b, ir = tx + 16 * a, c = c0 + ic, r = r0 + ir;
            pos[a][b] = -1;
            if (ic < nc && ir < nr && (r >= c || !S.sym))
                pos[a][b] = r >= c ? S.rel[tab[0][ic].rel0 + r] : S.rel[tab[1][ir].rel0 + c];
        }
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int ic = ty + 16 * b, ir = tx + 16 * a, c = c0 + ic, r = r0 + ir;
            const int p = pos[a][b];
            if (p < 0) continue;
            if (r >= c) {   // L entry of the front of R_F[c]
                const ScatterRow& Cc = tab[0][ic];
                if (Cc.pos >= 0) atomicAdd(&fac[Cc.loff + (ll)Cc.pos * Cc.ld + p], -acc[a][b]);
            } else {        // entry of the front of R_F[r]
                const ScatterRow& R = tab[1][ir];
                if (R.pos >= 0) {
                    const ll addr = p < R.nf ? R.loff + (ll)p * R.ld + R.pos : R.uoff + (ll)R.pos * R.m + (p - R.nf);
                    atomicAdd(&fac[addr], -acc[a][b]);
                }
            }
        }
}

// ---------------------------------------------------------------------------
// Rank updates of the FP32 fronts on the tensor cores (3xTF32), from the
// panels packed by k_block_panel.  Tiles are 128 x 128; the rows of a
// front are tiled in two regions, [c1, nf) from c1 (n1 tiles) and [nf, ld)
// from nf (n2 tiles), the columns likewise ([c1, nf) of the front, then the
// U12 columns), so that the packed tiles of every block line up with the
// Schur complement's.
//   TRAIL (block `step`): A = L panel row tile rt, B = U panel column tile
//     ct, K = the block's columns; tiles (rt < n1 + n2, ct < n1) update Lf,
//     tiles (rt < n1, n1 <= ct) update U12 in Uf.
//   SCHUR: A = L21 row tile, B = U12 column tile, K = all blocks' columns;
//     the product is scattered into the ancestors like k_schur.
// A launch covers local tiles tile_base.. of each front in its list (the
// trailing update is launched as tile 0, which holds the next block's
// diagonal block, and tiles 1.., so that the next block LU can start before
// the rest of the update is done).  SCHUR launches of part 1 / 2 cover the
// near / far tiles of each front (schur_part_tile), part 0 all of them.
// Persistent: CTA b takes tiles b, b + gridDim.x, ...  Warp 0 lane 0 issues
// the bulk copies, warp 1 lane 0 the MMAs, and the TC_EPI epilogue warps
// (from warp 4; warp w reads TMEM lanes 32 (w % 4).. and the 32 accumulator
// columns 32 ((w - 4) / 4)..) drain the accumulator.
// ---------------------------------------------------------------------------

constexpr int TC_TRAIL = 0, TC_SCHUR = 1;
constexpr int TC_EPI = 16, TC_THREADS = 32 * (4 + TC_EPI);

struct TcTile {
    DFront F;
    int rt, ct, n1, n2, nchunks;
    int nh;   // 128-column tiles of the (wide) tile that exist: ct .. ct + nh - 1
};

template <int MODE, int NH = 1>
__device__ __forceinline__ TcTile tc_decode(const Sched& S, const Launch& L, int step, int tile, int tile_base,
                                           int part) {
    TcTile T;
    int fid, t;
    locate(L, tile, fid, t);
    t += tile_base;
    T.F = S.fronts[fid];
    const int n2 = cdiv(T.F.m, umma::TM);
    T.n2 = n2;
    if (MODE == TC_TRAIL) {
        const int blk = T.F.block0 + step;
        const int c1 = S.blk_c1[blk], bw = c1 - S.blk_c0[blk];
        const int n1 = cdiv(T.F.nf - c1, umma::TM);
        T.n1 = n1;
        if (S.sym) {   // lower tiles of the front columns only
            lower_tile(t, n1 + n2, T.rt, T.ct);
        } else if (t < (n1 + n2) * n1) {
            T.rt = t % (n1 + n2);
            T.ct = t / (n1 + n2);
        } else {
            const int t2 = t - (n1 + n2) * n1;
            T.rt = t2 % n1;
            T.ct = n1 + t2 / n1;
        }
        T.nchunks = cdiv(bw, umma::KCH);
        T.nh = 1;
    } else {
        T.n1 = 0;
        t = schur_part_tile(part, t, n2, NH, T.F.sq, S.sym != 0);
        int g;
        if (S.sym) {
            lower_tile_w(t, n2, NH, T.rt, g);
        } else {
            T.rt = t % n2;
            g = t / n2;
        }
        T.ct = NH * g;
        T.nh = min(NH, n2 - T.ct);
        if (S.sym) T.nh = min(T.nh, T.rt - T.ct + 1);   // no tile above the diagonal
        int nc = 0;
        for (int b = 0; b < T.F.nblocks; ++b) {
            const int blk = T.F.block0 + b;
            nc += cdiv(S.blk_c1[blk] - S.blk_c0[blk], umma::KCH);
        }
        T.nchunks = nc;
    }
    return T;
}

// The K loop of one tile as a sequence of pipeline stages: (block, first
// chunk, chunks).  TRAIL: the chunks of block `step`; SCHUR: those of every
// block of the front in turn.  A stage holds one chunk (TF32: hi + lo of A
// and of B) or, in the BF16 form, up to umma::BF_GROUP consecutive chunks of
// one block.  The copy and the MMA threads walk the same sequence.
template <int MODE, bool BF>
struct ChunkWalk {
    static constexpr int G = BF ? umma::BF_GROUP : 1;
    int b, c, nb, left;   // current block, its next chunk, its chunks; chunks of the tile left
    __device__ __forceinline__ ChunkWalk(const Sched& S, const TcTile& T, int step) {
        b = MODE == TC_TRAIL ? T.F.block0 + step : T.F.block0;
        c = 0;
        nb = cdiv(S.blk_c1[b] - S.blk_c0[b], umma::KCH);
        left = T.nchunks;
    }
    // Next stage: block, first chunk, number of chunks; false when done.
    __device__ __forceinline__ bool next(const Sched& S, int& blk, int& c0, int& kc) {
        if (left <= 0) return false;
        while (c == nb) {   // SCHUR: the next block of the front
            ++b;
            c = 0;
            nb = cdiv(S.blk_c1[b] - S.blk_c0[b], umma::KCH);
        }
        blk = b;
        c0 = c;
        kc = min(G, nb - c);
        c += kc;
        left -= kc;
        return true;
    }
};

template <int MODE, bool BF, int NH = 1>
__global__ void __launch_bounds__(TC_THREADS, 1) k_tc_update(float* fac, const unsigned char* pack, Sched S, Launch L,
                                                              int step, int ntiles, int tile_base, int part, int* err) {
    static_assert(MODE == TC_SCHUR || NH == 1, "wide tiles are for the Schur complements");
    using G = umma::PGeo<NH>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ ScatterRow tab[NH + 1][umma::TM];   // SCHUR: [h] columns of tile h, [NH] tile rows
    __shared__ int dead;
    const umma::PCtx cx = umma::pctx_of<NH>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < G::NST; ++s) {
            umma::mbar_init(&cx.full[s], 1);
            umma::mbar_init(&cx.empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            umma::mbar_init(&cx.tfull[b], 1);
            umma::mbar_init(&cx.tempty[b], 32 * TC_EPI);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        dead = 0;
    }
    if (warp == 1) umma::tmem_alloc(cx.tmem_slot, G::TMEM_COLS);
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = *cx.tmem_slot;
    volatile int* vdead = &dead;
    // bytes of one chunk of one operand; B tile h of a stage at BOFF + h * BSTEP
    constexpr uint32_t CB = BF ? umma::PCHUNK16 : umma::PCHUNK;
    constexpr uint32_t BOFF = 2 * umma::OPB, BSTEP = 2 * umma::OPB;
    constexpr uint32_t ACC_COLS = NH * umma::TN;

    if (warp == 0) {
        if (lane == 0) {   // bulk copies
            int s = 0;
            uint32_t ph = 0;
            for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
                const TcTile T = tc_decode<MODE, NH>(S, L, step, tile, tile_base, part);
                ChunkWalk<MODE, BF> w(S, T, step);
                int b, c, kc;
                while (w.next(S, b, c, kc)) {
                    const int nch = w.nb;
                    const int n1b = MODE == TC_TRAIL ? T.n1 : cdiv(T.F.nf - S.blk_c1[b], umma::TM);
                    const int ra = MODE == TC_TRAIL ? T.rt : n1b + T.rt;
                    const int rb = MODE == TC_TRAIL ? T.ct : n1b + T.ct;
                    const ll lp = BF ? (S.blk_lpack[b] >> 2) : S.blk_lpack[b];
                    const ll up = BF ? (S.blk_upack[b] >> 2) : S.blk_upack[b];
                    const unsigned char* pa = pack + lp + ((ll)ra * nch + c) * CB;
                    umma::wait_bounded(&cx.empty[s], ph ^ 1, vdead, err);
                    umma::arrive_expect_tx(&cx.full[s], (1 + T.nh) * kc * CB);
                    const uint32_t dst = umma::saddr(cx.stage + s * G::STAGE);
                    umma::bulk_g2s(dst, pa, kc * CB, &cx.full[s]);
                    for (int h = 0; h < T.nh; ++h) {
                        const unsigned char* pb = pack + up + ((ll)(rb + h) * nch + c) * CB;
                        umma::bulk_g2s(dst + BOFF + h * BSTEP, pb, kc * CB, &cx.full[s]);
                    }
                    if (++s == G::NST) { s = 0; ph ^= 1; }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {   // MMAs
            constexpr uint32_t IDESC = BF ? umma::idesc_bf16(umma::TM, umma::TN) : umma::idesc_tf32(umma::TM, umma::TN);
            int s = 0;
            uint32_t ph = 0;
            int acc = 0;
            uint32_t aph = 0;
            for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
                const TcTile T = tc_decode<MODE, NH>(S, L, step, tile, tile_base, part);
                umma::wait_bounded(&cx.tempty[acc], aph ^ 1, vdead, err);
                umma::fence_after();
                ChunkWalk<MODE, BF> w(S, T, step);
                int b, c, kc;
                bool first = true;
                while (w.next(S, b, c, kc)) {
                    umma::wait_bounded(&cx.full[s], ph, vdead, err);
                    umma::fence_after();
                    const uint32_t a0 = umma::saddr(cx.stage + s * G::STAGE);
                    for (int h = 0; h < T.nh; ++h) {
                        const uint32_t d = tmem + acc * ACC_COLS + h * umma::TN;
                        const uint32_t b0 = a0 + BOFF + h * BSTEP;
                        if constexpr (BF) {
                            for (int j = 0; j < kc; ++j) {   // one K = 16 product per chunk
                                const uint64_t da = umma::desc_kmajor(a0 + j * CB, 128, umma::SBO16);
                                const uint64_t db = umma::desc_kmajor(b0 + j * CB, 128, umma::SBO16);
                                umma::mma_bf16(d, da, db, IDESC, (first && j == 0) ? 0u : 1u);
                            }
                        } else {
                            const uint32_t a_hi = a0, a_lo = a0 + umma::OPB;
                            const uint32_t b_hi = b0, b_lo = b0 + umma::OPB;
#pragma unroll
                            for (int kk = 0; kk < umma::KCH / 8; ++kk) {
                                const uint32_t o = kk * 256;
                                const uint64_t dah = umma::desc_kmajor(a_hi + o, 128, umma::SBO);
                                const uint64_t dal = umma::desc_kmajor(a_lo + o, 128, umma::SBO);
                                const uint64_t dbh = umma::desc_kmajor(b_hi + o, 128, umma::SBO);
                                const uint64_t dbl = umma::desc_kmajor(b_lo + o, 128, umma::SBO);
                                umma::mma_tf32(d, dah, dbh, IDESC, (first && kk == 0) ? 0u : 1u);
                                umma::mma_tf32(d, dah, dbl, IDESC, 1u);
                                umma::mma_tf32(d, dal, dbh, IDESC, 1u);
                            }
                        }
                    }
                    first = false;
                    umma::commit(&cx.empty[s]);
                    if (++s == G::NST) { s = 0; ph ^= 1; }
                }
                umma::commit(&cx.tfull[acc]);
                if (++acc == 2) { acc = 0; aph ^= 1; }
            }
        }
    } else if (warp >= 4) {   // epilogue: thread = one TMEM lane (tile row), 32 columns of each tile
        const int q4 = warp & 3, i = 32 * q4 + lane, cg = (warp - 4) >> 2, et = threadIdx.x - 128;
        int acc = 0;
        uint32_t aph = 0;
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            const TcTile T = tc_decode<MODE, NH>(S, L, step, tile, tile_base, part);
            const DFront& F = T.F;
            if (MODE == TC_SCHUR) {
                asm volatile("bar.sync 1, %0;" ::"n"(32 * TC_EPI) : "memory");   // previous tile's scatter done
                for (int e = et; e < (T.nh + 1) * umma::TM; e += 32 * TC_EPI) {
                    const int side = e / umma::TM, rows = side == T.nh;
                    const int x = (rows ? T.rt : T.ct + side) * umma::TM + (e % umma::TM);
                    tab[rows ? NH : side][e % umma::TM] = scatter_row<float>(S, F, x);
                }
                asm volatile("bar.sync 1, %0;" ::"n"(32 * TC_EPI) : "memory");
            }
            umma::wait_bounded(&cx.tfull[acc], aph, vdead, err);
            umma::fence_after();
            const uint32_t taddr = tmem + acc * ACC_COLS + ((uint32_t)(32 * q4) << 16);
            if (MODE == TC_TRAIL) {
                const int c1 = S.blk_c1[F.block0 + step];
                const bool rL = T.rt < T.n1;   // row region [c1, nf) else [nf, ld)
                const int row = rL ? c1 + T.rt * umma::TM + i : F.nf + (T.rt - T.n1) * umma::TM + i;
                const bool rok = rL ? row < F.nf : row < F.ld;
                const bool cL = T.ct < T.n1;   // column region: front columns [c1, nf) else U12
                const int col0 = cL ? c1 + T.ct * umma::TN : (T.ct - T.n1) * umma::TN;
                const int ncol = cL ? F.nf - col0 : F.m - col0;
                {
                    const int h = cg;
                    float v[32];
                    umma::tmem_ld32(taddr + h * 32, v);
                    if (rok) {
                        // all 32 loads before any store: the compiler cannot tell that the
                        // entries are distinct, and would otherwise serialise the round trips
                        float* dst = cL ? fac + F.loff + (ll)(col0 + h * 32) * F.ld + row
                                        : fac + F.uoff + (ll)row * F.m + col0 + h * 32;
                        const ll step_j = cL ? (ll)F.ld : 1;
#pragma unroll
                        for (int half = 0; half < 2; ++half) {   // 16 loads in flight, no spills
                            float old[16];
#pragma unroll
                            for (int j = 0; j < 16; ++j) {
                                const int jj = 16 * half + j;
                                old[j] = (h * 32 + jj < ncol) ? dst[(ll)jj * step_j] : 0.0f;
                            }
#pragma unroll
                            for (int j = 0; j < 16; ++j) {
                                const int jj = 16 * half + j;
                                if (h * 32 + jj < ncol) dst[(ll)jj * step_j] = old[j] - v[jj];
                            }
                        }
                    }
                }
            } else {
                const int r = T.rt * umma::TM + i;
                const ScatterRow& R = tab[NH][i];
                for (int th = 0; th < T.nh; ++th) {
                    const int c0 = (T.ct + th) * umma::TN;
                    const int h = cg;
                    float v[32];
                    umma::tmem_ld32(taddr + th * umma::TN + h * 32, v);
                    if (r < F.m) {
                        // positions of 16 entries first (their rel[] loads in flight
                        // together), then the 16 scatter-adds
#pragma unroll
                        for (int half = 0; half < 2; ++half) {
                            int pos[16];
#pragma unroll
                            for (int j = 0; j < 16; ++j) {
                                const int jj = 16 * half + j, c = c0 + h * 32 + jj;
                                pos[j] = -1;
                                if (c < F.m && (r >= c || !S.sym))
                                    pos[j] = r >= c ? S.rel[tab[th][h * 32 + jj].rel0 + r] : S.rel[R.rel0 + c];
                            }
#pragma unroll
                            for (int j = 0; j < 16; ++j) {
                                const int jj = 16 * half + j, c = c0 + h * 32 + jj;
                                if (c >= F.m || pos[j] < 0) continue;
                                if (r >= c) {   // L entry of the front of R_F[c]
                                    const ScatterRow& Cc = tab[th][h * 32 + jj];
                                    if (Cc.pos >= 0) atomicAdd(&fac[Cc.loff + (ll)Cc.pos * Cc.ld + pos[j]], -v[jj]);
                                } else if (R.pos >= 0) {   // entry of the front of R_F[r]
                                    const int pc = pos[j];
                                    const ll addr = pc < R.nf ? R.loff + (ll)pc * R.ld + R.pos
                                                              : R.uoff + (ll)R.pos * R.m + (pc - R.nf);
                                    atomicAdd(&fac[addr], -v[jj]);
                                }
                            }
                        }
                    }
                }
            }
            umma::fence_before();
            umma::arrive(&cx.tempty[acc]);
            if (++acc == 2) { acc = 0; aph ^= 1; }
        }
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    if (warp == 1) umma::tmem_dealloc(tmem, G::TMEM_COLS);
}

// ---------------------------------------------------------------------------
// Triangular solves.  Right-hand sides are column-major n x nrhs (ld = n),
// nrhs <= 16 per launch.
// ---------------------------------------------------------------------------
constexpr int TS = 128;
constexpr int MAXRHS = 16;

// Forward step for block `step`, tiled as (128 rows below the block) x (32
// columns of the block): a tile computes its 32 values of y_B = Minv b_B
// (the interchanges and unit-lower solves of the block's pieces, the
// reference's _lulsolve!, SpkLUFactor.jl:297-321), the first row tile stores
// them, and every tile subtracts L[rows, chunk] y_chunk from its rows with
// atomics (column chunks and sibling fronts share rows).  b is the running
// right-hand side, y receives the block's values.
constexpr int SC = 32;   // block columns per solve tile
template <typename T>
__global__ void __launch_bounds__(TS) k_fwd(const T* fac, const T* inv2, T* b, T* y, int n, int nrhs, Sched S,
                                            Launch L, int step) {
    constexpr int BM = BlockMax<T>::value;
    __shared__ T sm[BM * SC];   // Minv[:, chunk], sm[k * SC + j]
    __shared__ T sb[BM * MAXRHS];
    __shared__ T sp[4 * SC * MAXRHS];
    __shared__ T sy[SC * MAXRHS];
    griddep_launch();
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int blk = F.block0 + step;
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk], bw = c1 - c0;
    const int ncc = cdiv(bw, SC), cc = tile % ncc, rt = tile / ncc;
    const int j0 = cc * SC, nj = min(SC, bw - j0);
    const T* Mi = inv2 + S.blk_inv2[blk];
    const int tid = threadIdx.x;
    // Factor data (complete before the solve) first: the chunk of Minv into
    // shared memory, this thread's row of L[:, chunk] into registers.
    for (int e = tid; e < bw * SC; e += TS) {
        const int k = e / SC, j = e % SC;
        cp_elem(&sm[e], Mi + (ll)k * bw + j0 + min(j, nj - 1), j < nj);
    }
    const int row = c1 + rt * TS + tid;
    const bool has_row = row < F.ld;
    T lv[SC];
    int grow = 0;
    {
        const T* lcol = fac + F.loff + (ll)(c0 + j0) * F.ld + (has_row ? row : c1);
#pragma unroll
        for (int j = 0; j < SC; ++j) lv[j] = (has_row && j < nj) ? lcol[(ll)j * F.ld] : T(0);
        if (has_row) grow = row < F.nf ? F.f + row : S.rows[F.rows_off + row - F.nf];
    }
    griddep_wait();
    for (int e = tid; e < bw * nrhs; e += TS) {
        int k = e % bw, r = e / bw;
        sb[r * BM + k] = b[(ll)r * n + F.f + c0 + k];
    }
    cp_wait_all();
    __syncthreads();
    {   // y_chunk = Minv[j0:j0+nj, :] b_B : 32 columns x 4 partial sums over k
        const int j = tid & 31, kq = tid >> 5;
        T acc[MAXRHS];
#pragma unroll
        for (int r = 0; r < MAXRHS; ++r) acc[r] = T(0);
#pragma unroll 8
        for (int k = kq; k < bw; k += 4) {
            const T mk = sm[k * SC + j];
#pragma unroll
            for (int r = 0; r < MAXRHS; ++r)
                if (r < nrhs) acc[r] += mk * sb[r * BM + k];
        }
#pragma unroll
        for (int r = 0; r < MAXRHS; ++r)
            if (r < nrhs) sp[(kq * MAXRHS + r) * SC + j] = acc[r];
    }
    __syncthreads();
    for (int e = tid; e < SC * nrhs; e += TS) {
        int j = e % SC, r = e / SC;
        sy[r * SC + j] = sp[(0 * MAXRHS + r) * SC + j] + sp[(1 * MAXRHS + r) * SC + j] +
                         sp[(2 * MAXRHS + r) * SC + j] + sp[(3 * MAXRHS + r) * SC + j];
    }
    __syncthreads();
    if (rt == 0)
        for (int e = tid; e < nj * nrhs; e += TS) {
            int j = e % nj, r = e / nj;
            y[(ll)r * n + F.f + c0 + j0 + j] = sy[r * SC + j];
        }
    if (has_row) {
#pragma unroll
        for (int r = 0; r < MAXRHS; ++r) {
            if (r >= nrhs) break;
            T acc = T(0);
#pragma unroll
            for (int j = 0; j < SC; ++j) acc += lv[j] * sy[r * SC + j];
            atomicAdd(&b[(ll)r * n + grow], -acc);
        }
    }
}

// Products y[F.f + k] -= dot(line k, x[R_F]) over the lines of a front's
// off-diagonal part (U12 rows for the backward solve, L21 columns for the
// transposed one; line k at base + k * stride, F.m values, contiguous).  A
// CTA (256 threads) takes a tile of U12_ROWS lines x U12_COLS positions of
// R_F: it gathers x at those positions into shared memory (four right-hand
// sides at a time), then each warp streams four lines against it, the four
// lines' loads interleaved so that 16 are in flight per lane; partial sums go
// to y with atomics.  The tile count of a front is
// cdiv(F.nf, U12_ROWS) * cdiv(F.m, U12_COLS), enough CTAs to keep HBM busy
// on the wide fronts near the root.
constexpr int U12_ROWS = 32, U12_COLS = 512, U12_RG = 4;
template <typename T>
__device__ __forceinline__ void front_line_dots(const T* base, ll stride, T* y, const T* x, int n, int nrhs,
                                                const DFront& F, const int* rows, int tile) {
    __shared__ T sx[U12_COLS * U12_RG];   // sx[c * U12_RG + r]
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int ncc = cdiv(F.m, U12_COLS);
    const int i0 = (tile / ncc) * U12_ROWS + wid, c0 = (tile % ncc) * U12_COLS;
    const int nc = min(U12_COLS, F.m - c0);
    for (int r0 = 0; r0 < nrhs; r0 += U12_RG) {
        const int nr = min(U12_RG, nrhs - r0);
        if (r0 > 0) __syncthreads();
        for (int c = threadIdx.x; c < nc; c += 256) {
            const int g = rows[c0 + c];
#pragma unroll
            for (int r = 0; r < U12_RG; ++r) sx[c * U12_RG + r] = r < nr ? x[(ll)(r0 + r) * n + g] : T(0);
        }
        __syncthreads();
        T acc[4][U12_RG];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int r = 0; r < U12_RG; ++r) acc[a][r] = T(0);
        const T* u[4];
        bool live[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            live[a] = i0 + 8 * a < F.nf;
            u[a] = base + (ll)(live[a] ? i0 + 8 * a : 0) * stride + c0;
        }
#pragma unroll 4
        for (int c = lane; c < nc; c += 32) {
            T uv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) uv[a] = live[a] ? u[a][c] : T(0);
            T xv[U12_RG];
#pragma unroll
            for (int r = 0; r < U12_RG; ++r) xv[r] = sx[c * U12_RG + r];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int r = 0; r < U12_RG; ++r) acc[a][r] += uv[a] * xv[r];
        }
#pragma unroll
        for (int a = 0; a < 4; ++a) {
#pragma unroll
            for (int r = 0; r < U12_RG; ++r) {
                T v = acc[a][r];
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
                if (lane == 0 && live[a] && r < nr) atomicAdd(&y[(ll)(r0 + r) * n + F.f + i0 + 8 * a], -v);
            }
        }
    }
}

// Backward, part 1: y[F's columns] -= U12 * x[R_F] (U12 row i contiguous in Uf).
template <typename T>
__global__ void __launch_bounds__(256) k_bwd_u12(const T* fac, T* y, const T* x, int n, int nrhs, Sched S, Launch L) {
    griddep_launch();
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    griddep_wait();
    front_line_dots<T>(fac + F.uoff, F.m, y, x, n, nrhs, F, S.rows + F.rows_off, tile);
}

// Backward, part 2, for the block `step`-th from the last, tiled as (128
// rows above the block) x (32 block columns): x_chunk = Uinv[chunk, :] c_B
// (the upper solves of the block's pieces, the reference's _luusolve!,
// SpkLUFactor.jl:350-375), stored by the first row tile, then the rows
// above get U[rows, chunk] x_chunk subtracted (atomics across chunks).
template <typename T>
__global__ void __launch_bounds__(TS) k_bwd(const T* fac, const T* inv2, T* y, T* x, int n, int nrhs, Sched S,
                                            Launch L, int step) {
    constexpr int BM = BlockMax<T>::value;
    __shared__ T sm[BM * SC];   // Uinv[:, chunk], sm[k * SC + j] (rows k >= j0)
    __shared__ T sc[BM * MAXRHS];
    __shared__ T sp[4 * SC * MAXRHS];
    __shared__ T sx[SC * MAXRHS];
    griddep_launch();
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int blk = F.block0 + F.nblocks - 1 - step;
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk], bw = c1 - c0;
    const int ncc = cdiv(bw, SC), cc = tile % ncc, rt = tile / ncc;
    const int j0 = cc * SC, nj = min(SC, bw - j0);
    const T* Ui = inv2 + S.blk_inv2[blk] + (ll)bw * bw;
    const int tid = threadIdx.x;
    // Factor data first: the chunk of Uinv, this thread's row of U[:, chunk].
    for (int e = j0 * SC + tid; e < bw * SC; e += TS) {
        const int k = e / SC, j = e % SC;
        cp_elem(&sm[e], Ui + (ll)k * bw + j0 + min(j, nj - 1), j < nj);
    }
    const int row = rt * TS + tid;
    const bool has_row = row < c0;
    T uv[SC];
    {
        const T* ucol = fac + F.loff + (ll)(c0 + j0) * F.ld + (has_row ? row : 0);
#pragma unroll
        for (int j = 0; j < SC; ++j) uv[j] = (has_row && j < nj) ? ucol[(ll)j * F.ld] : T(0);
    }
    griddep_wait();
    for (int e = tid; e < bw * nrhs; e += TS) {
        int k = e % bw, r = e / bw;
        sc[r * BM + k] = y[(ll)r * n + F.f + c0 + k];
    }
    cp_wait_all();
    __syncthreads();
    {   // x_chunk = Uinv[j0:j0+nj, :] c_B (upper: k >= j)
        const int j = tid & 31, kq = tid >> 5;
        T acc[MAXRHS];
#pragma unroll
        for (int r = 0; r < MAXRHS; ++r) acc[r] = T(0);
        if (j < nj) {
            const int kstart = j0 + j;
#pragma unroll 8
            for (int k = kstart + kq; k < bw; k += 4) {
                const T uk = sm[k * SC + j];
#pragma unroll
                for (int r = 0; r < MAXRHS; ++r)
                    if (r < nrhs) acc[r] += uk * sc[r * BM + k];
            }
        }
#pragma unroll
        for (int r = 0; r < MAXRHS; ++r)
            if (r < nrhs) sp[(kq * MAXRHS + r) * SC + j] = acc[r];
    }
    __syncthreads();
    for (int e = tid; e < SC * nrhs; e += TS) {
        int j = e % SC, r = e / SC;
        sx[r * SC + j] = sp[(0 * MAXRHS + r) * SC + j] + sp[(1 * MAXRHS + r) * SC + j] +
                         sp[(2 * MAXRHS + r) * SC + j] + sp[(3 * MAXRHS + r) * SC + j];
    }
    __syncthreads();
    if (rt == 0)
        for (int e = tid; e < nj * nrhs; e += TS) {
            int j = e % nj, r = e / nj;
            x[(ll)r * n + F.f + c0 + j0 + j] = sx[r * SC + j];
        }
    if (has_row) {
#pragma unroll
        for (int r = 0; r < MAXRHS; ++r) {
            if (r >= nrhs) break;
            T acc = T(0);
#pragma unroll
            for (int j = 0; j < SC; ++j) acc += uv[j] * sx[r * SC + j];
            atomicAdd(&y[(ll)r * n + F.f + row], -acc);
        }
    }
}

// ---------------------------------------------------------------------------
// Solves of a front with many blocks by a cluster of NC CTAs (16 where the
// GPU can hold such clusters, else FC = 8), all its block steps in one
// launch.  Step t handles block t (forward) or block nb-1-t
// (backward); CTA rank (t mod FC) owns step t: it holds that block's
// right-hand side in shared memory, receives the updates of the earlier
// steps there, and computes the step's solution (Minv b_B forward, Uinv c_B
// backward).  The solution is published in the owner's shared memory; every
// CTA reads it through distributed shared memory and subtracts its product
// with the block's column of the factor (L below the block forward, U above
// it backward) from the blocks it owns.  The operator of an owned step and
// the block linking it to the previous step are prefetched into shared
// memory while the earlier steps run.  One cluster barrier phase per step,
// split: a CTA arrives as soon as it has read the step's solution (the
// owner of the next step after publishing it), so that only the next
// owner's work is on the chain.  Same operations as k_fwd / k_bwd per step
// inside the front; forward, the R_F rows get L21 y_F afterwards from
// k_fwd_l21 (all the GPU's SMs).  Right-hand sides FC_RG at a time.  Fronts
// with at least FC_MINB and at most FC * FC_OWN blocks take this path (the
// plan decides).
// ---------------------------------------------------------------------------
constexpr int FC = 8, FC_MINB = 4, FC_OWN = 16, FC_RG = 4, FC_THREADS = 1024;

// Vectors of a block for FC_RG right-hand sides: entry (k, r) at k * FC_RG + r.
template <typename T> struct RgVec;
template <> struct RgVec<float> {
    using type = float4;
    __device__ static void get(const float* p, float (&v)[FC_RG]) {
        const float4 q = *reinterpret_cast<const float4*>(p);
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    }
};
template <> struct RgVec<double> {
    __device__ static void get(const double* p, double (&v)[FC_RG]) {
        const double2 q0 = *reinterpret_cast<const double2*>(p), q1 = *reinterpret_cast<const double2*>(p + 2);
        v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
    }
};

template <typename T>
struct FcSmem {
    static constexpr int BM = BlockMax<T>::value, CS = FC_THREADS / BM;
    static constexpr size_t ypub = 0, ycur = ypub + BM * FC_RG, own = ycur + BM * FC_RG,
                            part = own + (size_t)FC_OWN * BM * FC_RG, preA = part + (size_t)CS * BM * FC_RG,
                            preM = preA + (size_t)BM * BM, total = preM + (size_t)BM * BM;   // in T's
    static constexpr size_t bytes = total * sizeof(T);
};

// v[i * FC_RG + r] -= sum_j A(i, j) w[j * FC_RG + r], i < nrow, j < ncol,
// with A(i, j) = a[j * lda + i] (a block of the factor in global memory, or
// its prefetched copy in shared memory).  Thread (i, cs) takes columns
// cs, cs + CS, ...; all its loads are issued before the first use.
template <typename T>
__device__ __forceinline__ void fc_tile_update(const T* a, ll lda, int nrow, int ncol, T* v, const T* w, T* part) {
    constexpr int BM = BlockMax<T>::value, CS = FC_THREADS / BM, NJ = BM / CS;
    const int i = threadIdx.x % BM, cs = threadIdx.x / BM;
    T av[NJ];
#pragma unroll
    for (int q = 0; q < NJ; ++q) {
        const int j = cs + q * CS;
        av[q] = (i < nrow && j < ncol) ? a[(ll)j * lda + i] : T(0);
    }
    T acc[FC_RG];
#pragma unroll
    for (int r = 0; r < FC_RG; ++r) acc[r] = T(0);
#pragma unroll
    for (int q = 0; q < NJ; ++q) {
        T wv[FC_RG];
        RgVec<T>::get(w + (cs + q * CS) * FC_RG, wv);
#pragma unroll
        for (int r = 0; r < FC_RG; ++r) acc[r] += av[q] * wv[r];
    }
#pragma unroll
    for (int r = 0; r < FC_RG; ++r) part[(cs * BM + i) * FC_RG + r] = acc[r];
    __syncthreads();
    for (int e = threadIdx.x; e < nrow * FC_RG; e += FC_THREADS) {
        T sum = T(0);
#pragma unroll
        for (int c = 0; c < CS; ++c) sum += part[c * BM * FC_RG + e];
        v[e] -= sum;
    }
    __syncthreads();
}

// out[j * FC_RG + r] = sum_k op(j, k) v[k * FC_RG + r] for the block's solve
// operator (forward Minv, backward Uinv; op(j, k) at m[k * BM + j]).
template <typename T, bool FWD>
__device__ __forceinline__ void fc_block_solve(const T* m, int bw, const T* v, T* out, T* part, int nr) {
    constexpr int BM = BlockMax<T>::value, CS = FC_THREADS / BM;
    const int j = threadIdx.x % BM, cs = threadIdx.x / BM;
    T acc[FC_RG];
#pragma unroll
    for (int r = 0; r < FC_RG; ++r) acc[r] = T(0);
    if (j < bw) {
#pragma unroll 4
        for (int k = (FWD ? 0 : j) + cs; k < bw; k += CS) {
            const T mv = m[k * BM + j];
            T vv[FC_RG];
            RgVec<T>::get(v + k * FC_RG, vv);
#pragma unroll
            for (int r = 0; r < FC_RG; ++r) acc[r] += mv * vv[r];
        }
    }
#pragma unroll
    for (int r = 0; r < FC_RG; ++r) part[(cs * BM + j) * FC_RG + r] = acc[r];
    __syncthreads();
    for (int e = threadIdx.x; e < BM * FC_RG; e += FC_THREADS) {
        const int jj = e / FC_RG, r = e % FC_RG;
        T sum = T(0);
        if (jj < bw && r < nr)
#pragma unroll
            for (int c = 0; c < CS; ++c) sum += part[c * BM * FC_RG + e];
        out[e] = sum;
    }
    __syncthreads();
}

template <typename T, bool FWD, int NC>
__global__ void __cluster_dims__(NC, 1, 1) __launch_bounds__(FC_THREADS, 1)
    k_front_solve(const T* fac, const T* inv2, T* in, T* out, int n, int nrhs, Sched S, Launch L) {
    constexpr int FC = NC;   // CTAs of the cluster
    namespace cg = cooperative_groups;
    constexpr int BM = BlockMax<T>::value;
    using SM = FcSmem<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = reinterpret_cast<T*>(smem_raw);
    T* ypub = sm + SM::ypub;
    T* ycur = sm + SM::ycur;
    T* own = sm + SM::own;
    T* part = sm + SM::part;
    T* preA = sm + SM::preA;   // A(block of step st, block of step st - 1), [j * BM + i]
    T* preM = sm + SM::preM;   // solve operator of step st, [k * BM + j]
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const DFront F = S.fronts[L.front_ids[blockIdx.x / FC]];
    const int nb = F.nblocks, tid = threadIdx.x;
    auto blk_of = [&](int step) { return F.block0 + (FWD ? step : nb - 1 - step); };
    auto a_of = [&](int bs, int bt) { return fac + F.loff + (ll)S.blk_c0[bt] * F.ld + S.blk_c0[bs]; };
    // The factor data of owned step st (its operator, and the block linking
    // it to step st - 1) is copied asynchronously while other steps run.
    auto prefetch = [&](int st) {
        if (st >= nb) return;
        const int bs = blk_of(st), bw = S.blk_c1[bs] - S.blk_c0[bs];
        const T* Mi = inv2 + S.blk_inv2[bs] + (FWD ? 0 : (ll)bw * bw);
        for (int e = tid; e < BM * BM; e += FC_THREADS) {
            const int j = e % BM, k = e / BM;
            const bool v = j < bw && k < bw;
            cp_elem(&preM[e], v ? Mi + (ll)k * bw + j : Mi, v);
        }
        if (st > 0) {
            const int bt = blk_of(st - 1), ncol = S.blk_c1[bt] - S.blk_c0[bt];
            const T* a = a_of(bs, bt);
            for (int e = tid; e < BM * BM; e += FC_THREADS) {
                const int i = e % BM, j = e / BM;
                const bool v = i < bw && j < ncol;
                cp_elem(&preA[e], v ? a + (ll)j * F.ld + i : a, v);
            }
        }
    };
    for (int r0 = 0; r0 < nrhs; r0 += FC_RG) {
        const int nr = min(FC_RG, nrhs - r0);
        prefetch(rank);
        for (int st = rank, o = 0; st < nb; st += FC, ++o) {   // the owned blocks' right-hand sides
            const int blk = blk_of(st), c0 = S.blk_c0[blk], bw = S.blk_c1[blk] - c0;
            T* v = own + (size_t)o * BM * FC_RG;
            for (int e = tid; e < BM * FC_RG; e += FC_THREADS) {
                const int k = e / FC_RG, r = e % FC_RG;
                v[e] = (k < bw && r < nr) ? in[(ll)(r0 + r) * n + F.f + c0 + k] : T(0);
            }
        }
        __syncthreads();
        auto solve_step = [&](int st) {   // owner: publish the solution of step st
            const int blk = blk_of(st), bw = S.blk_c1[blk] - S.blk_c0[blk];
            fc_block_solve<T, FWD>(preM, bw, own + (size_t)(st / FC) * BM * FC_RG, ypub, part, nr);
        };
        auto finish_step = [&](int st) {   // owner, after the barrier arrival: output and next prefetch
            const int blk = blk_of(st), c0 = S.blk_c0[blk], bw = S.blk_c1[blk] - c0;
            for (int e = tid; e < bw * nr; e += FC_THREADS) {
                const int j = e % bw, r = e / bw;
                out[(ll)(r0 + r) * n + F.f + c0 + j] = ypub[j * FC_RG + r];
            }
            prefetch(st + FC);   // preM / preA are free again
        };
        if (rank == 0) {
            cp_wait_all();
            __syncthreads();
            solve_step(0);
        }
        cl.barrier_arrive();
        if (rank == 0) finish_step(0);
        for (int t = 0; t < nb; ++t) {
            cl.barrier_wait();
            const T* src = cl.map_shared_rank(ypub, t % FC);
            for (int e = tid; e < BM * FC_RG; e += FC_THREADS) ycur[e] = src[e];
            __syncthreads();
            const int bt = blk_of(t), ncol = S.blk_c1[bt] - S.blk_c0[bt];
            const bool next = t + 1 < nb && (t + 1) % FC == rank;
            if (next) {   // the next step's block first, from its prefetched copy: it is on the chain
                cp_wait_all();
                __syncthreads();
                const int bs = blk_of(t + 1);
                fc_tile_update<T>(preA, BM, S.blk_c1[bs] - S.blk_c0[bs], ncol,
                                  own + (size_t)((t + 1) / FC) * BM * FC_RG, ycur, part);
                solve_step(t + 1);
            }
            cl.barrier_arrive();
            if (next) finish_step(t + 1);
            for (int st = rank, o = 0; st < nb; st += FC, ++o)
                if (st > t && !(next && st == t + 1)) {
                    const int bs = blk_of(st);
                    fc_tile_update<T>(a_of(bs, bt), F.ld, S.blk_c1[bs] - S.blk_c0[bs], ncol,
                                      own + (size_t)o * BM * FC_RG, ycur, part);
                }
            __syncthreads();
        }
        cl.barrier_wait();   // every CTA has read every published solution
        cp_wait_all();   // no copy outlives the group
        __syncthreads();
    }
}

// Solves of small fronts (one block of at most 32 columns, m <= LEAF_M), one
// warp per front, eight fronts per CTA: the whole front in one pass.
//   forward:  y_F = Minv b_F; b[R_F] -= L21 y_F (atomics, the rows are
//             shared with sibling fronts);
//   backward: c_F = y_F - U12 x[R_F]; x_F = Uinv c_F.
// Each launch holds fronts of one width class W (block width <= W, the
// classes of k_leaf_factor).  Lane j holds column j of the front; the
// front's right-hand side values are exchanged by shuffles.  Every factor
// load of a pass (a lane's column of the operator, its row of L21, its part
// of U12 for 32 rows) is issued before the first use, so that a pass waits
// for one memory round trip, not one per column.  U12 x[R_F]: for W <= 8 a
// lane per row accumulates all W columns and the warp reduces once at the
// end; wider fronts keep a lane per column and shuffle x.  Same operations as
// k_fwd / k_bwd_u12 / k_bwd.
constexpr int LEAF_M = 128;

// Warp reduce-scatter: N (a power of 2, at most 32) values per lane, summed
// over the 32 lanes; each step keeps the half of the values picked by a
// lane bit and adds the partner's copy of it, and once one value is left
// the remaining lane bits are summed by a butterfly (N/2 + N/4 + ... + the
// rest shuffles instead of 5 N).  Lane l ends with the sum of value
// l * N / 32.
template <int N, int OFF, typename T>
__device__ __forceinline__ void rs_halve(T* v, int lane) {
    const bool hi = (lane & OFF) != 0;
#pragma unroll
    for (int i = 0; i < N / 2; ++i) {
        const T keep = hi ? v[i + N / 2] : v[i];
        const T send = hi ? v[i] : v[i + N / 2];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, OFF);
    }
}
template <int N, int OFF, typename T>
__device__ __forceinline__ void rs_rec(T* v, int lane) {
    if constexpr (OFF > 0) {
        if constexpr (N > 1) {
            rs_halve<N, OFF>(v, lane);
            rs_rec<N / 2, OFF / 2>(v, lane);
        } else {
            v[0] += __shfl_xor_sync(0xffffffffu, v[0], OFF);
            rs_rec<1, OFF / 2>(v, lane);
        }
    }
}
template <int N, typename T>
__device__ __forceinline__ T warp_reduce_scatter(T (&v)[N]) {
    static_assert(N >= 1 && N <= 32 && (N & (N - 1)) == 0, "a power of 2, at most 32 values");
    rs_rec<N, 16>(v, threadIdx.x & 31);
    return v[0];
}

template <typename T, bool FWD, int W, int RG>
__global__ void __launch_bounds__(256) k_solve_leaf(const T* fac, const T* inv2, T* in, T* out, const T* xs, int n,
                                                     int nrhs, Sched S, Launch L) {
    // RG: right-hand sides per pass (1 for a single one, else 4)
    const unsigned FULL = 0xffffffffu;
    griddep_launch();
    const int lane = threadIdx.x & 31, idx = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (idx >= L.count) return;   // whole warp
    const DFront F = S.fronts[L.front_ids[idx]];
    const int blk = F.block0, bw = F.nf;
    const T* Mi = inv2 + S.blk_inv2[blk] + (FWD ? 0 : (ll)bw * bw);
    const int* rows = S.rows + F.rows_off;
    griddep_wait();
    for (int r0 = 0; r0 < nrhs; r0 += RG) {
        const int nr = min(RG, nrhs - r0);
        // narrow fronts: the loads that do not depend on the solve first (the
        // operator column, forward this lane's L21 row among the first 32
        // rows), so that a front waits for fewer round trips; wider ones
        // keep them where they are used (registers)
        constexpr bool EARLY = W <= 8;
        T mv[W];   // op(lane, k), op(j, k) at Mi[k * bw + j]
        auto load_mv = [&] {
#pragma unroll
            for (int k = 0; k < W; ++k)
                mv[k] = (k < bw && lane < bw && (FWD || k >= lane)) ? Mi[(ll)k * bw + lane] : T(0);
        };
        if constexpr (EARLY) load_mv();
        T lv0[FWD && EARLY ? W : 1];
        if constexpr (FWD && EARLY) {
#pragma unroll
            for (int k = 0; k < W; ++k) lv0[k] = (k < bw && lane < F.m) ? fac[F.loff + (ll)k * F.ld + F.nf + lane] : T(0);
        }
        T v[RG];
#pragma unroll
        for (int r = 0; r < RG; ++r) v[r] = (lane < bw && r < nr) ? in[(ll)(r0 + r) * n + F.f + lane] : T(0);
        if constexpr (!FWD) {   // c_F = y_F - U12 x[R_F] (U12 row j contiguous in Uf)
            T acc[RG];
#pragma unroll
            for (int r = 0; r < RG; ++r) acc[r] = T(0);
            if constexpr (W <= 8) {
                T pw[W][RG];   // lane: its rows' share of every column's sum
#pragma unroll
                for (int j = 0; j < W; ++j)
#pragma unroll
                    for (int r = 0; r < RG; ++r) pw[j][r] = T(0);
                for (int i0 = 0; i0 < F.m; i0 += 32) {
                    const int il = i0 + lane;
                    const bool ok = il < F.m;
                    const int g = ok ? rows[il] : 0;
                    T uv[W], xv[RG];
#pragma unroll
                    for (int j = 0; j < W; ++j) uv[j] = (ok && j < bw) ? fac[F.uoff + (ll)j * F.m + il] : T(0);
#pragma unroll
                    for (int r = 0; r < RG; ++r) xv[r] = (ok && r < nr) ? xs[(ll)(r0 + r) * n + g] : T(0);
#pragma unroll
                    for (int j = 0; j < W; ++j)
#pragma unroll
                        for (int r = 0; r < RG; ++r) pw[j][r] += uv[j] * xv[r];
                }
                constexpr int NV = W * RG;   // value j * RG + r
                T flat[NV];
#pragma unroll
                for (int j = 0; j < W; ++j)
#pragma unroll
                    for (int r = 0; r < RG; ++r) flat[j * RG + r] = pw[j][r];
                const T t = warp_reduce_scatter<NV>(flat);   // lane l: value l * NV / 32
#pragma unroll
                for (int r = 0; r < RG; ++r) {
                    const T vr = __shfl_sync(FULL, t, ((lane * RG + r) * 32 / NV) & 31);
                    if (lane < bw) acc[r] = vr;
                }
            } else {
                const T* u = fac + F.uoff + (ll)lane * F.m;
                for (int i0 = 0; i0 < F.m; i0 += 32) {
                    // lane l: x at row R_F[i0 + l]; lane j: U12(j, i0 ..)
                    const int il = i0 + lane;
                    T xv[RG];
                    const int g = il < F.m ? rows[il] : 0;
#pragma unroll
                    for (int r = 0; r < RG; ++r) xv[r] = (il < F.m && r < nr) ? xs[(ll)(r0 + r) * n + g] : T(0);
                    T uv[32];
#pragma unroll
                    for (int q = 0; q < 32; ++q) uv[q] = (lane < bw && i0 + q < F.m) ? u[i0 + q] : T(0);
#pragma unroll
                    for (int q = 0; q < 32; ++q) {
                        if (i0 + q < F.m) {   // uniform
#pragma unroll
                            for (int r = 0; r < RG; ++r) acc[r] += uv[q] * __shfl_sync(FULL, xv[r], q);
                        }
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < RG; ++r) v[r] -= acc[r];
        }
        if constexpr (!EARLY) load_mv();
        T y[RG];   // lane j: sum_k op(j, k) v_k
#pragma unroll
        for (int r = 0; r < RG; ++r) y[r] = T(0);
#pragma unroll
        for (int k = 0; k < W; ++k) {
            if (k < bw) {   // uniform
#pragma unroll
                for (int r = 0; r < RG; ++r) y[r] += mv[k] * __shfl_sync(FULL, v[r], k);
            }
        }
        if (lane < bw)
#pragma unroll
            for (int r = 0; r < RG; ++r)
                if (r < nr) out[(ll)(r0 + r) * n + F.f + lane] = y[r];
        if constexpr (FWD) {   // b[R_F] -= L21 y_F (L21 column k contiguous in Lf)
            for (int i0 = 0; i0 < F.m; i0 += 32) {
                const int i = i0 + lane;
                T lv[W];   // this lane's row of L21 (the first chunk's came in early)
#pragma unroll
                for (int k = 0; k < W; ++k) {
                    if constexpr (EARLY) {
                        if (i0 == 0) { lv[k] = lv0[k]; continue; }
                    }
                    lv[k] = (k < bw && i < F.m) ? fac[F.loff + (ll)k * F.ld + F.nf + i] : T(0);
                }
                T acc[RG];
#pragma unroll
                for (int r = 0; r < RG; ++r) acc[r] = T(0);
#pragma unroll
                for (int k = 0; k < W; ++k) {
                    if (k < bw) {   // uniform
#pragma unroll
                        for (int r = 0; r < RG; ++r) acc[r] += lv[k] * __shfl_sync(FULL, y[r], k);
                    }
                }
                if (i < F.m)
#pragma unroll
                    for (int r = 0; r < RG; ++r)
                        if (r < nr) atomicAdd(&in[(ll)(r0 + r) * n + rows[i]], -acc[r]);
            }
        }
    }
}

// Forward, after k_front_solve: b[R_F] -= L21 y_F for the fronts it solved.
// Tiles of 256 R_F rows x 128 front columns; a thread takes one row
// (L21 column k contiguous in Lf), y_F of the tile's columns in shared
// memory, partial sums added to b with atomics.
constexpr int L21_ROWS = 256, L21_COLS = 64;   // 64 columns: twice the CTAs and loads in flight of 128
template <typename T>
__global__ void __launch_bounds__(256) k_fwd_l21(const T* fac, T* b, const T* y, int n, int nrhs, Sched S, Launch L) {
    __shared__ T sy[L21_COLS * FC_RG];
    griddep_launch();
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int nrt = cdiv(F.m, L21_ROWS), i0 = (tile % nrt) * L21_ROWS, k0 = (tile / nrt) * L21_COLS;
    const int nk = min(L21_COLS, F.nf - k0), i = i0 + threadIdx.x;
    const bool ok = i < F.m;
    const int grow = ok ? S.rows[F.rows_off + i] : 0;
    const T* a = fac + F.loff + (ll)k0 * F.ld + F.nf + (ok ? i : 0);
    griddep_wait();
    for (int r0 = 0; r0 < nrhs; r0 += FC_RG) {
        const int nr = min(FC_RG, nrhs - r0);
        if (r0 > 0) __syncthreads();
        for (int e = threadIdx.x; e < L21_COLS * FC_RG; e += blockDim.x) {
            const int k = e % L21_COLS, r = e / L21_COLS;
            sy[e] = (k < nk && r < nr) ? y[(ll)(r0 + r) * n + F.f + k0 + k] : T(0);
        }
        __syncthreads();
        T acc[FC_RG];
#pragma unroll
        for (int r = 0; r < FC_RG; ++r) acc[r] = T(0);
        if (ok) {
#pragma unroll 16
            for (int k = 0; k < nk; ++k) {
                const T av = a[(ll)k * F.ld];
#pragma unroll
                for (int r = 0; r < FC_RG; ++r) acc[r] += av * sy[r * L21_COLS + k];
            }
#pragma unroll
            for (int r = 0; r < FC_RG; ++r)
                if (r < nr) atomicAdd(&b[(ll)(r0 + r) * n + grow], -acc[r]);
        }
    }
}

// A root front (no rows below it) of more blocks than a cluster solves well
// in one launch is solved in chunks of consecutive blocks, a cluster launch
// each; between two of them every SM takes part in the rectangular product
// that links them: out[f + r] -= sum_c A(r, c) in[f + c] over rows
// [r0, r1) and columns [c0, c1) of the front (A(r, c) = fac[loff + c ld +
// r]; forward the L rows below the chunk, backward the U rows above it).
// Tiles of L21_ROWS rows x L21_COLS columns, atomics as k_fwd_l21.
constexpr int FC_CHUNK = 16;   // blocks per chunk at most
template <typename T>
__global__ void __launch_bounds__(256) k_front_gemv(const T* fac, T* out, const T* in, int n, int nrhs, ll loff, int ld,
                                                    int f, int r0, int r1, int c0, int c1) {
    __shared__ T sv[L21_COLS * FC_RG];
    const int nrt = cdiv(r1 - r0, L21_ROWS);
    const int i0 = r0 + (int)(blockIdx.x % nrt) * L21_ROWS, k0 = c0 + (int)(blockIdx.x / nrt) * L21_COLS;
    const int nk = min(L21_COLS, c1 - k0), i = i0 + threadIdx.x;
    const bool ok = i < r1;
    const T* a = fac + loff + (ll)k0 * ld + (ok ? i : 0);
    for (int q0 = 0; q0 < nrhs; q0 += FC_RG) {
        const int nr = min(FC_RG, nrhs - q0);
        if (q0 > 0) __syncthreads();
        for (int e = threadIdx.x; e < L21_COLS * FC_RG; e += blockDim.x) {
            const int k = e % L21_COLS, r = e / L21_COLS;
            sv[e] = (k < nk && r < nr) ? in[(ll)(q0 + r) * n + f + k0 + k] : T(0);
        }
        __syncthreads();
        T acc[FC_RG];
#pragma unroll
        for (int r = 0; r < FC_RG; ++r) acc[r] = T(0);
        if (ok) {
#pragma unroll 16
            for (int k = 0; k < nk; ++k) {
                const T av = a[(ll)k * ld];
#pragma unroll
                for (int r = 0; r < FC_RG; ++r) acc[r] += av * sv[r * L21_COLS + k];
            }
#pragma unroll
            for (int r = 0; r < FC_RG; ++r)
                if (r < nr) atomicAdd(&out[(ll)(q0 + r) * n + f + i], -acc[r]);
        }
    }
}

// ---------------------------------------------------------------------------
// Transposed solves, A^T x = b with the same factors (no reference kernel:
// the reference's `transposetriangularsolve` is commented out,
// SpkSparseSpdSolver.jl:384).  With A~ = L U factored block by block, the
// forward operator is E_N ... E_1 (E_B: y_B = Minv_B b_B, b_below -=
// L_below,B y_B) and the backward one G_1 ... G_N (G_B: x_B = Uinv_B (y_B -
// U_B,right x_right)); A~^T = (G-chain)^T (E-chain)^T reversed:
//   pass 1, blocks in order (children first): z_B = Uinv_B^T c_B, then the
//     columns right of the block (front columns and U12, through R_F) get
//     U_B,right^T z_B subtracted;
//   pass 2, fronts top-down: the front's columns get L21^T x[R_F]
//     subtracted, then blocks in reverse: x_B = Minv_B^T z_B, and the
//     front's earlier columns get L_B,earlier^T x_B subtracted.
// The tiles and launch lists are those of k_fwd / k_bwd_u12 / k_bwd.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(TS) k_tfwd(const T* fac, const T* inv2, T* b, T* z, int n, int nrhs, Sched S,
                                             Launch L, int step) {
    constexpr int BM = BlockMax<T>::value;
    __shared__ T sb[BM * MAXRHS];
    __shared__ T sp[4 * SC * MAXRHS];
    __shared__ T sz[SC * MAXRHS];
    griddep_launch();
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int blk = F.block0 + step;
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk], bw = c1 - c0;
    const int ncc = cdiv(bw, SC), cc = tile % ncc, rt = tile / ncc;
    const int j0 = cc * SC, nj = min(SC, bw - j0);
    const T* Ui = inv2 + S.blk_inv2[blk] + (ll)bw * bw;   // Uinv(k, j) at Ui[j * bw + k], zero for k > j
    griddep_wait();
    const int tid = threadIdx.x;
    for (int e = tid; e < bw * nrhs; e += TS) {
        int k = e % bw, r = e / bw;
        sb[r * BM + k] = b[(ll)r * n + F.f + c0 + k];
    }
    __syncthreads();
    {   // z_chunk = (Uinv^T)[j0:j0+nj, :] c_B : 32 columns x 4 partial sums over k <= j
        const int j = tid & 31, kq = tid >> 5;
        T acc[MAXRHS];
#pragma unroll
        for (int r = 0; r < MAXRHS; ++r) acc[r] = T(0);
        if (j < nj) {
            const T* ucol = Ui + (ll)(j0 + j) * bw;
#pragma unroll 8
            for (int k = kq; k <= j0 + j; k += 4) {
                const T uk = ucol[k];
#pragma unroll
                for (int r = 0; r < MAXRHS; ++r)
                    if (r < nrhs) acc[r] += uk * sb[r * BM + k];
            }
        }
#pragma unroll
        for (int r = 0; r < MAXRHS; ++r)
            if (r < nrhs) sp[(kq * MAXRHS + r) * SC + j] = acc[r];
    }
    __syncthreads();
    for (int e = tid; e < SC * nrhs; e += TS) {
        int j = e % SC, r = e / SC;
        sz[r * SC + j] = sp[(0 * MAXRHS + r) * SC + j] + sp[(1 * MAXRHS + r) * SC + j] +
                         sp[(2 * MAXRHS + r) * SC + j] + sp[(3 * MAXRHS + r) * SC + j];
    }
    __syncthreads();
    if (rt == 0)
        for (int e = tid; e < nj * nrhs; e += TS) {
            int j = e % nj, r = e / nj;
            z[(ll)r * n + F.f + c0 + j0 + j] = sz[r * SC + j];
        }
    const int col = c1 + rt * TS + tid;   // a column right of the block: front column (< nf) or U12 column
    if (col < F.ld) {
        T uv[SC];
        int gcol;
        if (col < F.nf) {
            gcol = F.f + col;
            const T* u = fac + F.loff + (ll)col * F.ld + c0 + j0;      // U(c0 + j0 + jj, col), contiguous
#pragma unroll
            for (int jj = 0; jj < SC; ++jj) uv[jj] = jj < nj ? u[jj] : T(0);
        } else {
            const int uc = col - F.nf;
            gcol = S.rows[F.rows_off + uc];
            const T* u = fac + F.uoff + (ll)(c0 + j0) * F.m + uc;       // U12(c0 + j0 + jj, uc)
#pragma unroll
            for (int jj = 0; jj < SC; ++jj) uv[jj] = jj < nj ? u[(ll)jj * F.m] : T(0);
        }
#pragma unroll
        for (int r = 0; r < MAXRHS; ++r) {
            if (r >= nrhs) break;
            T acc = T(0);
#pragma unroll
            for (int jj = 0; jj < SC; ++jj) acc += uv[jj] * sz[r * SC + jj];
            atomicAdd(&b[(ll)r * n + gcol], -acc);
        }
    }
}

// Pass 2, per front: z[F's columns] -= L21^T x[R_F] (L21 column k contiguous in Lf).
template <typename T>
__global__ void __launch_bounds__(256) k_tbwd_l21(const T* fac, T* z, const T* x, int n, int nrhs, Sched S, Launch L) {
    griddep_launch();
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    griddep_wait();
    front_line_dots<T>(fac + F.loff + F.nf, F.ld, z, x, n, nrhs, F, S.rows + F.rows_off, tile);
}

// Pass 2, block `step`-th from the last: x_chunk = (Minv^T)[chunk, :] z_B,
// stored by the first tile, then the front's columns before the block get
// L[block rows, column]^T x_chunk subtracted (atomics across chunks).
template <typename T>
__global__ void __launch_bounds__(TS) k_tbwd(const T* fac, const T* inv2, T* z, T* x, int n, int nrhs, Sched S,
                                             Launch L, int step) {
    constexpr int BM = BlockMax<T>::value;
    __shared__ T sc[BM * MAXRHS];
    __shared__ T sp[4 * SC * MAXRHS];
    __shared__ T sx[SC * MAXRHS];
    griddep_launch();
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int blk = F.block0 + F.nblocks - 1 - step;
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk], bw = c1 - c0;
    const int ncc = cdiv(bw, SC), cc = tile % ncc, rt = tile / ncc;
    const int j0 = cc * SC, nj = min(SC, bw - j0);
    const T* Mi = inv2 + S.blk_inv2[blk];   // Minv(k, j) at Mi[j * bw + k]
    griddep_wait();
    const int tid = threadIdx.x;
    for (int e = tid; e < bw * nrhs; e += TS) {
        int k = e % bw, r = e / bw;
        sc[r * BM + k] = z[(ll)r * n + F.f + c0 + k];
    }
    __syncthreads();
    {
        const int j = tid & 31, kq = tid >> 5;
        T acc[MAXRHS];
#pragma unroll
        for (int r = 0; r < MAXRHS; ++r) acc[r] = T(0);
        if (j < nj) {
            const T* mcol = Mi + (ll)(j0 + j) * bw;
#pragma unroll 8
            for (int k = kq; k < bw; k += 4) {
                const T mk = mcol[k];
#pragma unroll
                for (int r = 0; r < MAXRHS; ++r)
                    if (r < nrhs) acc[r] += mk * sc[r * BM + k];
            }
        }
#pragma unroll
        for (int r = 0; r < MAXRHS; ++r)
            if (r < nrhs) sp[(kq * MAXRHS + r) * SC + j] = acc[r];
    }
    __syncthreads();
    for (int e = tid; e < SC * nrhs; e += TS) {
        int j = e % SC, r = e / SC;
        sx[r * SC + j] = sp[(0 * MAXRHS + r) * SC + j] + sp[(1 * MAXRHS + r) * SC + j] +
                         sp[(2 * MAXRHS + r) * SC + j] + sp[(3 * MAXRHS + r) * SC + j];
    }
    __syncthreads();
    if (rt == 0)
        for (int e = tid; e < nj * nrhs; e += TS) {
            int j = e % nj, r = e / nj;
            x[(ll)r * n + F.f + c0 + j0 + j] = sx[r * SC + j];
        }
    const int col = rt * TS + tid;   // a front column before the block
    if (col < c0) {
        T lv[SC];
        const T* l = fac + F.loff + (ll)col * F.ld + c0 + j0;   // L(c0 + j0 + jj, col), contiguous
#pragma unroll
        for (int jj = 0; jj < SC; ++jj) lv[jj] = jj < nj ? l[jj] : T(0);
#pragma unroll
        for (int r = 0; r < MAXRHS; ++r) {
            if (r >= nrhs) break;
            T acc = T(0);
#pragma unroll
            for (int jj = 0; jj < SC; ++jj) acc += lv[jj] * sx[r * SC + jj];
            atomicAdd(&z[(ll)r * n + F.f + col], -acc);
        }
    }
}

// dA (on A's pattern, CSC order) = -sum_r lambda_r x_r^T: the gradient of a
// loss of x = A^{-1} b with respect to A's stored entries, given the adjoint
// lambda = A^{-T} dloss/dx.
__global__ void k_grad_pattern(const int* __restrict__ row, const int* __restrict__ colof, const double* __restrict__ lam,
                               const double* __restrict__ x, ll ld, int nrhs, double* __restrict__ dA, ll nnz) {
    for (ll k = (ll)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (ll)gridDim.x * blockDim.x) {
        const int i = row[k], j = colof[k];
        double s = 0.0;
        for (int r = 0; r < nrhs; ++r) s += lam[(ll)r * ld + i] * x[(ll)r * ld + j];
        dA[k] = -s;
    }
}

// ---------------------------------------------------------------------------
// Assembly, permutation, residual.
// ---------------------------------------------------------------------------

// Zero-initialised factor storage += A's values at their slots (_inmatrix!).
// A's values in CSR order (aval in CSC order, src the CSC index of each CSR
// position), so that the residuals read each row's values contiguously.
__global__ void __launch_bounds__(256) k_gather_csr(const double* __restrict__ aval, const ll* __restrict__ src,
                                                    double* __restrict__ acsr, ll nnz) {
    for (ll k = blockIdx.x * (ll)blockDim.x + threadIdx.x; k < nnz; k += (ll)gridDim.x * blockDim.x)
        acsr[k] = aval[src[k]];
}

template <typename T>
__global__ void k_scatter_values(const double* __restrict__ aval, const ll* __restrict__ slot, T* fac, ll nnz) {
    ll k = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    ll stride = (ll)gridDim.x * blockDim.x;
    for (; k < nnz; k += stride) atomicAdd(&fac[slot[k]], (T)aval[k]);
}

// out[i + r*n] = in[perm[i] + r*ldin]: rhs into permuted order (and precision).
template <typename Tin, typename Tout>
__global__ void k_permute(const Tin* __restrict__ in, ll ldin, Tout* __restrict__ out, ll ldout, const int* __restrict__ perm,
                          int n, int nrhs) {
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (ll)n * nrhs) return;
    int i = (int)(t % n), r = (int)(t / n);
    out[(ll)r * ldout + i] = (Tout)in[(ll)r * ldin + perm[i]];
}

// x[j] (+)= xp[invp[j]]: solution back to original order.
template <typename Tin>
__global__ void k_unpermute(const Tin* __restrict__ xp, ll ldp, double* __restrict__ x, ll ldx, const int* __restrict__ invp,
                            int n, int nrhs, int accumulate) {
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (ll)n * nrhs) return;
    int j = (int)(t % n), r = (int)(t / n);
    double v = (double)xp[(ll)r * ldp + invp[j]];
    if (accumulate) x[(ll)r * ldx + j] += v; else x[(ll)r * ldx + j] = v;
}

// Sums of the squares of r and b for RES_RG right-hand sides over a CTA
// (256 threads), one atomic per sum and CTA.
constexpr int RES_RG = 4;
__device__ __forceinline__ void residual_sums(double (&rr)[RES_RG], double (&bb)[RES_RG], int r0, int nr,
                                              double* __restrict__ sums) {
    __shared__ double part[8][2 * RES_RG];
#pragma unroll
    for (int q = 0; q < RES_RG; ++q)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            rr[q] += __shfl_down_sync(0xffffffffu, rr[q], off);
            bb[q] += __shfl_down_sync(0xffffffffu, bb[q], off);
        }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int q = 0; q < RES_RG; ++q) {
            part[w][2 * q] = rr[q];
            part[w][2 * q + 1] = bb[q];
        }
    __syncthreads();
    if (threadIdx.x < 2 * nr) {
        double t = 0.0;
        for (int v = 0; v < (int)(blockDim.x >> 5); ++v) t += part[v][threadIdx.x];
        atomicAdd(&sums[2 * r0 + threadIdx.x], t);
    }
    __syncthreads();
}

// r = b - A x in FP64 with A in row order (values gathered from CSC order
// through src), or r = b - A^T x with A^T's rows = A's CSC columns (src
// null); the squares of r and b are accumulated per right-hand side.  A
// thread takes a row for RES_RG right-hand sides at a time.
__global__ void __launch_bounds__(256) k_residual(const double* __restrict__ aval, const int* __restrict__ rowptr,
                                                  const int* __restrict__ col, const ll* __restrict__ src,
                                                  const double* __restrict__ x, ll ldx, const double* __restrict__ b,
                                                  ll ldb, double* __restrict__ r, int n, int nrhs,
                                                  double* __restrict__ sums) {
    for (int r0 = 0; r0 < nrhs; r0 += RES_RG) {
        const int nr = min(RES_RG, nrhs - r0);
        double rr[RES_RG], bb[RES_RG];
#pragma unroll
        for (int q = 0; q < RES_RG; ++q) rr[q] = bb[q] = 0.0;
        // grid-stride over the rows: one partial sum per CTA and right-hand side
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
            double s[RES_RG];
#pragma unroll
            for (int q = 0; q < RES_RG; ++q) s[q] = 0.0;
            for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
                const double a = aval[src ? src[k] : k];
                const int c = col[k];
#pragma unroll
                for (int q = 0; q < RES_RG; ++q)
                    if (q < nr) s[q] += a * x[(ll)(r0 + q) * ldx + c];
            }
#pragma unroll
            for (int q = 0; q < RES_RG; ++q)
                if (q < nr) {
                    const double bi = b[(ll)(r0 + q) * ldb + i], ri = bi - s[q];
                    r[(ll)(r0 + q) * n + i] = ri;
                    rr[q] += ri * ri;
                    bb[q] += bi * bi;
                }
        }
        residual_sums(rr, bb, r0, nr, sums);
    }
}

// ---------------------------------------------------------------------------
// GMRES-IR (refinement whose correction equation A d = r is solved by GMRES
// in FP64, preconditioned on the right by the low-precision LU).  Vectors are
// n x nrhs column-major (ld n); a basis is an array of such blocks, vector j
// at V + j * n * nrhs.  Every right-hand side has its own Krylov space.
// ---------------------------------------------------------------------------

// w = A z (FP64, rows of A; values in CSR order, or gathered from CSC order
// through src).
__global__ void __launch_bounds__(256) k_gm_spmv(const double* __restrict__ aval, const int* __restrict__ rowptr,
                                                 const int* __restrict__ col, const ll* __restrict__ src,
                                                 const double* __restrict__ z, double* __restrict__ w, int n, int nrhs) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        for (int r0 = 0; r0 < nrhs; r0 += RES_RG) {
            double acc[RES_RG] = {0.0, 0.0, 0.0, 0.0};
            for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
                const double a = aval[src ? src[k] : k];
                const int c = col[k];
#pragma unroll
                for (int q = 0; q < RES_RG; ++q)
                    if (r0 + q < nrhs) acc[q] += a * z[(ll)(r0 + q) * n + c];
            }
#pragma unroll
            for (int q = 0; q < RES_RG; ++q)
                if (r0 + q < nrhs) w[(ll)(r0 + q) * n + i] = acc[q];
        }
    }
}

constexpr int GM_MAXRHS = 16;

// out[j * nrhs + r] += <V_j[:, r], w[:, r]> for the basis vectors j = blockIdx.y
// (w may be V itself with nv = 1: squared norms).
__global__ void __launch_bounds__(256) k_gm_dots(const double* __restrict__ V, const double* __restrict__ w, int n,
                                                 int nrhs, double* __restrict__ out) {
    __shared__ double part[8][GM_MAXRHS];
    const int j = blockIdx.y;
    const double* v = V + (ll)j * n * nrhs;
    double acc[GM_MAXRHS];
#pragma unroll
    for (int r = 0; r < GM_MAXRHS; ++r) acc[r] = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
#pragma unroll
        for (int r = 0; r < GM_MAXRHS; ++r)
            if (r < nrhs) acc[r] += v[(ll)r * n + i] * w[(ll)r * n + i];
    const int wp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int r = 0; r < GM_MAXRHS; ++r) {
        double t = acc[r];
        for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
        if (lane == 0) part[wp][r] = t;
    }
    __syncthreads();
    if ((int)threadIdx.x < nrhs) {
        double t = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += part[q][threadIdx.x];
        atomicAdd(&out[(ll)j * nrhs + threadIdx.x], t);
    }
}

// w[:, r] += sign * sum_{j < nv} c[j * nrhs + r] V_j[:, r]  (w has leading dimension ldw).
__global__ void __launch_bounds__(256) k_gm_axpy(const double* __restrict__ V, const double* __restrict__ c,
                                                 double* __restrict__ w, ll ldw, int n, int nrhs, int nv, double sign) {
    const ll tot = (ll)n * nrhs;
    for (ll e = (ll)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (ll)gridDim.x * blockDim.x) {
        const int r = (int)(e / n);
        const int i = (int)(e - (ll)r * n);
        double t = 0.0;
        for (int j = 0; j < nv; ++j) t += c[(ll)j * nrhs + r] * V[(ll)j * tot + e];
        w[(ll)r * ldw + i] += sign * t;
    }
}

// v[:, r] = w[:, r] / sqrt(nrm2[r]) (zero where the norm is zero).
__global__ void __launch_bounds__(256) k_gm_scale(const double* __restrict__ w, const double* __restrict__ nrm2,
                                                  double* __restrict__ v, int n, int nrhs) {
    const ll tot = (ll)n * nrhs;
    for (ll e = (ll)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (ll)gridDim.x * blockDim.x) {
        const double s = nrm2[e / n];
        v[e] = s > 0.0 ? w[e] / sqrt(s) : 0.0;
    }
}

// Norms only: sums[2r] += ||b_r - A x_r||^2 and sums[2r+1] += ||b_r||^2, with
// no residual vector written (used where no work space may be allocated).
__global__ void __launch_bounds__(256) k_residual_norms(const double* __restrict__ aval, const int* __restrict__ rowptr,
                                                        const int* __restrict__ col, const ll* __restrict__ src,
                                                        const double* __restrict__ x, ll ldx,
                                                        const double* __restrict__ b, ll ldb, int n, int nrhs,
                                                        double* __restrict__ sums) {
    for (int r0 = 0; r0 < nrhs; r0 += RES_RG) {
        const int nr = min(RES_RG, nrhs - r0);
        double rr[RES_RG], bb[RES_RG];
#pragma unroll
        for (int q = 0; q < RES_RG; ++q) rr[q] = bb[q] = 0.0;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
            double s[RES_RG];
#pragma unroll
            for (int q = 0; q < RES_RG; ++q) s[q] = 0.0;
            for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
                const double a = aval[src ? src[k] : k];
                const int c = col[k];
#pragma unroll
                for (int q = 0; q < RES_RG; ++q)
                    if (q < nr) s[q] += a * x[(ll)(r0 + q) * ldx + c];
            }
#pragma unroll
            for (int q = 0; q < RES_RG; ++q)
                if (q < nr) {
                    const double bi = b[(ll)(r0 + q) * ldb + i], ri = bi - s[q];
                    rr[q] += ri * ri;
                    bb[q] += bi * bi;
                }
        }
        residual_sums(rr, bb, r0, nr, sums);
    }
}

}  // namespace spk


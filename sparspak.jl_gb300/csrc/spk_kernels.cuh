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

#include <cuda_runtime.h>
#include <stdint.h>

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
    int pad;
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
    const ll* blk_inv;     // offset in inv[] of the pieces' inverses
    const ll* blk_inv2;    // offset in inv2[] of the block's Minv (then Uinv), bw x bw each
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

template <typename T> __device__ __forceinline__ T tabs(T x) { return x < T(0) ? -x : x; }

// Widest supernode handled.  The reference's splitting rule
// (src/SparseSpdMethod/SpkSymFct.jl:432-460) caps pieces near maxblocksize
// but lets the last piece of a long chain reach about 1.5x that (46 for 30).
constexpr int MAXW = 64;

// ---------------------------------------------------------------------------
// Blocks.  The pieces of a front are processed in *blocks* of consecutive
// pieces (at most BlockMax<T> columns).  k_block_lu factors a block in
// shared memory piece by piece with exactly the reference's in-block
// pivoting: ggetrf! on the piece's diagonal block (one warp), _luswap! of
// the piece's U rows and the two _trsm! panels inside the block, and the
// block-local trailing update.  For every piece p it also stores two w x w
// matrices in inv[] (at 2 * sum of the earlier pieces' w^2):
//   Ui_p = U_pp^{-1}            and   Li_p = L_pp^{-1} P_p
// (P_p the piece's interchanges), so that the L panel below a piece is
// X * Ui_p, the U panel to its right Li_p * Y, and the triangular-solve
// steps of the piece Li_p * b and Ui_p * c: small dense products.
// ---------------------------------------------------------------------------
template <typename T> struct BlockMax;
template <> struct BlockMax<float> { static constexpr int value = 128; };
template <> struct BlockMax<double> { static constexpr int value = 64; };

// ggetrf! of the w x w diagonal block of a piece (w <= 64), by one warp:
// A points at the block's first entry, column-major with leading dimension
// lda.  piv[k] = 0-based local pivot row; returns true on a zero pivot.
template <typename T>
__device__ bool warp_getrf(T* A, int lda, int w, int* piv) {
    const int lane = threadIdx.x & 31;
    bool sing = false;
    for (int k = 0; k < w; ++k) {
        double key = -1.0;
        int idx = w;
        for (int i = k + lane; i < w; i += 32) {
            double v = (double)tabs(A[k * lda + i]);
            double ki = (v != v) ? ((i == k) ? __longlong_as_double(0x7ff0000000000000LL) : -1.0) : v;
            if (ki > key || idx == w) { key = ki; idx = i; }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            double k2 = __shfl_xor_sync(0xffffffffu, key, off);
            int i2 = __shfl_xor_sync(0xffffffffu, idx, off);
            if (k2 > key || (k2 == key && i2 < idx)) { key = k2; idx = i2; }
        }
        const int kp = idx;
        if (lane == 0) piv[k] = kp;
        const T pv = A[k * lda + kp];
        __syncwarp();
        if (pv != T(0)) {
            if (kp != k)
                for (int j = lane; j < w; j += 32) {
                    T t = A[j * lda + k];
                    A[j * lda + k] = A[j * lda + kp];
                    A[j * lda + kp] = t;
                }
            __syncwarp();
            const T inv = T(1) / A[k * lda + k];
            for (int i = k + 1 + lane; i < w; i += 32) A[k * lda + i] *= inv;
        } else {
            sing = true;
        }
        __syncwarp();
        for (int i = k + 1 + lane; i < w; i += 32) {
            const T lik = A[k * lda + i];
            for (int j = k + 1; j < w; ++j) A[j * lda + i] -= lik * A[j * lda + k];
        }
        __syncwarp();
    }
    return sing;
}

// Inverses of a factored piece: Ui = U^{-1} (upper solve on the identity,
// as trsm 'l','u','n','n') and Li = L^{-1} P (laswp then unit-lower solve on
// the identity, as _lulsolve!), each w x w column-major (ld w), one lane per
// column.  Warp 0 of the caller forms Ui, warp 1 forms Li.
template <typename T>
__device__ void piece_inverses(const T* A, int lda, int w, const int* piv, T* Ui, T* Li) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        for (int j = lane; j < w; j += 32) {
            T* u = Ui + j * w;
            for (int i = 0; i < w; ++i) u[i] = T(i == j);
            for (int k = j; k >= 0; --k) {
                T uk = u[k];
                if (uk != T(0)) {
                    uk /= A[k * lda + k];
                    u[k] = uk;
                    for (int i = 0; i < k; ++i) u[i] -= uk * A[k * lda + i];
                }
            }
        }
    } else if (warp == 1) {
        for (int j = lane; j < w; j += 32) {
            T* v = Li + j * w;
            for (int i = 0; i < w; ++i) v[i] = T(i == j);
            for (int k = 0; k < w; ++k) {
                int kp = piv[k];
                if (kp != k) { T t = v[k]; v[k] = v[kp]; v[kp] = t; }
            }
            for (int k = 0; k < w; ++k) {
                T vk = v[k];
                if (vk != T(0))
                    for (int i = k + 1; i < w; ++i) v[i] -= vk * A[k * lda + i];
            }
        }
    }
}

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

// r[k] for a runtime k without indexing a register array dynamically.
template <typename T>
__device__ __forceinline__ T pick32(const T (&r)[32], int k) {
    T v = r[0];
#pragma unroll
    for (int j = 1; j < 32; ++j)
        if (j == k) v = r[j];
    return v;
}

// One right-looking LU sweep over the columns [0, ncols) of a register block
// held one row per lane (rows/columns below 32).  For column k in piece
// [a, b): pivot = first strict maximum among rows [k, b) (ggetrf!), whole
// rows interchanged over columns [a, 32) (the piece's columns, then
// _luswap! of its U rows), column k scaled below the diagonal (ggetrf!
// scaling, and the L-panel trsm 'r','u','n','n' for rows past the piece),
// rank-1 update of rows and columns after k (ggetrf!, the U-panel trsm
// 'r','l','t','u' and the block-local update).  `nrows` rows take part.
template <typename T>
__device__ bool warp_lu_sweep(T (&r)[32], int nrows, int ncols, const int* q0, int* piv) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    bool sing = false;
    int pc = 0;
#pragma unroll 1
    for (int k = 0; k < ncols; ++k) {
        while (q0[pc + 1] <= k) ++pc;
        const int a = q0[pc], b = q0[pc + 1];
        const T rk0 = pick32(r, k);
        const int kp = warp_first_max(pivot_key(rk0, lane >= k && lane < b, lane == k));
        if (lane == 0) piv[k] = kp - a;
        const T pv = __shfl_sync(FULL, rk0, kp);
        if (pv != T(0)) {
            if (kp != k) {
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const T vk = __shfl_sync(FULL, r[j], k), vp = __shfl_sync(FULL, r[j], kp);
                    if (j >= a) {
                        if (lane == k) r[j] = vp;
                        else if (lane == kp) r[j] = vk;
                    }
                }
            }
            const T inv = T(1) / pv;
            if (lane > k && lane < nrows) {
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    if (j == k) r[j] *= inv;
            }
        } else {
            sing = true;
        }
        const T lk = pick32(r, k);
        T u[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) u[j] = __shfl_sync(FULL, r[j], k);
        if (lane > k && lane < nrows) {
#pragma unroll
            for (int j = 0; j < 32; ++j)
                if (j > k) r[j] -= lk * u[j];
        }
    }
    return sing;
}

// ggetrf! of a piece of at most 32 columns by one warp, lane i holding row
// i in registers; A (w x w, column-major, leading dimension lda) is read and
// written back; piv[k] receives the local pivot row.
template <typename T>
__device__ bool warp_getrf32(T* A, int lda, int w, int* piv) {
    const int lane = threadIdx.x & 31;
    T r[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) r[j] = (lane < w && j < w) ? A[j * lda + lane] : T(0);
    const int q0[2] = {0, w};
    const bool sing = warp_lu_sweep(r, w, w, q0, piv);
    if (lane < w) {
#pragma unroll
        for (int j = 0; j < 32; ++j)
            if (j < w) A[j * lda + lane] = r[j];
    }
    return sing;
}

// Ui = U^{-1} of a factored piece (w <= 32) by one warp: trsm 'l','u','n','n'
// on the identity, lane j forming column j.
template <typename T>
__device__ void warp_inv_upper32(const T* A, int lda, int w, T* Ui) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    T r[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) r[j] = (lane < w && j < w) ? A[j * lda + lane] : T(0);
    T x[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) x[i] = T(i == lane);
#pragma unroll 1
    for (int k = w - 1; k >= 0; --k) {
        const T rk = pick32(r, k);
        T uk[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) uk[i] = __shfl_sync(FULL, rk, i);   // column k of U
        T xk = pick32(x, k);
        if (xk != T(0)) {
            xk /= pick32(uk, k);
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                if (i == k) x[i] = xk;
                else if (i < k) x[i] -= xk * uk[i];
            }
        }
    }
    if (lane < w) {
#pragma unroll
        for (int i = 0; i < 32; ++i)
            if (i < w) Ui[lane * w + i] = x[i];
    }
}

// Li = L^{-1} P of a factored piece (w <= 32) by one warp: laswp then trsm
// 'l','l','n','u' on the identity, lane j forming column j.
template <typename T>
__device__ void warp_inv_lower32(const T* A, int lda, int w, const int* piv, T* Li) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    T r[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) r[j] = (lane < w && j < w) ? A[j * lda + lane] : T(0);
    int pos = lane;
    for (int k = 0; k < w; ++k) {
        const int kp = piv[k];
        if (pos == k) pos = kp;
        else if (pos == kp) pos = k;
    }
    T x[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) x[i] = T(i == pos);
#pragma unroll 1
    for (int k = 0; k < w; ++k) {
        const T rk = pick32(r, k);
        T lk[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) lk[i] = __shfl_sync(FULL, rk, i);   // column k of L
        const T xk = pick32(x, k);
        if (xk != T(0)) {
#pragma unroll
            for (int i = 0; i < 32; ++i)
                if (i > k && i < w) x[i] -= xk * lk[i];
        }
    }
    if (lane < w) {
#pragma unroll
        for (int i = 0; i < 32; ++i)
            if (i < w) Li[lane * w + i] = x[i];
    }
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
template <typename T>
__device__ bool warp_block_lu32(T* A, int lda, int bw, const int* q0, int np, int* piv) {
    const int lane = threadIdx.x & 31;
    (void)np;
    T r[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) r[j] = (lane < bw && j < bw) ? A[j * lda + lane] : T(0);
    const bool sing = warp_lu_sweep(r, bw, bw, q0, piv);
    if (lane < bw) {
#pragma unroll
        for (int j = 0; j < 32; ++j)
            if (j < bw) A[j * lda + lane] = r[j];
    }
    __syncwarp();
    return sing;
}

// Blocks of at most 32 columns: one warp per block, four blocks per CTA (the
// launch holds one block per front).  Same outputs as k_block_lu.
template <typename T>
__global__ void __launch_bounds__(128) k_block_lu_small(T* fac, int* ipiv, int* info, T* inv, Sched S, Launch L,
                                                         int step) {
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
    for (int j = 0; j < bw; ++j)
        if (lane < bw) A[j * lda + lane] = fac[F.loff + (ll)(c0 + j) * F.ld + c0 + lane];
    __syncwarp();
    const bool sing = warp_block_lu32(A, lda, bw, q0, np, piv);
    for (int j = 0; j < bw; ++j)
        if (lane < bw) fac[F.loff + (ll)(c0 + j) * F.ld + c0 + lane] = A[j * lda + lane];
    if (lane < bw) ipiv[F.f + c0 + lane] = piv[lane];
    T* out = inv + S.blk_inv[blk];
    int woff = 0;
    for (int pc = 0; pc < np; ++pc) {
        const int a = q0[pc], w = q0[pc + 1] - a;
        warp_inv_upper32(A + a * lda + a, lda, w, out + woff);
        warp_inv_lower32(A + a * lda + a, lda, w, piv + a, out + woff + w * w);
        woff += 2 * w * w;
    }
    if (lane == 0 && sing) {   // sing is uniform across the warp
        for (int pc = 0; pc < np; ++pc) {
            bool z = false;
            for (int k = q0[pc]; k < q0[pc + 1]; ++k) z |= A[k * lda + k] == T(0);
            if (z) { atomicMin(info, p0 + pc + 1); break; }
        }
    }
}

// One CTA (256 threads) per front: factor block `step` of the front in shared
// memory, write it back with its pivots and the pieces' inverses.
// Dynamic shared memory: bwmax * (bwmax | 1) + 2 * bwmax * MAXW T's, and
// 2 * (BlockMax + 1) ints.
template <typename T>
__global__ void __launch_bounds__(256) k_block_lu(T* fac, int* ipiv, int* info, T* inv, Sched S, Launch L, int step,
                                                   int bwmax) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* A = reinterpret_cast<T*>(smem_raw);
    T* W = A + bwmax * (bwmax | 1);                 // the pieces' inverses, packed as in inv[]
    int* q0 = reinterpret_cast<int*>(W + 2 * bwmax * MAXW);
    int* piv = q0 + BlockMax<T>::value + 1;
    __shared__ int ssing;
    __shared__ int src[32];
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int blk = F.block0 + step;
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk], bw = c1 - c0;
    const int lda = bw | 1;
    const int p0 = S.blk_p0[blk], np = S.blk_np[blk];
    const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31, nw = nt >> 5;
    if (tid == 0) ssing = 0;
    for (int k = tid; k <= np; k += nt) q0[k] = S.xsuper[p0 + k] - F.f - c0;
#pragma unroll 4
    for (int j = warp; j < bw; j += nw) {
        const T* src = fac + F.loff + (ll)(c0 + j) * F.ld + c0;
#pragma unroll
        for (int q = 0; q < BlockMax<T>::value / 32; ++q) {
            const int i = lane + 32 * q;
            if (i < bw) A[j * lda + i] = src[i];
        }
    }
    __syncthreads();
    int woff = 0;
    for (int pc = 0; pc < np; ++pc) {
        const int a = q0[pc], b = q0[pc + 1], w = b - a;
        T* Ui = W + woff;
        T* Li = Ui + w * w;
        if (w <= 32) {
            if (warp == 0 && warp_getrf32(A + a * lda + a, lda, w, piv + a)) ssing = 1;
            __syncthreads();
            if (tid == 0) {                          // the piece's interchanges as a gather map
                for (int k = 0; k < w; ++k) src[k] = k;
                for (int k = 0; k < w; ++k) {
                    const int kp = piv[a + k];
                    const int t0 = src[k];
                    src[k] = src[kp];
                    src[kp] = t0;
                }
            }
            __syncthreads();
            if (warp == 0) {
                warp_inv_upper32(A + a * lda + a, lda, w, Ui);
            } else if (warp == 1) {
                warp_inv_lower32(A + a * lda + a, lda, w, piv + a, Li);
            } else if (b < bw) {
                // warps 2..: U panel to the right inside the block (one thread per
                // column: _luswap! as a gather, then the unit-lower solve) and L
                // panel below (one thread per row: X := X * inv(U_pp)), in registers
                const int ncol = bw - b, nrow = bw - b;
                for (int t = tid - 64; t < ncol + nrow; t += nt - 64) {
                    if (t < ncol) {
                        T* col = A + (b + t) * lda + a;
                        T y[32];
#pragma unroll
                        for (int k = 0; k < 32; ++k) y[k] = k < w ? col[src[k]] : T(0);
#pragma unroll 1
                        for (int k = 0; k < w; ++k) {
                            const T yk = pick32(y, k);
                            const T* lcol = A + (a + k) * lda + a;
#pragma unroll
                            for (int i = 0; i < 32; ++i)
                                if (i > k && i < w) y[i] -= lcol[i] * yk;
                        }
#pragma unroll
                        for (int k = 0; k < 32; ++k)
                            if (k < w) col[k] = y[k];
                    } else {
                        const int i = b + (t - ncol);
                        T x[32];
#pragma unroll
                        for (int k = 0; k < 32; ++k) x[k] = k < w ? A[(a + k) * lda + i] : T(0);
#pragma unroll 1
                        for (int j = 0; j < w; ++j) {
                            const T* ucol = A + (a + j) * lda + a;
                            T acc = pick32(x, j);
#pragma unroll
                            for (int k = 0; k < 32; ++k)
                                if (k < j) acc -= ucol[k] * x[k];
                            acc *= T(1) / ucol[j];
#pragma unroll
                            for (int k = 0; k < 32; ++k)
                                if (k == j) x[k] = acc;
                        }
#pragma unroll
                        for (int k = 0; k < 32; ++k)
                            if (k < w) A[(a + k) * lda + i] = x[k];
                    }
                }
            }
            __syncthreads();
            if (b < bw) {
                for (int j = b + warp; j < bw; j += nw) {   // block-local trailing update
                    for (int i = b + lane; i < bw; i += 32) {
                        T acc = T(0);
                        for (int k = 0; k < w; ++k) acc += A[(a + k) * lda + i] * A[j * lda + a + k];
                        A[j * lda + i] -= acc;
                    }
                }
                __syncthreads();
            }
        } else {
            if (warp == 0 && warp_getrf(A + a * lda + a, lda, w, piv + a)) ssing = 1;
            __syncthreads();
            piece_inverses(A + a * lda + a, lda, w, piv + a, Ui, Li);
            __syncthreads();
            if (b < bw) {
                for (int j = b + warp; j < bw; j += nw) {
                    T yv[2];
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        const int i = lane + 32 * q;
                        T acc = T(0);
                        if (i < w)
                            for (int k = 0; k < w; ++k) acc += Li[k * w + i] * A[j * lda + a + k];
                        yv[q] = acc;
                    }
                    __syncwarp();
#pragma unroll
                    for (int q = 0; q < 2; ++q)
                        if (lane + 32 * q < w) A[j * lda + a + lane + 32 * q] = yv[q];
                }
                for (int i = b + tid; i < bw; i += nt) {
                    for (int j = w - 1; j >= 0; --j) {
                        T acc = T(0);
                        for (int k = 0; k <= j; ++k) acc += A[(a + k) * lda + i] * Ui[j * w + k];
                        A[(a + j) * lda + i] = acc;
                    }
                }
                __syncthreads();
                for (int j = b + warp; j < bw; j += nw) {
                    for (int i = b + lane; i < bw; i += 32) {
                        T acc = T(0);
                        for (int k = 0; k < w; ++k) acc += A[(a + k) * lda + i] * A[j * lda + a + k];
                        A[j * lda + i] -= acc;
                    }
                }
                __syncthreads();
            }
        }
        woff += 2 * w * w;
    }
    for (int j = warp; j < bw; j += nw)
        for (int i = lane; i < bw; i += 32) fac[F.loff + (ll)(c0 + j) * F.ld + c0 + i] = A[j * lda + i];
    for (int c = tid; c < bw; c += nt) ipiv[F.f + c0 + c] = piv[c];
    T* out = inv + S.blk_inv[blk];
    for (int e = tid; e < woff; e += nt) out[e] = W[e];
    if (tid == 0 && ssing) {
        for (int pc = 0; pc < np; ++pc) {   // first singular piece of the block
            bool z = false;
            for (int k = q0[pc]; k < q0[pc + 1]; ++k) z |= A[k * lda + k] == T(0);
            if (z) { atomicMin(info, p0 + pc + 1); break; }
        }
    }
}

// After the factorisation, one CTA per block (all blocks of all fronts in
// one launch) turns the pieces' inverses into whole-block operators:
//   Minv rows of piece q = Li_q (E_q - L_q,<q Minv_<q)     (forward, pieces in order)
//   Uinv rows of piece p = Ui_p (E_p - U_p,>p Uinv_>p)     (backward, pieces reversed)
// so that a triangular-solve step of the block is one product, Minv * b or
// Uinv * c.  Both are written column-major (bw x bw) to inv2[].
// Dynamic shared memory: 3 * bwmax * (bwmax | 1) T's.
template <typename T>
__global__ void __launch_bounds__(256) k_block_inv(const T* fac, const T* inv, T* inv2, Sched S, const int* blk_front,
                                                    const int* blk_ids, int bwmax) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int q0[BlockMax<T>::value + 1];
    __shared__ int wo[BlockMax<T>::value + 1];
    const int blk = blk_ids[blockIdx.x];
    const DFront F = S.fronts[blk_front[blk]];
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk], bw = c1 - c0, lda = bw | 1;
    const int p0 = S.blk_p0[blk], np = S.blk_np[blk];
    T* A = reinterpret_cast<T*>(smem_raw);        // block, column-major
    T* M = A + bwmax * (bwmax | 1);               // Minv, row-major (i, j) at i * lda + j
    T* U = M + bwmax * (bwmax | 1);               // Uinv, row-major
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nw = blockDim.x >> 5;
    for (int k = tid; k <= np; k += blockDim.x) q0[k] = S.xsuper[p0 + k] - F.f - c0;
    for (int j = warp; j < bw; j += nw)
        for (int i = lane; i < bw; i += 32) A[j * lda + i] = fac[F.loff + (ll)(c0 + j) * F.ld + c0 + i];
    __syncthreads();
    if (tid == 0) {
        int o = 0;
        for (int pc = 0; pc < np; ++pc) {
            wo[pc] = o;
            const int w = q0[pc + 1] - q0[pc];
            o += 2 * w * w;
        }
    }
    __syncthreads();
    const T* W = inv + S.blk_inv[blk];
    for (int pc = 0; pc < np; ++pc) {               // forward operator
        const int a = q0[pc], b = q0[pc + 1], w = b - a;
        const T* Li = W + wo[pc] + w * w;
        for (int i = a + warp; i < b; i += nw)      // T = E_q - L_q,<q Minv_<q  (into M rows of q)
            for (int j = lane; j < bw; j += 32) {
                T acc = T(i == j);
                for (int k = 0; k < a; ++k) acc -= A[k * lda + i] * M[k * lda + j];
                M[i * lda + j] = acc;
            }
        __syncthreads();
        for (int j = tid; j < bw; j += blockDim.x) {   // rows of q := Li_q T, one thread per column
            T t[64];
#pragma unroll
            for (int k = 0; k < 64; ++k) t[k] = k < w ? M[(a + k) * lda + j] : T(0);
            for (int i = 0; i < w; ++i) {
                T acc = T(0);
#pragma unroll
                for (int k = 0; k < 64; ++k)
                    if (k < w) acc += Li[k * w + i] * t[k];
                M[(a + i) * lda + j] = acc;
            }
        }
        __syncthreads();
    }
    for (int pc = np - 1; pc >= 0; --pc) {          // backward operator
        const int a = q0[pc], b = q0[pc + 1], w = b - a;
        const T* Ui = W + wo[pc];
        for (int i = a + warp; i < b; i += nw)      // T = E_p - U_p,>p Uinv_>p
            for (int j = lane; j < bw; j += 32) {
                T acc = T(i == j);
                for (int k = b; k < bw; ++k) acc -= A[k * lda + i] * U[k * lda + j];
                U[i * lda + j] = acc;
            }
        __syncthreads();
        for (int j = tid; j < bw; j += blockDim.x) {
            T t[64];
#pragma unroll
            for (int k = 0; k < 64; ++k) t[k] = k < w ? U[(a + k) * lda + j] : T(0);
            for (int i = 0; i < w; ++i) {
                T acc = T(0);
#pragma unroll
                for (int k = 0; k < 64; ++k)
                    if (k >= i && k < w) acc += Ui[k * w + i] * t[k];
                U[(a + i) * lda + j] = acc;
            }
        }
        __syncthreads();
    }
    T* out = inv2 + S.blk_inv2[blk];
    for (int j = warp; j < bw; j += nw)
        for (int i = lane; i < bw; i += 32) {
            out[(ll)j * bw + i] = M[i * lda + j];
            out[(ll)bw * bw + (ll)j * bw + i] = U[i * lda + j];
        }
}

// ---------------------------------------------------------------------------
// 64 x 64 register-tiled block product, 256 threads, 4 x 4 outputs each.
// sA[k][i] (k < kc, i < 64), sB[k][j]; thread (tx, ty) owns rows tx+16a and
// columns ty+16b when rows_fast, else rows ty+16a and columns tx+16b.
// ---------------------------------------------------------------------------
constexpr int TT = 64;
constexpr int KC = 32;

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

// Panels of block `step`: 64-row tiles of the L panel below the block and
// 64-column tiles of the U panel to its right (inside the front, stored in
// Lf, and in U12, stored in Uf).  Piece by piece: an L row gets
//   X_p := (X_p - X_<p U_<p,p) Ui_p,
// a U column gets
//   Y_p := Li_p (Y_p - L_p,<p Y_<p),
// the reference's two _trsm! panels (after _luswap!) for every piece of the
// block.  Block entries and inverses are read through the cache.
// Dynamic shared memory: 64 * bwmax T's.
template <typename T>
__global__ void __launch_bounds__(256) k_block_panel(T* fac, const T* inv, Sched S, Launch L, int step, int bwmax) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sX = reinterpret_cast<T*>(smem_raw);   // sX[k * 64 + t], k < bw, t < 64
    __shared__ int q0[BlockMax<T>::value + 1];
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int blk = F.block0 + step;
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk], bw = c1 - c0;
    const int p0 = S.blk_p0[blk], np = S.blk_np[blk];
    const int tid = threadIdx.x, t = tid & 63, g = tid >> 6;
    const int nL = cdiv(F.ld - c1, 64), nUa = cdiv(F.nf - c1, 64);
    const T* blockA = fac + F.loff + (ll)c0 * F.ld + c0;   // (i, j) of the block at j * ld + i
    const T* W = inv + S.blk_inv[blk];
    for (int k = tid; k <= np; k += 256) q0[k] = S.xsuper[p0 + k] - F.f - c0;
    if (tile < nL) {
        const int r0 = c1 + tile * 64, nr = min(64, F.ld - r0);
        for (int e = tid; e < 64 * bw; e += 256) {
            int i = e & 63, k = e >> 6;
            sX[k * 64 + i] = i < nr ? fac[F.loff + (ll)(c0 + k) * F.ld + r0 + i] : T(0);
        }
        __syncthreads();
        int woff = 0;
        for (int pc = 0; pc < np; ++pc) {
            const int a = q0[pc], b = q0[pc + 1], w = b - a;
            const T* Ui = W + woff;
            for (int j = a + g; j < b; j += 4) {       // X_p -= X_<p U_<p,p
                T acc = T(0);
                for (int k = 0; k < a; ++k) acc += sX[k * 64 + t] * blockA[(ll)j * F.ld + k];
                sX[j * 64 + t] -= acc;
            }
            __syncthreads();
            T out[16];                                  // X_p := X_p Ui_p, columns a+g+4q
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const int j = g + 4 * q;
                T acc = T(0);
                if (j < w)
                    for (int k = 0; k <= j; ++k) acc += sX[(a + k) * 64 + t] * Ui[j * w + k];
                out[q] = acc;
            }
            __syncthreads();
#pragma unroll
            for (int q = 0; q < 16; ++q)
                if (g + 4 * q < w) sX[(a + g + 4 * q) * 64 + t] = out[q];
            __syncthreads();
            woff += 2 * w * w;
        }
        for (int e = tid; e < 64 * bw; e += 256) {
            int i = e & 63, k = e >> 6;
            if (i < nr) fac[F.loff + (ll)(c0 + k) * F.ld + r0 + i] = sX[k * 64 + i];
        }
    } else {
        const bool inner = tile < nL + nUa;
        const int col0 = inner ? c1 + (tile - nL) * 64 : (tile - nL - nUa) * 64;
        const int nc = inner ? min(64, F.nf - col0) : min(64, F.m - col0);
        if (inner) {
            for (int e = tid; e < bw * 64; e += 256) {
                int k = e % bw, c = e / bw;
                sX[k * 64 + c] = c < nc ? fac[F.loff + (ll)(col0 + c) * F.ld + c0 + k] : T(0);
            }
        } else {
            for (int e = tid; e < bw * 64; e += 256) {
                int c = e & 63, k = e >> 6;
                sX[k * 64 + c] = c < nc ? fac[F.uoff + (ll)(c0 + k) * F.m + col0 + c] : T(0);
            }
        }
        __syncthreads();
        int woff = 0;
        for (int pc = 0; pc < np; ++pc) {
            const int a = q0[pc], b = q0[pc + 1], w = b - a;
            const T* Li = W + woff + w * w;
            for (int i = a + g; i < b; i += 4) {       // Y_p -= L_p,<p Y_<p
                T acc = T(0);
                for (int k = 0; k < a; ++k) acc += blockA[(ll)k * F.ld + i] * sX[k * 64 + t];
                sX[i * 64 + t] -= acc;
            }
            __syncthreads();
            T out[16];                                  // Y_p := Li_p Y_p, rows a+g+4q
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const int i = g + 4 * q;
                T acc = T(0);
                if (i < w)
                    for (int k = 0; k < w; ++k) acc += Li[k * w + i] * sX[(a + k) * 64 + t];
                out[q] = acc;
            }
            __syncthreads();
#pragma unroll
            for (int q = 0; q < 16; ++q)
                if (g + 4 * q < w) sX[(a + g + 4 * q) * 64 + t] = out[q];
            __syncthreads();
            woff += 2 * w * w;
        }
        if (inner) {
            for (int e = tid; e < bw * 64; e += 256) {
                int k = e % bw, c = e / bw;
                if (c < nc) fac[F.loff + (ll)(col0 + c) * F.ld + c0 + k] = sX[k * 64 + c];
            }
        } else {
            for (int e = tid; e < bw * 64; e += 256) {
                int c = e & 63, k = e >> 6;
                if (c < nc) fac[F.uoff + (ll)(c0 + k) * F.m + col0 + c] = sX[k * 64 + c];
            }
        }
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
    const bool isL = tile < nrL * ncL;
    int r0, col0, nr, nc;
    if (isL) {
        r0 = c1 + (tile % nrL) * TT;
        col0 = c1 + (tile / nrL) * TT;
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
    if (isL) {
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            int c = ty + 16 * b;
            if (c >= nc) continue;
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                int r = tx + 16 * a;
                if (r < nr) fac[F.loff + (ll)(col0 + c) * F.ld + r0 + r] -= acc[a][b];
            }
        }
    } else {
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            int r = ty + 16 * a;
            if (r >= nr) continue;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                int c = tx + 16 * b;
                if (c < nc) fac[F.uoff + (ll)(r0 + r) * F.m + col0 + c] -= acc[a][b];
            }
        }
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
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int tid = threadIdx.x;
    const int nt = cdiv(F.m, TT);
    const int r0 = (tile % nt) * TT, c0 = (tile / nt) * TT;
    const int nr = min(TT, F.m - r0), nc = min(TT, F.m - c0);
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
    const int tx = tid & 15, ty = tid >> 4;
    const int* runid = S.runid + F.runid_off;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const int c = c0 + ty + 16 * b;
        if (c - c0 >= nc) continue;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int r = r0 + tx + 16 * a;
            if (r - r0 >= nr) continue;
            const int x = min(r, c);
            const int g = runid[x];
            const DFront G = S.fronts[S.run_tgt[g]];
            const ll base = S.run_rel[g] - S.run_start[g];
            const int pr = S.rel[base + r], pc = S.rel[base + c];
            if (pr < 0 || pc < 0) continue;     // exact zero: (r, c) is padding of F only
            ll addr;
            if (r >= c || pc < G.nf) addr = G.loff + (ll)pc * G.ld + pr;
            else addr = G.uoff + (ll)pr * G.m + (pc - G.nf);
            atomicAdd(&fac[addr], -acc[a][b]);
        }
    }
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
    __shared__ T sb[BM * MAXRHS];
    __shared__ T sp[4 * SC * MAXRHS];
    __shared__ T sy[SC * MAXRHS];
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int blk = F.block0 + step;
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk], bw = c1 - c0;
    const int ncc = cdiv(bw, SC), cc = tile % ncc, rt = tile / ncc;
    const int j0 = cc * SC, nj = min(SC, bw - j0);
    const T* Mi = inv2 + S.blk_inv2[blk];
    const int tid = threadIdx.x;
    for (int e = tid; e < bw * nrhs; e += TS) {
        int k = e % bw, r = e / bw;
        sb[r * BM + k] = b[(ll)r * n + F.f + c0 + k];
    }
    __syncthreads();
    {   // y_chunk = Minv[j0:j0+nj, :] b_B : 32 columns x 4 partial sums over k
        const int j = tid & 31, kq = tid >> 5;
        T acc[MAXRHS];
#pragma unroll
        for (int r = 0; r < MAXRHS; ++r) acc[r] = T(0);
        if (j < nj) {
#pragma unroll 8
            for (int k = kq; k < bw; k += 4) {
                const T mk = Mi[(ll)k * bw + j0 + j];
#pragma unroll
                for (int r = 0; r < MAXRHS; ++r)
                    if (r < nrhs) acc[r] += mk * sb[r * BM + k];
            }
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
    const int row = c1 + rt * TS + tid;
    if (row < F.ld) {
        const int grow = row < F.nf ? F.f + row : S.rows[F.rows_off + row - F.nf];
        T lv[SC];
        const T* lcol = fac + F.loff + (ll)(c0 + j0) * F.ld + row;
#pragma unroll
        for (int j = 0; j < SC; ++j) lv[j] = j < nj ? lcol[(ll)j * F.ld] : T(0);
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

// Backward, part 1: y[F's columns] -= U12 * x[R_F] (one warp per row).
template <typename T>
__global__ void __launch_bounds__(TS) k_bwd_u12(const T* fac, T* y, const T* x, int n, int nrhs, Sched S, Launch L) {
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int i = tile * (TS / 32) + wid;
    if (i >= F.nf) return;
    for (int r = 0; r < nrhs; ++r) {
        T acc = T(0);
#pragma unroll 8
        for (int c = lane; c < F.m; c += 32)
            acc += fac[F.uoff + (ll)i * F.m + c] * x[(ll)r * n + S.rows[F.rows_off + c]];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        if (lane == 0) y[(ll)r * n + F.f + i] -= acc;
    }
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
    __shared__ T sc[BM * MAXRHS];
    __shared__ T sp[4 * SC * MAXRHS];
    __shared__ T sx[SC * MAXRHS];
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int blk = F.block0 + F.nblocks - 1 - step;
    const int c0 = S.blk_c0[blk], c1 = S.blk_c1[blk], bw = c1 - c0;
    const int ncc = cdiv(bw, SC), cc = tile % ncc, rt = tile / ncc;
    const int j0 = cc * SC, nj = min(SC, bw - j0);
    const T* Ui = inv2 + S.blk_inv2[blk] + (ll)bw * bw;
    const int tid = threadIdx.x;
    for (int e = tid; e < bw * nrhs; e += TS) {
        int k = e % bw, r = e / bw;
        sc[r * BM + k] = y[(ll)r * n + F.f + c0 + k];
    }
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
                const T uk = Ui[(ll)k * bw + j0 + j];
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
    const int row = rt * TS + tid;
    if (row < c0) {
        T uv[SC];
        const T* ucol = fac + F.loff + (ll)(c0 + j0) * F.ld + row;
#pragma unroll
        for (int j = 0; j < SC; ++j) uv[j] = j < nj ? ucol[(ll)j * F.ld] : T(0);
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
// Assembly, permutation, residual.
// ---------------------------------------------------------------------------

// Zero-initialised factor storage += A's values at their slots (_inmatrix!).
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

// r = b - A x in FP64 with A in row order (values gathered from CSC order);
// the squares of r and b are accumulated per right-hand side.
__global__ void k_residual(const double* __restrict__ aval, const int* __restrict__ rowptr, const int* __restrict__ col,
                           const ll* __restrict__ src, const double* __restrict__ x, ll ldx, const double* __restrict__ b,
                           ll ldb, double* __restrict__ r, int n, int nrhs, double* __restrict__ sums) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int rhs = blockIdx.y;
    double rr = 0.0, bb = 0.0;
    if (i < n) {
        double s = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) s += aval[src[k]] * x[(ll)rhs * ldx + col[k]];
        double bi = b[(ll)rhs * ldb + i];
        double ri = bi - s;
        r[(ll)rhs * n + i] = ri;
        rr = ri * ri;
        bb = bi * bi;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        rr += __shfl_down_sync(0xffffffffu, rr, off);
        bb += __shfl_down_sync(0xffffffffu, bb, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&sums[2 * rhs], rr);
        atomicAdd(&sums[2 * rhs + 1], bb);
    }
}

// Norms only: sums[2r] += ||b_r - A x_r||^2 and sums[2r+1] += ||b_r||^2, with
// no residual vector written (used where no work space may be allocated).
__global__ void k_residual_norms(const double* __restrict__ aval, const int* __restrict__ rowptr,
                                 const int* __restrict__ col, const ll* __restrict__ src, const double* __restrict__ x,
                                 ll ldx, const double* __restrict__ b, ll ldb, int n, double* __restrict__ sums) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int rhs = blockIdx.y;
    double rr = 0.0, bb = 0.0;
    if (i < n) {
        double s = 0.0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) s += aval[src[k]] * x[(ll)rhs * ldx + col[k]];
        double bi = b[(ll)rhs * ldb + i];
        double ri = bi - s;
        rr = ri * ri;
        bb = bi * bi;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        rr += __shfl_down_sync(0xffffffffu, rr, off);
        bb += __shfl_down_sync(0xffffffffu, bb, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&sums[2 * rhs], rr);
        atomicAdd(&sums[2 * rhs + 1], bb);
    }
}

}  // namespace spk


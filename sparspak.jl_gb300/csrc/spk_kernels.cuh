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
// In-block partial pivoting LU of a w x w block held in shared memory
// (column-major, leading dimension w, w <= MAXW).  Pivot = first row with the
// strictly largest |a| (ggetrf!, src/Utilities/GenericBlasLapackFragments.jl:
// 56-100): NaN never wins, except a NaN on the diagonal, which keeps k; a
// zero pivot skips the interchange and the scaling and sets *sing.
// piv[k] receives the 0-based local pivot row.
// ---------------------------------------------------------------------------
template <typename T>
__device__ void block_getrf(T* A, int w, int* piv, int* sing) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int k = 0; k < w; ++k) {
        if (tid < 32) {
            double key = -1.0;
            int idx = w;
            for (int i = k + tid; i < w; i += 32) {   // first strict maximum among this lane's rows
                double a = (double)tabs(A[k * w + i]);
                double ki = (a != a) ? ((i == k) ? __longlong_as_double(0x7ff0000000000000LL) : -1.0) : a;
                if (ki > key || idx == w) { key = ki; idx = i; }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                double k2 = __shfl_down_sync(0xffffffffu, key, off);
                int i2 = __shfl_down_sync(0xffffffffu, idx, off);
                if (k2 > key || (k2 == key && i2 < idx)) { key = k2; idx = i2; }
            }
            if (tid == 0) piv[k] = idx;
        }
        __syncthreads();
        const int kp = piv[k];
        const bool nz = A[k * w + kp] != T(0);
        if (nz) {
            if (kp != k)
                for (int j = tid; j < w; j += nt) {
                    T t = A[j * w + k];
                    A[j * w + k] = A[j * w + kp];
                    A[j * w + kp] = t;
                }
            __syncthreads();
            const T inv = T(1) / A[k * w + k];
            for (int i = k + 1 + tid; i < w; i += nt) A[k * w + i] *= inv;
        } else if (tid == 0) {
            *sing = 1;
        }
        __syncthreads();
        const int r = w - k - 1;
        for (int e = tid; e < r * r; e += nt) {
            int i = k + 1 + e % r, j = k + 1 + e / r;
            A[j * w + i] -= A[k * w + i] * A[j * w + k];
        }
        __syncthreads();
    }
}

// Factor the diagonal block of piece p of front F in place and record its
// pivots (0-based local) in ipiv[column].  Used by k_getrf_first and by the
// corner tile of k_trail.
template <typename T>
__device__ void factor_diag(T* fac, int* ipiv, int* info, const DFront& F, int p, int p0, int w, T* sD,
                            int* spiv, int* ssing) {
    const int tid = threadIdx.x, nt = blockDim.x;
    if (tid == 0) *ssing = 0;
    for (int e = tid; e < w * w; e += nt) {
        int i = e % w, k = e / w;
        sD[k * w + i] = fac[F.loff + (ll)(p0 + k) * F.ld + p0 + i];
    }
    __syncthreads();
    block_getrf(sD, w, spiv, ssing);
    for (int e = tid; e < w * w; e += nt) {
        int i = e % w, k = e / w;
        fac[F.loff + (ll)(p0 + k) * F.ld + p0 + i] = sD[k * w + i];
    }
    if (tid < w) ipiv[F.f + p0 + tid] = spiv[tid];
    if (tid == 0 && *ssing) atomicMin(info, p + 1);
}

template <typename T>
__global__ void __launch_bounds__(128) k_getrf_first(T* fac, int* ipiv, int* info, Sched S, Launch L) {
    __shared__ T sD[MAXW * MAXW];
    __shared__ int spiv[MAXW];
    __shared__ int ssing;
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int p = F.piece0;
    const int p0 = S.xsuper[p] - F.f, w = S.xsuper[p + 1] - S.xsuper[p];
    factor_diag(fac, ipiv, info, F, p, p0, w, sD, spiv, &ssing);
}

// ---------------------------------------------------------------------------
// Panel kernel for piece `step` of every front in the launch.  Tiles:
//   [0, nL)          : 128 rows of the L panel, X := X * inv(U11) (trsm 'r','u','n','n')
//   [nL, nL+nUa)     : 128 U columns inside the front (stored in Lf)
//   [nL+nUa, ...)    : 128 U columns of U12 (stored in Uf)
// U columns get the block's row interchanges (_luswap!) and then
// X := inv(L11) X (the reference's trsm 'r','l','t','u' on U12').
// ---------------------------------------------------------------------------
constexpr int TP = 128;

// Dynamic shared memory: (wmax^2 + wmax*TP) T's and MAXW ints, wmax the widest piece.
template <typename T>
__global__ void __launch_bounds__(TP) k_panel(T* fac, const int* ipiv, Sched S, Launch L, int step, int wmax) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sD = reinterpret_cast<T*>(smem_raw);
    T* sX = sD + wmax * wmax;
    int* spiv = reinterpret_cast<int*>(sX + wmax * TP);
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int p = F.piece0 + step;
    const int p0 = S.xsuper[p] - F.f, p1 = S.xsuper[p + 1] - F.f, w = p1 - p0;
    const int tid = threadIdx.x;
    for (int e = tid; e < w * w; e += TP) {
        int i = e % w, k = e / w;
        sD[k * w + i] = fac[F.loff + (ll)(p0 + k) * F.ld + p0 + i];
    }
    if (tid < w) spiv[tid] = ipiv[F.f + p0 + tid];
    const int nL = cdiv(F.ld - p1, TP), nUa = cdiv(F.nf - p1, TP);
    if (tile < nL) {
        const int r0 = p1 + tile * TP;
        const int nr = min(TP, F.ld - r0);
        for (int k = 0; k < w; ++k)
            if (tid < nr) sX[k * TP + tid] = fac[F.loff + (ll)(p0 + k) * F.ld + r0 + tid];
        __syncthreads();
        if (tid < nr) {
            for (int j = 0; j < w; ++j) {
                T s = sX[j * TP + tid];
                for (int k = 0; k < j; ++k) {
                    T u = sD[j * w + k];
                    if (u != T(0)) s -= u * sX[k * TP + tid];
                }
                sX[j * TP + tid] = s * (T(1) / sD[j * w + j]);
            }
        }
        __syncthreads();
        for (int k = 0; k < w; ++k)
            if (tid < nr) fac[F.loff + (ll)(p0 + k) * F.ld + r0 + tid] = sX[k * TP + tid];
    } else {
        const bool inner = tile < nL + nUa;
        const int c0 = inner ? p1 + (tile - nL) * TP : (tile - nL - nUa) * TP;   // inner: front column; else U12 column
        const int nc = inner ? min(TP, F.nf - c0) : min(TP, F.m - c0);
        // cooperative load of the w x nc block into sX[k*TP + c]
        if (inner) {
            for (int e = tid; e < w * nc; e += TP) {
                int k = e % w, c = e / w;
                sX[k * TP + c] = fac[F.loff + (ll)(c0 + c) * F.ld + p0 + k];
            }
        } else {
            for (int k = 0; k < w; ++k)
                if (tid < nc) sX[k * TP + tid] = fac[F.uoff + (ll)(p0 + k) * F.m + c0 + tid];
        }
        __syncthreads();
        if (tid < nc) {
            for (int k = 0; k < w; ++k) {
                int kp = spiv[k];
                if (kp != k) {
                    T t = sX[k * TP + tid];
                    sX[k * TP + tid] = sX[kp * TP + tid];
                    sX[kp * TP + tid] = t;
                }
            }
            for (int k = 0; k < w; ++k) {
                T xk = sX[k * TP + tid];
                for (int j = k + 1; j < w; ++j) {
                    T l = sD[k * w + j];
                    if (l != T(0)) sX[j * TP + tid] -= l * xk;
                }
            }
        }
        __syncthreads();
        if (inner) {
            for (int e = tid; e < w * nc; e += TP) {
                int k = e % w, c = e / w;
                fac[F.loff + (ll)(c0 + c) * F.ld + p0 + k] = sX[k * TP + c];
            }
        } else {
            for (int k = 0; k < w; ++k)
                if (tid < nc) fac[F.uoff + (ll)(p0 + k) * F.m + c0 + tid] = sX[k * TP + tid];
        }
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

// Trailing update after piece `step`: A[R, C] -= L[R, piece] * U[piece, C]
// over the front minus its Schur-complement block.  L tiles: rows in
// [p1, nf+m), columns in [p1, nf) (stored in Lf).  U tiles: rows in
// [p1, nf), columns in U12 (stored in Uf).  The L tile at the corner then
// factors the next piece's diagonal block.
template <typename T>
__global__ void __launch_bounds__(256) k_trail(T* fac, int* ipiv, int* info, Sched S, Launch L, int step) {
    __shared__ T sAB[2 * KC * TT];     // also the MAXW x MAXW scratch of the corner factorisation
    __shared__ int spiv[MAXW];
    __shared__ int ssing;
    T* sA = sAB;
    T* sB = sAB + KC * TT;
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int p = F.piece0 + step;
    const int p0 = S.xsuper[p] - F.f, p1 = S.xsuper[p + 1] - F.f, w = p1 - p0;
    const int tid = threadIdx.x;
    const int nrL = cdiv(F.ld - p1, TT), ncL = cdiv(F.nf - p1, TT);
    const bool isL = tile < nrL * ncL;
    int r0, c0, nr, nc;
    if (isL) {
        r0 = p1 + (tile % nrL) * TT;
        c0 = p1 + (tile / nrL) * TT;
        nr = min(TT, F.ld - r0);
        nc = min(TT, F.nf - c0);
    } else {
        const int t2 = tile - nrL * ncL, nrU = cdiv(F.nf - p1, TT);
        r0 = p1 + (t2 % nrU) * TT;
        c0 = (t2 / nrU) * TT;            // U12 column index
        nr = min(TT, F.nf - r0);
        nc = min(TT, F.m - c0);
    }
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
    for (int k0 = 0; k0 < w; k0 += KC) {
        const int kc = min(KC, w - k0);
        for (int e = tid; e < kc * TT; e += 256) {
            int i = e % TT, k = e / TT;
            sA[k * TT + i] = (i < nr) ? fac[F.loff + (ll)(p0 + k0 + k) * F.ld + r0 + i] : T(0);
        }
        if (isL) {
            for (int e = tid; e < kc * TT; e += 256) {
                int k = e % kc, j = e / kc;
                sB[k * TT + j] = (j < nc) ? fac[F.loff + (ll)(c0 + j) * F.ld + p0 + k0 + k] : T(0);
            }
        } else {
            for (int e = tid; e < kc * TT; e += 256) {
                int j = e % TT, k = e / TT;
                sB[k * TT + j] = (j < nc) ? fac[F.uoff + (ll)(p0 + k0 + k) * F.m + c0 + j] : T(0);
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
                if (r < nr) fac[F.loff + (ll)(c0 + c) * F.ld + r0 + r] -= acc[a][b];
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
                if (c < nc) fac[F.uoff + (ll)(r0 + r) * F.m + c0 + c] -= acc[a][b];
            }
        }
    }
    if (isL && tile == 0 && step + 1 < F.npieces) {
        __syncthreads();
        const int q = p + 1;
        const int q0 = S.xsuper[q] - F.f, wq = S.xsuper[q + 1] - S.xsuper[q];
        factor_diag(fac, ipiv, info, F, q, q0, wq, sAB, spiv, &ssing);
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

// Forward step for piece `step`: interchanges (laswp), unit-lower solve of
// the piece (the reference's _lulsolve!, SpkLUFactor.jl:297-321) and the
// update of every row below it in the front; rows of R_F are updated with
// atomics because sibling fronts share them.  b is the running right-hand
// side, y receives the solved values of the piece.
template <typename T>
__global__ void __launch_bounds__(TS) k_fwd(const T* fac, const int* ipiv, T* b, T* y, int n, int nrhs, Sched S,
                                            Launch L, int step) {
    __shared__ T sD[MAXW * MAXW];
    __shared__ T sy[MAXW * MAXRHS];
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int p = F.piece0 + step;
    const int p0 = S.xsuper[p] - F.f, p1 = S.xsuper[p + 1] - F.f, w = p1 - p0;
    const int tid = threadIdx.x;
    for (int e = tid; e < w * w; e += TS) {
        int i = e % w, k = e / w;
        sD[k * w + i] = fac[F.loff + (ll)(p0 + k) * F.ld + p0 + i];
    }
    for (int e = tid; e < w * nrhs; e += TS) {
        int k = e % w, r = e / w;
        sy[r * MAXW + k] = b[(ll)r * n + F.f + p0 + k];
    }
    __syncthreads();
    if (tid < nrhs) {
        T* v = sy + tid * MAXW;
        for (int k = 0; k < w; ++k) {
            int kp = ipiv[F.f + p0 + k];
            if (kp != k) { T t = v[k]; v[k] = v[kp]; v[kp] = t; }
        }
        for (int k = 0; k < w; ++k) {
            T vk = v[k];
            if (vk != T(0))
                for (int i = k + 1; i < w; ++i) v[i] -= vk * sD[k * w + i];
        }
    }
    __syncthreads();
    if (tile == 0)
        for (int e = tid; e < w * nrhs; e += TS) {
            int k = e % w, r = e / w;
            y[(ll)r * n + F.f + p0 + k] = sy[r * MAXW + k];
        }
    const int row = p1 + tile * TS + tid;
    if (row < F.ld) {
        const int grow = row < F.nf ? F.f + row : S.rows[F.rows_off + row - F.nf];
        for (int r = 0; r < nrhs; ++r) {
            T acc = T(0);
            for (int k = 0; k < w; ++k) acc += sy[r * MAXW + k] * fac[F.loff + (ll)(p0 + k) * F.ld + row];
            if (row < F.nf) b[(ll)r * n + grow] -= acc;
            else atomicAdd(&b[(ll)r * n + grow], -acc);
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
        for (int c = lane; c < F.m; c += 32)
            acc += fac[F.uoff + (ll)i * F.m + c] * x[(ll)r * n + S.rows[F.rows_off + c]];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        if (lane == 0) y[(ll)r * n + F.f + i] -= acc;
    }
}

// Backward, part 2, for the piece `step`-th from the last: upper solve of
// the piece (the reference's _luusolve!, SpkLUFactor.jl:350-375), then the
// update of the front's rows above it.
template <typename T>
__global__ void __launch_bounds__(TS) k_bwd(const T* fac, T* y, T* x, int n, int nrhs, Sched S, Launch L, int step) {
    __shared__ T sD[MAXW * MAXW];
    __shared__ T sx[MAXW * MAXRHS];
    int fid, tile;
    locate(L, blockIdx.x, fid, tile);
    const DFront F = S.fronts[fid];
    const int p = F.piece0 + F.npieces - 1 - step;
    const int p0 = S.xsuper[p] - F.f, p1 = S.xsuper[p + 1] - F.f, w = p1 - p0;
    const int tid = threadIdx.x;
    for (int e = tid; e < w * w; e += TS) {
        int i = e % w, k = e / w;
        sD[k * w + i] = fac[F.loff + (ll)(p0 + k) * F.ld + p0 + i];
    }
    for (int e = tid; e < w * nrhs; e += TS) {
        int k = e % w, r = e / w;
        sx[r * MAXW + k] = y[(ll)r * n + F.f + p0 + k];
    }
    __syncthreads();
    if (tid < nrhs) {
        T* v = sx + tid * MAXW;
        for (int k = w - 1; k >= 0; --k) {
            if (v[k] != T(0)) {
                v[k] /= sD[k * w + k];
                T vk = v[k];
                for (int i = 0; i < k; ++i) v[i] -= vk * sD[k * w + i];
            }
        }
    }
    __syncthreads();
    if (tile == 0)
        for (int e = tid; e < w * nrhs; e += TS) {
            int k = e % w, r = e / w;
            x[(ll)r * n + F.f + p0 + k] = sx[r * MAXW + k];
        }
    const int row = tile * TS + tid;
    if (row < p0) {
        for (int r = 0; r < nrhs; ++r) {
            T acc = T(0);
            for (int k = 0; k < w; ++k) acc += fac[F.loff + (ll)(p0 + k) * F.ld + row] * sx[r * MAXW + k];
            y[(ll)r * n + F.f + row] -= acc;
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

}  // namespace spk

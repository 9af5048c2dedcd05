/*
 * ORACLE - TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference package's numeric phase, used by
 * the tests, by __graft_entry__.smoke() and by bench.py's CPU baseline to
 * check and time the CUDA library.  Nothing in the product links it.
 *
 * It follows, in the reference's own call order and storage layout:
 *   _inmatrix!   (CSC)  src/SparseCSCInterface/SparseCSCInterface.jl:101-169
 *   _lufactor!          src/SparseMethod/SpkLUFactor.jl:60-255
 *   _lulsolve!          src/SparseMethod/SpkLUFactor.jl:269-323
 *   _luusolve!          src/SparseMethod/SpkLUFactor.jl:325-377
 *   _triangularsolve!   src/SparseMethod/SpkSparseBase.jl:400-416
 * with the dense kernels of the generic path
 *   ggetrf!, ggemm!, ggemv!, gtrsm!, glaswp!
 *                       src/Utilities/GenericBlasLapackFragments.jl:56-495
 * and the index helpers _assmb!, _ldindx!, _igathr!, _mmpyi!, _luswap!
 *                       src/SparseSpdMethod/SpkSpdMMOps.jl:41-175.
 *
 * Every array argument is 1-based in the reference's sense: the C pointer
 * passed in addresses element 1 (so a[i] in the reference is A1(a, i)).
 * Pinned by the reference's golden vectors (tests/golden/).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t i64;

#define A1(p, i) ((p)[(i) - 1])

/* ---- dense kernels (generic path semantics) ---------------------------- */

/* ggetrf!: unblocked right-looking LU, first strict maximum as pivot. */
static void o_getrf(i64 m, i64 n, double* a, i64 lda, i64* ipiv) {
#define A(i, j) a[((j) - 1) * lda + (i) - 1]
    i64 mn = m < n ? m : n;
    for (i64 k = 1; k <= mn; ++k) {
        i64 kp = k;
        if (k < m) {
            double amax = fabs(A(k, k));
            for (i64 i = k + 1; i <= m; ++i) {
                double ai = fabs(A(i, k));
                if (ai > amax) { kp = i; amax = ai; }
            }
        }
        ipiv[k - 1] = kp;
        if (A(kp, k) != 0.0) {
            if (k != kp)
                for (i64 i = 1; i <= n; ++i) { double t = A(k, i); A(k, i) = A(kp, i); A(kp, i) = t; }
            double inv = 1.0 / A(k, k);
            for (i64 i = k + 1; i <= m; ++i) A(i, k) *= inv;
        }
        for (i64 j = k + 1; j <= n; ++j)
            for (i64 i = k + 1; i <= m; ++i) A(i, j) -= A(i, k) * A(k, j);
    }
#undef A
}

/* ggemm!('n','t'): C := alpha*A*B' + beta*C */
static void o_gemm_nt(i64 m, i64 n, i64 k, double alpha, const double* a, i64 lda, const double* b, i64 ldb,
                      double beta, double* c, i64 ldc) {
    if (m == 0 || n == 0) return;
    for (i64 j = 0; j < n; ++j) {
        if (beta == 0.0) for (i64 i = 0; i < m; ++i) c[j * ldc + i] = 0.0;
        else if (beta != 1.0) for (i64 i = 0; i < m; ++i) c[j * ldc + i] *= beta;
        for (i64 l = 0; l < k; ++l) {
            double t = alpha * b[l * ldb + j];
            for (i64 i = 0; i < m; ++i) c[j * ldc + i] += t * a[l * lda + i];
        }
    }
}

/* gtrsm!('r','u','n','n'): B := B * inv(U), U upper non-unit. */
static void o_trsm_runn(i64 m, i64 n, const double* a, i64 lda, double* b, i64 ldb) {
    if (m == 0 || n == 0) return;
    for (i64 j = 0; j < n; ++j) {
        for (i64 k = 0; k < j; ++k) {
            double akj = a[j * lda + k];
            if (akj != 0.0)
                for (i64 i = 0; i < m; ++i) b[j * ldb + i] -= akj * b[k * ldb + i];
        }
        double t = 1.0 / a[j * lda + j];
        for (i64 i = 0; i < m; ++i) b[j * ldb + i] *= t;
    }
}

/* gtrsm!('r','l','t','u'): B := B * inv(L'), L unit lower. */
static void o_trsm_rltu(i64 m, i64 n, const double* a, i64 lda, double* b, i64 ldb) {
    if (m == 0 || n == 0) return;
    for (i64 k = 0; k < n; ++k)
        for (i64 j = k + 1; j < n; ++j) {
            double ajk = a[k * lda + j];
            if (ajk != 0.0)
                for (i64 i = 0; i < m; ++i) b[j * ldb + i] -= ajk * b[k * ldb + i];
        }
}

/* gtrsm!('l','l','n','u') with one column: b := inv(L) b, L unit lower. */
static void o_trsv_llnu(i64 m, const double* a, i64 lda, double* b) {
    for (i64 k = 0; k < m; ++k)
        if (b[k] != 0.0)
            for (i64 i = k + 1; i < m; ++i) b[i] -= b[k] * a[k * lda + i];
}

/* gtrsm!('l','u','n','n') with one column: b := inv(U) b. */
static void o_trsv_lunn(i64 m, const double* a, i64 lda, double* b) {
    for (i64 k = m - 1; k >= 0; --k)
        if (b[k] != 0.0) {
            b[k] /= a[k * lda + k];
            for (i64 i = 0; i < k; ++i) b[i] -= b[k] * a[k * lda + i];
        }
}


/* ---- optional BLAS/LAPACK mode ------------------------------------------- */

/* The reference calls BLAS/LAPACK for Float64 (dgemm_, dgetrf_, dtrsm_,
 * dlaswp_, dgemv_: src/SparseSpdMethod/SpkSpdMMOps.jl:222-351).  With
 * oracle_set_blas the same calls go to the given routines (LP64 Fortran
 * interface, e.g. the OpenBLAS bundled with scipy); without it the generic
 * loops above are used (the reference's path for other element types). */
typedef void (*dgemm_f)(char*, char*, int*, int*, int*, double*, double*, int*, double*, int*, double*, double*, int*);
typedef void (*dtrsm_f)(char*, char*, char*, char*, int*, int*, double*, double*, int*, double*, int*);
typedef void (*dgetrf_f)(int*, int*, double*, int*, int*, int*);
typedef void (*dlaswp_f)(int*, double*, int*, int*, int*, int*, int*);
typedef void (*dgemv_f)(char*, int*, int*, double*, double*, int*, double*, int*, double*, double*, int*);
static struct {
    dgemm_f gemm;
    dtrsm_f trsm;
    dgetrf_f getrf;
    dlaswp_f laswp;
    dgemv_f gemv;
} g_blas;

/* All five pointers, or all NULL to return to the generic loops. */
void oracle_set_blas(void* gemm, void* trsm, void* getrf, void* laswp, void* gemv) {
    g_blas.gemm = (dgemm_f)gemm;
    g_blas.trsm = (dtrsm_f)trsm;
    g_blas.getrf = (dgetrf_f)getrf;
    g_blas.laswp = (dlaswp_f)laswp;
    g_blas.gemv = (dgemv_f)gemv;
}

int oracle_blas_mode(void) { return g_blas.gemm != NULL; }

/* _gemm!('n','t') */
static void x_gemm_nt(i64 m, i64 n, i64 k, double alpha, double* a, i64 lda, double* b, i64 ldb, double beta, double* c,
                      i64 ldc) {
    if (!g_blas.gemm) { o_gemm_nt(m, n, k, alpha, a, lda, b, ldb, beta, c, ldc); return; }
    char tn = 'N', tt = 'T';
    int im = (int)m, in = (int)n, ik = (int)k, ia = (int)lda, ib = (int)ldb, ic = (int)ldc;
    g_blas.gemm(&tn, &tt, &im, &in, &ik, &alpha, a, &ia, b, &ib, &beta, c, &ic);
}

/* _getrf! on an n x n block; ipiv local 1..n */
static void x_getrf(i64 n, double* a, i64 lda, i64* ipiv) {
    if (!g_blas.getrf) { o_getrf(n, n, a, lda, ipiv); return; }
    int in = (int)n, ia = (int)lda, info = 0;
    int* p = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    g_blas.getrf(&in, &in, a, &ia, p, &info);
    for (i64 k = 0; k < n; ++k) ipiv[k] = p[k];
    free(p);
}

/* _trsm!(side, uplo, transa, diag) with alpha = 1 */
static void x_trsm(char side, char uplo, char ta, char diag, i64 m, i64 n, double* a, i64 lda, double* b, i64 ldb) {
    int im = (int)m, in = (int)n, ia = (int)lda, ib = (int)ldb;
    double one = 1.0;
    g_blas.trsm(&side, &uplo, &ta, &diag, &im, &in, &one, a, &ia, b, &ib);
}

/* ---- _inmatrix! (CSC) ---------------------------------------------------- */

/* Returns 0, or -(1 + position) of the first entry with no slot. */
i64 oracle_inmatrix_csc(i64 n, i64 ncols, const i64* colptr, const i64* rowval, const double* nzval,
                        const i64* rinvp, const i64* cinvp, const i64* snode, const i64* xsuper,
                        const i64* xlindx, const i64* lindx, const i64* xlnz, double* lnz, const i64* xunz,
                        double* unz) {
    (void)n;
    for (i64 i = 1; i <= ncols; ++i) {
        for (i64 p = A1(colptr, i); p <= A1(colptr, i + 1) - 1; ++p) {
            i64 inew = A1(rinvp, A1(rowval, p));
            i64 jnew = A1(cinvp, i);
            double v = A1(nzval, p);
            int placed = 0;
            if (inew >= A1(xsuper, A1(snode, jnew))) {
                i64 js = A1(snode, jnew);
                i64 loc = 0;
                for (i64 s = A1(xlindx, js); s <= A1(xlindx, js + 1) - 1; ++s) {
                    i64 r = A1(lindx, s);
                    if (r > inew) break;
                    if (r == inew) { A1(lnz, A1(xlnz, jnew) + loc) += v; placed = 1; break; }
                    ++loc;
                }
            } else {
                i64 js = A1(snode, inew);
                i64 w = A1(xsuper, js + 1) - A1(xsuper, js);
                i64 loc = 0;
                for (i64 s = A1(xlindx, js) + w; s <= A1(xlindx, js + 1) - 1; ++s) {
                    i64 r = A1(lindx, s);
                    if (r > jnew) break;
                    if (r == jnew) { A1(unz, A1(xunz, inew) + loc) += v; placed = 1; break; }
                    ++loc;
                }
            }
            if (!placed) return -(p);
        }
    }
    return 0;
}

/* ---- _lufactor! ---------------------------------------------------------- */

/* State of one left-looking factorisation, so that it can run in slices of
 * consecutive supernodes (bench.py's reference arm times the slices of one
 * complete factorisation as its steps). */
typedef struct {
    i64 n, nsuper;
    const i64 *xsuper, *snode, *xlindx, *lindx, *xlnz, *xunz;
    double *lnz, *unz;
    i64* ipvt;
    i64 *link, *lngth, *map, *relind;
    double* temp;
    i64 tmpsiz, iflag, first_singular, next;
} LuCtx;

void* oracle_lu_begin(i64 n, i64 nsuper, const i64* xsuper, const i64* snode, const i64* xlindx, const i64* lindx,
                      const i64* xlnz, double* lnz, const i64* xunz, double* unz, i64* ipvt) {
    LuCtx* c = (LuCtx*)calloc(1, sizeof(LuCtx));
    c->n = n; c->nsuper = nsuper;
    c->xsuper = xsuper; c->snode = snode; c->xlindx = xlindx; c->lindx = lindx; c->xlnz = xlnz; c->xunz = xunz;
    c->lnz = lnz; c->unz = unz; c->ipvt = ipvt;
    c->link = (i64*)calloc((size_t)nsuper + 1, sizeof(i64));
    c->lngth = (i64*)calloc((size_t)nsuper + 1, sizeof(i64));
    c->map = (i64*)calloc((size_t)n + 1, sizeof(i64));
    c->relind = (i64*)calloc((size_t)n + 1, sizeof(i64));
    for (i64 i = 1; i <= nsuper; ++i) {
        c->lngth[i] = A1(xlindx, i + 1) - A1(xlindx, i);
        i64 w = A1(xsuper, i + 1) - A1(xsuper, i);
        i64 need = w * (A1(xlnz, A1(xsuper, i) + 1) - A1(xlnz, A1(xsuper, i)));
        if (need > c->tmpsiz) c->tmpsiz = need;
    }
    c->temp = (double*)calloc((size_t)c->tmpsiz + 1, sizeof(double));
    c->next = 1;
    return c;
}

/* Factor supernodes c->next .. js_end (the body of _lufactor!'s jsup loop,
 * SpkLUFactor.jl:89-252); returns the next supernode to factor. */
i64 oracle_lu_run(void* ctx, i64 js_end) {
    LuCtx* c = (LuCtx*)ctx;
    const i64 *xsuper = c->xsuper, *snode = c->snode, *xlindx = c->xlindx, *lindx = c->lindx, *xlnz = c->xlnz,
              *xunz = c->xunz;
    i64* ipvt = c->ipvt;
    i64 *link = c->link, *lngth = c->lngth, *map = c->map, *relind = c->relind;
    double* temp = c->temp;
    const i64 tmpsiz = c->tmpsiz;
    i64 iflag = c->iflag;
    double* L = c->lnz - 1; /* L[p] == reference lnz[p] */
    double* U = c->unz - 1;
    if (js_end > c->nsuper) js_end = c->nsuper;
    for (i64 js = c->next; js <= js_end; ++js) {
        i64 fj = A1(xsuper, js), lj = A1(xsuper, js + 1) - 1, nj = lj - fj + 1;
        i64 jlen = A1(xlnz, fj + 1) - A1(xlnz, fj);
        i64 jx = A1(xlindx, js), jl = A1(xlnz, fj), ju = A1(xunz, fj);
        /* _ldindx!: distance of each row from the bottom of jsup */
        for (i64 j = 1, kk = jlen - 1; j <= jlen; ++j, --kk) map[A1(lindx, jx + j - 1)] = kk;
        i64 nxt = 0;
        for (;;) {
            i64 ks = link[js];
            if (ks == 0) break;
            link[js] = link[ks];
            link[ks] = 0;
            i64 fk = A1(xsuper, ks), lk = A1(xsuper, ks + 1) - 1, nk = lk - fk + 1;
            i64 kslen = A1(xlnz, fk + 1) - A1(xlnz, fk);
            i64 klen = lngth[ks];
            i64 kx = A1(xlindx, ks + 1) - klen;
            i64 kl = A1(xlnz, fk + 1) - klen;
            i64 ku = A1(xunz, fk + 1) - klen;
            i64 nups;
            if (klen == jlen) {
                x_gemm_nt(jlen, nj, nk, -1.0, &L[kl], kslen, &U[ku], kslen - nk, 1.0, &L[jl], jlen);
                if (jlen > nj)
                    x_gemm_nt(jlen - nj, nj, nk, -1.0, &U[ku + nj], kslen - nk, &L[kl], kslen, 1.0, &U[ju],
                              jlen - nj);
                nups = nj;
                if (klen > nj) nxt = A1(lindx, jx + nj);
            } else {
                nups = klen;
                for (i64 i = 0; i <= klen - 1; ++i) {
                    nxt = A1(lindx, kx + i);
                    if (nxt > lj) { nups = i; break; }
                }
                if (nk == 1) {
                    /* _mmpyi! twice: rank-one update by a one-column supernode */
                    for (i64 k = 1; k <= nups; ++k) {
                        double t = U[ku + k - 1];
                        i64 zl = A1(xlnz, A1(lindx, kx + k - 1) + 1) - 1;
                        for (i64 j = 1; j <= klen; ++j) L[zl - map[A1(lindx, kx + j - 1)]] -= t * L[kl + j - 1];
                    }
                    for (i64 k = 1; k <= nups; ++k) {
                        double t = L[kl + k - 1];
                        i64 zl = A1(xunz, A1(lindx, kx + k - 1) + 1) - 1;
                        for (i64 j = 1; j <= klen - nups; ++j)
                            U[zl - map[A1(lindx, kx + nups + j - 1)]] -= t * U[ku + nups + j - 1];
                    }
                } else {
                    i64 kfirst = A1(lindx, kx), klast = A1(lindx, kx + klen - 1);
                    i64 inddif = map[kfirst] - map[klast];
                    if (inddif < klen) {
                        i64 il = A1(xlnz, kfirst) + (kfirst - fj);
                        x_gemm_nt(klen, nups, nk, -1.0, &L[kl], kslen, &U[ku], kslen - nk, 1.0, &L[il], jlen);
                        i64 iu = A1(xunz, kfirst);
                        if (klen > nups)
                            x_gemm_nt(klen - nups, nups, nk, -1.0, &U[ku + nups], kslen - nk, &L[kl], kslen, 1.0,
                                      &U[iu], jlen - nj);
                    } else {
                        if (klen * nups > tmpsiz) iflag = -2;
                        for (i64 j = 1; j <= klen; ++j) relind[j] = map[A1(lindx, kx + j - 1)];
                        x_gemm_nt(klen, nups, nk, -1.0, &L[kl], kslen, &U[ku], kslen - nk, 0.0, temp, klen);
                        /* _assmb! into the columns of L */
                        for (i64 j = 1; j <= nups; ++j) {
                            i64 lbot = A1(xlnz, fj + jlen - relind[j]) - 1;
                            for (i64 k = 1; k <= klen; ++k) L[lbot - relind[k]] += temp[(j - 1) * klen + k - 1];
                        }
                        if (klen > nups) {
                            x_gemm_nt(klen - nups, nups, nk, -1.0, &U[ku + nups], kslen - nk, &L[kl], kslen, 0.0,
                                      temp, klen - nups);
                            for (i64 j = 1; j <= nups; ++j) {
                                i64 lbot = A1(xunz, fj + jlen - relind[j]) - 1;
                                for (i64 k = 1; k <= klen - nups; ++k)
                                    U[lbot - relind[nups + k]] += temp[(j - 1) * (klen - nups) + k - 1];
                            }
                        }
                    }
                }
            }
            if (klen > nups) {
                i64 ns = A1(snode, nxt);
                link[ks] = link[ns];
                link[ns] = ks;
                lngth[ks] = klen - nups;
            } else {
                lngth[ks] = 0;
            }
        }
        /* diagonal block, then the two panels */
        x_getrf(nj, &L[jl], jlen, &A1(ipvt, fj));
        {
            int sing = 0;
            for (i64 k = 0; k < nj; ++k)
                if (L[jl + k * jlen + k] == 0.0) sing = 1;
            iflag = sing ? -1 : 0;
            if (sing && c->first_singular == 0) c->first_singular = js;
        }
        if (g_blas.trsm) x_trsm('R', 'U', 'N', 'N', jlen - nj, nj, &L[jl], jlen, &L[jl + nj], jlen);
        else o_trsm_runn(jlen - nj, nj, &L[jl], jlen, &L[jl + nj], jlen);
        if (jlen > nj) {
            /* _luswap!: swap U-panel rows k <-> ipvt[k], in order */
            i64 ld = jlen - nj;
            for (i64 k = 1; k <= nj; ++k) {
                i64 ip = A1(ipvt, fj + k - 1);
                double* ca = &U[ju + (k - 1) * ld];
                double* cb = &U[ju + (ip - 1) * ld];
                for (i64 t = 0; t < ld; ++t) { double x = cb[t]; cb[t] = ca[t]; ca[t] = x; }
            }
            if (g_blas.trsm) x_trsm('R', 'L', 'T', 'U', jlen - nj, nj, &L[jl], jlen, &U[ju], jlen - nj);
            else o_trsm_rltu(jlen - nj, nj, &L[jl], jlen, &U[ju], jlen - nj);
        }
        if (jlen > nj) {
            nxt = A1(lindx, jx + nj);
            i64 ns = A1(snode, nxt);
            link[js] = link[ns];
            link[ns] = js;
            lngth[js] = jlen - nj;
        } else {
            lngth[js] = 0;
        }
    }
    c->iflag = iflag;
    c->next = js_end + 1;
    return c->next;
}

/* Returns iflag as the reference computes it (last diagonal block wins),
 * and in *first_singular the first supernode whose block had a zero pivot;
 * releases the state. */
i64 oracle_lu_end(void* ctx, i64* first_singular) {
    LuCtx* c = (LuCtx*)ctx;
    i64 iflag = c->iflag;
    *first_singular = c->first_singular;
    free(c->link); free(c->lngth); free(c->map); free(c->relind); free(c->temp);
    free(c);
    return iflag;
}

/* _lufactor! in one call. */
i64 oracle_lufactor(i64 n, i64 nsuper, const i64* xsuper, const i64* snode, const i64* xlindx, const i64* lindx,
                    const i64* xlnz, double* lnz, const i64* xunz, double* unz, i64* ipvt, i64* first_singular) {
    void* c = oracle_lu_begin(n, nsuper, xsuper, snode, xlindx, lindx, xlnz, lnz, xunz, unz, ipvt);
    oracle_lu_run(c, nsuper);
    return oracle_lu_end(c, first_singular);
}

/* ---- supernodal Cholesky on the LU partition ------------------------------ */

/* The symmetric form of _lufactor! for symmetric positive definite A: the
 * same left-looking loop over supernodes and the same link lists
 * (SpkLUFactor.jl:89-252), with L alone: the update of jsup by ksup is
 * L_j -= L_k L_k(jsup rows)^T (the _gemm!('n','t') of the L part with the
 * U-panel operand replaced by L's own rows), the diagonal block is factored
 * by a POTRF (lower, no interchanges: the correct form of the SPD solver's
 * _pchole!, SpkLDLtFactor.jl:347-378, whose scaling is misplaced) and the
 * rows below by _trsm!('r','l','t','n').  On return lnz holds the Cholesky
 * factor C (A = C C^T) in the lower part of every supernode block; the
 * upper part of the diagonal blocks is not meaningful.  Returns 0, or the
 * 1-based column of the first non-positive pivot. */
i64 oracle_cholfactor(i64 n, i64 nsuper, const i64* xsuper, const i64* snode, const i64* xlindx, const i64* lindx,
                      const i64* xlnz, double* lnz) {
    i64* link = (i64*)calloc((size_t)nsuper + 1, sizeof(i64));
    i64* lngth = (i64*)calloc((size_t)nsuper + 1, sizeof(i64));
    i64* map = (i64*)calloc((size_t)n + 1, sizeof(i64));
    i64* relind = (i64*)calloc((size_t)n + 1, sizeof(i64));
    i64 tmpsiz = 0, bad = 0;
    for (i64 i = 1; i <= nsuper; ++i) {
        lngth[i] = A1(xlindx, i + 1) - A1(xlindx, i);
        i64 w = A1(xsuper, i + 1) - A1(xsuper, i);
        i64 need = w * (A1(xlnz, A1(xsuper, i) + 1) - A1(xlnz, A1(xsuper, i)));
        if (need > tmpsiz) tmpsiz = need;
    }
    double* temp = (double*)calloc((size_t)tmpsiz + 1, sizeof(double));
    double* L = lnz - 1;
    for (i64 js = 1; js <= nsuper; ++js) {
        i64 fj = A1(xsuper, js), lj = A1(xsuper, js + 1) - 1, nj = lj - fj + 1;
        i64 jlen = A1(xlnz, fj + 1) - A1(xlnz, fj);
        i64 jx = A1(xlindx, js), jl = A1(xlnz, fj);
        for (i64 j = 1, kk = jlen - 1; j <= jlen; ++j, --kk) map[A1(lindx, jx + j - 1)] = kk;
        i64 nxt = 0;
        for (;;) {
            i64 ks = link[js];
            if (ks == 0) break;
            link[js] = link[ks];
            link[ks] = 0;
            i64 fk = A1(xsuper, ks);
            i64 kslen = A1(xlnz, fk + 1) - A1(xlnz, fk);
            i64 nk = A1(xsuper, ks + 1) - fk;
            i64 klen = lngth[ks];
            i64 kx = A1(xlindx, ks + 1) - klen;
            i64 kl = A1(xlnz, fk + 1) - klen;
            i64 nups;
            if (klen == jlen) {
                x_gemm_nt(jlen, nj, nk, -1.0, &L[kl], kslen, &L[kl], kslen, 1.0, &L[jl], jlen);
                nups = nj;
                if (klen > nj) nxt = A1(lindx, jx + nj);
            } else {
                nups = klen;
                for (i64 i = 0; i <= klen - 1; ++i) {
                    nxt = A1(lindx, kx + i);
                    if (nxt > lj) { nups = i; break; }
                }
                for (i64 j = 1; j <= klen; ++j) relind[j] = map[A1(lindx, kx + j - 1)];
                x_gemm_nt(klen, nups, nk, -1.0, &L[kl], kslen, &L[kl], kslen, 0.0, temp, klen);
                for (i64 j = 1; j <= nups; ++j) {   /* _assmb! into the columns of L */
                    i64 lbot = A1(xlnz, fj + jlen - relind[j]) - 1;
                    for (i64 k = j; k <= klen; ++k) L[lbot - relind[k]] += temp[(j - 1) * klen + k - 1];
                }
            }
            (void)nk;
            if (klen > nups) {
                i64 ns = A1(snode, nxt);
                link[ks] = link[ns];
                link[ns] = ks;
                lngth[ks] = klen - nups;
            } else {
                lngth[ks] = 0;
            }
        }
        /* POTRF of the diagonal block (lower), then L21 := A21 L11^-T */
        for (i64 k = 0; k < nj; ++k) {
            double* ck = &L[jl + k * jlen];
            for (i64 p = 0; p < k; ++p) {
                const double* cp = &L[jl + p * jlen];
                for (i64 i = k; i < jlen; ++i) ck[i] -= cp[i] * cp[k];
            }
            if (!(ck[k] > 0.0)) {
                if (bad == 0) bad = fj + k;
                ck[k] = 1.0;
            }
            double d = sqrt(ck[k]);
            ck[k] = d;
            for (i64 i = k + 1; i < jlen; ++i) ck[i] /= d;
        }
        if (jlen > nj) {
            nxt = A1(lindx, jx + nj);
            i64 ns = A1(snode, nxt);
            link[js] = link[ns];
            link[ns] = js;
            lngth[js] = jlen - nj;
        } else {
            lngth[js] = 0;
        }
    }
    free(link);
    free(lngth);
    free(map);
    free(relind);
    free(temp);
    return bad;
}

/* ---- _lulsolve! / _luusolve! ---------------------------------------------- */

void oracle_lulsolve(i64 nsuper, const i64* xsuper, const i64* xlindx, const i64* lindx, const i64* xlnz,
                     const double* lnz, const i64* ipiv, double* rhs) {
    const double* L = lnz - 1;
    double* R = rhs - 1;
    i64 maxlen = 1;
    for (i64 js = 1; js <= nsuper; ++js)
        if (A1(xlindx, js + 1) - A1(xlindx, js) > maxlen) maxlen = A1(xlindx, js + 1) - A1(xlindx, js);
    double* temp = g_blas.gemv ? (double*)calloc((size_t)maxlen, sizeof(double)) : NULL;
    int* ip32 = g_blas.laswp ? (int*)calloc((size_t)maxlen, sizeof(int)) : NULL;
    for (i64 js = 1; js <= nsuper; ++js) {
        i64 fj = A1(xsuper, js), nj = A1(xsuper, js + 1) - fj;
        i64 jlen = A1(xlnz, fj + 1) - A1(xlnz, fj);
        i64 jx = A1(xlindx, js), jl = A1(xlnz, fj);
        if (g_blas.gemv) {   /* _laswp!, _trsm!('l','l','n','u'), _gemv!('n'), scatter-add */
            int one = 1, inj = (int)nj, im = (int)(jlen - nj), ild = (int)jlen, inc = 1;
            double mone = -1.0, zero = 0.0;
            for (i64 i = 0; i < nj; ++i) ip32[i] = (int)A1(ipiv, fj + i);
            g_blas.laswp(&one, &R[fj], &inj, &one, &inj, ip32, &inc);
            x_trsm('L', 'L', 'N', 'U', nj, 1, (double*)&L[jl], jlen, &R[fj], nj);
            if (im > 0) {
                g_blas.gemv("N", &im, &inj, &mone, (double*)&L[jl + nj], &ild, &R[fj], &inc, &zero, temp, &inc);
                for (i64 j = 1; j <= jlen - nj; ++j) R[A1(lindx, jx + nj + j - 1)] += temp[j - 1];
            }
            continue;
        }
        for (i64 i = 1; i <= nj; ++i) { /* glaswp! */
            i64 ip = A1(ipiv, fj + i - 1);
            if (ip != i) { double t = R[fj + i - 1]; R[fj + i - 1] = R[fj + ip - 1]; R[fj + ip - 1] = t; }
        }
        o_trsv_llnu(nj, &L[jl], jlen, &R[fj]);
        for (i64 j = 1; j <= jlen - nj; ++j) { /* ggemv!('n') then scatter-add */
            double t = 0.0;
            for (i64 k = 0; k < nj; ++k) t += -R[fj + k] * L[jl + nj + k * jlen + j - 1];
            R[A1(lindx, jx + nj + j - 1)] += t;
        }
    }
    free(temp);
    free(ip32);
}

void oracle_luusolve(i64 n, i64 nsuper, const i64* xsuper, const i64* xlindx, const i64* lindx, const i64* xlnz,
                     const double* lnz, const i64* xunz, const double* unz, double* rhs) {
    (void)n;
    const double* L = lnz - 1;
    const double* U = unz - 1;
    double* R = rhs - 1;
    i64 maxlen = 1;
    for (i64 js = 1; js <= nsuper; ++js)
        if (A1(xlindx, js + 1) - A1(xlindx, js) > maxlen) maxlen = A1(xlindx, js + 1) - A1(xlindx, js);
    double* temp = g_blas.gemv ? (double*)calloc((size_t)maxlen, sizeof(double)) : NULL;
    for (i64 js = nsuper; js >= 1; --js) {
        i64 fj = A1(xsuper, js), nj = A1(xsuper, js + 1) - fj;
        i64 jlen = A1(xlnz, fj + 1) - A1(xlnz, fj);
        i64 jx = A1(xlindx, js), jl = A1(xlnz, fj), ju = A1(xunz, fj);
        if (g_blas.gemv) {   /* gather, _gemv!('t'), _trsm!('l','u','n','n') */
            if (jlen > nj) {
                int im = (int)(jlen - nj), inj = (int)nj, inc = 1;
                double mone = -1.0, one = 1.0;
                for (i64 j = 1; j <= jlen - nj; ++j) temp[j - 1] = R[A1(lindx, jx + nj + j - 1)];
                g_blas.gemv("T", &im, &inj, &mone, (double*)&U[ju], &im, temp, &inc, &one, &R[fj], &inc);
            }
            x_trsm('L', 'U', 'N', 'N', nj, 1, (double*)&L[jl], jlen, &R[fj], nj);
            continue;
        }
        if (jlen > nj) { /* gather, then ggemv!('t') */
            for (i64 k = 0; k < nj; ++k) {
                double t = 0.0;
                for (i64 j = 1; j <= jlen - nj; ++j) t += U[ju + k * (jlen - nj) + j - 1] * R[A1(lindx, jx + nj + j - 1)];
                R[fj + k] += -t;
            }
        }
        o_trsv_lunn(nj, &L[jl], jlen, &R[fj]);
    }
    free(temp);
}

/* _triangularsolve!: permute, forward, backward, unpermute (in place). */
void oracle_triangularsolve(i64 n, i64 nsuper, const i64* xsuper, const i64* xlindx, const i64* lindx,
                            const i64* xlnz, const double* lnz, const i64* xunz, const double* unz, const i64* ipiv,
                            const i64* rperm, const i64* rinvp, double* solution) {
    double* r = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    for (i64 i = 1; i <= n; ++i) r[i - 1] = A1(solution, A1(rperm, i));
    oracle_lulsolve(nsuper, xsuper, xlindx, lindx, xlnz, lnz, ipiv, r);
    oracle_luusolve(n, nsuper, xsuper, xlindx, lindx, xlnz, lnz, xunz, unz, r);
    for (i64 i = 1; i <= n; ++i) A1(solution, i) = r[A1(rinvp, i) - 1];
    free(r);
}

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

/* Returns iflag as the reference computes it (last diagonal block wins),
 * and in *first_singular the first supernode whose block had a zero pivot. */
i64 oracle_lufactor(i64 n, i64 nsuper, const i64* xsuper, const i64* snode, const i64* xlindx, const i64* lindx,
                    const i64* xlnz, double* lnz, const i64* xunz, double* unz, i64* ipvt, i64* first_singular) {
    i64* link = (i64*)calloc((size_t)nsuper + 1, sizeof(i64));
    i64* lngth = (i64*)calloc((size_t)nsuper + 1, sizeof(i64));
    i64* map = (i64*)calloc((size_t)n + 1, sizeof(i64));
    i64* relind = (i64*)calloc((size_t)n + 1, sizeof(i64));
    i64 tmpsiz = 0, iflag = 0;
    *first_singular = 0;
    for (i64 i = 1; i <= nsuper; ++i) {
        lngth[i] = A1(xlindx, i + 1) - A1(xlindx, i);
        i64 w = A1(xsuper, i + 1) - A1(xsuper, i);
        i64 need = w * (A1(xlnz, A1(xsuper, i) + 1) - A1(xlnz, A1(xsuper, i)));
        if (need > tmpsiz) tmpsiz = need;
    }
    double* temp = (double*)calloc((size_t)tmpsiz + 1, sizeof(double));
    double* L = lnz - 1; /* L[p] == reference lnz[p] */
    double* U = unz - 1;

    for (i64 js = 1; js <= nsuper; ++js) {
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
                o_gemm_nt(jlen, nj, nk, -1.0, &L[kl], kslen, &U[ku], kslen - nk, 1.0, &L[jl], jlen);
                if (jlen > nj)
                    o_gemm_nt(jlen - nj, nj, nk, -1.0, &U[ku + nj], kslen - nk, &L[kl], kslen, 1.0, &U[ju],
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
                        o_gemm_nt(klen, nups, nk, -1.0, &L[kl], kslen, &U[ku], kslen - nk, 1.0, &L[il], jlen);
                        i64 iu = A1(xunz, kfirst);
                        if (klen > nups)
                            o_gemm_nt(klen - nups, nups, nk, -1.0, &U[ku + nups], kslen - nk, &L[kl], kslen, 1.0,
                                      &U[iu], jlen - nj);
                    } else {
                        if (klen * nups > tmpsiz) iflag = -2;
                        for (i64 j = 1; j <= klen; ++j) relind[j] = map[A1(lindx, kx + j - 1)];
                        o_gemm_nt(klen, nups, nk, -1.0, &L[kl], kslen, &U[ku], kslen - nk, 0.0, temp, klen);
                        /* _assmb! into the columns of L */
                        for (i64 j = 1; j <= nups; ++j) {
                            i64 lbot = A1(xlnz, fj + jlen - relind[j]) - 1;
                            for (i64 k = 1; k <= klen; ++k) L[lbot - relind[k]] += temp[(j - 1) * klen + k - 1];
                        }
                        if (klen > nups) {
                            o_gemm_nt(klen - nups, nups, nk, -1.0, &U[ku + nups], kslen - nk, &L[kl], kslen, 0.0,
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
        o_getrf(nj, nj, &L[jl], jlen, &A1(ipvt, fj));
        {
            int sing = 0;
            for (i64 k = 0; k < nj; ++k)
                if (L[jl + k * jlen + k] == 0.0) sing = 1;
            iflag = sing ? -1 : 0;
            if (sing && *first_singular == 0) *first_singular = js;
        }
        o_trsm_runn(jlen - nj, nj, &L[jl], jlen, &L[jl + nj], jlen);
        if (jlen > nj) {
            /* _luswap!: swap U-panel rows k <-> ipvt[k], in order */
            i64 ld = jlen - nj;
            for (i64 k = 1; k <= nj; ++k) {
                i64 ip = A1(ipvt, fj + k - 1);
                double* ca = &U[ju + (k - 1) * ld];
                double* cb = &U[ju + (ip - 1) * ld];
                for (i64 t = 0; t < ld; ++t) { double x = cb[t]; cb[t] = ca[t]; ca[t] = x; }
            }
            o_trsm_rltu(jlen - nj, nj, &L[jl], jlen, &U[ju], jlen - nj);
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
    return iflag;
}

/* ---- _lulsolve! / _luusolve! ---------------------------------------------- */

void oracle_lulsolve(i64 nsuper, const i64* xsuper, const i64* xlindx, const i64* lindx, const i64* xlnz,
                     const double* lnz, const i64* ipiv, double* rhs) {
    const double* L = lnz - 1;
    double* R = rhs - 1;
    for (i64 js = 1; js <= nsuper; ++js) {
        i64 fj = A1(xsuper, js), nj = A1(xsuper, js + 1) - fj;
        i64 jlen = A1(xlnz, fj + 1) - A1(xlnz, fj);
        i64 jx = A1(xlindx, js), jl = A1(xlnz, fj);
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
}

void oracle_luusolve(i64 n, i64 nsuper, const i64* xsuper, const i64* xlindx, const i64* lindx, const i64* xlnz,
                     const double* lnz, const i64* xunz, const double* unz, double* rhs) {
    (void)n;
    const double* L = lnz - 1;
    const double* U = unz - 1;
    double* R = rhs - 1;
    for (i64 js = nsuper; js >= 1; --js) {
        i64 fj = A1(xsuper, js), nj = A1(xsuper, js + 1) - fj;
        i64 jlen = A1(xlnz, fj + 1) - A1(xlnz, fj);
        i64 jx = A1(xlindx, js), jl = A1(xlnz, fj), ju = A1(xunz, fj);
        if (jlen > nj) { /* gather, then ggemv!('t') */
            for (i64 k = 0; k < nj; ++k) {
                double t = 0.0;
                for (i64 j = 1; j <= jlen - nj; ++j) t += U[ju + k * (jlen - nj) + j - 1] * R[A1(lindx, jx + nj + j - 1)];
                R[fj + k] += -t;
            }
        }
        o_trsv_lunn(nj, &L[jl], jlen, &R[fj]);
    }
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

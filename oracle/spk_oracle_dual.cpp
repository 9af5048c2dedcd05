// ORACLE - TEST INFRASTRUCTURE ONLY.
//
// Forward-mode derivatives through the reference's LU path, the way the
// reference computes them: its generic Julia code run on ForwardDiff.Dual
// numbers (test/test_generic.jl:19-43 and the gradient test :58-98).  This
// file restates, templated on the element type, the same steps as
// spk_oracle.c - _inmatrix! (CSC, src/SparseCSCInterface/SparseCSCInterface.jl:101-169),
// _lufactor! (src/SparseMethod/SpkLUFactor.jl:60-255) with the generic
// fragments ggetrf!, ggemm!, gtrsm! (src/Utilities/GenericBlasLapackFragments.jl:56-480),
// _lulsolve! / _luusolve! (SpkLUFactor.jl:269-377) and _triangularsolve!
// (src/SparseMethod/SpkSparseBase.jl:400-416) - and runs them on a dual
// number with NP partials.  As in ForwardDiff, comparisons of duals (the
// pivot search, the tests for zero) look at the value alone.  The tests use
// it to check the GPU adjoint gradient on reduced problems.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

typedef int64_t i64;

namespace {

constexpr int NP = 16;   // partials per dual number

struct Dual {
    double v;
    double d[NP];
};

inline Dual dconst(double x) {
    Dual r;
    r.v = x;
    for (int k = 0; k < NP; ++k) r.d[k] = 0.0;
    return r;
}
inline Dual operator+(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v + b.v;
    for (int k = 0; k < NP; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
inline Dual operator-(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v - b.v;
    for (int k = 0; k < NP; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
inline Dual operator-(const Dual& a) {
    Dual r;
    r.v = -a.v;
    for (int k = 0; k < NP; ++k) r.d[k] = -a.d[k];
    return r;
}
inline Dual operator*(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v * b.v;
    for (int k = 0; k < NP; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
inline Dual operator/(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v / b.v;
    const double ib2 = 1.0 / (b.v * b.v);
    for (int k = 0; k < NP; ++k) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) * ib2;
    return r;
}
inline Dual& operator+=(Dual& a, const Dual& b) { return a = a + b; }
inline Dual& operator-=(Dual& a, const Dual& b) { return a = a - b; }
inline Dual& operator*=(Dual& a, const Dual& b) { return a = a * b; }
inline double val(const Dual& a) { return a.v; }   // ForwardDiff compares values only

#define A1(p, i) ((p)[(i) - 1])

// ggetrf!: unblocked right-looking LU, first strict maximum of |a| as pivot.
template <typename T>
void g_getrf(i64 m, i64 n, T* a, i64 lda, i64* ipiv) {
    auto A = [&](i64 i, i64 j) -> T& { return a[(j - 1) * lda + i - 1]; };
    const i64 mn = m < n ? m : n;
    for (i64 k = 1; k <= mn; ++k) {
        i64 kp = k;
        if (k < m) {
            double amax = std::fabs(val(A(k, k)));
            for (i64 i = k + 1; i <= m; ++i) {
                const double ai = std::fabs(val(A(i, k)));
                if (ai > amax) { kp = i; amax = ai; }
            }
        }
        ipiv[k - 1] = kp;
        if (val(A(kp, k)) != 0.0) {
            if (k != kp)
                for (i64 i = 1; i <= n; ++i) { T t = A(k, i); A(k, i) = A(kp, i); A(kp, i) = t; }
            const T inv = dconst(1.0) / A(k, k);
            for (i64 i = k + 1; i <= m; ++i) A(i, k) *= inv;
        }
        for (i64 j = k + 1; j <= n; ++j)
            for (i64 i = k + 1; i <= m; ++i) A(i, j) -= A(i, k) * A(k, j);
    }
}

// ggemm!('n','t'): C := alpha A B' + beta C (alpha = -1; beta 0 or 1).
template <typename T>
void g_gemm_nt(i64 m, i64 n, i64 k, const T* a, i64 lda, const T* b, i64 ldb, bool beta1, T* c, i64 ldc) {
    for (i64 j = 0; j < n; ++j) {
        if (!beta1)
            for (i64 i = 0; i < m; ++i) c[j * ldc + i] = dconst(0.0);
        for (i64 l = 0; l < k; ++l) {
            const T t = -b[l * ldb + j];
            for (i64 i = 0; i < m; ++i) c[j * ldc + i] += t * a[l * lda + i];
        }
    }
}

// gtrsm!('r','u','n','n'): B := B inv(U).
template <typename T>
void g_trsm_runn(i64 m, i64 n, const T* a, i64 lda, T* b, i64 ldb) {
    for (i64 j = 0; j < n; ++j) {
        for (i64 k = 0; k < j; ++k) {
            const T akj = a[j * lda + k];
            if (val(akj) != 0.0)
                for (i64 i = 0; i < m; ++i) b[j * ldb + i] -= akj * b[k * ldb + i];
        }
        const T t = dconst(1.0) / a[j * lda + j];
        for (i64 i = 0; i < m; ++i) b[j * ldb + i] *= t;
    }
}

// gtrsm!('r','l','t','u'): B := B inv(L'), L unit lower.
template <typename T>
void g_trsm_rltu(i64 m, i64 n, const T* a, i64 lda, T* b, i64 ldb) {
    for (i64 k = 0; k < n; ++k)
        for (i64 j = k + 1; j < n; ++j) {
            const T ajk = a[k * lda + j];
            if (val(ajk) != 0.0)
                for (i64 i = 0; i < m; ++i) b[j * ldb + i] -= ajk * b[k * ldb + i];
        }
}

// _lufactor! with the generic fragments (the same steps as oracle_lufactor).
template <typename T>
void g_lufactor(i64 n, i64 nsuper, const i64* xsuper, const i64* snode, const i64* xlindx, const i64* lindx,
                const i64* xlnz, T* lnz, const i64* xunz, T* unz, i64* ipvt) {
    std::vector<i64> link(nsuper + 1, 0), lngth(nsuper + 1, 0), map(n + 1, 0), relind(n + 1, 0);
    i64 tmpsiz = 0;
    for (i64 i = 1; i <= nsuper; ++i) {
        lngth[i] = A1(xlindx, i + 1) - A1(xlindx, i);
        const i64 w = A1(xsuper, i + 1) - A1(xsuper, i);
        tmpsiz = std::max(tmpsiz, w * (A1(xlnz, A1(xsuper, i) + 1) - A1(xlnz, A1(xsuper, i))));
    }
    std::vector<T> temp(tmpsiz + 1);
    T* L = lnz - 1;
    T* U = unz - 1;
    for (i64 js = 1; js <= nsuper; ++js) {
        const i64 fj = A1(xsuper, js), lj = A1(xsuper, js + 1) - 1, nj = lj - fj + 1;
        const i64 jlen = A1(xlnz, fj + 1) - A1(xlnz, fj);
        const i64 jx = A1(xlindx, js), jl = A1(xlnz, fj), ju = A1(xunz, fj);
        for (i64 j = 1, kk = jlen - 1; j <= jlen; ++j, --kk) map[A1(lindx, jx + j - 1)] = kk;
        i64 nxt = 0;
        for (;;) {
            const i64 ks = link[js];
            if (ks == 0) break;
            link[js] = link[ks];
            link[ks] = 0;
            const i64 fk = A1(xsuper, ks), nk = A1(xsuper, ks + 1) - fk;
            const i64 kslen = A1(xlnz, fk + 1) - A1(xlnz, fk);
            const i64 klen = lngth[ks];
            const i64 kx = A1(xlindx, ks + 1) - klen;
            const i64 kl = A1(xlnz, fk + 1) - klen;
            const i64 ku = A1(xunz, fk + 1) - klen;
            i64 nups;
            if (klen == jlen) {
                g_gemm_nt(jlen, nj, nk, &L[kl], kslen, &U[ku], kslen - nk, true, &L[jl], jlen);
                if (jlen > nj) g_gemm_nt(jlen - nj, nj, nk, &U[ku + nj], kslen - nk, &L[kl], kslen, true, &U[ju], jlen - nj);
                nups = nj;
                if (klen > nj) nxt = A1(lindx, jx + nj);
            } else {
                nups = klen;
                for (i64 i = 0; i <= klen - 1; ++i) {
                    nxt = A1(lindx, kx + i);
                    if (nxt > lj) { nups = i; break; }
                }
                for (i64 j = 1; j <= klen; ++j) relind[j] = map[A1(lindx, kx + j - 1)];
                g_gemm_nt(klen, nups, nk, &L[kl], kslen, &U[ku], kslen - nk, false, temp.data(), klen);
                for (i64 j = 1; j <= nups; ++j) {   // _assmb! into the columns of L
                    const i64 lbot = A1(xlnz, fj + jlen - relind[j]) - 1;
                    for (i64 k = 1; k <= klen; ++k) L[lbot - relind[k]] += temp[(j - 1) * klen + k - 1];
                }
                if (klen > nups) {
                    g_gemm_nt(klen - nups, nups, nk, &U[ku + nups], kslen - nk, &L[kl], kslen, false, temp.data(),
                              klen - nups);
                    for (i64 j = 1; j <= nups; ++j) {
                        const i64 lbot = A1(xunz, fj + jlen - relind[j]) - 1;
                        for (i64 k = 1; k <= klen - nups; ++k)
                            U[lbot - relind[nups + k]] += temp[(j - 1) * (klen - nups) + k - 1];
                    }
                }
            }
            if (klen > nups) {
                const i64 ns = A1(snode, nxt);
                link[ks] = link[ns];
                link[ns] = ks;
                lngth[ks] = klen - nups;
            } else {
                lngth[ks] = 0;
            }
        }
        g_getrf(nj, nj, &L[jl], jlen, &A1(ipvt, fj));
        g_trsm_runn(jlen - nj, nj, &L[jl], jlen, &L[jl + nj], jlen);
        if (jlen > nj) {
            const i64 ld = jlen - nj;
            for (i64 k = 1; k <= nj; ++k) {   // _luswap!
                const i64 ip = A1(ipvt, fj + k - 1);
                T* ca = &U[ju + (k - 1) * ld];
                T* cb = &U[ju + (ip - 1) * ld];
                for (i64 t = 0; t < ld; ++t) { T x = cb[t]; cb[t] = ca[t]; ca[t] = x; }
            }
            g_trsm_rltu(jlen - nj, nj, &L[jl], jlen, &U[ju], jlen - nj);
            nxt = A1(lindx, jx + nj);
            const i64 ns = A1(snode, nxt);
            link[js] = link[ns];
            link[ns] = js;
            lngth[js] = jlen - nj;
        } else {
            lngth[js] = 0;
        }
    }
}

// _lulsolve! then _luusolve! on a permuted right-hand side.
template <typename T>
void g_solve(i64 nsuper, const i64* xsuper, const i64* xlindx, const i64* lindx, const i64* xlnz, const T* lnz,
             const i64* xunz, const T* unz, const i64* ipiv, T* rhs) {
    const T* L = lnz - 1;
    const T* U = unz - 1;
    T* R = rhs - 1;
    for (i64 js = 1; js <= nsuper; ++js) {
        const i64 fj = A1(xsuper, js), nj = A1(xsuper, js + 1) - fj;
        const i64 jlen = A1(xlnz, fj + 1) - A1(xlnz, fj);
        const i64 jx = A1(xlindx, js), jl = A1(xlnz, fj);
        for (i64 i = 1; i <= nj; ++i) {   // glaswp!
            const i64 ip = A1(ipiv, fj + i - 1);
            if (ip != i) { T t = R[fj + i - 1]; R[fj + i - 1] = R[fj + ip - 1]; R[fj + ip - 1] = t; }
        }
        for (i64 k = 0; k < nj; ++k)   // gtrsm!('l','l','n','u'), one column
            if (val(R[fj + k]) != 0.0)
                for (i64 i = k + 1; i < nj; ++i) R[fj + i] -= R[fj + k] * L[jl + k * jlen + i];
        for (i64 j = 1; j <= jlen - nj; ++j) {   // ggemv!('n'), scatter-add
            T t = dconst(0.0);
            for (i64 k = 0; k < nj; ++k) t += (-R[fj + k]) * L[jl + nj + k * jlen + j - 1];
            R[A1(lindx, jx + nj + j - 1)] += t;
        }
    }
    for (i64 js = nsuper; js >= 1; --js) {
        const i64 fj = A1(xsuper, js), nj = A1(xsuper, js + 1) - fj;
        const i64 jlen = A1(xlnz, fj + 1) - A1(xlnz, fj);
        const i64 jx = A1(xlindx, js), jl = A1(xlnz, fj), ju = A1(xunz, fj);
        if (jlen > nj)
            for (i64 k = 0; k < nj; ++k) {   // gather, ggemv!('t')
                T t = dconst(0.0);
                for (i64 j = 1; j <= jlen - nj; ++j) t += U[ju + k * (jlen - nj) + j - 1] * R[A1(lindx, jx + nj + j - 1)];
                R[fj + k] -= t;
            }
        for (i64 k = nj - 1; k >= 0; --k)   // gtrsm!('l','u','n','n'), one column
            if (val(R[fj + k]) != 0.0) {
                R[fj + k] = R[fj + k] / L[jl + k * jlen + k];
                for (i64 i = 0; i < k; ++i) R[fj + i] -= R[fj + k] * L[jl + k * jlen + i];
            }
    }
}

}  // namespace

// x = A^{-1} b with A's values dual: nzval[nnz] the values, dnz[nnz * NP]
// (entry-major) their partials; b has no partials.  Runs _inmatrix! (CSC),
// _lufactor! and _triangularsolve! on duals for the given structure.
// Returns 0, or -(1 + p) if entry p has no slot; x[n], dx[n * NP] (row-major).
extern "C" i64 oracle_dual_solve(i64 n, i64 nsuper, const i64* xsuper, const i64* snode, const i64* xlindx,
                                 const i64* lindx, const i64* xlnz, const i64* xunz, const i64* rperm, const i64* rinvp,
                                 const i64* colptr, const i64* rowval, const double* nzval, const double* dnz,
                                 const double* b, double* x, double* dx) {
    std::vector<Dual> lnz(A1(xlnz, n + 1) - 1, dconst(0.0)), unz(std::max<i64>(A1(xunz, n + 1) - 1, 1), dconst(0.0));
    std::vector<i64> ipiv(n, 0);
    // _inmatrix! (CSC): the same slot search as oracle_inmatrix_csc
    for (i64 i = 1; i <= n; ++i)
        for (i64 p = A1(colptr, i); p <= A1(colptr, i + 1) - 1; ++p) {
            const i64 inew = A1(rinvp, A1(rowval, p)), jnew = A1(rinvp, i);
            Dual v;
            v.v = A1(nzval, p);
            for (int k = 0; k < NP; ++k) v.d[k] = dnz[(p - 1) * NP + k];
            bool placed = false;
            if (inew >= A1(xsuper, A1(snode, jnew))) {
                const i64 js = A1(snode, jnew);
                i64 loc = 0;
                for (i64 s = A1(xlindx, js); s <= A1(xlindx, js + 1) - 1; ++s) {
                    const i64 r = A1(lindx, s);
                    if (r > inew) break;
                    if (r == inew) { lnz[A1(xlnz, jnew) + loc - 1] += v; placed = true; break; }
                    ++loc;
                }
            } else {
                const i64 js = A1(snode, inew), w = A1(xsuper, js + 1) - A1(xsuper, js);
                i64 loc = 0;
                for (i64 s = A1(xlindx, js) + w; s <= A1(xlindx, js + 1) - 1; ++s) {
                    const i64 r = A1(lindx, s);
                    if (r > jnew) break;
                    if (r == jnew) { unz[A1(xunz, inew) + loc - 1] += v; placed = true; break; }
                    ++loc;
                }
            }
            if (!placed) return -p;
        }
    g_lufactor(n, nsuper, xsuper, snode, xlindx, lindx, xlnz, lnz.data(), xunz, unz.data(), ipiv.data());
    std::vector<Dual> r(n);
    for (i64 i = 1; i <= n; ++i) r[i - 1] = dconst(A1(b, A1(rperm, i)));
    g_solve(nsuper, xsuper, xlindx, lindx, xlnz, lnz.data(), xunz, unz.data(), ipiv.data(), r.data());
    for (i64 i = 1; i <= n; ++i) {
        const Dual& v = r[A1(rinvp, i) - 1];
        x[i - 1] = v.v;
        for (int k = 0; k < NP; ++k) dx[(i - 1) * NP + k] = v.d[k];
    }
    return 0;
}

extern "C" int oracle_dual_partials(void) { return NP; }

// Reference-order BLAS / LAPACK / MKL-extension subset for the one-process CPU
// build of chiML's own sources (test infrastructure only).
//
// Each routine follows the published netlib (or Intel MKL, for the mkl_*
// routines) definition with plain loops in column-major order. Nothing here is
// tuned; the point is a deterministic, dependency-free stand-in so that the
// unmodified reference sources link and run on this machine.
#include <cmath>
#include <complex>
#include <cstdlib>
#include <stdexcept>
#include <vector>

typedef std::complex<double> cplx;

namespace {
inline bool is(const char* c, char u) { return (*c == u) || (*c == u + 32); }
inline cplx opval(const cplx* a, int lda, int i, int j, char t) {
    // element (i, j) of op(A), op in {N, T, C, R}
    if (t == 'N' || t == 'n') return a[i + j * lda];
    if (t == 'T' || t == 't') return a[j + i * lda];
    if (t == 'C' || t == 'c') return std::conj(a[j + i * lda]);
    return std::conj(a[i + j * lda]);  // 'R': conjugate, no transpose
}
}  // namespace

extern "C" {

void daxpy_(const int* n, const double* a, const double* x, const int* incx, double* y, const int* incy) {
    for (int i = 0; i < *n; ++i) y[i * *incy] += *a * x[i * *incx];
}
void dcopy_(const int* n, const double* x, const int* incx, double* y, const int* incy) {
    for (int i = 0; i < *n; ++i) y[i * *incy] = x[i * *incx];
}
void dscal_(const int* n, const double* a, double* x, const int* incx) {
    for (int i = 0; i < *n; ++i) x[i * *incx] *= *a;
}
double ddot_(const int* n, const double* x, const int* incx, const double* y, const int* incy) {
    double s = 0.0;
    for (int i = 0; i < *n; ++i) s += x[i * *incx] * y[i * *incy];
    return s;
}
double dasum_(const int* n, const double* x, const int* incx) {
    double s = 0.0;
    for (int i = 0; i < *n; ++i) s += std::abs(x[i * *incx]);
    return s;
}
void zaxpy_(const int* n, const cplx* a, const cplx* x, const int* incx, cplx* y, const int* incy) {
    for (int i = 0; i < *n; ++i) y[i * *incy] += *a * x[i * *incx];
}
void zcopy_(const int* n, const cplx* x, const int* incx, cplx* y, const int* incy) {
    for (int i = 0; i < *n; ++i) y[i * *incy] = x[i * *incx];
}
void zscal_(const int* n, const cplx* a, cplx* x, const int* incx) {
    for (int i = 0; i < *n; ++i) x[i * *incx] *= *a;
}
void zdotc_(cplx* res, const int* n, const cplx* x, const int* incx, const cplx* y, const int* incy) {
    cplx s = 0.0;
    for (int i = 0; i < *n; ++i) s += std::conj(x[i * *incx]) * y[i * *incy];
    *res = s;
}
// Integer "single" routines: the reference calls these on int arrays. For the
// non-negative values it passes, float ordering of the bit patterns equals
// integer ordering, so comparing the integers directly gives the same index.
void saxpy_(const int* n, const int* a, const int* x, const int* incx, int* y, const int* incy) {
    for (int i = 0; i < *n; ++i) y[i * *incy] += *a * x[i * *incx];
}
void scopy_(const int* n, const int* x, const int* incx, int* y, const int* incy) {
    for (int i = 0; i < *n; ++i) y[i * *incy] = x[i * *incx];
}
void sscal_(const int* n, const int* a, int* x, const int* incx) {
    for (int i = 0; i < *n; ++i) x[i * *incx] *= *a;
}
int sasum_(const int* n, const int* x, const int* incx) {
    int s = 0;
    for (int i = 0; i < *n; ++i) s += std::abs(x[i * *incx]);
    return s;
}
int isamin_(const int* n, const int* x, const int* incx) {
    if (*n < 1) return 0;
    int best = 0;
    for (int i = 1; i < *n; ++i)
        if (std::abs(x[i * *incx]) < std::abs(x[best * *incx])) best = i;
    return best + 1;
}
int isamax_(const int* n, const int* x, const int* incx) {
    if (*n < 1) return 0;
    int best = 0;
    for (int i = 1; i < *n; ++i)
        if (std::abs(x[i * *incx]) > std::abs(x[best * *incx])) best = i;
    return best + 1;
}
int idamin_(const int* n, const double* x, const int* incx) {
    if (*n < 1) return 0;
    int best = 0;
    for (int i = 1; i < *n; ++i)
        if (std::abs(x[i * *incx]) < std::abs(x[best * *incx])) best = i;
    return best + 1;
}
int idamax_(const int* n, const double* x, const int* incx) {
    if (*n < 1) return 0;
    int best = 0;
    for (int i = 1; i < *n; ++i)
        if (std::abs(x[i * *incx]) > std::abs(x[best * *incx])) best = i;
    return best + 1;
}
// BLAS i?amax for complex uses |Re| + |Im|
int izamin_(const int* n, const cplx* x, const int* incx) {
    if (*n < 1) return 0;
    int best = 0;
    auto m = [](cplx v) { return std::abs(v.real()) + std::abs(v.imag()); };
    for (int i = 1; i < *n; ++i)
        if (m(x[i * *incx]) < m(x[best * *incx])) best = i;
    return best + 1;
}
int izamax_(const int* n, const cplx* x, const int* incx) {
    if (*n < 1) return 0;
    int best = 0;
    auto m = [](cplx v) { return std::abs(v.real()) + std::abs(v.imag()); };
    for (int i = 1; i < *n; ++i)
        if (m(x[i * *incx]) > m(x[best * *incx])) best = i;
    return best + 1;
}

void dger_(const int* m, const int* n, const double* alpha, const double* x, const int* incx, const double* y,
           const int* incy, double* a, const int* lda) {
    for (int j = 0; j < *n; ++j) {
        const double t = *alpha * y[j * *incy];
        for (int i = 0; i < *m; ++i) a[i + j * *lda] += x[i * *incx] * t;
    }
}
void zgerc_(const int* m, const int* n, const cplx* alpha, const cplx* x, const int* incx, const cplx* y,
            const int* incy, cplx* a, const int* lda) {
    for (int j = 0; j < *n; ++j) {
        const cplx t = *alpha * std::conj(y[j * *incy]);
        for (int i = 0; i < *m; ++i) a[i + j * *lda] += x[i * *incx] * t;
    }
}
void zgeru_(const int* m, const int* n, const cplx* alpha, const cplx* x, const int* incx, const cplx* y,
            const int* incy, cplx* a, const int* lda) {
    for (int j = 0; j < *n; ++j) {
        const cplx t = *alpha * y[j * *incy];
        for (int i = 0; i < *m; ++i) a[i + j * *lda] += x[i * *incx] * t;
    }
}
void dgemv_(const char* trans, const int* m, const int* n, const double* alpha, const double* a, const int* lda,
            const double* x, const int* incx, const double* beta, double* y, const int* incy) {
    const bool t = !is(trans, 'N');
    const int ly = t ? *n : *m, lx = t ? *m : *n;
    for (int i = 0; i < ly; ++i) {
        double s = 0.0;
        for (int k = 0; k < lx; ++k) s += (t ? a[k + i * *lda] : a[i + k * *lda]) * x[k * *incx];
        y[i * *incy] = (*beta == 0.0 ? 0.0 : *beta * y[i * *incy]) + *alpha * s;
    }
}
void zgemv_(const char* trans, const int* m, const int* n, const cplx* alpha, const cplx* a, const int* lda,
            const cplx* x, const int* incx, const cplx* beta, cplx* y, const int* incy) {
    const char tc = *trans;
    const bool t = !(tc == 'N' || tc == 'n');
    const int ly = t ? *n : *m, lx = t ? *m : *n;
    for (int i = 0; i < ly; ++i) {
        cplx s = 0.0;
        for (int k = 0; k < lx; ++k) s += opval(a, *lda, i, k, tc) * x[k * *incx];
        y[i * *incy] = (*beta == 0.0 ? cplx(0.0) : *beta * y[i * *incy]) + *alpha * s;
    }
}
void dgemm_(const char* ta, const char* tb, const int* m, const int* n, const int* k, const double* alpha,
            const double* a, const int* lda, const double* b, const int* ldb, const double* beta, double* c,
            const int* ldc) {
    const bool at = !is(ta, 'N'), bt = !is(tb, 'N');
    for (int j = 0; j < *n; ++j)
        for (int i = 0; i < *m; ++i) {
            double s = 0.0;
            for (int l = 0; l < *k; ++l)
                s += (at ? a[l + i * *lda] : a[i + l * *lda]) * (bt ? b[j + l * *ldb] : b[l + j * *ldb]);
            c[i + j * *ldc] = (*beta == 0.0 ? 0.0 : *beta * c[i + j * *ldc]) + *alpha * s;
        }
}
void zgemm_(const char* ta, const char* tb, const int* m, const int* n, const int* k, const cplx* alpha,
            const cplx* a, const int* lda, const cplx* b, const int* ldb, const cplx* beta, cplx* c, const int* ldc) {
    for (int j = 0; j < *n; ++j)
        for (int i = 0; i < *m; ++i) {
            cplx s = 0.0;
            for (int l = 0; l < *k; ++l) s += opval(a, *lda, i, l, *ta) * opval(b, *ldb, l, j, *tb);
            c[i + j * *ldc] = (*beta == 0.0 ? cplx(0.0) : *beta * c[i + j * *ldc]) + *alpha * s;
        }
}
void zgemm3m_(const char* ta, const char* tb, const int* m, const int* n, const int* k, const cplx* alpha,
              const cplx* a, const int* lda, const cplx* b, const int* ldb, const cplx* beta, cplx* c,
              const int* ldc) {
    zgemm_(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
void zhemm_(const char* side, const char* uplo, const int* m, const int* n, const cplx* alpha, const cplx* a,
            const int* lda, const cplx* b, const int* ldb, const cplx* beta, cplx* c, const int* ldc) {
    // A Hermitian, referenced triangle given by uplo
    const bool left = is(side, 'L'), up = is(uplo, 'U');
    const int na = left ? *m : *n;
    std::vector<cplx> full(static_cast<std::size_t>(na) * na);
    for (int j = 0; j < na; ++j)
        for (int i = 0; i < na; ++i) {
            cplx v;
            if (i == j) v = cplx(a[i + j * *lda].real(), 0.0);
            else if ((i < j) == up) v = a[i + j * *lda];
            else v = std::conj(a[j + i * *lda]);
            full[i + j * na] = v;
        }
    for (int j = 0; j < *n; ++j)
        for (int i = 0; i < *m; ++i) {
            cplx s = 0.0;
            if (left) for (int l = 0; l < *m; ++l) s += full[i + l * na] * b[l + j * *ldb];
            else for (int l = 0; l < *n; ++l) s += b[i + l * *ldb] * full[l + j * na];
            c[i + j * *ldc] = (*beta == 0.0 ? cplx(0.0) : *beta * c[i + j * *ldc]) + *alpha * s;
        }
}
// MKL out-of-place matrix add: C = alpha*op(A) + beta*op(B); ordering 'R' (row-major) or 'C'
void mkl_zomatadd(const char* ordering, const char* ta, const char* tb, const int* m, const int* n,
                  const cplx* alpha, const cplx* A, const int* lda, const cplx* beta, const cplx* B, const int* ldb,
                  cplx* C, const int* ldc) {
    const bool row = is(ordering, 'R');
    std::vector<cplx> out(static_cast<std::size_t>(*m) * *n);
    for (int i = 0; i < *m; ++i)
        for (int j = 0; j < *n; ++j) {
            // element (i, j) of op(X) for a matrix stored with leading dimension ld in the given ordering
            auto get = [&](const cplx* X, int ld, char t) -> cplx {
                const bool tr = (t == 'T' || t == 't' || t == 'C' || t == 'c');
                const bool cj = (t == 'C' || t == 'c' || t == 'R' || t == 'r');
                const int r = tr ? j : i, c = tr ? i : j;
                cplx v = row ? X[r * ld + c] : X[r + c * ld];
                return cj ? std::conj(v) : v;
            };
            out[i * *n + j] = *alpha * get(A, *lda, *ta) + *beta * get(B, *ldb, *tb);
        }
    for (int i = 0; i < *m; ++i)
        for (int j = 0; j < *n; ++j) {
            if (row) C[i * *ldc + j] = out[i * *n + j];
            else C[i + j * *ldc] = out[i * *n + j];
        }
}
void mkl_zomatadd_(const char* o, const char* ta, const char* tb, const int* m, const int* n, const cplx* alpha,
                   const cplx* A, const int* lda, const cplx* beta, const cplx* B, const int* ldb, cplx* C,
                   const int* ldc) {
    mkl_zomatadd(o, ta, tb, m, n, alpha, A, lda, beta, B, ldb, C, ldc);
}
void mkl_zomatcopy_(const char* ordering, const char* trans, const int* r, const int* c, const cplx* alpha,
                    const cplx* A, const int* lda, cplx* B, const int* ldb) {
    const bool row = is(ordering, 'R');
    const bool tr = (*trans == 'T' || *trans == 't' || *trans == 'C' || *trans == 'c');
    const bool cj = (*trans == 'C' || *trans == 'c' || *trans == 'R' || *trans == 'r');
    for (int i = 0; i < *r; ++i)
        for (int j = 0; j < *c; ++j) {
            cplx v = row ? A[i * *lda + j] : A[i + j * *lda];
            if (cj) v = std::conj(v);
            v *= *alpha;
            const int oi = tr ? j : i, oj = tr ? i : j;
            if (row) B[oi * *ldb + oj] = v;
            else B[oi + oj * *ldb] = v;
        }
}
void mkl_domatcopy_(const char* ordering, const char* trans, const int* r, const int* c, const double* alpha,
                    const double* A, const int* lda, double* B, const int* ldb) {
    const bool row = is(ordering, 'R');
    const bool tr = !is(trans, 'N');
    for (int i = 0; i < *r; ++i)
        for (int j = 0; j < *c; ++j) {
            double v = (row ? A[i * *lda + j] : A[i + j * *lda]) * *alpha;
            const int oi = tr ? j : i, oj = tr ? i : j;
            if (row) B[oi * *ldb + oj] = v;
            else B[oi + oj * *ldb] = v;
        }
}
// LU with partial pivoting (LAPACK dgetrf semantics, unblocked)
void dgetrf_(const int* m, const int* n, double* a, const int* lda, int* ipiv, int* info) {
    *info = 0;
    const int mn = std::min(*m, *n);
    for (int j = 0; j < mn; ++j) {
        int p = j;
        for (int i = j + 1; i < *m; ++i)
            if (std::abs(a[i + j * *lda]) > std::abs(a[p + j * *lda])) p = i;
        ipiv[j] = p + 1;
        if (a[p + j * *lda] == 0.0) {
            if (*info == 0) *info = j + 1;
            continue;
        }
        if (p != j)
            for (int k = 0; k < *n; ++k) std::swap(a[j + k * *lda], a[p + k * *lda]);
        for (int i = j + 1; i < *m; ++i) a[i + j * *lda] /= a[j + j * *lda];
        for (int k = j + 1; k < *n; ++k)
            for (int i = j + 1; i < *m; ++i) a[i + k * *lda] -= a[i + j * *lda] * a[j + k * *lda];
    }
}
// Inverse from the LU factors (LAPACK dgetri semantics)
void dgetri_(const int* n, double* a, const int* lda, const int* ipiv, double* work, const int* lwork, int* info) {
    *info = 0;
    const int N = *n;
    if (*lwork == -1) {
        work[0] = N;
        return;
    }
    std::vector<double> inv(static_cast<std::size_t>(N) * N, 0.0);
    for (int col = 0; col < N; ++col) {
        std::vector<double> e(N, 0.0);
        e[col] = 1.0;
        // apply the row interchanges of P to e (P A = L U  =>  A^{-1} = U^{-1} L^{-1} P)
        for (int i = 0; i < N; ++i) std::swap(e[i], e[ipiv[i] - 1]);
        for (int i = 0; i < N; ++i)
            for (int k = 0; k < i; ++k) e[i] -= a[i + k * *lda] * e[k];
        for (int i = N - 1; i >= 0; --i) {
            for (int k = i + 1; k < N; ++k) e[i] -= a[i + k * *lda] * e[k];
            if (a[i + i * *lda] == 0.0) {
                *info = i + 1;
                return;
            }
            e[i] /= a[i + i * *lda];
        }
        for (int i = 0; i < N; ++i) inv[i + col * N] = e[i];
    }
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) a[i + j * *lda] = inv[i + j * N];
}
// Symmetric eigen-solver (Jacobi rotations), LAPACK dsyev semantics for jobz 'N'/'V'
void dsyev_(const char* jobz, const char* uplo, const int* n, double* a, const int* lda, double* w, double* work,
            const int* lwork, int* info) {
    const int N = *n;
    *info = 0;
    if (*lwork == -1) {
        work[0] = 3 * N;
        return;
    }
    std::vector<double> A(static_cast<std::size_t>(N) * N), V(static_cast<std::size_t>(N) * N, 0.0);
    const bool up = is(uplo, 'U');
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            const bool stored = up ? (i <= j) : (i >= j);
            A[i + j * N] = stored ? a[i + j * *lda] : a[j + i * *lda];
        }
    for (int i = 0; i < N; ++i) V[i + i * N] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0;
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < j; ++i) off += A[i + j * N] * A[i + j * N];
        if (off < 1e-30) break;
        for (int p = 0; p < N; ++p)
            for (int q = p + 1; q < N; ++q) {
                const double apq = A[p + q * N];
                if (apq == 0.0) continue;
                const double theta = (A[q + q * N] - A[p + p * N]) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::abs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < N; ++k) {
                    const double akp = A[k + p * N], akq = A[k + q * N];
                    A[k + p * N] = c * akp - s * akq;
                    A[k + q * N] = s * akp + c * akq;
                }
                for (int k = 0; k < N; ++k) {
                    const double apk = A[p + k * N], aqk = A[q + k * N];
                    A[p + k * N] = c * apk - s * aqk;
                    A[q + k * N] = s * apk + c * aqk;
                }
                for (int k = 0; k < N; ++k) {
                    const double vkp = V[k + p * N], vkq = V[k + q * N];
                    V[k + p * N] = c * vkp - s * vkq;
                    V[k + q * N] = s * vkp + c * vkq;
                }
            }
    }
    std::vector<int> order(N);
    for (int i = 0; i < N; ++i) order[i] = i;
    for (int i = 0; i < N; ++i)
        for (int j = i + 1; j < N; ++j)
            if (A[order[j] + order[j] * N] < A[order[i] + order[i] * N]) std::swap(order[i], order[j]);
    for (int i = 0; i < N; ++i) w[i] = A[order[i] + order[i] * N];
    if (is(jobz, 'V'))
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) a[i + j * *lda] = V[i + order[j] * N];
}
void zheev_(const char*, const char*, const int*, cplx*, const int*, double*, cplx*, const int*, double*, int* info) {
    throw std::logic_error("zheev_ is not provided by the one-process reference build");
}
void dgesvd_(const char*, const char*, const int*, const int*, double*, const int*, double*, double*, const int*,
             double*, const int*, double*, const int*, int* info) {
    throw std::logic_error("dgesvd_ is not provided by the one-process reference build");
}
}  // extern "C"

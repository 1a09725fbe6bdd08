// Small dense FP64 linear algebra on the host CPU: the projected (Rayleigh-Ritz) and Gram
// eigenproblems and Cholesky factors of the eigensolvers, at most a few hundred on a side.
//
// Why the host: on GB300 the GPU's FP64 rate is about 1.25 TFLOP/s in total, a few GFLOP/s per
// SM, while one Grace core reaches tens of GFLOP/s in FP64.  A 48 x 48 symmetric eigenproblem
// is ~0.5 MFLOP of strictly sequential work; it finishes sooner on one host core than on one SM,
// and the host is where the reference solves these too (src/chebyshev.jl:71-73,123,139 call
// LAPACK `eigen`/`cholesky` on the host).
//
// Algorithms (published methods, written here from their mathematics):
//   symmetric eigenproblem: Householder reduction to tridiagonal form, then the implicit
//   symmetric tridiagonal QR iteration with Wilkinson shifts and Givens bulge chasing, the
//   rotations accumulated into the Householder basis (Golub & Van Loan, Matrix Computations,
//   algorithms 8.3.1-8.3.3).
//   Cholesky: the column-oriented A = U'U recurrence.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

#include "kf_internal.h"

namespace kf {

// Eigenvalues (ascending) w[0..n) and orthonormal eigenvectors V (columns) of the symmetric A
// (column-major, both triangles read as their average).  Returns 0, or -1 without convergence.
int sym_eig(int n, const double *A, int lda, double *w, double *V, int ldv) {
    if (n <= 0) return 0;
    // working copy, symmetrised
    std::vector<double> a((size_t)n * n);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) a[i + (size_t)n * j] = 0.5 * (A[i + (size_t)lda * j] + A[j + (size_t)lda * i]);
    auto at = [&](int i, int j) -> double & { return a[i + (size_t)n * j]; };
    // Householder tridiagonalisation; reflector k acts on rows/cols k+1..n-1
    std::vector<std::vector<double>> refl(n > 2 ? n - 2 : 0);
    std::vector<double> p(n), q(n);
    for (int k = 0; k + 2 < n; ++k) {
        const int m = n - k - 1;
        double nx = 0;
        for (int i = 0; i < m; ++i) nx += at(k + 1 + i, k) * at(k + 1 + i, k);
        nx = std::sqrt(nx);
        std::vector<double> &v = refl[k];
        if (nx == 0) continue;
        const double x0 = at(k + 1, k);
        const double alpha = x0 > 0 ? -nx : nx;
        v.assign(m, 0.0);
        for (int i = 0; i < m; ++i) v[i] = at(k + 1 + i, k);
        v[0] -= alpha;
        double vn = 0;
        for (int i = 0; i < m; ++i) vn += v[i] * v[i];
        vn = std::sqrt(vn);
        if (vn == 0) { v.clear(); continue; }
        for (int i = 0; i < m; ++i) v[i] /= vn;
        // p = A22 v, K = v'p, q = 2 (p - K v), A22 -= v q' + q v'
        double K = 0;
        for (int i = 0; i < m; ++i) {
            // A22 is symmetric: row i read down column i (contiguous)
            const double *col = &a[(size_t)(k + 1) + (size_t)n * (k + 1 + i)];
            double s = 0;
            for (int j = 0; j < m; ++j) s += col[j] * v[j];
            p[i] = s;
            K += v[i] * s;
        }
        for (int i = 0; i < m; ++i) q[i] = 2.0 * (p[i] - K * v[i]);
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < m; ++i) at(k + 1 + i, k + 1 + j) -= v[i] * q[j] + q[i] * v[j];
        at(k + 1, k) = alpha;
        at(k, k + 1) = alpha;
        for (int i = 1; i < m; ++i) {
            at(k + 1 + i, k) = 0;
            at(k, k + 1 + i) = 0;
        }
    }
    std::vector<double> d(n), e(n > 1 ? n - 1 : 1, 0.0);
    for (int i = 0; i < n; ++i) d[i] = at(i, i);
    for (int i = 0; i + 1 < n; ++i) e[i] = at(i + 1, i);
    // Q = H_0 H_1 ... H_{n-3}, built by applying the reflectors right to left to the identity
    std::vector<double> Z((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) Z[i + (size_t)n * i] = 1.0;
    for (int k = n - 3; k >= 0; --k) {
        const std::vector<double> &v = refl[k];
        if (v.empty()) continue;
        const int m = n - k - 1;
        for (int c = 0; c < n; ++c) {
            double s = 0;
            for (int i = 0; i < m; ++i) s += v[i] * Z[(k + 1 + i) + (size_t)n * c];
            s *= 2.0;
            if (s == 0) continue;
            for (int i = 0; i < m; ++i) Z[(k + 1 + i) + (size_t)n * c] -= s * v[i];
        }
    }
    // implicit symmetric tridiagonal QR with Wilkinson shifts
    const double eps = std::numeric_limits<double>::epsilon();
    int hi = n - 1;
    int iters = 0;
    const int maxit = 60 * n + 60;
    while (hi > 0) {
        // deflate negligible off-diagonals
        for (int i = 0; i < hi; ++i)
            if (std::fabs(e[i]) <= eps * (std::fabs(d[i]) + std::fabs(d[i + 1]))) e[i] = 0.0;
        while (hi > 0 && e[hi - 1] == 0.0) --hi;
        if (hi == 0) break;
        int lo = hi - 1;
        while (lo > 0 && e[lo - 1] != 0.0) --lo;
        if (++iters > maxit) return -1;
        // Wilkinson shift from the trailing 2 x 2 of the unreduced block lo..hi
        const double delta = 0.5 * (d[hi - 1] - d[hi]);
        const double eh = e[hi - 1];
        const double sg = delta >= 0 ? 1.0 : -1.0;
        const double mu = d[hi] - eh * eh / (delta + sg * std::hypot(delta, eh));
        double x = d[lo] - mu, z = e[lo];
        for (int k = lo; k < hi; ++k) {
            const double r = std::hypot(x, z);
            const double c = r == 0 ? 1.0 : x / r;
            const double s = r == 0 ? 0.0 : z / r;
            if (k > lo) e[k - 1] = r;
            const double a0 = d[k], b0 = e[k], g0 = d[k + 1];
            d[k] = c * c * a0 + 2 * c * s * b0 + s * s * g0;
            d[k + 1] = s * s * a0 - 2 * c * s * b0 + c * c * g0;
            e[k] = c * s * (g0 - a0) + (c * c - s * s) * b0;
            if (k + 1 < hi) {
                z = s * e[k + 1];
                e[k + 1] = c * e[k + 1];
                x = e[k];
            }
            double *zk = &Z[(size_t)n * k], *zk1 = &Z[(size_t)n * (k + 1)];
            for (int i = 0; i < n; ++i) {
                const double u = zk[i], v = zk1[i];
                zk[i] = c * u + s * v;
                zk1[i] = -s * u + c * v;
            }
        }
    }
    // sort ascending
    std::vector<int> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int i, int j) { return d[i] < d[j]; });
    for (int jj = 0; jj < n; ++jj) {
        const int j = ord[jj];
        w[jj] = d[j];
        for (int i = 0; i < n; ++i) V[i + (size_t)ldv * jj] = Z[i + (size_t)n * j];
    }
    return 0;
}

// A = U'U with U upper triangular, written into A's upper triangle (the strict lower triangle
// is zeroed).  False when a pivot is not positive and finite.
bool cholesky_upper(int n, double *A, int lda) {
    for (int j = 0; j < n; ++j) {
        double s = A[j + (size_t)lda * j];
        for (int k = 0; k < j; ++k) s -= A[k + (size_t)lda * j] * A[k + (size_t)lda * j];
        if (!(s > 0) || !std::isfinite(s)) return false;
        const double ujj = std::sqrt(s);
        A[j + (size_t)lda * j] = ujj;
        for (int i = j + 1; i < n; ++i) {
            double t = A[j + (size_t)lda * i];
            for (int k = 0; k < j; ++k) t -= A[k + (size_t)lda * j] * A[k + (size_t)lda * i];
            A[j + (size_t)lda * i] = t / ujj;
        }
    }
    for (int j = 0; j < n; ++j)
        for (int i = j + 1; i < n; ++i) A[i + (size_t)lda * j] = 0.0;
    return true;
}

// Ui = U^{-1} for upper-triangular U (column by column back substitution).
void tri_upper_inverse(int n, const double *U, int ldu, double *Ui, int ldi) {
    for (int j = 0; j < n; ++j) {
        for (int i = 0; i < n; ++i) Ui[i + (size_t)ldi * j] = 0.0;
        Ui[j + (size_t)ldi * j] = 1.0 / U[j + (size_t)ldu * j];
        for (int i = j - 1; i >= 0; --i) {
            double s = 0;
            for (int k = i + 1; k <= j; ++k) s += U[i + (size_t)ldu * k] * Ui[k + (size_t)ldi * j];
            Ui[i + (size_t)ldi * j] = -s / U[i + (size_t)ldu * i];
        }
    }
}

}  // namespace kf

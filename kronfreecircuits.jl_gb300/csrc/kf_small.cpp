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
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <thread>
#include <vector>

#include "kf_internal.h"

namespace kf {

namespace {

// y += alpha x (n entries); no aliasing between x and y
inline void axpy(int n, double alpha, const double *__restrict__ x, double *__restrict__ y) {
    for (int i = 0; i < n; ++i) y[i] += alpha * x[i];
}

// y -= a x' + b (rank-2 column update): y[i] -= a[i] bj + b[i] aj
inline void rank2_col(int n, const double *__restrict__ a, double bj, const double *__restrict__ b, double aj,
                      double *__restrict__ y) {
    for (int i = 0; i < n; ++i) y[i] -= a[i] * bj + b[i] * aj;
}

// plane rotation of two columns: (x, y) <- (c x + s y, -s x + c y)
inline void rot(int n, double *__restrict__ x, double *__restrict__ y, double c, double s) {
    for (int i = 0; i < n; ++i) {
        const double u = x[i], v = y[i];
        x[i] = c * u + s * v;
        y[i] = c * v - s * u;
    }
}

// dot product with four partial sums (independent FMA chains)
inline double dot(int n, const double *__restrict__ x, const double *__restrict__ y) {
    double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    int i = 0;
    for (; i + 4 <= n; i += 4) {
        s0 += x[i] * y[i];
        s1 += x[i + 1] * y[i + 1];
        s2 += x[i + 2] * y[i + 2];
        s3 += x[i + 3] * y[i + 3];
    }
    for (; i < n; ++i) s0 += x[i] * y[i];
    return (s0 + s1) + (s2 + s3);
}

}  // namespace

// Eigenvalues (ascending) w[0..n) and orthonormal eigenvectors V (columns) of the symmetric A
// (column-major, both triangles read as their average).  Returns 0, or -1 without convergence.
// Every O(n^3) loop is a column axpy, a rank-2 column update or a plane rotation of two columns
// (no reductions in the inner loops, so the compiler vectorises them); the reflectors are
// accumulated right to left in the transposed layout for the same reason.
int sym_eig(int n, const double *A, int lda, double *w, double *V, int ldv) {
    if (n <= 0) return 0;
    const size_t nn = (size_t)n;
    std::vector<double> a(nn * nn);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) a[i + nn * j] = 0.5 * (A[i + (size_t)lda * j] + A[j + (size_t)lda * i]);
    // Householder tridiagonalisation, both triangles kept: reflector k (unit vector in column k of
    // R, rows k+1..n-1) maps column k below the diagonal onto its first entry
    std::vector<double> R(nn * nn, 0.0), p(n), q(n), d(n), e(n > 1 ? n - 1 : 1, 0.0);
    std::vector<char> has(n, 0);
    for (int k = 0; k + 2 < n; ++k) {
        const int m = n - k - 1;
        double *x = &a[(k + 1) + nn * k];
        const double nx = std::sqrt(dot(m, x, x));
        if (nx == 0) continue;
        const double x0 = x[0];
        const double alpha = x0 > 0 ? -nx : nx;
        double *v = &R[(k + 1) + nn * k];
        std::memcpy(v, x, sizeof(double) * m);
        v[0] -= alpha;
        const double vn = std::sqrt(dot(m, v, v));
        if (vn == 0) continue;
        const double iv = 1.0 / vn;
        for (int i = 0; i < m; ++i) v[i] *= iv;
        has[k] = 1;
        // p = A22 v as a sum of columns, K = v'p, q = 2 (p - K v), A22 -= v q' + q v'
        std::fill(p.begin(), p.begin() + m, 0.0);
        for (int j = 0; j < m; ++j) axpy(m, v[j], &a[(k + 1) + nn * (k + 1 + j)], p.data());
        const double K = dot(m, v, p.data());
        for (int i = 0; i < m; ++i) q[i] = 2.0 * (p[i] - K * v[i]);
        for (int j = 0; j < m; ++j) rank2_col(m, v, q[j], q.data(), v[j], &a[(k + 1) + nn * (k + 1 + j)]);
        x[0] = alpha;
        a[k + nn * (k + 1)] = alpha;
        for (int i = 1; i < m; ++i) {
            x[i] = 0;
            a[k + nn * (k + 1 + i)] = 0;
        }
    }
    for (int i = 0; i < n; ++i) d[i] = a[i + nn * i];
    for (int i = 0; i + 1 < n; ++i) e[i] = a[(i + 1) + nn * i];
    // Large problems (the per-axis eigenbases, n >= 128) record the QR rotations and then build the
    // eigenvectors by row blocks on several host threads: a block of rows of Q = H_0 ... H_{n-3}
    // (built left to right, Z <- Z H_k) followed by every recorded rotation depends on no other
    // rows, so the blocks need no synchronisation and every row gets the same arithmetic whatever
    // the thread count.  Small problems (every Rayleigh-Ritz and SVQB step) stay on one thread.
    const bool par = n >= 128;
    std::vector<double> Z;
    if (!par) {
        // Q built right to left on the identity in the transposed layout (Zt = Q'): Q <- H_k Q
        // touches rows k+1.. of Q's columns k+1.., i.e. Zt <- Zt H_k on that block, y = Zt v (a sum
        // of columns) then Zt -= 2 y v'
        std::vector<double> Zt(nn * nn, 0.0), y(n);
        for (int i = 0; i < n; ++i) Zt[i + nn * i] = 1.0;
        for (int k = n - 3; k >= 0; --k) {
            if (!has[k]) continue;
            const int m = n - k - 1;
            const double *v = &R[(k + 1) + nn * k];
            std::fill(y.begin(), y.begin() + m, 0.0);
            for (int i = 0; i < m; ++i) axpy(m, v[i], &Zt[(k + 1) + nn * (k + 1 + i)], y.data());
            for (int i = 0; i < m; ++i) axpy(m, -2.0 * v[i], y.data(), &Zt[(k + 1) + nn * (k + 1 + i)]);
        }
        Z.resize(nn * nn);
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) Z[i + nn * j] = Zt[j + nn * i];
    }
    std::vector<double> rc, rs;   // recorded rotations (large problems)
    std::vector<int> rk;
    // implicit symmetric tridiagonal QR with Wilkinson shifts
    const double eps = std::numeric_limits<double>::epsilon();
    int hi = n - 1;
    int iters = 0;
    const int maxit = 60 * n + 60;
    while (hi > 0) {
        for (int i = 0; i < hi; ++i)
            if (std::fabs(e[i]) <= eps * (std::fabs(d[i]) + std::fabs(d[i + 1]))) e[i] = 0.0;
        while (hi > 0 && e[hi - 1] == 0.0) --hi;
        if (hi == 0) break;
        int lo = hi - 1;
        while (lo > 0 && e[lo - 1] != 0.0) --lo;
        if (++iters > maxit) return -1;
        const double delta = 0.5 * (d[hi - 1] - d[hi]);
        const double eh = e[hi - 1];
        const double sg = delta >= 0 ? 1.0 : -1.0;
        const double mu = d[hi] - eh * eh / (delta + sg * std::hypot(delta, eh));
        double x = d[lo] - mu, z = e[lo];
        for (int k = lo; k < hi; ++k) {
            // sqrt(x^2 + z^2) directly where neither square can overflow or underflow
            const double ax = std::fabs(x), az = std::fabs(z), big = ax > az ? ax : az;
            const double r = (big < 1e150 && big > 1e-150) ? std::sqrt(x * x + z * z) : std::hypot(x, z);
            const double ir = r == 0 ? 0.0 : 1.0 / r;
            const double c = r == 0 ? 1.0 : x * ir;
            const double s = z * ir;
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
            if (par) {
                rc.push_back(c);
                rs.push_back(s);
                rk.push_back(k);
            } else {
                rot(n, &Z[nn * k], &Z[nn * (k + 1)], c, s);
            }
        }
    }
    // the row-block form's storage: 64-byte aligned, column stride padded past a power of two (so
    // that the columns of a block spread over the cache sets and no two threads share a line)
    std::vector<double> Zbuf;
    double *Zp = nullptr;
    const size_t ldz = nn + 8;
    if (par) {
        Zbuf.assign(ldz * nn + 8, 0.0);
        Zp = Zbuf.data() + ((64 - (reinterpret_cast<uintptr_t>(Zbuf.data()) & 63)) & 63) / sizeof(double);
        // rows [r0, r1) of Q, then of Q times the rotations
        auto rows = [&](int r0, int r1) {
            const int rb = r1 - r0;
            if (rb <= 0) return;
            for (int i = r0; i < r1; ++i) Zp[i + ldz * i] = 1.0;
            std::vector<double> y(rb);
            for (int k = 0; k + 2 < n; ++k) {
                if (!has[k]) continue;
                const int m = n - k - 1;
                const double *v = &R[(k + 1) + nn * k];
                std::fill(y.begin(), y.end(), 0.0);
                for (int i = 0; i < m; ++i) axpy(rb, v[i], &Zp[r0 + ldz * (k + 1 + i)], y.data());
                for (int i = 0; i < m; ++i) axpy(rb, -2.0 * v[i], y.data(), &Zp[r0 + ldz * (k + 1 + i)]);
            }
            const size_t nrot = rk.size();
            for (size_t t = 0; t < nrot; ++t) {
                double *zk = &Zp[r0 + ldz * rk[t]];
                rot(rb, zk, zk + ldz, rc[t], rs[t]);
            }
        };
        const unsigned hw = std::thread::hardware_concurrency();
        const int nt = (int)std::max(1u, std::min(8u, hw));
        // row blocks on 8-row (64-byte) boundaries: no two threads write one cache line
        const int per = ((n + nt - 1) / nt + 7) / 8 * 8;
        std::vector<std::thread> pool;
        for (int t = 1; t < nt && t * per < n; ++t) pool.emplace_back(rows, t * per, std::min(n, (t + 1) * per));
        rows(0, std::min(n, per));
        for (auto &th : pool) th.join();
    }
    std::vector<int> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int i, int j) { return d[i] < d[j]; });
    for (int jj = 0; jj < n; ++jj) {
        const int j = ord[jj];
        w[jj] = d[j];
        for (int i = 0; i < n; ++i) V[i + (size_t)ldv * jj] = par ? Zp[i + ldz * j] : Z[i + nn * j];
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

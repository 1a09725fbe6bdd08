// Batched leaf solves: the lowest m eigenpairs of many small single-axis operators (the leaves of a
// parameter sweep, or sibling leaves of a tree) in ONE persistent kernel launch, captured in a CUDA
// graph.  The reference solves them one node at a time (src/materialize.jl:713-731), each through
// the Chebyshev filter on a device (src/chebyshev.jl:310-406) or Dense.
//
// Each CTA takes leaves from an atomic work queue (largest first, for balance) and runs, for its
// leaf, a Chebyshev-filtered subspace iteration on a block of nb = m + 4 columns:
//   filter (three-term recurrence, degree d, on [lambda_cut, lambda_max] with lambda_max the
//   Gershgorin bound), two Cholesky-QR passes, Rayleigh-Ritz, residual norms, locking of the
//   converged prefix; the filter runs in FP32 until the residuals reach the FP32 floor
//   (1e-5 ||H||), then in FP64.  Gram matrices accumulate in FP64; the small Cholesky and the
//   Rayleigh-Ritz eigenproblem (cyclic Jacobi) are FP64, in shared memory.  Acceptance: every
//   returned pair's FP64 residual ||H v - E v|| <= tol.
//
// The block lives in a per-CTA slice of global scratch (L2-resident: nb x N x (3 FP32 + 4 FP64)
// values); every wait is a __syncthreads inside one CTA -- no CTA waits on another, and the
// iteration count is capped, so the kernel always finishes.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <vector>

#include "kf_internal.h"

namespace kf {
namespace {

constexpr int BMAXB = 9;        // bands of a leaf stencil
constexpr int BMAXNB = 32;      // block columns
constexpr int BMAXN = 4096;     // leaf dimension

struct LeafDesc {
    int N, m, nb, nbands;
    int off[BMAXB];
    int64_t data;               // D at data, band weights at data + N (band-major, zero at invalid rows)
    double lmax;                // Gershgorin bound
    int64_t outE, outV;
};

struct BatchParams {
    int count;
    double tol;
    int maxiter;
    int degree;
    int64_t scratch_per_cta;    // doubles
    int *err;                   // the host-mapped error words (KF_CHECK builds record bounds-check sites)
};

// ---- block helpers (all threads of the CTA call them) ---------------------------------------

// Y = alpha H X + beta X + gamma Z on an N x nb block (column stride N); T = float or double
template <typename T>
__device__ void leaf_apply(const LeafDesc &L, const T *D, const T *W, const T *X, T *Y, int nb, T alpha, T beta,
                           const T *Z, T gamma, int *err) {
    const int N = L.N;
    // element e = (column c, row r); one division per thread, then (c, r) advance by the block's
    // stride without dividing (each element's arithmetic is unchanged)
    const int sc = (int)blockDim.x / N, sr = (int)blockDim.x % N;
    int c = (int)threadIdx.x / N, r = (int)threadIdx.x % N;
    for (int e = threadIdx.x; e < N * nb; e += blockDim.x) {
        // KF_CHECK site 201: the incremental decode stays inside the N x nb block
        if (!KF_CHK(c < nb && r >= 0 && r < N, err, 201)) break;
        const T *x = X + (int64_t)c * N;
        T acc = D[r] * x[r];
        for (int b = 0; b < L.nbands; ++b) {
            const int j = r + L.off[b];
            if (j >= 0 && j < N) acc += W[(int64_t)b * N + r] * x[j];
        }
        T v = alpha * acc + beta * x[r];
        if (Z) v += gamma * Z[(int64_t)c * N + r];
        Y[(int64_t)c * N + r] = v;
        c += sc;
        r += sr;
        if (r >= N) {
            r -= N;
            ++c;
        }
    }
    __syncthreads();
}

// G (nb x nb, FP64 shared) = A' B over N rows; each thread owns output pairs
template <typename T>
__device__ void leaf_gram(const T *A, const T *B, int N, int nb, double *G) {
    for (int p = threadIdx.x; p < nb * nb; p += blockDim.x) {
        const int i = p % nb, j = p / nb;
        const T *a = A + (int64_t)i * N, *b = B + (int64_t)j * N;
        double s = 0;
        for (int r = 0; r < N; ++r) s += (double)a[r] * (double)b[r];
        G[p] = s;
    }
    __syncthreads();
}

// Y (N x k) = X (N x kk) C (kk x k, FP64 shared, column-major ldc)
template <typename T>
__device__ void leaf_update(T *Y, const T *X, int N, int kk, int k, const double *C, int ldc, int *err) {
    const int sc = (int)blockDim.x / N, sr = (int)blockDim.x % N;
    int c = (int)threadIdx.x / N, r = (int)threadIdx.x % N;
    for (int e = threadIdx.x; e < N * k; e += blockDim.x) {
        // KF_CHECK site 202: the element inside the N x k block, C's last entry inside its shared array
        if (!KF_CHK(c < k && r >= 0 && r < N && (kk - 1) + ldc * c < BMAXNB * BMAXNB, err, 202)) break;
        double s = 0;
        for (int q = 0; q < kk; ++q) s += (double)X[(int64_t)q * N + r] * C[q + ldc * c];
        Y[(int64_t)c * N + r] = (T)s;
        c += sc;
        r += sr;
        if (r >= N) {
            r -= N;
            ++c;
        }
    }
    __syncthreads();
}

// In shared memory, by thread 0: cyclic Jacobi eigen-decomposition of the symmetric n x n A
// (destroyed), eigenvalues ascending into w, eigenvectors into V (column-major).
__device__ void jacobi_eig(double *A, double *V, double *w, int n) {
    if (threadIdx.x == 0) {
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) V[i + n * j] = (i == j) ? 1.0 : 0.0;
        for (int sweep = 0; sweep < 30; ++sweep) {
            double off = 0, tot = 0;
            for (int j = 0; j < n; ++j)
                for (int i = 0; i < n; ++i) {
                    const double a = A[i + n * j] * A[i + n * j];
                    tot += a;
                    if (i != j) off += a;
                }
            if (off <= 1e-30 * tot || off == 0) break;
            for (int p = 0; p < n - 1; ++p)
                for (int q = p + 1; q < n; ++q) {
                    const double apq = A[p + n * q];
                    if (apq == 0) continue;
                    const double app = A[p + n * p], aqq = A[q + n * q];
                    const double tau = (aqq - app) / (2 * apq);
                    const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1 + tau * tau));
                    const double c = 1 / sqrt(1 + t * t), s = t * c;
                    for (int k = 0; k < n; ++k) {          // columns p, q
                        const double akp = A[k + n * p], akq = A[k + n * q];
                        A[k + n * p] = c * akp - s * akq;
                        A[k + n * q] = s * akp + c * akq;
                    }
                    for (int k = 0; k < n; ++k) {          // rows p, q
                        const double apk = A[p + n * k], aqk = A[q + n * k];
                        A[p + n * k] = c * apk - s * aqk;
                        A[q + n * k] = s * apk + c * aqk;
                    }
                    for (int k = 0; k < n; ++k) {
                        const double vkp = V[k + n * p], vkq = V[k + n * q];
                        V[k + n * p] = c * vkp - s * vkq;
                        V[k + n * q] = s * vkp + c * vkq;
                    }
                }
        }
        for (int i = 0; i < n; ++i) w[i] = A[i + n * i];
        // selection sort ascending with the vectors
        for (int i = 0; i < n; ++i) {
            int k = i;
            for (int j = i + 1; j < n; ++j)
                if (w[j] < w[k]) k = j;
            if (k != i) {
                const double t = w[i]; w[i] = w[k]; w[k] = t;
                for (int r = 0; r < n; ++r) {
                    const double u = V[r + n * i]; V[r + n * i] = V[r + n * k]; V[r + n * k] = u;
                }
            }
        }
    }
    __syncthreads();
}

// Cholesky-QR coefficients: G = U'U, C = U^{-1} (upper), by thread 0; returns false if G is not SPD
__device__ bool chol_inv(const double *G, double *C, double *U, int n, int *flag) {
    if (threadIdx.x == 0) {
        bool ok = true;
        for (int i = 0; i < n * n; ++i) U[i] = 0;
        for (int j = 0; j < n && ok; ++j) {
            double s = G[j + n * j];
            for (int k = 0; k < j; ++k) s -= U[k + n * j] * U[k + n * j];
            if (!(s > 0)) { ok = false; break; }
            const double ujj = sqrt(s);
            U[j + n * j] = ujj;
            for (int i = j + 1; i < n; ++i) {
                double t = G[j + n * i];
                for (int k = 0; k < j; ++k) t -= U[k + n * j] * U[k + n * i];
                U[j + n * i] = t / ujj;
            }
        }
        if (ok) {
            for (int j = 0; j < n; ++j) {
                for (int i = 0; i < n; ++i) C[i + n * j] = 0;
                C[j + n * j] = 1 / U[j + n * j];
                for (int i = j - 1; i >= 0; --i) {
                    double s = 0;
                    for (int k = i + 1; k <= j; ++k) s += U[i + n * k] * C[k + n * j];
                    C[i + n * j] = -s / U[i + n * i];
                }
            }
        }
        *flag = ok ? 1 : 0;
    }
    __syncthreads();
    return *flag != 0;
}

__device__ inline uint64_t bmix(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// ---- the persistent kernel -------------------------------------------------------------------

__global__ void k_batch_chfsi(const LeafDesc *__restrict__ leaves, const int *__restrict__ order, BatchParams P,
                              const double *__restrict__ data64, const float *__restrict__ data32, double *Eout,
                              double *Vout, int *iters_out, double *resid_out, double *scratch, int *counter) {
    __shared__ double G[BMAXNB * BMAXNB], Vs[BMAXNB * BMAXNB], Us[BMAXNB * BMAXNB];
    __shared__ double theta[BMAXNB], res[BMAXNB], wv[BMAXNB];
    __shared__ int s_leaf, s_flag;
    double *base = scratch + (int64_t)blockIdx.x * P.scratch_per_cta;
    while (true) {
        if (threadIdx.x == 0) s_leaf = atomicAdd(counter, 1);
        __syncthreads();
        const int q = s_leaf;
        __syncthreads();
        if (q >= P.count) break;
        const int li = order[q];
        const LeafDesc L = leaves[li];
        const int N = L.N, nb = L.nb, m = L.m;
        const double *D64 = data64 + L.data, *W64 = D64 + N;
        const float *D32 = data32 + L.data, *W32 = D32 + N;
        // scratch: FP64 X, HX, A, B ; FP32 A32, B32, C32 (all N x nb)
        double *X = base, *HX = X + (int64_t)N * nb, *A = HX + (int64_t)N * nb, *B = A + (int64_t)N * nb;
        float *A32 = (float *)(B + (int64_t)N * nb), *B32 = A32 + (int64_t)N * nb, *C32 = B32 + (int64_t)N * nb;
        // KF_CHECK site 203: the leaf's blocks fit this CTA's scratch and its block the shared arrays
        // (the same for every thread: the leaf is skipped as a whole)
        if (!KF_CHK(nb >= 1 && nb <= BMAXNB && N >= 1 &&
                        (int64_t)N * nb * 4 + ((int64_t)N * nb * 3 + 1) / 2 <= P.scratch_per_cta,
                    P.err, 203))
            continue;
        // random start, orthonormalised
        for (int e = threadIdx.x; e < N * nb; e += blockDim.x) {
            const uint64_t h = bmix(bmix(0x4346ull + li) ^ (uint64_t)e);
            X[e] = ((double)(h >> 11) * (1.0 / 9007199254740992.0)) - 0.5;
        }
        __syncthreads();
        const double hn = L.lmax;
        const double floor32 = 1e-5 * fabs(hn);
        // acceptance and locking threshold: max(tol, the roundoff floor 10 eps ||H||), as the
        // reference's Chebyshev filter (src/solvers.jl:75, src/chebyshev.jl:359,401)
        const double thr = fmax(P.tol, 10 * 2.220446049250313e-16 * fabs(hn));
        bool use32 = true;
        int it = 0, nlock = 0;
        bool done = false;
        double lcut = 0;
        for (; it <= P.maxiter && !done; ++it) {
            if (it > 0) {
                // filter the active columns: T_d((H - c)/e) X, FP32 or FP64
                const int na = nb - nlock;
                const double c = (hn + lcut) / 2, e = (hn - lcut) / 2;
                // degree cap: amplify the lowest Ritz value at most 1/sqrt(eps) over the cut
                // (src/chebyshev.jl:169-174), with eps of the filter's precision
                int deg = P.degree;
                {
                    const double x = fabs((theta[0] - c) / e);
                    const double cap = x > 1 ? acosh(use32 ? 2896.3 : 67108864.0) / acosh(x) : 1e9;
                    if (cap < deg) deg = max((int)floor(cap), 1);
                }
                if (use32) {
                    for (int k = threadIdx.x; k < N * na; k += blockDim.x) A32[k] = (float)X[(int64_t)nlock * N + k];
                    __syncthreads();
                    float *a = A32, *b = B32, *cc = C32;
                    leaf_apply<float>(L, D32, W32, a, b, na, (float)(1 / e), (float)(-c / e), nullptr, 0.f, P.err);
                    for (int k = 2; k <= deg; ++k) {
                        leaf_apply<float>(L, D32, W32, b, cc, na, (float)(2 / e), (float)(-2 * c / e), a, -1.f, P.err);
                        float *t = a; a = b; b = cc; cc = t;
                        if (k % 10 == 0) {   // rescale the live pair by the newer member's column norms
                            for (int col = threadIdx.x; col < na; col += blockDim.x) {
                                double s = 0;
                                for (int r = 0; r < N; ++r) s += (double)b[(int64_t)col * N + r] * b[(int64_t)col * N + r];
                                wv[col] = s > 0 ? 1 / sqrt(s) : 1;
                            }
                            __syncthreads();
                            for (int k2 = threadIdx.x; k2 < N * na; k2 += blockDim.x) {
                                a[k2] *= (float)wv[k2 / N];
                                b[k2] *= (float)wv[k2 / N];
                            }
                            __syncthreads();
                        }
                    }
                    for (int k = threadIdx.x; k < N * na; k += blockDim.x) A[k] = (double)b[k];
                    __syncthreads();
                } else {
                    for (int k = threadIdx.x; k < N * na; k += blockDim.x) A[k] = X[(int64_t)nlock * N + k];
                    __syncthreads();
                    // FP64: reuse HX (free until Rayleigh-Ritz) and B as the recurrence buffers
                    double *a = A, *b = B, *cc = HX;
                    leaf_apply<double>(L, D64, W64, a, b, na, 1 / e, -c / e, nullptr, 0.0, P.err);
                    for (int k = 2; k <= deg; ++k) {
                        leaf_apply<double>(L, D64, W64, b, cc, na, 2 / e, -2 * c / e, a, -1.0, P.err);
                        double *t = a; a = b; b = cc; cc = t;
                        if (k % 10 == 0) {
                            for (int col = threadIdx.x; col < na; col += blockDim.x) {
                                double s = 0;
                                for (int r = 0; r < N; ++r) s += b[(int64_t)col * N + r] * b[(int64_t)col * N + r];
                                wv[col] = s > 0 ? 1 / sqrt(s) : 1;
                            }
                            __syncthreads();
                            for (int k2 = threadIdx.x; k2 < N * na; k2 += blockDim.x) {
                                a[k2] *= wv[k2 / N];
                                b[k2] *= wv[k2 / N];
                            }
                            __syncthreads();
                        }
                    }
                    if (b != A)
                        for (int k = threadIdx.x; k < N * na; k += blockDim.x) A[k] = b[k];
                    __syncthreads();
                }
                // project out the locked columns (twice) and put the filtered block back
                for (int pass = 0; pass < 2 && nlock > 0; ++pass) {
                    for (int p = threadIdx.x; p < nlock * na; p += blockDim.x) {
                        const int i = p % nlock, j = p / nlock;
                        double s = 0;
                        for (int r = 0; r < N; ++r) s += X[(int64_t)i * N + r] * A[(int64_t)j * N + r];
                        G[i + BMAXNB * j] = s;
                    }
                    __syncthreads();
                    for (int k = threadIdx.x; k < N * na; k += blockDim.x) {
                        const int j = k / N, r = k % N;
                        double s = 0;
                        for (int i = 0; i < nlock; ++i) s += X[(int64_t)i * N + r] * G[i + BMAXNB * j];
                        A[k] -= s;
                    }
                    __syncthreads();
                }
                for (int k = threadIdx.x; k < N * na; k += blockDim.x) X[(int64_t)nlock * N + k] = A[k];
                __syncthreads();
            }
            // Cholesky-QR twice on the active columns X[:, nlock:]
            const int na = nb - nlock;
            double *Xa = X + (int64_t)nlock * N;
            bool ok = true;
            for (int pass = 0; pass < 2 && ok; ++pass) {
                leaf_gram<double>(Xa, Xa, N, na, G);
                ok = chol_inv(G, Vs, Us, na, &s_flag);
                if (ok) {
                    leaf_update<double>(A, Xa, N, na, na, Vs, na, P.err);
                    for (int k = threadIdx.x; k < N * na; k += blockDim.x) Xa[k] = A[k];
                    __syncthreads();
                }
            }
            if (!ok) break;   // rank-deficient block: reported as not converged
            // Rayleigh-Ritz on the active columns
            leaf_apply<double>(L, D64, W64, Xa, HX, na, 1.0, 0.0, nullptr, 0.0, P.err);
            leaf_gram<double>(Xa, HX, N, na, G);
            if (threadIdx.x == 0)
                for (int j = 0; j < na; ++j)
                    for (int i = 0; i < j; ++i) {
                        const double s = 0.5 * (G[i + na * j] + G[j + na * i]);
                        G[i + na * j] = G[j + na * i] = s;
                    }
            __syncthreads();
            jacobi_eig(G, Vs, wv, na);
            leaf_update<double>(A, Xa, N, na, na, Vs, na, P.err);
            for (int k = threadIdx.x; k < N * na; k += blockDim.x) Xa[k] = A[k];
            __syncthreads();
            if (threadIdx.x < na) theta[nlock + threadIdx.x] = wv[threadIdx.x];
            __syncthreads();
            // residual norms of the active columns (FP64)
            leaf_apply<double>(L, D64, W64, Xa, HX, na, 1.0, 0.0, nullptr, 0.0, P.err);
            for (int col = threadIdx.x; col < na; col += blockDim.x) {
                double s = 0;
                const double th = theta[nlock + col];
                for (int r = 0; r < N; ++r) {
                    const double d = HX[(int64_t)col * N + r] - th * Xa[(int64_t)col * N + r];
                    s += d * d;
                }
                res[nlock + col] = sqrt(s);
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                // lock the converged prefix (after at least one filter); switch FP32 -> FP64 at the floor
                int nl = nlock;
                if (it >= 1)
                    while (nl < nb - 1 && res[nl] <= 0.5 * thr) ++nl;
                double best = 1e300;
                for (int j = nl; j < nb; ++j) best = fmin(best, res[j]);
                s_flag = nl;
                if (best <= floor32) wv[0] = 0.0; else wv[0] = 1.0;
            }
            __syncthreads();
            nlock = s_flag;
            if (use32 && wv[0] == 0.0) use32 = false;
            lcut = theta[nb - 1];
            done = nlock >= m;
            __syncthreads();
        }
        // outputs: the lowest m pairs (already ascending within locking order; sort the locked set)
        if (threadIdx.x == 0) {
            iters_out[li] = it;
            double worst = 0;
            for (int j = 0; j < m; ++j) worst = fmax(worst, res[j]);
            resid_out[li] = done ? worst : -1.0;   // -1: not converged within maxiter
            for (int j = 0; j < m; ++j) Eout[L.outE + j] = theta[j];
        }
        for (int k = threadIdx.x; k < N * m; k += blockDim.x) Vout[L.outV + k] = X[k];
        __syncthreads();
    }
}

// the tuned threads-per-CTA per batch size class
std::mutex g_tune_mu;
std::map<int, int> g_tuned;

int size_class(int count, int maxN) { return (count > 256 ? 2 : count > 32 ? 1 : 0) * 16 + (maxN > 2048 ? 2 : maxN > 512 ? 1 : 0); }

struct Prepared {
    std::vector<LeafDesc> leaves;
    std::vector<double> data;
    std::vector<int> order;
    int maxN = 0, maxnb = 0;
    double total_m = 0;
};

Prepared prepare(const kf_op_desc *descs, int count, const int32_t *m) {
    Prepared P;
    int64_t eoff = 0, voff = 0;
    for (int i = 0; i < count; ++i) {
        const kf_op_desc &d = descs[i];
        KF_REQUIRE(d.ndims == 1, KF_EINVAL, "kf_batch_solve: batched operators must have one axis");
        const int N = (int)d.dims[0];
        KF_REQUIRE(N >= 1 && N <= BMAXN, KF_EINVAL, "kf_batch_solve: operator dimension must lie in 1:4096");
        KF_REQUIRE(m[i] >= 1 && m[i] + 4 <= BMAXNB && m[i] + 4 <= N, KF_EINVAL,
                   "kf_batch_solve: need 1 <= m and m + 4 <= min(32, N)");
        LeafDesc L{};
        L.N = N;
        L.m = m[i];
        L.nb = m[i] + 4;
        L.data = (int64_t)P.data.size();
        std::vector<double> D(N, d.constant);
        if (d.diag)
            for (int r = 0; r < N; ++r) D[r] += d.diag[r];
        std::map<int, std::vector<double>> bands;
        for (int t = 0; t < d.nterms; ++t) {
            const kf_term &T = d.terms[t];
            KF_REQUIRE(T.nfactors <= 1, KF_EINVAL, "kf_batch_solve: one-axis terms only");
            if (T.nfactors == 0) {
                for (int r = 0; r < N; ++r) D[r] += T.coeff;
                continue;
            }
            const kf_factor &f = T.factors[0];
            KF_REQUIRE(f.n == N && f.axis == 0, KF_EDIM, "kf_batch_solve: factor dimension mismatch");
            if (f.kind == KF_DIAG) {
                for (int r = 0; r < N; ++r) D[r] += T.coeff * f.data[r];
            } else if (f.kind == KF_SHIFT) {
                auto &w = bands[(int)(-f.shift)];
                w.resize(N, 0.0);
                for (int r = 0; r < N; ++r)
                    if (r - f.shift >= 0 && r - f.shift < N) w[r] += T.coeff * f.factor;
            } else if (f.kind == KF_BANDED) {
                for (int b = 0; b < f.nbands; ++b) {
                    const int o = (int)f.offsets[b];
                    if (o == 0) {
                        for (int r = 0; r < N; ++r) D[r] += T.coeff * f.data[(size_t)b * N + r];
                        continue;
                    }
                    auto &w = bands[o];
                    w.resize(N, 0.0);
                    for (int r = 0; r < N; ++r)
                        if (r + o >= 0 && r + o < N) w[r] += T.coeff * f.data[(size_t)b * N + r];
                }
            } else {
                throw Error(KF_EINVAL, "kf_batch_solve: dense factors are not supported in batched leaves");
            }
        }
        KF_REQUIRE((int)bands.size() <= BMAXB, KF_EINVAL, "kf_batch_solve: too many bands");
        L.nbands = 0;
        P.data.insert(P.data.end(), D.begin(), D.end());
        double gmax = -INFINITY;
        std::vector<double> rowsum(N, 0.0);
        for (auto &kv : bands) {
            L.off[L.nbands++] = kv.first;
            P.data.insert(P.data.end(), kv.second.begin(), kv.second.end());
            for (int r = 0; r < N; ++r) rowsum[r] += std::fabs(kv.second[r]);
        }
        for (int r = 0; r < N; ++r) gmax = std::max(gmax, D[r] + rowsum[r]);
        L.lmax = gmax;
        L.outE = eoff;
        L.outV = voff;
        eoff += m[i];
        voff += (int64_t)N * m[i];
        P.leaves.push_back(L);
        P.maxN = std::max(P.maxN, N);
        P.maxnb = std::max(P.maxnb, L.nb);
    }
    P.order.resize(count);
    std::iota(P.order.begin(), P.order.end(), 0);
    std::stable_sort(P.order.begin(), P.order.end(), [&](int a, int b) { return P.leaves[a].N > P.leaves[b].N; });
    return P;
}

// One persistent launch over the batch, captured in a CUDA graph; returns the kernel time (ms).
float run_batch(const Prepared &P, double tol, int maxiter, int threads, int degree, double *E_out, double *V_out,
                int32_t *iters_out, double *resid_out) {
    const int count = (int)P.leaves.size();
    int dev = 0, nsm = 0;
    KF_CUDA(cudaGetDevice(&dev));
    KF_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int ctas = std::min(count, nsm * 2);
    const int64_t per = (int64_t)P.maxN * P.maxnb * 6;     // 4 FP64 blocks + 3 FP32 blocks (as 1.5 FP64)
    int64_t sumE = 0, sumV = 0;
    for (auto &L : P.leaves) {
        sumE += L.m;
        sumV += (int64_t)L.N * L.m;
    }
    std::vector<float> d32(P.data.begin(), P.data.end());
    void *dL, *dO, *d64, *df32, *dE, *dV, *dI, *dR, *dS, *dC;
    KF_CUDA(cudaMalloc(&dL, sizeof(LeafDesc) * count));
    KF_CUDA(cudaMalloc(&dO, sizeof(int) * count));
    KF_CUDA(cudaMalloc(&d64, sizeof(double) * P.data.size()));
    KF_CUDA(cudaMalloc(&df32, sizeof(float) * d32.size()));
    KF_CUDA(cudaMalloc(&dE, sizeof(double) * sumE));
    KF_CUDA(cudaMalloc(&dV, sizeof(double) * sumV));
    KF_CUDA(cudaMalloc(&dI, sizeof(int) * count));
    KF_CUDA(cudaMalloc(&dR, sizeof(double) * count));
    KF_CUDA(cudaMalloc(&dS, sizeof(double) * per * ctas));
    KF_CUDA(cudaMalloc(&dC, sizeof(int)));
    cudaStream_t s;
    KF_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    KF_CUDA(cudaMemcpyAsync(dL, P.leaves.data(), sizeof(LeafDesc) * count, cudaMemcpyHostToDevice, s));
    KF_CUDA(cudaMemcpyAsync(dO, P.order.data(), sizeof(int) * count, cudaMemcpyHostToDevice, s));
    KF_CUDA(cudaMemcpyAsync(d64, P.data.data(), sizeof(double) * P.data.size(), cudaMemcpyHostToDevice, s));
    KF_CUDA(cudaMemcpyAsync(df32, d32.data(), sizeof(float) * d32.size(), cudaMemcpyHostToDevice, s));
    BatchParams bp{count, tol, maxiter, degree, per, tc_error_word()};
    // capture: reset the work counter, then the persistent kernel
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    KF_CUDA(cudaStreamSynchronize(s));
    KF_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(dC, 0, sizeof(int), s);
    k_batch_chfsi<<<ctas, threads, 0, s>>>((const LeafDesc *)dL, (const int *)dO, bp, (const double *)d64,
                                           (const float *)df32, (double *)dE, (double *)dV, (int *)dI, (double *)dR,
                                           (double *)dS, (int *)dC);
    KF_CUDA(cudaStreamEndCapture(s, &graph));
    KF_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaEvent_t e0, e1;
    KF_CUDA(cudaEventCreate(&e0));
    KF_CUDA(cudaEventCreate(&e1));
    KF_CUDA(cudaEventRecord(e0, s));
    KF_CUDA(cudaGraphLaunch(exec, s));
    KF_CUDA(cudaEventRecord(e1, s));
    KF_CUDA(cudaStreamSynchronize(s));
    KF_CUDA(cudaGetLastError());
    float ms = 0;
    KF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (E_out) KF_CUDA(cudaMemcpy(E_out, dE, sizeof(double) * sumE, cudaMemcpyDeviceToHost));
    if (V_out) KF_CUDA(cudaMemcpy(V_out, dV, sizeof(double) * sumV, cudaMemcpyDeviceToHost));
    if (iters_out) KF_CUDA(cudaMemcpy(iters_out, dI, sizeof(int) * count, cudaMemcpyDeviceToHost));
    if (resid_out) KF_CUDA(cudaMemcpy(resid_out, dR, sizeof(double) * count, cudaMemcpyDeviceToHost));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    cudaStreamDestroy(s);
    for (void *p : {dL, dO, d64, df32, dE, dV, dI, dR, dS, dC}) cudaFree(p);
    return ms;
}

const int kThreadCandidates[] = {128, 256, 512};

}  // namespace
}  // namespace kf

using namespace kf;

extern "C" {

int kf_batch_solve(const kf_op_desc *descs, int32_t count, const int32_t *m, double tol, int32_t maxiter, int32_t tile,
                   double *E_out, double *V_out, int32_t *iters_out, double *resid_out) {
    try {
        KF_REQUIRE(descs && m && count >= 1, KF_EINVAL, "kf_batch_solve: empty batch");
        KF_REQUIRE(tol > 0 && std::isfinite(tol), KF_EINVAL, "kf_batch_solve: tol must be positive and finite");
        KF_REQUIRE(maxiter >= 1 && maxiter <= 10000, KF_EINVAL, "kf_batch_solve: maxiter must lie in 1:10000");
        KF_REQUIRE(tile == 0 || tile == 128 || tile == 256 || tile == 512, KF_EINVAL,
                   "kf_batch_solve: tile must be 0 (tuned), 128, 256 or 512");
        Prepared P = prepare(descs, count, m);
        int threads = tile;
        if (threads == 0) {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            auto it = g_tuned.find(size_class(count, P.maxN));
            threads = it == g_tuned.end() ? 256 : it->second;
        }
        std::vector<int32_t> iters(count);
        std::vector<double> resid(count);
        run_batch(P, tol, maxiter, threads, 40, E_out, V_out, iters.data(), resid.data());
        if (iters_out) std::memcpy(iters_out, iters.data(), sizeof(int32_t) * count);
        if (resid_out) std::memcpy(resid_out, resid.data(), sizeof(double) * count);
        int bad = 0;
        for (int i = 0; i < count; ++i) {
            const double thr = std::max(tol, 10 * 2.220446049250313e-16 * std::fabs(P.leaves[i].lmax));
            bad += !(resid[i] >= 0 && resid[i] <= thr);
        }
        if (bad) {
            set_last_error("kf_batch_solve: " + std::to_string(bad) + " of " + std::to_string(count) +
                           " operators did not converge within maxiter = " + std::to_string(maxiter));
            return KF_ENOCONV;
        }
        return KF_OK;
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return KF_EINVAL;
    }
}

int kf_batch_autotune(const kf_op_desc *descs, int32_t count, const int32_t *m, double tol, int32_t maxiter,
                      int32_t *best_tile) {
    try {
        KF_REQUIRE(descs && m && count >= 1 && best_tile, KF_EINVAL, "kf_batch_autotune: bad arguments");
        Prepared P = prepare(descs, count, m);
        float best = 1e30f;
        int bt = 256;
        for (int th : kThreadCandidates) {
            const float ms = run_batch(P, tol, maxiter, th, 40, nullptr, nullptr, nullptr, nullptr);
            if (ms < best) {
                best = ms;
                bt = th;
            }
        }
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            g_tuned[size_class(count, P.maxN)] = bt;
        }
        *best_tile = bt;
        return KF_OK;
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return KF_EINVAL;
    }
}

}  // extern "C"

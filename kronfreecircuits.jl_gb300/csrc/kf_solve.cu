// Eigensolver drivers: LOBPCG, Chebyshev-filtered subspace iteration and Lanczos on the GPU.
//
// Reference semantics (KronFreeCircuits.jl):
//   src/lobpcg.jl:217-301      lobpcg_solve: product seed perturbed by sqrt(eps) along a fixed
//                              random direction, guard columns g = min(guard, (N-5)/3 - m),
//                              n_conv_check = m + g, one retry from a random block, acceptance
//                              on the residual norms of the lowest m
//   src/lobpcg.jl:51-135       per-Ritz Jacobi preconditioner R_j / hypot(D - theta_j, eta)
//   src/chebyshev.jl:310-406   Chebyshev-filtered subspace iteration, its locking, guards, degree
//                              cap, SVQB / Cholesky-QR and final true-residual acceptance
//   src/solvers.jl:65-75       true residuals and the roundoff floor
//   src/solvers.jl:85-106      Lanczos
//
// The block LOBPCG iteration (the reference calls the unvendored LOBPCGEigensolver 0.1.4): X
// holds the Ritz vectors (a converged prefix is hard-locked), W the preconditioned residuals of
// the active columns, P the previous update directions.  Per iteration [W P] is orthogonalised
// against all of X and against itself, twice: a classical Gram-Schmidt projection followed by
// SVQB (directions below a relative cutoff dropped); H is applied to that basis, and Rayleigh-Ritz on
// [X_active, W, P] gives the new active Ritz pairs; P is the [W P] part of the update.
//
// Precision (KF_PREC_MIXED): the bulk of the iterations run with FP32 blocks (FP32 applies,
// FP32 Gram products accumulated in FP64 across CTAs, FP64 Rayleigh-Ritz on the host, or with
// KF_DEVICE_RR=1 by FP32 Jacobi on the device, kf_rr.cu, so that an iteration waits once); when
// every active residual is below mixed_switch * ||H|| (or the FP32 residuals stop falling),
// the block is widened to FP64 and the same iteration finishes in FP64 with FP64 residuals,
// the last sweep being the FP64 refinement that the acceptance test measures.
#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <numeric>
#include <random>

#include "kf_internal.h"

namespace kf {

// ------------------------------------------------------------------------------------------
// device / pinned memory helpers
//
// Inside a solve (AllocScope), device work blocks come from the device's default stream-ordered
// memory pool on the solve's stream (cudaMallocAsync / cudaFreeAsync); the pool keeps freed
// memory for the next solve (release threshold raised once per device), so back-to-back solves
// do not pay cudaMalloc / cudaFree (and cudaFree's device-wide synchronisation) for their
// gigabyte-sized workspaces.  Pinned host staging buffers are recycled the same way.

static thread_local cudaStream_t g_alloc_stream = nullptr;
static thread_local bool g_alloc_async = false;

struct AllocScope {
    cudaStream_t prev_s;
    bool prev_a;
    explicit AllocScope(cudaStream_t s) : prev_s(g_alloc_stream), prev_a(g_alloc_async) {
        static std::mutex mu;
        static uint64_t done_mask = 0;
        int dev = 0;
        KF_CUDA(cudaGetDevice(&dev));
        {
            std::lock_guard<std::mutex> lk(mu);
            if (dev < 64 && !(done_mask & (1ull << dev))) {
                cudaMemPool_t pool;
                KF_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
                uint64_t thr = UINT64_MAX;
                KF_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
                done_mask |= 1ull << dev;
            }
        }
        g_alloc_stream = s;
        g_alloc_async = true;
    }
    ~AllocScope() {
        g_alloc_stream = prev_s;
        g_alloc_async = prev_a;
    }
    AllocScope(const AllocScope &) = delete;
    AllocScope &operator=(const AllocScope &) = delete;
};

struct DevMem {
    void *p = nullptr;
    cudaStream_t s = nullptr;
    bool async = false;
    DevMem() = default;
    explicit DevMem(size_t bytes) {
        if (!bytes) return;
        if (g_alloc_async) {
            KF_CUDA(cudaMallocAsync(&p, bytes, g_alloc_stream));
            s = g_alloc_stream;
            async = true;
        } else {
            KF_CUDA(cudaMalloc(&p, bytes));
        }
    }
    ~DevMem() {
        if (!p) return;
        if (async) cudaFreeAsync(p, s);
        else cudaFree(p);
    }
    DevMem(const DevMem &) = delete;
    DevMem &operator=(const DevMem &) = delete;
    template <typename T>
    T *as() const { return (T *)p; }
};

// pinned host blocks, recycled per thread by size
static thread_local std::vector<std::pair<size_t, void *>> g_pinned_free;

struct HostMem {
    void *p = nullptr;
    size_t n = 0;
    explicit HostMem(size_t bytes) : n(bytes ? bytes : 8) {
        for (size_t i = 0; i < g_pinned_free.size(); ++i)
            if (g_pinned_free[i].first == n) {
                p = g_pinned_free[i].second;
                g_pinned_free.erase(g_pinned_free.begin() + (long)i);
                return;
            }
        KF_CUDA(cudaMallocHost(&p, n));
    }
    ~HostMem() {
        if (!p) return;
        if (g_pinned_free.size() < 64) g_pinned_free.emplace_back(n, p);
        else cudaFreeHost(p);
    }
    HostMem(const HostMem &) = delete;
    HostMem &operator=(const HostMem &) = delete;
    template <typename T>
    T *as() const { return (T *)p; }
};

// KF_TRACE=1 in the environment prints one line per LOBPCG iteration to stderr (phase,
// iteration, locked columns, smallest / largest active residual, SVQB rank) -- the per-iteration
// information the reference hands to its solver callbacks (src/tree.jl:55-56).
static bool trace_on() {
    static const bool on = [] {
        const char *e = std::getenv("KF_TRACE");
        return e && e[0] && e[0] != '0';
    }();
    return on;
}

static double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// KF_TRACE: host time spent blocked on the stream (waiting for the GPU) and in the small host
// eigenproblems, per LOBPCG phase
struct TraceTimes {
    double sync = 0, eig = 0;
    int nsync = 0;
};
static thread_local TraceTimes g_tt;

static int timed_sym_eig(int n, const double *A, int lda, double *w, double *V, int ldv) {
    const double t0 = now_s();
    const int r = sym_eig(n, A, lda, w, V, ldv);
    g_tt.eig += now_s() - t0;
    return r;
}

// ------------------------------------------------------------------------------------------
// SVQB coefficients on the host: for the Gram matrix G (k x k) of a block Z, T (k x r) with
// Z T orthonormal, dropping directions whose unit-diagonal Gram eigenvalue is below
// cutoff * the largest (src/chebyshev.jl:68-81).  Returns r.
static int svqb_coeffs(int k, const double *G, double cutoff, std::vector<double> &T) {
    std::vector<double> d(k), Gs((size_t)k * k), w(k), U((size_t)k * k);
    for (int i = 0; i < k; ++i) d[i] = 1.0 / std::sqrt(std::max(G[i + (size_t)k * i], 1e-300));
    for (int j = 0; j < k; ++j)
        for (int i = 0; i < k; ++i) Gs[i + (size_t)k * j] = d[i] * G[i + (size_t)k * j] * d[j];
    if (timed_sym_eig(k, Gs.data(), k, w.data(), U.data(), k) != 0)
        throw Error(KF_EBREAKDOWN, "SVQB: the Gram eigenproblem did not converge");
    const double top = w[k - 1];
    std::vector<int> keep;
    if (top > 0 && std::isfinite(top))
        for (int j = 0; j < k; ++j)
            if (w[j] > cutoff * top) keep.push_back(j);
    const int r = (int)keep.size();
    T.assign((size_t)k * std::max(r, 1), 0.0);
    for (int c = 0; c < r; ++c) {
        const int j = keep[c];
        const double s = 1.0 / std::sqrt(w[j]);
        for (int i = 0; i < k; ++i) T[i + (size_t)k * c] = d[i] * U[i + (size_t)k * j] * s;
    }
    return r;
}

// ------------------------------------------------------------------------------------------
// LOBPCG on one precision

struct LobParams {
    double lock_tol;        // a column locks (and counts as converged) below this residual
    int maxiter;
    int precond;            // KF_PRECOND_*
    double eta;
    int n_conv_check;
    double cutoff;          // SVQB relative cutoff
    bool stall_exit;        // FP32 phase: leave when the residuals stop falling
    int judge_iters;        // warm-start judge: iteration at which ...
    double judge_resid;     // ... a largest residual above this aborts (0 = off)
    int judge_cols = 0;     // ... among the first judge_cols columns (the warm block's m; 0: all checked)
};

struct LobOut {
    int iters = 0;
    int fast_updates = 0;   // refinement: updates that took the FP64-diagonal + FP32-mixing form
    int ortho_fallbacks = 0;  // FP32 iterations whose device second orthogonalisation pass gave way to the host
    int64_t nmv = 0;
    int nlocked = 0;
    bool converged = false;
    bool judged_bad = false;
    std::vector<double> theta, resid;
};

template <typename T>
struct LobWork {
    int64_t N;
    int w;
    DevMem X, HX, Xn, HXn, Z, HZ, Zt, Pn, F1, F2, dG, dC, dpart, dth, dthp, dnorm, dD, dstat, dtheta;
    HostMem hG, hC, hv, hstat;
    size_t part_bytes;
    LobWork(int64_t N_, int w_)
        : N(N_), w(w_),
          X((size_t)N_ * w_ * sizeof(T)), HX((size_t)N_ * w_ * sizeof(T)), Xn((size_t)N_ * w_ * sizeof(T)),
          HXn((size_t)N_ * w_ * sizeof(T)), Z((size_t)N_ * 2 * w_ * sizeof(T)), HZ((size_t)N_ * 2 * w_ * sizeof(T)),
          Zt((size_t)N_ * 2 * w_ * sizeof(T)), Pn((size_t)N_ * w_ * sizeof(T)),
          F1((size_t)N_ * w_ * sizeof(float)), F2((size_t)N_ * w_ * sizeof(float)),
          dG((size_t)9 * w_ * w_ * sizeof(double)), dC((size_t)9 * w_ * w_ * sizeof(double)),
          dpart(gram_partials_size(3 * w_, 3 * w_, N_)), dth(w_ * sizeof(double)), dthp(w_ * sizeof(double)),
          dnorm(2 * w_ * sizeof(double)), dD(0), dstat(16), dtheta(w_ * sizeof(double)),
          hG((size_t)9 * w_ * w_ * sizeof(double)), hC((size_t)9 * w_ * w_ * sizeof(double)),
          hv((size_t)4 * w_ * sizeof(double)), hstat(16), part_bytes(gram_partials_size(3 * w_, 3 * w_, N_)) {}
};

template <typename T>
static void d2h_sync(double *h, const double *d, size_t n, cudaStream_t s) {
    KF_CUDA(cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    const double t0 = now_s();
    KF_CUDA(cudaStreamSynchronize(s));
    g_tt.sync += now_s() - t0;
    ++g_tt.nsync;
    if (const int e = tc_take_error()) throw Error(e, "a tensor-core mode product timed out on the device");
}

static void h2d(double *d, const double *h, size_t n, cudaStream_t s) {
    KF_CUDA(cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, s));
}

// Orthonormalise Zb (N x k, leading dimension N) against X (N x w) and itself, twice; the
// result lands in `out` (N x r, may be Zt or Z).  Returns r.  `tmp` is an N x k scratch.
//
// FP32 blocks take one Gram launch and one update per pass: G = X'Z and S = Z'Z come from one
// pass over [X Z]' Z; the Gram of the projected block (I - XX')Z is S - G'G (X orthonormal), its
// SVQB transform T is computed on the host, and the projection and T are applied together,
// Z_new = Z T - X (G T).  The second pass absorbs what the first lost to cancellation in S - G'G.
// FP64 blocks project with one classical Gram-Schmidt step and then run SVQB, per pass.
template <typename T>
static int ortho_against(kf_op *op, LobWork<T> &W, T *Zb, int k, const T *X, int wx, T *tmp, T *&result,
                         double cutoff, cudaStream_t s, int npass = 2) {
    const int64_t N = W.N;
    double *G = W.dG.template as<double>();
    double *part = W.dpart.template as<double>();
    double *hG = W.hG.template as<double>();
    double *hC = W.hC.template as<double>();
    double *C = W.dC.template as<double>();
    T *cur = Zb, *other = tmp;
    int r = k;
    for (int pass = 0; pass < npass; ++pass) {
        if constexpr (sizeof(T) == 4) {
            if (wx > 0) {
                // [X Z]' Z: rows 0..wx-1 = G = X'Z, rows wx.. = S = Z'Z ((wx + r) x r, column-major)
                gram32_sets((const float *)X, N, wx, (const float *)cur, N, r, (const float *)cur, N, r, nullptr, 0, 0,
                            N, G, part, s);
                const int ld = wx + r;
                d2h_sync<T>(hG, G, (size_t)ld * r, s);
                std::vector<double> Sp((size_t)r * r);
                for (int j = 0; j < r; ++j)
                    for (int i = 0; i < r; ++i) {
                        double v = hG[wx + i + (size_t)ld * j];
                        for (int q = 0; q < wx; ++q) v -= hG[q + (size_t)ld * i] * hG[q + (size_t)ld * j];
                        Sp[i + (size_t)r * j] = v;
                    }
                std::vector<double> Tc;
                const int r2 = svqb_coeffs(r, Sp.data(), cutoff, Tc);
                if (r2 == 0) { result = cur; return 0; }
                // coefficients of [Z X]: T on top, -G T below ((r + wx) x r2)
                const int lc = r + wx;
                for (int j = 0; j < r2; ++j) {
                    for (int i = 0; i < r; ++i) hC[i + (size_t)lc * j] = Tc[i + (size_t)r * j];
                    for (int q = 0; q < wx; ++q) {
                        double v = 0;
                        for (int i = 0; i < r; ++i) v += hG[q + (size_t)ld * i] * Tc[i + (size_t)r * j];
                        hC[r + q + (size_t)lc * j] = -v;
                    }
                }
                h2d(C, hC, (size_t)lc * r2, s);
                update2<T>(other, N, r2, cur, N, r, X, N, wx, C, lc, 1.0, 0.0, N, s);
                std::swap(cur, other);
                r = r2;
                continue;
            }
        }
        if (wx > 0) {
            // one classical Gram-Schmidt projection per pass; with the SVQB between the two passes
            // this is "twice is enough" against X
            gram<T>(X, N, wx, cur, N, r, N, G, part, s);
            update<T>(cur, N, r, X, N, wx, G, wx, -1.0, 1.0, N, s);
        }
        gram<T>(cur, N, r, cur, N, r, N, G, part, s);
        d2h_sync<T>(hG, G, (size_t)r * r, s);
        std::vector<double> Tc;
        const int r2 = svqb_coeffs(r, hG, cutoff, Tc);
        if (r2 == 0) { result = cur; return 0; }
        std::memcpy(hC, Tc.data(), sizeof(double) * (size_t)r * r2);
        h2d(C, hC, (size_t)r * r2, s);
        update<T>(other, N, r2, cur, N, r, C, r, 1.0, 0.0, N, s);
        std::swap(cur, other);
        r = r2;
    }
    result = cur;
    return r;
}

// ---- FP32 search directions with two host waits per iteration instead of four --------------
//
// merged_gram_sync: for Z = [W P] (nz = na + np columns; W for every active column, P for every
// previous one), one Gram [X Z]'Z and, in the same host wait, the active residual norms.
// merged_finish: after the caller's lock decision (`newly` leading active columns lock), the
// directions of the newly locked columns get zero coefficients; SVQB of the projected Gram
// Z'Z - G'G over the kept columns (host), one update to Z1 = (I - XX') Z T; then the second pass on
// the device -- Gram [X Z1]'Z1, Cholesky coefficients (k_chol2_coeffs), one update -- so no host
// wait.  Its failure flag travels with the Rayleigh-Ritz blocks; the caller falls back to the host
// pass from Z1 (left in Zt) when it is set.
// the separable preconditioner on n FP32 columns in place (column j shifted by dth[j])
static void precondition_f32(kf_op *op, LobWork<float> &W, const LobParams &prm, float *Wb, int n, const double *dth,
                             cudaStream_t s) {
    if (prm.precond != KF_PRECOND_SEPARABLE || n <= 0) return;
    const double eta_s = std::max(prm.eta, 1e-3 * std::fabs(op->gershgorin));
    float *outp = sep_apply(op, Wb, W.F1.as<float>(), n, dth, eta_s, s);
    if (outp != Wb) copy_block<float>(outp, W.N, Wb, W.N, n, W.N, s);
}

static void merged_gram_sync(LobWork<float> &W, const float *X, int wx, const float *Zb, int nz, const double *dnorm,
                             int na, double *hnorm, cudaStream_t s) {
    const int64_t N = W.N;
    double *G = W.dG.as<double>();
    gram32_sets(X, N, wx, Zb, N, nz, Zb, N, nz, nullptr, 0, 0, N, G, W.dpart.as<double>(), s);
    if (na > 0) KF_CUDA(cudaMemcpyAsync(hnorm, dnorm, sizeof(double) * na, cudaMemcpyDeviceToHost, s));
    d2h_sync<float>(W.hG.as<double>(), G, (size_t)(wx + nz) * nz, s);
}

// returns k (columns of Q, in W.Z) or 0 when the directions vanished
static int merged_finish(kf_op *op, LobWork<float> &W, const float *X, int wx, float *Zb, int na, int np, int newly,
                         double cutoff, cudaStream_t s, bool host_second = false) {
    const int64_t N = W.N;
    const int nz = na + np, ld = wx + nz;
    const double *hG = W.hG.as<double>();
    std::vector<int> keep;
    for (int c = newly; c < na; ++c) keep.push_back(c);
    for (int c = na + newly; c < nz; ++c) keep.push_back(c);
    const int r0 = (int)keep.size();
    if (r0 == 0) return 0;
    std::vector<double> Sp((size_t)r0 * r0);
    for (int jj = 0; jj < r0; ++jj)
        for (int ii = 0; ii < r0; ++ii) {
            const int i = keep[ii], j = keep[jj];
            double v = hG[wx + i + (size_t)ld * j];
            for (int q = 0; q < wx; ++q) v -= hG[q + (size_t)ld * i] * hG[q + (size_t)ld * j];
            Sp[ii + (size_t)r0 * jj] = v;
        }
    std::vector<double> Tc;
    const int r1 = svqb_coeffs(r0, Sp.data(), cutoff, Tc);
    if (r1 == 0) return 0;
    // coefficients of [Z X]: T (rows of the kept columns, zero elsewhere), then -G T
    const int lc = nz + wx;
    double *hC = W.hC.as<double>();
    std::fill(hC, hC + (size_t)lc * r1, 0.0);
    for (int j = 0; j < r1; ++j) {
        for (int ii = 0; ii < r0; ++ii) hC[keep[ii] + (size_t)lc * j] = Tc[ii + (size_t)r0 * j];
        for (int q = 0; q < wx; ++q) {
            double v = 0;
            for (int ii = 0; ii < r0; ++ii) v += hG[q + (size_t)ld * keep[ii]] * Tc[ii + (size_t)r0 * j];
            hC[nz + q + (size_t)lc * j] = -v;
        }
    }
    double *C = W.dC.as<double>();
    h2d(C, hC, (size_t)lc * r1, s);
    float *Z1 = W.Zt.as<float>();
    update2<float>(Z1, N, r1, Zb, N, nz, X, N, wx, C, lc, 1.0, 0.0, N, s);
    if (r1 > CHOL2_MAX_R || host_second) {
        // wider than the device Cholesky takes (or its previous attempt failed): the second pass on
        // the host, result in W.Z
        float *Q = nullptr;
        const int r2 = ortho_against<float>(op, W, Z1, r1, X, wx, Zb, Q, cutoff, s, 1);
        KF_CUDA(cudaMemsetAsync(W.dstat.as<int>(), 0, sizeof(int), s));
        return r2;
    }
    // second pass on the device
    double *G = W.dG.as<double>();
    gram32_sets(X, N, wx, Z1, N, r1, Z1, N, r1, nullptr, 0, 0, N, G, W.dpart.as<double>(), s);
    chol2_coeffs(G, wx, r1, C, W.dstat.as<int>(), s);
    update2<float>(W.Z.as<float>(), N, r1, Z1, N, r1, X, N, wx, C, r1 + wx, 1.0, 0.0, N, s);
    return r1;
}

// The Rayleigh-Ritz Gram blocks of [X_a Q] against [Y HZ] in one tensor-core launch when it fits
// (rows X_a, Q; columns Y, HZ): the caller unpacks the blocks it needs from the (na + k)^2 result.
static bool rr_gram_merged(LobWork<float> &W, const float *Xa, const float *Q, const float *Y, const float *HZ, int na,
                           int k, cudaStream_t s) {
    if (W.N < GRAM_TC_MIN_ROWS) return false;
    const int64_t N = W.N;
    const GramTcSrc src[4] = {{Xa, N, na}, {Q, N, k}, {Y, N, na}, {HZ, N, k}};
    return gram_tc(src, 4, 0, 2, 2, 4, N, W.dG.as<double>(), W.dpart.as<double>(), W.part_bytes, s);
}

template <typename T>
static LobOut lobpcg_run(kf_op *op, LobWork<T> &Wk, const double *D, const LobParams &prm, cudaStream_t s,
                         std::vector<double> &theta) {
    const int64_t N = Wk.N;
    const int w = Wk.w;
    const bool f32 = sizeof(T) == 4;
    // FP32 blocks: norms and the first Gram of [W P] share one wait, the second orthogonalisation
    // pass runs on the device (merged_gram_sync / merged_finish); FP64 keeps the plain sequence
    constexpr bool merged = sizeof(T) == 4;
    // FP32 blocks with KF_DEVICE_RR=1 (read per solve): the Rayleigh-Ritz eigenproblem on the device
    // (kf_rr.cu) -- the Ritz values live in Wk.dtheta and come back with the next residual norms --
    // except with the fixed Jacobi preconditioner (its shift travels in the theta buffer).  Off by
    // default: on GB300 the one-CTA FP32 Jacobi takes longer than the host round trip it saves
    // (111.9 against 122.8 eigenpairs/s on the three-mode leaf)
    const char *dev_rr_env = std::getenv("KF_DEVICE_RR");
    const bool dev_rr = merged && prm.precond != KF_PRECOND_JACOBI && dev_rr_env && dev_rr_env[0] &&
                        dev_rr_env[0] != '0';
    double *dtheta = Wk.dtheta.template as<double>();
    bool host_second = false;   // the previous device Cholesky failed: host second pass this time
    LobOut out;
    T *X = Wk.X.template as<T>(), *HX = Wk.HX.template as<T>();
    T *Xn = Wk.Xn.template as<T>(), *HXn = Wk.HXn.template as<T>();
    T *Z = Wk.Z.template as<T>(), *HZ = Wk.HZ.template as<T>(), *Zt = Wk.Zt.template as<T>();
    T *Pn = Wk.Pn.template as<T>();
    double *G = Wk.dG.template as<double>(), *C = Wk.dC.template as<double>();
    double *part = Wk.dpart.template as<double>();
    double *hG = Wk.hG.template as<double>(), *hC = Wk.hC.template as<double>();
    double *dth = Wk.dth.template as<double>(), *dthp = Wk.dthp.template as<double>();
    double *dnorm = Wk.dnorm.template as<double>();
    double *hv = Wk.hv.template as<double>();

    // orthonormalise the initial block (in X) and Rayleigh-Ritz on it
    {
        T *res = nullptr;
        const int r = ortho_against<T>(op, Wk, X, w, nullptr, 0, Zt, res, prm.cutoff, s);
        if (r < w) throw Error(KF_EBREAKDOWN, "LOBPCG: the initial block is numerically rank deficient");
        if (res != X) copy_block<T>(res, N, X, N, w, N, s);
        launch_apply(op, f32, X, HX, N, N, w, 1, 0, nullptr, 0, 0, s);
        out.nmv += w;
        gram<T>(X, N, w, HX, N, w, N, G, part, s);
        d2h_sync<T>(hG, G, (size_t)w * w, s);
        theta.assign(w, 0.0);
        std::vector<double> V((size_t)w * w);
        if (sym_eig(w, hG, w, theta.data(), V.data(), w) != 0)
            throw Error(KF_EBREAKDOWN, "LOBPCG: Rayleigh-Ritz eigenproblem did not converge");
        std::memcpy(hC, V.data(), sizeof(double) * w * w);
        h2d(C, hC, (size_t)w * w, s);
        if (dev_rr) {
            std::memcpy(hv + 2 * w, theta.data(), sizeof(double) * w);
            h2d(dtheta, hv + 2 * w, w, s);
        }
        update<T>(Xn, N, w, X, N, w, C, w, 1.0, 0.0, N, s);
        update<T>(HXn, N, w, HX, N, w, C, w, 1.0, 0.0, N, s);
        std::swap(X, Xn);
        std::swap(HX, HXn);
    }
    std::vector<double> res(w, INFINITY);
    int nl = 0, np = 0, na_prev = w;
    const TraceTimes tt0 = g_tt;
    const double tw0 = now_s();
    double best = INFINITY;
    int since_best = 0;
    for (int it = 0;; ++it) {
        const int na = w - nl;
        // residuals of the active columns, preconditioned into Z[:, 0:na]; with the device
        // Rayleigh-Ritz the Ritz values are read where it wrote them
        double *dth_it = dth, *dthp_it = dthp;
        if (dev_rr) {
            dth_it = dthp_it = dtheta + nl;
        } else {
            std::memcpy(hv, theta.data() + nl, sizeof(double) * na);
            h2d(dth, hv, na, s);
            h2d(dthp, hv, na, s);
        }
        if (prm.precond == KF_PRECOND_JACOBI) {
            // fixed Jacobi: sigma = min(D) - 1, passed in thetap[0]
            double dmin = op->h_fulldiag.empty() ? 0.0
                                                 : *std::min_element(op->h_fulldiag.begin(), op->h_fulldiag.end());
            double sig = dmin - 1.0;
            h2d(dthp, &sig, 1, s);
        }
        const int mode = prm.precond == KF_PRECOND_RITZ ? 0 : prm.precond == KF_PRECOND_JACOBI ? 1 : 2;  // separable: 2, then below
        residual_precond<T>(X + (int64_t)nl * N, HX + (int64_t)nl * N, N, na, N, dth_it, dthp_it, D, prm.eta, mode, Z,
                            N, dnorm, part, s);
        if constexpr (merged) {
            // W for every active column (those that lock now get zero weight later), P after it
            precondition_f32(op, Wk, prm, (float *)Z, na, dth_it, s);
            if (np > 0) copy_block<float>((const float *)Pn, N, (float *)Z + (int64_t)na * N, N, np, N, s);
            if (dev_rr) {
                // the Ritz values and the last device Cholesky's status ride on the same wait
                KF_CUDA(cudaMemcpyAsync(hv + 2 * w, dtheta, sizeof(double) * w, cudaMemcpyDeviceToHost, s));
                KF_CUDA(cudaMemcpyAsync(Wk.hstat.template as<int>(), Wk.dstat.template as<int>(), sizeof(int),
                                        cudaMemcpyDeviceToHost, s));
            }
            merged_gram_sync(Wk, (const float *)X, w, (const float *)Z, na + np, dnorm, na, hv + w, s);
            if (dev_rr) {
                std::memcpy(theta.data(), hv + 2 * w, sizeof(double) * w);
                if (it > 0 && *Wk.hstat.template as<int>() != 0) {
                    // the previous iteration's device Cholesky met a nearly dependent direction: that
                    // iteration kept X and dropped P; the host takes the second pass this time
                    ++out.ortho_fallbacks;
                    host_second = true;
                }
            }
        } else {
            d2h_sync<T>(hv + w, dnorm, na, s);
        }
        for (int j = 0; j < na; ++j) res[nl + j] = std::sqrt(hv[w + j]);
        int newly = 0;
        while (nl + newly < w && res[nl + newly] <= prm.lock_tol) ++newly;
        if (newly > 0) {
            // locked columns never change again: keep both buffers' copies in sync
            copy_block<T>(X + (int64_t)nl * N, N, Xn + (int64_t)nl * N, N, newly, N, s);
            copy_block<T>(HX + (int64_t)nl * N, N, HXn + (int64_t)nl * N, N, newly, N, s);
        }
        out.iters = it;
        if (nl + newly >= prm.n_conv_check) {
            nl += newly;
            out.converged = true;
            break;
        }
        // the checked columns (m + guards); buffer columns beyond them do not enter the warm-start check,
        // the stall test or the convergence count
        const int ncc = prm.n_conv_check;
        double worst = 0, bestr = INFINITY;
        for (int j = nl; j < ncc; ++j) {
            worst = std::max(worst, res[j]);
            bestr = std::min(bestr, res[j]);
        }
        if (trace_on())
            std::fprintf(stderr, "kf lobpcg %s it=%d locked=%d(+%d) active_resid=[%.3e, %.3e]\n", sizeof(T) == 4 ? "f32" : "f64",
                         it, nl, newly, bestr, worst);
        if (!std::isfinite(worst)) throw Error(KF_ENOTFINITE, "LOBPCG: the residual block is not finite");
        double judged = worst;
        if (prm.judge_cols > 0) {
            judged = 0;
            for (int j = nl; j < std::min(prm.judge_cols, ncc); ++j) judged = std::max(judged, res[j]);
        }
        if (prm.judge_resid > 0 && it == prm.judge_iters && judged > prm.judge_resid) {
            out.judged_bad = true;
            break;
        }
        if (prm.stall_exit) {
            // FP32 has reached its floor when, for 30 iterations, no column has locked and the
            // geometric mean of the active residuals has not halved (single columns stall for
            // stretches while the block as a whole still converges)
            double lg = 0;
            for (int j = nl; j < ncc; ++j) lg += std::log(std::max(res[j], 1e-300));
            lg /= std::max(ncc - nl, 1);
            if (newly > 0 || lg < best - std::log(2.0)) {
                best = std::min(best, lg);
                since_best = 0;
            } else if (++since_best >= 30) {
                break;
            }
        }
        if (it >= prm.maxiter) break;
        T *Qc = nullptr;
        int k = 0, r1 = 0;
        if constexpr (merged) {
            k = r1 = merged_finish(op, Wk, (const float *)X, w, (float *)Z, na, np, newly, prm.cutoff, s, host_second);
            host_second = false;
            Qc = Z;
            nl += newly;
        } else {
            // W = Z[:, newly : na] (na2 columns), P = previous Pn[:, newly : na] placed right after it
            const int na2 = na - newly;
            T *Wb = Z + (int64_t)newly * N;
            if (prm.precond == KF_PRECOND_SEPARABLE && na2 > 0) {
                // the separable preconditioner always runs in FP32: it only steers the search
                // directions, the FP64 orthogonalisation and Rayleigh-Ritz keep the accuracy
                const double eta_s = std::max(prm.eta, 1e-3 * std::fabs(op->gershgorin));
                float *f1 = Wk.F1.template as<float>(), *f2 = Wk.F2.template as<float>();
                convert<double, float>((const double *)Wb, N, f2, N, na2, N, s);
                float *outp = sep_apply(op, f2, f1, na2, dth + newly, eta_s, s);
                convert<float, double>(outp, N, (double *)Wb, N, na2, N, s);
            }
            int nz = na2;
            if (np > 0) {
                const int np2 = np - newly;
                if (np2 > 0) {
                    copy_block<T>(Pn + (int64_t)newly * N, N, Wb + (int64_t)na2 * N, N, np2, N, s);
                    nz += np2;
                }
            }
            nl += newly;
            // orthonormalise [W P] against X and itself (result in Z or Zt)
            k = ortho_against<T>(op, Wk, Wb, nz, X, w, Zt, Qc, prm.cutoff, s);   // Qc in Zt, or in Z
        }
        if (k == 0) throw Error(KF_EBREAKDOWN, "LOBPCG: the search directions vanished");
        // Rayleigh-Ritz on S = [X_act, Q]: A = S' H S assembled from three Gram blocks
        const int na3 = w - nl;
        T *Xa = X + (int64_t)nl * N, *HXa = HX + (int64_t)nl * N;
        // the device Rayleigh-Ritz takes this iteration when its eigenproblem fits one CTA
        const bool dev_it = dev_rr && na3 + k <= 64;
        bool rr_done_on_device = false;
        auto apply_rr = [&]() {
            launch_apply(op, f32, Qc, HZ, N, N, k, 1, 0, nullptr, 0, 0, s);
            out.nmv += k;
            bool one = false;
            if constexpr (merged)
                one = rr_gram_merged(Wk, (const float *)Xa, (const float *)Qc, (const float *)HXa, (const float *)HZ,
                                     na3, k, s);
            if (!one) {
                double *G2 = G + (size_t)na3 * na3, *G3 = G2 + (size_t)na3 * k;
                gram<T>(Xa, N, na3, HXa, N, na3, N, G, part, s);
                gram<T>(Xa, N, na3, HZ, N, k, N, G2, part, s);
                gram<T>(Qc, N, k, HZ, N, k, N, G3, part, s);
            }
            if (dev_it) {
                // eigenpairs, C and the Ritz values on the device; no host wait
                rr_done_on_device = rr_eig_device(G, na3 + k, !one, na3, k, C, dtheta + nl, Wk.dstat.template as<int>(), s);
                if (rr_done_on_device) return;
            }
            if (merged)
                KF_CUDA(cudaMemcpyAsync(Wk.hstat.template as<int>(), Wk.dstat.template as<int>(), sizeof(int),
                                        cudaMemcpyDeviceToHost, s));
            const int ld = na3 + k;
            d2h_sync<T>(hG, G, one ? (size_t)ld * ld : (size_t)na3 * na3 + (size_t)na3 * k + (size_t)k * k, s);
            if (one) {
                // [X_a Q]'[HX_a HZ] -> X_a' H X_a, X_a' H Z, Q' H Z as three packed blocks
                std::vector<double> g(hG, hG + (size_t)ld * ld);
                double *b1 = hG, *b2 = hG + (size_t)na3 * na3, *b3 = b2 + (size_t)na3 * k;
                for (int j = 0; j < na3; ++j)
                    for (int i = 0; i < na3; ++i) b1[i + (size_t)na3 * j] = g[i + (size_t)ld * j];
                for (int j = 0; j < k; ++j)
                    for (int i = 0; i < na3; ++i) b2[i + (size_t)na3 * j] = g[i + (size_t)ld * (na3 + j)];
                for (int j = 0; j < k; ++j)
                    for (int i = 0; i < k; ++i) b3[i + (size_t)k * j] = g[(na3 + i) + (size_t)ld * (na3 + j)];
            }
        };
        apply_rr();
        if constexpr (merged) {
            if (!rr_done_on_device && *Wk.hstat.template as<int>() != 0) {
                // the device Cholesky met a nearly dependent direction: the host SVQB pass from Z1
                ++out.ortho_fallbacks;
                T *Q2 = nullptr;
                k = ortho_against<T>(op, Wk, Zt, r1, X, w, Z, Q2, prm.cutoff, s, 1);
                if (k == 0) throw Error(KF_EBREAKDOWN, "LOBPCG: the search directions vanished");
                Qc = Q2;
                apply_rr();
            }
        }
        const int ns = na3 + k;
        std::vector<double> A, lam, V;
        if (!rr_done_on_device) {
            A.assign((size_t)ns * ns, 0.0);
            const double *h1 = hG, *h2 = hG + (size_t)na3 * na3, *h3 = h2 + (size_t)na3 * k;
            for (int j = 0; j < na3; ++j)
                for (int i = 0; i < na3; ++i) A[i + (size_t)ns * j] = h1[i + (size_t)na3 * j];
            for (int j = 0; j < k; ++j)
                for (int i = 0; i < na3; ++i) {
                    A[i + (size_t)ns * (na3 + j)] = h2[i + (size_t)na3 * j];
                    A[(na3 + j) + (size_t)ns * i] = h2[i + (size_t)na3 * j];
                }
            for (int j = 0; j < k; ++j)
                for (int i = 0; i < k; ++i) A[(na3 + i) + (size_t)ns * (na3 + j)] = h3[i + (size_t)k * j];
            lam.resize(ns);
            V.resize((size_t)ns * ns);
            if (timed_sym_eig(ns, A.data(), ns, lam.data(), V.data(), ns) != 0)
                throw Error(KF_EBREAKDOWN, "LOBPCG: Rayleigh-Ritz eigenproblem did not converge");
            // C = V[:, 0:na3] (ns x na3), then [0; C_z] beside it: [X_new P_new] = [X_a Q] [C | [0; C_z]]
            std::memcpy(hC, V.data(), sizeof(double) * (size_t)ns * na3);
            for (int j = 0; j < na3; ++j)
                for (int i = 0; i < ns; ++i) hC[(size_t)ns * (na3 + j) + i] = i < na3 ? 0.0 : V[i + (size_t)ns * j];
            h2d(C, hC, (size_t)ns * 2 * na3, s);
            if (dev_rr) {
                // keep the device copy of the Ritz values current for the next iteration's kernels
                std::memcpy(hv + 2 * w + nl, lam.data(), sizeof(double) * na3);
                h2d(dtheta + nl, hv + 2 * w + nl, na3, s);
            }
        }
        // X_act <- Xa Cx + Q Cz ; HX likewise ; P <- Q Cz
        T *Xna = Xn + (int64_t)nl * N, *HXna = HXn + (int64_t)nl * N;
        bool fused = false;
        if constexpr (merged) {
            if (update_tc_prefer(na3 + k, 2 * na3, N, (const float *)Xa, N, (const float *)Qc, N)) {
                update_tc2((float *)Xna, N, na3, (float *)Pn, N, na3, (const float *)Xa, N, na3, (const float *)Qc, N,
                           k, C, ns, 1.0, 0.0, N, s, -1);
                fused = true;
            } else {
                fused = update_pipe((float *)Xna, N, na3, (float *)Pn, N, na3, (const float *)Xa, N, na3,
                                    (const float *)Qc, N, k, C, ns, 1.0, 0.0, N, s);
            }
        }
        if (!fused) update2<T>(Xna, N, na3, Xa, N, na3, Qc, N, k, C, ns, 1.0, 0.0, N, s);
        update2<T>(HXna, N, na3, HXa, N, na3, HZ, N, k, C, ns, 1.0, 0.0, N, s);
        if (!fused) update<T>(Pn, N, na3, Qc, N, k, C + na3, ns, 1.0, 0.0, N, s);
        np = na3;
        std::swap(X, Xn);
        std::swap(HX, HXn);
        if (!rr_done_on_device)
            for (int j = 0; j < na3; ++j) theta[nl + j] = lam[j];
        na_prev = na3;
    }
    (void)na_prev;
    if (trace_on())
        std::fprintf(stderr,
                     "kf lobpcg %s: %d iterations, %.4f s; blocked on the stream %.4f s (%d syncs), host eig %.4f s, "
                     "%d host second passes\n",
                     f32 ? "f32" : "f64", out.iters, now_s() - tw0, g_tt.sync - tt0.sync, g_tt.nsync - tt0.nsync,
                     g_tt.eig - tt0.eig, out.ortho_fallbacks);
    // make sure the final block sits in Wk.X / Wk.HX
    if (X != Wk.X.template as<T>()) {
        copy_block<T>(X, N, Wk.X.template as<T>(), N, w, N, s);
        copy_block<T>(HX, N, Wk.HX.template as<T>(), N, w, N, s);
    }
    KF_CUDA(cudaStreamSynchronize(s));
    out.nlocked = nl;
    out.theta = theta;
    out.resid = res;
    return out;
}

// ------------------------------------------------------------------------------------------
// Mixed-precision refinement: the FP64 phase of precision = mixed.
//
// GB300 runs FP64 arithmetic at about 1/64 of its FP32 rate, so FP64 is kept to what sets the
// final accuracy: the iterate X and HX (FP64), the residual R = HX - X theta and its norms (FP64),
// and the X-part of each update (X C_x, HX C_x).  The search block Z = [W P], its orthogonalisation
// against X (through an FP32 copy of X), H Z, and the Rayleigh-Ritz blocks are FP32.  Every FP32
// rounding then enters the next iterate multiplied by the correction coefficients C_z, which
// shrink with the residual, so the iteration converges to FP64 accuracy (mixed-precision
// iterative refinement):
//   A_xx = X_a' H X_a = theta + X_a' R          (X' X = I in FP64; X_a' R from FP32 blocks)
//   A_xz = X_a' H Z   = theta X_a' Z + R' Z  ~  R' Z
// Dropping theta X_a' Z (FP32-small, since Z is orthogonalised against X) is the exact
// Rayleigh-Ritz for the basis [X_a, Z - X_a (X_a' Z)], whose X-part differs from the update
// actually formed by X_a (X_a' Z) C_z -- again proportional to C_z.
// Locking, guards, the convergence count and the final FP64 acceptance are those of the FP64
// phase (src/lobpcg.jl:217-301).
struct RefineWork {
    int64_t N;
    int w;
    DevMem X, HX, Xn, HXn, R32, T32, HX32, dd;
    RefineWork(int64_t N_, int w_)
        : N(N_), w(w_), X((size_t)N_ * w_ * sizeof(double)), HX((size_t)N_ * w_ * sizeof(double)),
          Xn((size_t)N_ * w_ * sizeof(double)), HXn((size_t)N_ * w_ * sizeof(double)),
          R32((size_t)N_ * w_ * sizeof(float)), T32((size_t)N_ * w_ * sizeof(float)),
          HX32((size_t)N_ * w_ * sizeof(float)), dd((size_t)w_ * sizeof(double)) {}
};

// Y = X C for FP64 blocks (C w x w): the double-float kernel on the FP32 pipes where it takes the
// shape (about 2^-46 relative, twice as fast as the FP64 pipe on GB300), else the FP64 kernel
static void update64_square(double *Y, const double *X, const double *C, int w, int64_t N, cudaStream_t s) {
    if (!update_f64_df(Y, N, w, X, N, w, C, w, N, s)) update<double>(Y, N, w, X, N, w, C, w, 1.0, 0.0, N, s);
}

// X64 (in R.X) on entry: orthonormalise it in FP64, H X64 with a fresh FP64 apply, Rayleigh-Ritz
// in FP64; leaves X, HX, theta and the FP32 copy W32.X consistent.
static void refine_start(kf_op *op, RefineWork &R, LobWork<float> &W32, double cutoff, cudaStream_t s,
                         std::vector<double> &theta, int64_t &nmv) {
    const int64_t N = R.N;
    const int w = R.w;
    double *X = R.X.as<double>(), *HX = R.HX.as<double>(), *Xn = R.Xn.as<double>(), *HXn = R.HXn.as<double>();
    double *G = W32.dG.as<double>(), *C = W32.dC.as<double>(), *part = W32.dpart.as<double>();
    double *hG = W32.hG.as<double>(), *hC = W32.hC.as<double>();
    gram<double>(X, N, w, X, N, w, N, G, part, s);
    d2h_sync<double>(hG, G, (size_t)w * w, s);
    std::vector<double> Tc;
    const int r = svqb_coeffs(w, hG, cutoff, Tc);
    if (r < w) throw Error(KF_EBREAKDOWN, "LOBPCG: the refinement block is numerically rank deficient");
    std::memcpy(hC, Tc.data(), sizeof(double) * (size_t)w * w);
    h2d(C, hC, (size_t)w * w, s);
    update64_square(Xn, X, C, w, N, s);
    launch_apply(op, false, Xn, HXn, N, N, w, 1, 0, nullptr, 0, 0, s);
    nmv += w;
    gram<double>(Xn, N, w, HXn, N, w, N, G, part, s);
    d2h_sync<double>(hG, G, (size_t)w * w, s);
    theta.assign(w, 0.0);
    std::vector<double> V((size_t)w * w);
    if (sym_eig(w, hG, w, theta.data(), V.data(), w) != 0)
        throw Error(KF_EBREAKDOWN, "LOBPCG: Rayleigh-Ritz eigenproblem did not converge");
    std::memcpy(hC, V.data(), sizeof(double) * w * w);
    h2d(C, hC, (size_t)w * w, s);
    update64_square(X, Xn, C, w, N, s);
    update64_square(HX, HXn, C, w, N, s);
    convert<double, float>(X, N, W32.X.as<float>(), N, w, N, s);
    convert<double, float>(HX, N, R.HX32.as<float>(), N, w, N, s);
}

static LobOut lobpcg_refine(kf_op *op, RefineWork &Rw, LobWork<float> &Wk, const double *D, const LobParams &prm,
                            cudaStream_t s, std::vector<double> &theta) {
    const int64_t N = Wk.N;
    const int w = Wk.w;
    LobOut out;
    const double ts0 = now_s();
    refine_start(op, Rw, Wk, 1e-12, s, theta, out.nmv);
    if (trace_on()) {
        KF_CUDA(cudaStreamSynchronize(s));
        std::fprintf(stderr, "kf lobpcg refine start (FP64 SVQB, apply, Rayleigh-Ritz) %.4f s\n", now_s() - ts0);
    }
    double *X = Rw.X.as<double>(), *HX = Rw.HX.as<double>();
    double *Xn = Rw.Xn.as<double>(), *HXn = Rw.HXn.as<double>();
    float *X32 = Wk.X.as<float>();
    float *R32 = Rw.R32.as<float>(), *T32 = Rw.T32.as<float>();
    float *Z = Wk.Z.as<float>(), *HZ = Wk.HZ.as<float>(), *Zt = Wk.Zt.as<float>(), *Pn = Wk.Pn.as<float>();
    double *G = Wk.dG.as<double>(), *C = Wk.dC.as<double>();
    double *part = Wk.dpart.as<double>();
    double *hG = Wk.hG.as<double>(), *hC = Wk.hC.as<double>();
    double *dth = Wk.dth.as<double>(), *dthp = Wk.dthp.as<double>();
    double *dnorm = Wk.dnorm.as<double>();
    double *hv = Wk.hv.as<double>();

    std::vector<double> res(w, INFINITY);
    int nl = 0, np = 0;
    const TraceTimes tt0 = g_tt;
    const double tw0 = now_s();
    for (int it = 0;; ++it) {
        const int na = w - nl;
        std::memcpy(hv, theta.data() + nl, sizeof(double) * na);
        h2d(dth, hv, na, s);
        h2d(dthp, hv, na, s);
        if (prm.precond == KF_PRECOND_JACOBI) {
            double dmin = op->h_fulldiag.empty() ? 0.0
                                                 : *std::min_element(op->h_fulldiag.begin(), op->h_fulldiag.end());
            double sig = dmin - 1.0;
            h2d(dthp, &sig, 1, s);
        }
        const int mode = prm.precond == KF_PRECOND_RITZ ? 0 : prm.precond == KF_PRECOND_JACOBI ? 1 : 2;
        residual_mixed(X + (int64_t)nl * N, HX + (int64_t)nl * N, N, na, N, dth, dthp, D, prm.eta, mode, R32, N, Z, N,
                       dnorm, part, s);
        // W for every active column, P after it: one wait for the norms and the first Gram
        precondition_f32(op, Wk, prm, Z, na, dth, s);
        if (np > 0) copy_block<float>(Pn, N, Z + (int64_t)na * N, N, np, N, s);
        merged_gram_sync(Wk, X32, w, Z, na + np, dnorm, na, hv + w, s);
        for (int j = 0; j < na; ++j) res[nl + j] = std::sqrt(hv[w + j]);
        int newly = 0;
        while (nl + newly < w && res[nl + newly] <= prm.lock_tol) ++newly;
        if (newly > 0) {
            copy_block<double>(X + (int64_t)nl * N, N, Xn + (int64_t)nl * N, N, newly, N, s);
            copy_block<double>(HX + (int64_t)nl * N, N, HXn + (int64_t)nl * N, N, newly, N, s);
        }
        out.iters = it;
        if (nl + newly >= prm.n_conv_check) {
            nl += newly;
            out.converged = true;
            break;
        }
        // the checked columns (m + guards); buffer columns beyond them do not enter the warm-start check,
        // the stall test or the convergence count
        const int ncc = prm.n_conv_check;
        double worst = 0, bestr = INFINITY;
        for (int j = nl; j < ncc; ++j) {
            worst = std::max(worst, res[j]);
            bestr = std::min(bestr, res[j]);
        }
        if (trace_on())
            std::fprintf(stderr, "kf lobpcg refine it=%d locked=%d(+%d) active_resid=[%.3e, %.3e]\n", it, nl, newly,
                         bestr, worst);
        if (!std::isfinite(worst)) throw Error(KF_ENOTFINITE, "LOBPCG: the residual block is not finite");
        if (it >= prm.maxiter) break;
        nl += newly;
        // the FP32 blocks' Gram eigenvalues below 1e-6 of the largest are rounding noise
        int k = merged_finish(op, Wk, X32, w, Z, na, np, newly, 1e-6, s);
        const int r1 = k;
        if (k == 0) throw Error(KF_EBREAKDOWN, "LOBPCG: the search directions vanished");
        float *Q = Z;
        // Rayleigh-Ritz on [X_a, Q]: X_a' R, R' Q and Q' H Q, one transfer
        const int na3 = w - nl;
        const float *Ra = R32 + (int64_t)newly * N;
        const float *Xa32 = X32 + (int64_t)nl * N;
        auto apply_rr = [&]() {
            launch_apply(op, true, Q, HZ, N, N, k, 1, 0, nullptr, 0, 0, s);
            out.nmv += k;
            // one tensor-core Gram [X_a Q]'[R HZ] holds X_a' R, (R' Q)' and Q' H Z
            const bool one = rr_gram_merged(Wk, Xa32, Q, Ra, HZ, na3, k, s);
            if (!one) {
                double *G2 = G + (size_t)na3 * na3, *G3 = G2 + (size_t)na3 * k;
                gram<float>(Xa32, N, na3, Ra, N, na3, N, G, part, s);
                gram<float>(Ra, N, na3, Q, N, k, N, G2, part, s);
                gram<float>(Q, N, k, HZ, N, k, N, G3, part, s);
            }
            KF_CUDA(cudaMemcpyAsync(Wk.hstat.as<int>(), Wk.dstat.as<int>(), sizeof(int), cudaMemcpyDeviceToHost, s));
            const int ld = na3 + k;
            d2h_sync<double>(hG, G, one ? (size_t)ld * ld : (size_t)na3 * na3 + (size_t)na3 * k + (size_t)k * k, s);
            if (one) {
                std::vector<double> g(hG, hG + (size_t)ld * ld);
                double *b1 = hG, *b2 = hG + (size_t)na3 * na3, *b3 = b2 + (size_t)na3 * k;
                for (int j = 0; j < na3; ++j)
                    for (int i = 0; i < na3; ++i) b1[i + (size_t)na3 * j] = g[i + (size_t)ld * j];
                for (int j = 0; j < k; ++j)   // R' Q = (Q' R)'
                    for (int i = 0; i < na3; ++i) b2[i + (size_t)na3 * j] = g[(na3 + j) + (size_t)ld * i];
                for (int j = 0; j < k; ++j)
                    for (int i = 0; i < k; ++i) b3[i + (size_t)k * j] = g[(na3 + i) + (size_t)ld * (na3 + j)];
            }
        };
        apply_rr();
        if (*Wk.hstat.as<int>() != 0) {
            // the device Cholesky met a nearly dependent direction: the host SVQB pass from Z1
            ++out.ortho_fallbacks;
            k = ortho_against<float>(op, Wk, Zt, r1, X32, w, Z, Q, 1e-6, s, 1);
            if (k == 0) throw Error(KF_EBREAKDOWN, "LOBPCG: the search directions vanished");
            apply_rr();
        }
        const int ns = na3 + k;
        const double *h1 = hG, *h2 = hG + (size_t)na3 * na3, *h3 = h2 + (size_t)na3 * k;
        std::vector<double> A((size_t)ns * ns);
        for (int j = 0; j < na3; ++j)
            for (int i = 0; i < na3; ++i)
                A[i + (size_t)ns * j] = 0.5 * (h1[i + (size_t)na3 * j] + h1[j + (size_t)na3 * i]) +
                                        (i == j ? theta[nl + i] : 0.0);
        for (int j = 0; j < k; ++j)
            for (int i = 0; i < na3; ++i) {
                A[i + (size_t)ns * (na3 + j)] = h2[i + (size_t)na3 * j];
                A[(na3 + j) + (size_t)ns * i] = h2[i + (size_t)na3 * j];
            }
        for (int j = 0; j < k; ++j)
            for (int i = 0; i < k; ++i)
                A[(na3 + i) + (size_t)ns * (na3 + j)] = 0.5 * (h3[i + (size_t)k * j] + h3[j + (size_t)k * i]);
        std::vector<double> lam(ns), V((size_t)ns * ns);
        if (timed_sym_eig(ns, A.data(), ns, lam.data(), V.data(), ns) != 0)
            throw Error(KF_EBREAKDOWN, "LOBPCG: Rayleigh-Ritz eigenproblem did not converge");
        // Ritz vectors' signs are free: make diag(C_x) non-negative
        for (int j = 0; j < na3; ++j)
            if (V[j + (size_t)ns * j] < 0)
                for (int i = 0; i < ns; ++i) V[i + (size_t)ns * j] = -V[i + (size_t)ns * j];
        // X and HX are both updated, so the FP32 roundings of X_a E and HX_a E (E = C_x - D) do not
        // cancel in R = HX - X theta: they move the tracked residual by ~ eps32 |theta| max|E|.
        // The FP32 form is taken only while max|E| <= 1e-4 (a drift below ~1e-11 |theta|).
        bool near_identity = true;
        for (int j = 0; j < na3; ++j)
            for (int i = 0; i < na3; ++i)
                if (i != j && std::fabs(V[i + (size_t)ns * j]) > 1e-4) near_identity = false;
        if (near_identity) ++out.fast_updates;
        double *Xa = X + (int64_t)nl * N, *HXa = HX + (int64_t)nl * N;
        double *Xna = Xn + (int64_t)nl * N, *HXna = HXn + (int64_t)nl * N;
        float *X32a = X32 + (int64_t)nl * N, *HX32a = Rw.HX32.as<float>() + (int64_t)nl * N;
        if (near_identity) {
            // X_a C_x = X_a D + X_a (C_x - D), D = diag(C_x): the scaling in FP64, the rest in FP32
            // with Q C_z -- its rounding is proportional to the mixing C_x - D, which is small
            // unless two Ritz values are close (then their mixing moves the residual little)
            double *dg = hv + 2 * w;   // pinned staging, rewritten only after later synchronisations
            for (int j = 0; j < na3; ++j) {
                dg[j] = V[j + (size_t)ns * j];
                V[j + (size_t)ns * j] = 0.0;
            }
            std::memcpy(hC, V.data(), sizeof(double) * (size_t)ns * na3);
            h2d(C, hC, (size_t)ns * na3, s);
            h2d(Rw.dd.as<double>(), dg, na3, s);
            update2<float>(T32, N, na3, X32a, N, na3, Q, N, k, C, ns, 1.0, 0.0, N, s);
            scale_add(Xna, Xa, Rw.dd.as<double>(), T32, X32a, na3, N, s);
            update2<float>(T32, N, na3, HX32a, N, na3, HZ, N, k, C, ns, 1.0, 0.0, N, s);
            scale_add(HXna, HXa, Rw.dd.as<double>(), T32, HX32a, na3, N, s);
            update<float>(Pn, N, na3, Q, N, k, C + na3, ns, 1.0, 0.0, N, s);
        } else {
            // a large rotation inside X (Ritz values reordered): X_a C_x at FP64 accuracy, in
            // double-float arithmetic where it applies
            std::memcpy(hC, V.data(), sizeof(double) * (size_t)ns * na3);
            h2d(C, hC, (size_t)ns * na3, s);
            if (!update_f64_df(Xna, N, na3, Xa, N, na3, C, ns, N, s))
                update<double>(Xna, N, na3, Xa, N, na3, C, ns, 1.0, 0.0, N, s);
            update<float>(Pn, N, na3, Q, N, k, C + na3, ns, 1.0, 0.0, N, s);
            add_f32_into_f64(Xna, N, Pn, N, X32a, N, na3, N, s);
            if (!update_f64_df(HXna, N, na3, HXa, N, na3, C, ns, N, s))
                update<double>(HXna, N, na3, HXa, N, na3, C, ns, 1.0, 0.0, N, s);
            update<float>(T32, N, na3, HZ, N, k, C + na3, ns, 1.0, 0.0, N, s);
            add_f32_into_f64(HXna, N, T32, N, HX32a, N, na3, N, s);
        }
        np = na3;
        std::swap(X, Xn);
        std::swap(HX, HXn);
        for (int j = 0; j < na3; ++j) theta[nl + j] = lam[j];
    }
    if (trace_on())
        std::fprintf(stderr,
                     "kf lobpcg refine: %d iterations (%d FP32-mixing updates), %.4f s; blocked on the stream %.4f s "
                     "(%d syncs), host eig %.4f s, %d host second passes\n",
                     out.iters, out.fast_updates, now_s() - tw0, g_tt.sync - tt0.sync, g_tt.nsync - tt0.nsync,
                     g_tt.eig - tt0.eig, out.ortho_fallbacks);
    if (X != Rw.X.as<double>()) {
        copy_block<double>(X, N, Rw.X.as<double>(), N, w, N, s);
        copy_block<double>(HX, N, Rw.HX.as<double>(), N, w, N, s);
    }
    KF_CUDA(cudaStreamSynchronize(s));
    out.nlocked = nl;
    out.theta = theta;
    out.resid = res;
    return out;
}

// ------------------------------------------------------------------------------------------
// final FP64 acceptance: sort, true residuals with a fresh apply (src/solvers.jl:65-69)

static void accept_and_copy(kf_op *op, const double *Xd, int w, const std::vector<double> &theta, int m,
                            double *E_out, double *V_out, std::vector<double> &resid_out, cudaStream_t s) {
    const int64_t N = op->N;
    std::vector<int> ord(w);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return theta[a] < theta[b]; });
    DevMem V((size_t)N * m * sizeof(double)), HV((size_t)N * m * sizeof(double)), dth(m * sizeof(double)),
        dn(m * sizeof(double)), part(gram_partials_size(1, 1, N));
    std::vector<double> th(m);
    for (int j = 0; j < m; ++j) {
        th[j] = theta[ord[j]];
        KF_CUDA(cudaMemcpyAsync(V.as<double>() + (int64_t)j * N, Xd + (int64_t)ord[j] * N, N * sizeof(double),
                                cudaMemcpyDeviceToDevice, s));
    }
    launch_apply(op, false, V.as<double>(), HV.as<double>(), N, N, m, 1, 0, nullptr, 0, 0, s);
    KF_CUDA(cudaMemcpyAsync(dth.p, th.data(), m * sizeof(double), cudaMemcpyHostToDevice, s));
    residual_block<double>(V.as<double>(), HV.as<double>(), N, m, N, dth.as<double>(), HV.as<double>(), N, s);
    colnorms2<double>(HV.as<double>(), N, m, N, dn.as<double>(), part.as<double>(), s);
    std::vector<double> r2(m);
    KF_CUDA(cudaMemcpyAsync(r2.data(), dn.p, m * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (V_out) KF_CUDA(cudaMemcpyAsync(V_out, V.p, (size_t)N * m * sizeof(double), cudaMemcpyDeviceToHost, s));
    KF_CUDA(cudaStreamSynchronize(s));
    resid_out.resize(m);
    for (int j = 0; j < m; ++j) {
        resid_out[j] = std::sqrt(r2[j]);
        if (E_out) E_out[j] = th[j];
    }
}

// ------------------------------------------------------------------------------------------
// LOBPCG solve (src/lobpcg.jl:217-301)

static void solve_lobpcg(kf_op *op, const kf_solver_opts &o, int m, const double *X0, const double *seed,
                         double *E_out, double *V_out, kf_solve_stats &st) {
    const int64_t N = op->N;
    cudaStream_t s = op->stream;
    KF_REQUIRE(m >= 1, KF_EINVAL, "LOBPCG requires m >= 1, got " + std::to_string(m));
    KF_REQUIRE(N >= 3 * (int64_t)m + 5, KF_EINVAL,
               "LOBPCG needs N ≥ 3m + 5, got N = " + std::to_string(N) + " for m = " + std::to_string(m) +
                   "; the block eigensolver is unreliable on so small a problem, use Dense()");
    KF_REQUIRE(o.tol > 0 && std::isfinite(o.tol), KF_EINVAL, "LOBPCG: tol must be positive and finite");
    KF_REQUIRE(o.maxiter >= 1, KF_EINVAL, "LOBPCG: maxiter must be at least 1");
    KF_REQUIRE(o.eta > 0 && std::isfinite(o.eta), KF_EINVAL, "eta must be positive and finite");
    KF_REQUIRE(o.preconditioner >= KF_PRECOND_RITZ && o.preconditioner <= KF_PRECOND_SEPARABLE, KF_EINVAL,
               "LOBPCG: preconditioner must be :ritz, :jacobi, :none or :separable");
    KF_REQUIRE(o.precision == KF_PREC_F64 || o.precision == KF_PREC_MIXED, KF_EINVAL, "LOBPCG: unknown precision mode");
    KF_REQUIRE(o.guard >= 0, KF_EINVAL, "LOBPCG: guard must be nonnegative");
    KF_REQUIRE(o.buffer >= KF_BUFFER_AUTO, KF_EINVAL, "LOBPCG: buffer must be nonnegative (or KF_BUFFER_AUTO)");
    if (X0) {
        for (int j = 0; j < m; ++j) {
            bool nz = false;
            for (int64_t i = 0; i < N; ++i) {
                const double v = X0[i + N * j];
                KF_REQUIRE(std::isfinite(v), KF_EINVAL, "LOBPCG: X0 has non-finite entries");
                nz = nz || v != 0.0;
            }
            KF_REQUIRE(nz, KF_EINVAL, "LOBPCG: column " + std::to_string(j + 1) + " of X0 is zero");
        }
    }
    const int g = (int)std::min<int64_t>(o.guard, (N - 5) / 3 - m);
    const int w = m + g;
    // buffer columns: carried in the block (the iteration runs on wi columns) but never checked,
    // locked for the count or returned; the same N >= 3 wi + 5 bound as the guards
    const int b_req = o.buffer == KF_BUFFER_AUTO ? (o.precision == KF_PREC_MIXED ? 2 : 0) : o.buffer;
    const int b = (int)std::max<int64_t>(0, std::min<int64_t>(b_req, (N - 5) / 3 - w));
    const int wi = w + b;
    const double hn = op->gershgorin;
    st.hnorm = hn;
    DevMem dD((size_t)N * sizeof(double));
    KF_CUDA(cudaMemcpyAsync(dD.p, op->h_fulldiag.data(), N * sizeof(double), cudaMemcpyHostToDevice, s));
    LobWork<double> W64(N, wi);
    // the initial block, built on the device (src/lobpcg.jl:179-190): the warm start's / the
    // product seed's columns with the sqrt(eps) perturbation, random normal columns otherwise
    const double delta = std::sqrt(std::numeric_limits<double>::epsilon());
    auto build_block = [&](bool use_inputs, uint64_t rkey) {
        double *Xd = W64.X.as<double>();
        double *R = W64.Z.as<double>();   // scratch, 2 N w
        double *nrm = W64.dnorm.as<double>();
        double *part = W64.dpart.as<double>();
        bool guards_random = true, buffer_random = true;
        if (use_inputs && X0) {
            if (!seed && o.seed_kind == KF_SEED_PRODUCT && g + b > 0) {
                // the guards of a warm start are the product seed's columns m+1:w (src/lobpcg.jl:182-190),
                // the buffer columns its next ones
                product_seed_device(op, wi, Xd, s);
                perturb_block(Xd + (size_t)N * m, N, g + b, delta, 0x4b47, R, nrm, part, s);
                guards_random = buffer_random = false;
            }
            KF_CUDA(cudaMemcpyAsync(Xd, X0, sizeof(double) * (size_t)N * m, cudaMemcpyHostToDevice, s));
            perturb_block(Xd, N, m, delta, 0x4b46, R, nrm, part, s);
            if (seed) {
                KF_CUDA(cudaMemcpyAsync(Xd + (size_t)N * m, seed + (size_t)N * m, sizeof(double) * (size_t)N * g,
                                        cudaMemcpyHostToDevice, s));
                perturb_block(Xd + (size_t)N * m, N, g, delta, 0x4b47, R, nrm, part, s);
                guards_random = false;
                buffer_random = true;
            }
        } else if (use_inputs && seed) {
            KF_CUDA(cudaMemcpyAsync(Xd, seed, sizeof(double) * (size_t)N * w, cudaMemcpyHostToDevice, s));
            perturb_block(Xd, N, w, delta, 0x4b46, R, nrm, part, s);
            guards_random = false;
        } else if (use_inputs && o.seed_kind == KF_SEED_PRODUCT) {
            product_seed_device(op, wi, Xd, s);
            perturb_block(Xd, N, wi, delta, 0x4b46, R, nrm, part, s);
            guards_random = buffer_random = false;
        } else {
            fill_normal<double>(Xd, N, m, N, rkey, 1, s);
        }
        if (guards_random) fill_normal<double>(Xd + (size_t)N * m, N, g, N, rkey, 2, s);
        if (buffer_random && b > 0) fill_normal<double>(Xd + (size_t)N * w, N, b, N, rkey, 3, s);
    };
    if (X0) st.warm = 1;
    LobParams p64{o.tol, o.maxiter, o.preconditioner, o.eta, w, 1e-12, false, o.fallback_iters,
                  o.fallback_resid > 0 ? o.fallback_resid : 0.0};
    // the warm-start check looks at the warm block's m columns: the guards and buffers come from the product
    // seed, the method without the warm start
    p64.judge_cols = m;
    std::vector<double> theta;
    LobOut r;
    const double t0 = now_s();
    auto attempt = [&](bool allow_judge) {
        LobParams q = p64;
        if (!allow_judge) q.judge_resid = 0;
        int iters32 = 0;
        int64_t nmv32 = 0;
        if (o.precision == KF_PREC_MIXED) {
            LobWork<float> W32(N, wi);
            // every width class the solve applies H to is tuned here, not in the middle of the
            // iteration (the active block narrows one column at a time as columns lock)
            pretune_apply(op, true, W32.Z.p, W32.HZ.p, N, 2 * wi, s);
            pretune_apply(op, false, W64.Z.p, W64.HZ.p, N, wi, s);
            convert<double, float>(W64.X.as<double>(), N, W32.X.as<float>(), N, wi, N, s);
            LobParams p32 = q;
            p32.lock_tol = std::max(o.tol, o.mixed_switch * hn);
            p32.cutoff = 1e-6;
            p32.stall_exit = true;
            LobOut r32 = lobpcg_run<float>(op, W32, dD.as<double>(), p32, s, theta);
            iters32 = r32.iters;
            nmv32 = r32.nmv;
            if (r32.judged_bad) {
                r = r32;
                return;
            }
            q.judge_resid = 0;
            // FP64 refinement with FP32 search directions
            RefineWork RW(N, wi);
            convert<float, double>(W32.X.as<float>(), N, RW.X.as<double>(), N, wi, N, s);
            const double tf = now_s();
            r = lobpcg_refine(op, RW, W32, dD.as<double>(), q, s, theta);
            KF_CUDA(cudaMemcpyAsync(W64.X.p, RW.X.p, sizeof(double) * (size_t)N * wi, cudaMemcpyDeviceToDevice, s));
            st.seconds_f64 = now_s() - tf;
            st.iterations_f64 = r.iters;
            r.iters += iters32;
            r.nmv += nmv32;
            return;
        }
        pretune_apply(op, false, W64.Z.p, W64.HZ.p, N, 2 * wi, s);
        const double tf = now_s();
        r = lobpcg_run<double>(op, W64, dD.as<double>(), q, s, theta);
        st.seconds_f64 = now_s() - tf;
        st.iterations_f64 = r.iters;
        r.iters += iters32;
        r.nmv += nmv32;
    };
    const double tb0 = now_s();
    build_block(true, o.rng_seed);
    if (trace_on()) {
        KF_CUDA(cudaStreamSynchronize(s));
        std::fprintf(stderr, "kf lobpcg setup: initial block (upload + perturbation) %.4f s\n", now_s() - tb0);
    }
    bool failed = false;
    try {
        attempt(X0 != nullptr);
    } catch (const Error &e) {
        if (e.code != KF_EBREAKDOWN && e.code != KF_ENOTFINITE) throw;
        if (!X0 && !seed) throw Error(KF_EBREAKDOWN, std::string("LOBPCG: the eigensolver failed (") + e.what() + ")");
        failed = true;
    }
    if (failed || r.judged_bad) {
        // one retry from a random block (src/lobpcg.jl:272-289); also the warm-start fallback
        if (r.judged_bad) st.fell_back = 1;
        build_block(false, o.rng_seed ^ 0x52455452ull);
        const int it0 = r.judged_bad ? r.iters : 0;
        const int64_t nmv0 = r.judged_bad ? r.nmv : 0;
        try {
            attempt(false);
        } catch (const Error &e) {
            throw Error(e.code, std::string("LOBPCG: the eigensolver failed (") + e.what() +
                                    "). An exactly zero residual block (an operator proportional to the identity on "
                                    "the block, or exact eigenvectors) can break its orthogonalization; use Dense() "
                                    "for such operators");
        }
        r.iters += it0;
        r.nmv += nmv0;
    }
    st.iterations = r.iters;
    st.n_matvec = r.nmv;
    std::vector<double> resid;
    const double ta0 = now_s();
    accept_and_copy(op, W64.X.as<double>(), w, theta, m, E_out, V_out, resid, s);
    if (trace_on()) std::fprintf(stderr, "kf lobpcg acceptance (FP64 residuals + V to the host) %.4f s\n", now_s() - ta0);
    st.seconds = now_s() - t0;
    double worst = 0;
    int bad = 0;
    for (int j = 0; j < m; ++j) {
        worst = std::max(worst, resid[j]);
        if (!(resid[j] <= o.tol)) ++bad;
    }
    st.max_residual = worst;
    st.converged = m - bad;
    if (bad) {
        char buf[256];
        snprintf(buf, sizeof buf,
                 "LOBPCG: %d of %d eigenpairs did not converge within %d iterations (only %d converged; maximum "
                 "residual %.3e > tol = %.3e)",
                 bad, m, o.maxiter, m - bad, worst, o.tol);
        throw Error(KF_ENOCONV, buf);
    }
}

// ------------------------------------------------------------------------------------------
// Chebyshev-filtered subspace iteration (src/chebyshev.jl:310-406), FP64 or FP32 filter

static constexpr double SVQB_CUTOFF = 1e-12;
static constexpr double LOCK_FRACTION = 0.5;
static constexpr double SEED_ADMIXTURE = 1e-2;
static constexpr int CHEB_GUARDS = 4;
static constexpr double GUARD_GAIN_FRACTION = 0.1;

static double log_gain(double t, double lcut, double lmax) {
    const double x = std::fabs((t - (lmax + lcut) / 2) / ((lmax - lcut) / 2));
    return x > 1 ? std::acosh(x) : 0.0;
}

static double kth_smallest(std::vector<double> v, int k) {
    std::nth_element(v.begin(), v.begin() + (k - 1), v.end());
    return v[k - 1];
}

static void solve_chebyshev(kf_op *op, const kf_solver_opts &o, int m, const double *seed, double *E_out,
                            double *V_out, kf_solve_stats &st) {
    const int64_t N = op->N;
    cudaStream_t s = op->stream;
    KF_REQUIRE(m >= 1, KF_EINVAL, "ChebyshevFilter requires m >= 1, got " + std::to_string(m));
    KF_REQUIRE(m <= N, KF_EINVAL, "ChebyshevFilter: m exceeds the operator dimension");
    KF_REQUIRE(o.tol > 0 && std::isfinite(o.tol), KF_EINVAL, "ChebyshevFilter: tol must be positive and finite");
    KF_REQUIRE(o.degree >= 1 && o.degree <= 200, KF_EINVAL, "ChebyshevFilter: degree must lie in 1:200");
    KF_REQUIRE(o.extra >= 2, KF_EINVAL,
               "ChebyshevFilter: extra must be at least 2 so at least one column serves as a convergence guard");
    KF_REQUIRE(o.maxiter >= 1 && o.rescale_every >= 1, KF_EINVAL, "ChebyshevFilter: maxiter and rescale_every must be at least 1");
    const int nb = (int)std::min<int64_t>(m + o.extra, N);
    KF_REQUIRE(nb <= 110, KF_EINVAL, "ChebyshevFilter: this build supports blocks of at most 110 columns (m + extra)");
    const double hb = op->gershgorin;
    st.hnorm = hb;
    const double lmax = std::isnan(o.bound) ? hb : o.bound;
    const double eps = std::numeric_limits<double>::epsilon();
    const int g = std::max(std::min(std::min(o.extra - 1, CHEB_GUARDS), nb - 1 - m), 0);
    const double t0 = now_s();
    // buffers (FP64): X, HX, A, B, C, S
    const size_t blk = (size_t)N * nb * sizeof(double);
    DevMem dX(blk), dHX(blk), dA(blk), dB(blk), dC(blk), dS(blk), dG((size_t)nb * nb * 8), dM((size_t)nb * nb * 8),
        dpart(gram_partials_size(nb, nb, N)), dv(2 * nb * 8);
    HostMem hG((size_t)nb * nb * 8), hv(2 * nb * 8);
    double *X = dX.as<double>(), *HX = dHX.as<double>();
    double *bufs[3] = {dA.as<double>(), dB.as<double>(), dC.as<double>()};
    double *S = dS.as<double>(), *G = dG.as<double>(), *M = dM.as<double>(), *part = dpart.as<double>();
    uint64_t refill_stream = 1;
    // the starting block on the device: product seed + 1e-2 admixture (src/chebyshev.jl), or random
    if (seed) {
        KF_CUDA(cudaMemcpyAsync(bufs[0], seed, blk, cudaMemcpyHostToDevice, s));
        perturb_block(bufs[0], N, nb, SEED_ADMIXTURE, 0x4346, bufs[1], dv.as<double>(), part, s);
    } else if (o.seed_kind == KF_SEED_PRODUCT) {
        product_seed_device(op, nb, bufs[0], s);
        perturb_block(bufs[0], N, nb, SEED_ADMIXTURE, 0x4346, bufs[1], dv.as<double>(), part, s);
    } else {
        fill_normal<double>(bufs[0], N, nb, N, o.rng_seed, 3, s);
    }

    auto colnorms_host = [&](const double *Z, int k, std::vector<double> &out) {
        colnorms2<double>(Z, N, k, N, dv.as<double>(), part, s);
        KF_CUDA(cudaMemcpyAsync(hv.p, dv.p, k * 8, cudaMemcpyDeviceToHost, s));
        KF_CUDA(cudaStreamSynchronize(s));
        out.resize(k);
        for (int j = 0; j < k; ++j) out[j] = std::sqrt(hv.as<double>()[j]);
    };
    auto normalize = [&](double *Z, int k) {
        std::vector<double> nrm;
        colnorms_host(Z, k, nrm);
        for (int j = 0; j < k; ++j) hv.as<double>()[j] = 1.0 / std::max(nrm[j], 1e-300);
        KF_CUDA(cudaMemcpyAsync(dv.p, hv.p, k * 8, cudaMemcpyHostToDevice, s));
        scale_columns<double>(Z, N, k, N, dv.as<double>(), s);
    };
    // Z <- Z - L (L' Z), twice
    auto project_out = [&](double *Z, int k, const double *L, int nl) {
        if (nl == 0 || k == 0) return;
        for (int q = 0; q < 2; ++q) {
            gram<double>(L, N, nl, Z, N, k, N, G, part, s);
            update<double>(Z, N, k, L, N, nl, G, nl, -1.0, 1.0, N, s);
        }
    };
    // one SVQB pass: dst[:, 0:r] = orthonormal basis of Z; returns r
    auto svqb_pass = [&](double *dst, const double *Z, int k) -> int {
        if (k == 0) return 0;
        gram<double>(Z, N, k, Z, N, k, N, G, part, s);
        KF_CUDA(cudaMemcpyAsync(hG.p, G, (size_t)k * k * 8, cudaMemcpyDeviceToHost, s));
        KF_CUDA(cudaStreamSynchronize(s));
        std::vector<double> T;
        const int r = svqb_coeffs(k, hG.as<double>(), SVQB_CUTOFF, T);
        if (r == 0) return 0;
        KF_CUDA(cudaMemcpyAsync(M, T.data(), (size_t)k * r * 8, cudaMemcpyHostToDevice, s));
        update<double>(dst, N, r, Z, N, k, M, k, 1.0, 0.0, N, s);
        return r;
    };
    // orthonormalise Z (na columns) against the locked L into Wd; Z and Sd are scratch
    auto orthonormalize = [&](double *Wd, double *Z, int na, const double *L, int nl, double *Sd) {
        project_out(Z, na, L, nl);
        if (o.ortho == KF_ORTHO_CHOLQR) {
            const double *src = Z;
            double *dsts[2] = {Sd, Wd};
            for (int q = 0; q < 2; ++q) {
                gram<double>(src, N, na, src, N, na, N, G, part, s);
                KF_CUDA(cudaMemcpyAsync(hG.p, G, (size_t)na * na * 8, cudaMemcpyDeviceToHost, s));
                KF_CUDA(cudaStreamSynchronize(s));
                std::vector<double> U(hG.as<double>(), hG.as<double>() + (size_t)na * na), Ui((size_t)na * na);
                for (int j = 0; j < na; ++j)
                    for (int i = 0; i < j; ++i) U[j + (size_t)na * i] = U[i + (size_t)na * j] = 0.5 * (U[i + (size_t)na * j] + U[j + (size_t)na * i]);
                if (!cholesky_upper(na, U.data(), na))
                    throw Error(KF_EBREAKDOWN,
                                "ChebyshevFilter: Cholesky-QR failed, the filtered block is numerically rank "
                                "deficient; use ortho=:svqb (it drops and refills dependent directions)");
                tri_upper_inverse(na, U.data(), na, Ui.data(), na);
                KF_CUDA(cudaMemcpyAsync(M, Ui.data(), (size_t)na * na * 8, cudaMemcpyHostToDevice, s));
                update<double>(dsts[q], N, na, src, N, na, M, na, 1.0, 0.0, N, s);
                src = dsts[q];
            }
            project_out(Wd, na, L, nl);
            return;
        }
        int k1 = svqb_pass(Sd, Z, na);
        int k = svqb_pass(Wd, Sd, k1);
        int refills = 0;
        while (k < na) {
            if (++refills > 10)
                throw Error(KF_EBREAKDOWN,
                            "ChebyshevFilter: SVQB could not refill " + std::to_string(na - k) +
                                " dropped directions with random vectors; the block is wider than the space left "
                                "beside the locked columns");
            const int r = na - k;
            double *Rr = Z;
            fill_normal<double>(Rr, N, r, N, o.rng_seed, refill_stream++, s);
            std::vector<double> before, after;
            colnorms_host(Rr, r, before);
            project_out(Rr, r, L, nl);
            project_out(Rr, r, Wd, k);
            colnorms_host(Rr, r, after);
            for (int j = 0; j < r; ++j) {
                const bool room = after[j] > std::sqrt(eps) * before[j];
                hv.as<double>()[j] = room ? 1.0 / std::max(after[j], 1e-300) : 0.0;
            }
            KF_CUDA(cudaMemcpyAsync(dv.p, hv.p, r * 8, cudaMemcpyHostToDevice, s));
            scale_columns<double>(Rr, N, r, N, dv.as<double>(), s);
            const int j1 = svqb_pass(Sd, Rr, r);
            if (j1 == 0) continue;
            project_out(Sd, j1, Wd, k);
            k += svqb_pass(Wd + (int64_t)k * N, Sd, j1);
        }
        project_out(Wd, na, L, nl);
    };
    // Rayleigh-Ritz on W with HW: Xa = W Q, HXa = HW Q, theta (host)
    auto rayleigh_ritz = [&](double *Xa, double *HXa, const double *Wd, const double *HWd, int k,
                             std::vector<double> &th) {
        gram<double>(Wd, N, k, HWd, N, k, N, G, part, s);
        KF_CUDA(cudaMemcpyAsync(hG.p, G, (size_t)k * k * 8, cudaMemcpyDeviceToHost, s));
        KF_CUDA(cudaStreamSynchronize(s));
        std::vector<double> V((size_t)k * k);
        th.resize(k);
        if (sym_eig(k, hG.as<double>(), k, th.data(), V.data(), k) != 0)
            throw Error(KF_EBREAKDOWN, "ChebyshevFilter: Rayleigh-Ritz eigenproblem did not converge");
        KF_CUDA(cudaMemcpyAsync(M, V.data(), (size_t)k * k * 8, cudaMemcpyHostToDevice, s));
        update<double>(Xa, N, k, Wd, N, k, M, k, 1.0, 0.0, N, s);
        update<double>(HXa, N, k, HWd, N, k, M, k, 1.0, 0.0, N, s);
    };
    auto check_bound = [&](const double *th, int k) {
        const double slack = std::sqrt(eps) * std::max(std::fabs(lmax), 1.0);
        double top = -INFINITY;
        for (int j = 0; j < k; ++j) top = std::max(top, th[j]);
        if (!(top <= lmax + slack)) {
            char buf[320];
            snprintf(buf, sizeof buf,
                     "ChebyshevFilter: a Ritz value %.6g exceeds the upper end λ_max = %.6g of the filter interval, "
                     "so the bound is below the true largest eigenvalue; use bound=:gershgorin",
                     top, lmax);
            throw Error(KF_ENOCONV, buf);
        }
    };

    // the seed's Rayleigh-Ritz
    normalize(bufs[0], nb);
    orthonormalize(bufs[1], bufs[0], nb, nullptr, 0, bufs[2]);
    launch_apply(op, false, bufs[1], bufs[0], N, N, nb, 1, 0, nullptr, 0, 0, s);
    int64_t nmv = nb;
    std::vector<double> theta;
    rayleigh_ritz(X, HX, bufs[1], bufs[0], nb, theta);
    check_bound(theta.data(), nb);
    std::vector<double> res(nb, INFINITY);
    int nlock = 0, it = 0, deg = 0;
    double lcut = NAN;
    // mixed precision: the filter runs in FP32 until the smallest unlocked residual reaches the
    // FP32 floor region (1e-4 ||H||) or stops halving, then in FP64 (the FP32 filter cannot
    // resolve residuals below ~1e-6 ||H||, so the last iterations must be FP64)
    const bool mixed = o.precision == KF_PREC_MIXED;
    bool f32 = mixed;
    double prev_best = INFINITY;
    DevMem fA(mixed ? (size_t)N * nb * 4 : 0), fB(mixed ? (size_t)N * nb * 4 : 0), fC(mixed ? (size_t)N * nb * 4 : 0);
    while (true) {
        const int na = nb - nlock;
        // residual norms of the active columns
        KF_CUDA(cudaMemcpyAsync(dv.p, theta.data() + nlock, na * 8, cudaMemcpyHostToDevice, s));
        residual_block<double>(X + (int64_t)nlock * N, HX + (int64_t)nlock * N, N, na, N, dv.as<double>(), bufs[0], N, s);
        std::vector<double> rn;
        colnorms_host(bufs[0], na, rn);
        for (int j = 0; j < na; ++j) res[nlock + j] = rn[j];
        if (f32 && it >= 1) {
            double best = INFINITY;
            for (int j = nlock; j < nb; ++j) best = std::min(best, res[j]);
            if (best <= 1e-4 * std::fabs(hb) || best > 0.5 * prev_best) f32 = false;
            prev_best = std::min(prev_best, best);
        }
        const bool filtered = it >= 1 || nb == N;
        const double tmin = *std::min_element(theta.begin(), theta.end());
        const double floor_ = 10 * eps * std::max(std::fabs(hb), std::fabs(tmin));
        while (filtered && nlock < nb && res[nlock] <= LOCK_FRACTION * std::max(o.tol, floor_)) ++nlock;
        // counted guards
        int counted = g;
        if (deg > 0 && std::isfinite(lcut)) {
            const double ref = log_gain(kth_smallest(theta, m), lcut, lmax);
            if (ref > 0) {
                counted = 0;
                for (int j = m; j < m + g; ++j) {
                    if (log_gain(theta[j], lcut, lmax) < GUARD_GAIN_FRACTION * ref) break;
                    ++counted;
                }
            }
        }
        const int need = m + counted;
        bool done = false;
        if (nlock >= need) {
            if (nlock == nb)
                done = true;
            else
                done = theta[nlock] >= kth_smallest(std::vector<double>(theta.begin(), theta.begin() + nlock), m);
        }
        if (done) break;
        if (it >= o.maxiter) {
            char buf[256];
            snprintf(buf, sizeof buf, "ChebyshevFilter: within maxiter = %d iterations only %d of %d eigenpairs converged",
                     o.maxiter, std::min(nlock, need), need);
            throw Error(KF_ENOCONV, buf);
        }
        ++it;
        const int nact = nb - nlock;
        lcut = theta[nb - 1];
        if (!(lcut < lmax)) throw Error(KF_ENOCONV, "ChebyshevFilter: the block's largest Ritz value reaches the upper end λ_max of the filter interval; use Dense()");
        // degree cap (src/chebyshev.jl:169-174)
        deg = o.degree;
        {
            const double x = std::fabs((tmin - (lmax + lcut) / 2) / ((lmax - lcut) / 2));
            if (x > 1) {
                const double cap = std::acosh(1.0 / std::sqrt(eps)) / std::acosh(x);
                if (cap < o.degree) deg = std::max((int)std::floor(cap), 1);
            }
        }
        const double c = (lmax + lcut) / 2, e = (lmax - lcut) / 2;
        const double *Xa = X + (int64_t)nlock * N;
        double *Zres;
        int zi;
        if (!f32) {
            double *A = bufs[0], *B = bufs[1], *Cc = bufs[2];
            copy_block<double>(Xa, N, A, N, nact, N, s);
            launch_apply(op, false, A, B, N, N, nact, 1.0 / e, -c / e, nullptr, N, 0.0, s);   // T1 = (H - c) X / e
            for (int k = 2; k <= deg; ++k) {
                launch_apply(op, false, B, Cc, N, N, nact, 2.0 / e, -2.0 * c / e, A, N, -1.0, s);
                std::swap(A, B);
                std::swap(B, Cc);   // (A, B, C) <- (B, C, A)
                if (k % o.rescale_every == 0) {
                    std::vector<double> nrm;
                    colnorms_host(B, nact, nrm);
                    for (int j = 0; j < nact; ++j) hv.as<double>()[j] = 1.0 / std::max(nrm[j], 1e-300);
                    KF_CUDA(cudaMemcpyAsync(dv.p, hv.p, nact * 8, cudaMemcpyHostToDevice, s));
                    scale_columns<double>(A, N, nact, N, dv.as<double>(), s);
                    scale_columns<double>(B, N, nact, N, dv.as<double>(), s);
                }
            }
            Zres = B;
        } else {
            // FP32 filter: the recurrence in FP32, result widened to FP64
            float *A = fA.as<float>(), *B = fB.as<float>(), *Cc = fC.as<float>();
            convert<double, float>(Xa, N, A, N, nact, N, s);
            launch_apply(op, true, A, B, N, N, nact, 1.0 / e, -c / e, nullptr, N, 0.0, s);
            for (int k = 2; k <= deg; ++k) {
                launch_apply(op, true, B, Cc, N, N, nact, 2.0 / e, -2.0 * c / e, A, N, -1.0, s);
                std::swap(A, B);
                std::swap(B, Cc);
                if (k % o.rescale_every == 0) {
                    colnorms2<float>(B, N, nact, N, dv.as<double>(), part, s);
                    KF_CUDA(cudaMemcpyAsync(hv.p, dv.p, nact * 8, cudaMemcpyDeviceToHost, s));
                    KF_CUDA(cudaStreamSynchronize(s));
                    for (int j = 0; j < nact; ++j) hv.as<double>()[j] = 1.0 / std::max(std::sqrt(hv.as<double>()[j]), 1e-300);
                    KF_CUDA(cudaMemcpyAsync(dv.p, hv.p, nact * 8, cudaMemcpyHostToDevice, s));
                    scale_columns<float>(A, N, nact, N, dv.as<double>(), s);
                    scale_columns<float>(B, N, nact, N, dv.as<double>(), s);
                }
            }
            convert<float, double>(B, N, bufs[0], N, nact, N, s);
            Zres = bufs[0];
        }
        nmv += (int64_t)deg * nact;
        zi = Zres == bufs[0] ? 0 : Zres == bufs[1] ? 1 : 2;
        double *Wv = bufs[(zi + 1) % 3], *Sv = bufs[(zi + 2) % 3];
        {
            std::vector<double> nrm;
            colnorms_host(Zres, nact, nrm);
            for (int j = 0; j < nact; ++j)
                if (!std::isfinite(nrm[j]))
                    throw Error(KF_ENOTFINITE,
                                "ChebyshevFilter: the filtered block is not finite: the upper end λ_max of the filter "
                                "interval is below the true largest eigenvalue, so the filter amplifies the top of the "
                                "spectrum; use bound=:gershgorin");
        }
        normalize(Zres, nact);
        orthonormalize(Wv, Zres, nact, X, nlock, Sv);
        launch_apply(op, false, Wv, Zres, N, N, nact, 1, 0, nullptr, 0, 0, s);
        nmv += nact;
        std::vector<double> th;
        rayleigh_ritz(X + (int64_t)nlock * N, HX + (int64_t)nlock * N, Wv, Zres, nact, th);
        for (int j = 0; j < nact; ++j) theta[nlock + j] = th[j];
        check_bound(th.data(), nact);
    }
    st.iterations = it;
    st.n_matvec = nmv;
    // the lowest m locked pairs, accepted with a fresh application (src/chebyshev.jl:395-405)
    std::vector<double> thl(theta.begin(), theta.begin() + nlock);
    std::vector<double> resid;
    accept_and_copy(op, X, nlock, thl, m, E_out, V_out, resid, s);
    double worst = 0;
    int jw = 0;
    for (int j = 0; j < m; ++j)
        if (resid[j] > worst) { worst = resid[j]; jw = j; }
    std::vector<int> ord(nlock);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return thl[a] < thl[b]; });
    const double floor_ = 10 * eps * std::max(std::fabs(hb), std::fabs(thl[ord[0]]));
    st.max_residual = worst;
    st.converged = 0;
    for (int j = 0; j < m; ++j) st.converged += resid[j] <= std::max(o.tol, floor_);
    st.seconds = now_s() - t0;
    if (!(worst <= std::max(o.tol, floor_))) {
        char buf[256];
        snprintf(buf, sizeof buf, "ChebyshevFilter: the true residual ‖H v − E v‖ = %.3e of pair %d exceeds %.3e on return",
                 worst, jw + 1, std::max(o.tol, floor_));
        throw Error(KF_ENOCONV, buf);
    }
}

// ------------------------------------------------------------------------------------------
// Lanczos (src/solvers.jl:85-106): thick-restart Lanczos with full reorthogonalisation in FP64
// (KrylovKit's eigsolve is a Krylov-Schur method; both keep the Ritz vectors of the wanted end
// at each restart).

static void solve_lanczos(kf_op *op, const kf_solver_opts &o, int m, double *E_out, double *V_out,
                          kf_solve_stats &st) {
    const int64_t N = op->N;
    cudaStream_t s = op->stream;
    KF_REQUIRE(m >= 1, KF_EINVAL, "Lanczos requires m >= 1, got " + std::to_string(m));
    KF_REQUIRE(m <= N, KF_EINVAL, "Lanczos: m = " + std::to_string(m) + " exceeds the operator dimension " + std::to_string(N));
    const int kd = (int)std::min<int64_t>(std::max(2 * m + 10, o.krylovdim > 0 ? o.krylovdim : 40), N);
    KF_REQUIRE(kd <= 128, KF_EINVAL, "Lanczos: this build supports krylovdim <= 128");
    const double t0 = now_s();
    DevMem dV((size_t)N * (kd + 1) * 8), dHV((size_t)N * 8), dW((size_t)N * kd * 8), dG((size_t)(kd + 1) * 8 * 2),
        dC((size_t)(kd + 1) * (kd + 1) * 8), dpart(gram_partials_size(kd + 1, 1, N)), dn(8);
    HostMem hG((size_t)(kd + 1) * (kd + 1) * 8);
    double *V = dV.as<double>(), *G = dG.as<double>(), *part = dpart.as<double>();
    // start vector
    fill_normal<double>(V, N, 1, N, o.rng_seed, 7, s);
    double nrm2;
    colnorms2<double>(V, N, 1, N, dn.as<double>(), part, s);
    KF_CUDA(cudaMemcpyAsync(&nrm2, dn.p, 8, cudaMemcpyDeviceToHost, s));
    KF_CUDA(cudaStreamSynchronize(s));
    double sc = 1.0 / std::sqrt(nrm2);
    KF_CUDA(cudaMemcpyAsync(dn.p, &sc, 8, cudaMemcpyHostToDevice, s));
    scale_columns<double>(V, N, 1, N, dn.as<double>(), s);
    // T: the projected matrix in the current basis (k x k, symmetric, arrow + tridiagonal)
    std::vector<double> T((size_t)(kd + 1) * (kd + 1), 0.0);
    int k = 0;          // vectors kept from the last restart (T[0:k, 0:k] diagonal, row k the arrow)
    int64_t nmv = 0;
    int restarts = 0;
    std::vector<double> theta, resid(m, INFINITY);
    const double tol = o.tol;
    while (true) {
        // extend the basis from column j = k to kd
        for (int j = k; j < kd; ++j) {
            double *vj = V + (int64_t)j * N, *w = V + (int64_t)(j + 1) * N;
            launch_apply(op, false, vj, w, N, N, 1, 1, 0, nullptr, 0, 0, s);
            ++nmv;
            // full reorthogonalisation, twice: h = V[:, 0:j+1]' w, w -= V h
            std::vector<double> h(j + 1, 0.0);
            for (int q = 0; q < 2; ++q) {
                gram<double>(V, N, j + 1, w, N, 1, N, G, part, s);
                KF_CUDA(cudaMemcpyAsync(hG.p, G, (j + 1) * 8, cudaMemcpyDeviceToHost, s));
                update<double>(w, N, 1, V, N, j + 1, G, j + 1, -1.0, 1.0, N, s);
                KF_CUDA(cudaStreamSynchronize(s));
                for (int i = 0; i <= j; ++i) h[i] += hG.as<double>()[i];
            }
            colnorms2<double>(w, N, 1, N, dn.as<double>(), part, s);
            KF_CUDA(cudaMemcpyAsync(&nrm2, dn.p, 8, cudaMemcpyDeviceToHost, s));
            KF_CUDA(cudaStreamSynchronize(s));
            const double beta = std::sqrt(nrm2);
            for (int i = 0; i <= j; ++i) {
                T[i + (size_t)(kd + 1) * j] = h[i];
                T[j + (size_t)(kd + 1) * i] = h[i];
            }
            T[(j + 1) + (size_t)(kd + 1) * j] = beta;
            T[j + (size_t)(kd + 1) * (j + 1)] = beta;
            if (beta <= 1e-14 * std::max(1.0, std::fabs(op->gershgorin))) {
                // invariant subspace: restart the new direction randomly, orthogonalised
                fill_normal<double>(w, N, 1, N, o.rng_seed, 1000 + nmv, s);
                for (int q = 0; q < 2; ++q) {
                    gram<double>(V, N, j + 1, w, N, 1, N, G, part, s);
                    update<double>(w, N, 1, V, N, j + 1, G, j + 1, -1.0, 1.0, N, s);
                }
                colnorms2<double>(w, N, 1, N, dn.as<double>(), part, s);
                KF_CUDA(cudaMemcpyAsync(&nrm2, dn.p, 8, cudaMemcpyDeviceToHost, s));
                KF_CUDA(cudaStreamSynchronize(s));
                T[(j + 1) + (size_t)(kd + 1) * j] = 0;
                T[j + (size_t)(kd + 1) * (j + 1)] = 0;
                sc = 1.0 / std::sqrt(nrm2);
            } else {
                sc = 1.0 / beta;
            }
            KF_CUDA(cudaMemcpyAsync(dn.p, &sc, 8, cudaMemcpyHostToDevice, s));
            scale_columns<double>(w, N, 1, N, dn.as<double>(), s);
        }
        // Ritz pairs of T[0:kd, 0:kd]; residual of pair i = |beta_kd * y[kd-1, i]|
        std::vector<double> Ts((size_t)kd * kd), lam(kd), Y((size_t)kd * kd);
        for (int j = 0; j < kd; ++j)
            for (int i = 0; i < kd; ++i) Ts[i + (size_t)kd * j] = T[i + (size_t)(kd + 1) * j];
        if (sym_eig(kd, Ts.data(), kd, lam.data(), Y.data(), kd) != 0)
            throw Error(KF_EBREAKDOWN, "Lanczos: the projected eigenproblem did not converge");
        const double bk = T[kd + (size_t)(kd + 1) * (kd - 1)];
        int conv = 0;
        for (int i = 0; i < m; ++i) {
            resid[i] = std::fabs(bk * Y[(kd - 1) + (size_t)kd * i]);
            if (resid[i] <= tol) ++conv;
        }
        theta.assign(lam.begin(), lam.begin() + m);
        const int keep = std::min(kd - 1, std::max(m + (kd - m) / 2, m));
        if (conv == m || restarts >= o.maxiter) {
            // Ritz vectors of the lowest m into dW
            KF_CUDA(cudaMemcpyAsync(dC.p, Y.data(), (size_t)kd * m * 8, cudaMemcpyHostToDevice, s));
            update<double>(dW.as<double>(), N, m, V, N, kd, dC.as<double>(), kd, 1.0, 0.0, N, s);
            break;
        }
        // thick restart: keep the lowest `keep` Ritz vectors and the residual direction
        KF_CUDA(cudaMemcpyAsync(dC.p, Y.data(), (size_t)kd * keep * 8, cudaMemcpyHostToDevice, s));
        update<double>(dW.as<double>(), N, keep, V, N, kd, dC.as<double>(), kd, 1.0, 0.0, N, s);
        copy_block<double>(V + (int64_t)kd * N, N, V + (int64_t)keep * N, N, 1, N, s);
        copy_block<double>(dW.as<double>(), N, V, N, keep, N, s);
        std::fill(T.begin(), T.end(), 0.0);
        for (int i = 0; i < keep; ++i) {
            T[i + (size_t)(kd + 1) * i] = lam[i];
            const double a = bk * Y[(kd - 1) + (size_t)kd * i];
            T[keep + (size_t)(kd + 1) * i] = a;
            T[i + (size_t)(kd + 1) * keep] = a;
        }
        k = keep;
        ++restarts;
    }
    st.iterations = restarts;
    st.n_matvec = nmv;
    std::vector<double> r2;
    accept_and_copy(op, dW.as<double>(), m, theta, m, E_out, V_out, r2, s);
    double worst = 0;
    int bad = 0;
    for (int j = 0; j < m; ++j) {
        worst = std::max(worst, r2[j]);
        bad += !(r2[j] <= std::max(tol, 10 * std::numeric_limits<double>::epsilon() * std::fabs(op->gershgorin)));
    }
    st.max_residual = worst;
    st.converged = m - bad;
    st.seconds = now_s() - t0;
    if (bad) {
        char buf[200];
        snprintf(buf, sizeof buf, "Lanczos: only %d of %d eigenpairs converged (normres = %.3e)", m - bad, m, worst);
        throw Error(KF_ENOCONV, buf);
    }
}

void solve_dispatch(kf_op *op, const kf_solver_opts &o, int m, const double *X0, const double *seed, double *E_out,
                    double *V_out, kf_solve_stats &st) {
    std::memset(&st, 0, sizeof(st));
    AllocScope scope(op->stream);
    switch (o.kind) {
        case KF_SOLVER_LOBPCG: solve_lobpcg(op, o, m, X0, seed, E_out, V_out, st); break;
        case KF_SOLVER_CHEBYSHEV: solve_chebyshev(op, o, m, seed, E_out, V_out, st); break;
        case KF_SOLVER_LANCZOS: solve_lanczos(op, o, m, E_out, V_out, st); break;
        default: throw Error(KF_EINVAL, "kf_solve: unknown solver kind " + std::to_string(o.kind));
    }
}

}  // namespace kf

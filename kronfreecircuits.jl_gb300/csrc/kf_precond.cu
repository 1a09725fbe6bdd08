// The separable preconditioner: P = U diag(1 / hypot(S - theta_j, eta)) U', with U = (x)_a U_a the
// eigenbases of the per-axis sums of the single-axis terms and S = sum_a lambda_a the separable
// spectrum -- the reference's separable_eigenbases (src/apply.jl:606-642, the same basis its
// product_seed uses, src/apply.jl:655-685) turned into a "fast diagonalisation" preconditioner
// for LOBPCG.  The coupling terms (products over two or more axes) are left out, so P inverts the
// stiff single-axis kinetic parts exactly (the 1/Delta^2 finite-difference stencils that make
// ||H|| large) and the coupling only shifts the spectrum.  Each application costs 2 mode products
// per non-diagonal axis (tcgen05 tensor-core GEMMs with BF16 operands for axes up to 256 long,
// SIMT FP32 beyond) and one scaling pass.
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <set>
#include <queue>
#include <numeric>

#include "kf_internal.h"

namespace kf {

// The per-axis eigendecompositions (host FP64), no CUDA calls: run on a host thread started by
// kf_op_create, so that by the first solve they are usually done.
void sep_host_prepare(kf_op *op) {
    auto &S = op->sep;
    const int nd = (int)op->dims.size();
    KF_REQUIRE((int)S.M.size() == nd, KF_EINVAL, "separable preconditioner: the operator has no per-axis sums");
    S.ident.assign(nd, 0);
    S.Uh.assign(nd, std::vector<double>());
    S.lam.clear();
    for (int a = 0; a < nd; ++a) {
        const int d = (int)op->dims[a];
        const std::vector<double> &M = S.M[a];
        {
            // src/apply.jl:627-630: a non-Hermitian single-axis sum means H is not Hermitian
            double asym = 0, nrm = 0;
            for (int j = 0; j < d; ++j)
                for (int i = 0; i < d; ++i) {
                    const double x = M[i + (size_t)d * j], y = M[j + (size_t)d * i];
                    asym += (x - y) * (x - y);
                    nrm += x * x;
                }
            asym = std::sqrt(asym);
            nrm = std::sqrt(nrm);
            if (!(asym <= std::sqrt(2.220446049250313e-16) * nrm))
                throw Error(KF_EINVAL, "separable_eigenbases: the single-axis terms on axis " + std::to_string(a + 1) +
                                           " sum to a non-Hermitian matrix, so the operator is not Hermitian");
        }
        bool diag = true;
        for (int j = 0; j < d && diag; ++j)
            for (int i = 0; i < d; ++i)
                if (i != j && M[i + (size_t)d * j] != 0.0) { diag = false; break; }
        if (diag) {
            S.ident[a] = 1;
            for (int i = 0; i < d; ++i) S.lam.push_back(M[i + (size_t)d * i]);
            continue;
        }
        std::vector<double> w(d), U((size_t)d * d);
        if (sym_eig(d, M.data(), d, w.data(), U.data(), d) != 0)
            throw Error(KF_EBREAKDOWN, "separable preconditioner: an axis eigenproblem did not converge");
        S.lam.insert(S.lam.end(), w.begin(), w.end());
        S.Uh[a] = std::move(U);
    }
    S.host_ready = true;
}

void sep_prepare(kf_op *op) {
    auto &S = op->sep;
    if (S.ready) return;
    const auto t0 = std::chrono::steady_clock::now();
    if (S.host_job.valid()) S.host_job.get();   // rethrows the host job's error, if any
    if (!S.host_ready) sep_host_prepare(op);
    const int nd = (int)op->dims.size();
    S.dU.assign(nd, nullptr);
    S.dUt.assign(nd, nullptr);
    S.dU64.assign(nd, nullptr);
    S.tU.assign(nd, TcMatrix());
    S.tUt.assign(nd, TcMatrix());
    std::vector<int> off(nd), dims(nd);
    int acc = 0;
    for (int a = 0; a < nd; ++a) {
        const int d = (int)op->dims[a];
        dims[a] = d;
        off[a] = acc;
        acc += d;
        if (S.ident[a]) continue;
        const std::vector<double> &U = S.Uh[a];
        KF_CUDA(cudaMalloc(&S.dU64[a], U.size() * 8));
        KF_CUDA(cudaMemcpy(S.dU64[a], U.data(), U.size() * 8, cudaMemcpyHostToDevice));
        std::vector<float> u32((size_t)d * d), ut32((size_t)d * d);
        for (int j = 0; j < d; ++j)
            for (int i = 0; i < d; ++i) {
                u32[i + (size_t)d * j] = (float)U[i + (size_t)d * j];
                ut32[j + (size_t)d * i] = (float)U[i + (size_t)d * j];
            }
        KF_CUDA(cudaMalloc(&S.dU[a], u32.size() * 4));
        KF_CUDA(cudaMalloc(&S.dUt[a], ut32.size() * 4));
        KF_CUDA(cudaMemcpy(S.dU[a], u32.data(), u32.size() * 4, cudaMemcpyHostToDevice));
        KF_CUDA(cudaMemcpy(S.dUt[a], ut32.data(), ut32.size() * 4, cudaMemcpyHostToDevice));
        if (tc_mode_layout_ok(d)) {
            S.tU[a] = tc_matrix_create(U.data(), d, false);
            S.tUt[a] = tc_matrix_create(U.data(), d, true);
        }
    }
    KF_CUDA(cudaMalloc(&S.d_lam, S.lam.size() * 8));
    KF_CUDA(cudaMalloc(&S.d_lam_off, nd * sizeof(int)));
    KF_CUDA(cudaMalloc(&S.d_dims, nd * sizeof(int)));
    KF_CUDA(cudaMemcpy(S.d_lam, S.lam.data(), S.lam.size() * 8, cudaMemcpyHostToDevice));
    KF_CUDA(cudaMemcpy(S.d_lam_off, off.data(), nd * sizeof(int), cudaMemcpyHostToDevice));
    KF_CUDA(cudaMemcpy(S.d_dims, dims.data(), nd * sizeof(int), cudaMemcpyHostToDevice));
    // S(p) per point as FP32 hi / lo, once per operator (every scaling pass reads it)
    KF_CUDA(cudaMalloc(&S.d_shl, (size_t)2 * op->N * sizeof(float)));
    sep_spectrum(S.d_shl, op->N, nd, S.d_dims, S.d_lam, S.d_lam_off, op->stream);
    KF_CUDA(cudaStreamSynchronize(op->stream));
    S.ready = true;
    const char *tr = std::getenv("KF_TRACE");
    if (tr && tr[0] && tr[0] != '0')
        std::fprintf(stderr, "kf separable preconditioner set-up (wait for the host job + uploads) %.4f s\n",
                     std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
}

// ---- product_seed (src/apply.jl:655-685) ---------------------------------------------------

namespace {

struct SeedArgs {
    int nd;
    int dims[MAXDIMS];
    const double *U[MAXDIMS];   // FP64 eigenbasis of each axis (nullptr: identity)
};

// X[p, c] = prod_a U_a[i_a(p), idx[c, a]] (axis 1 fastest), the product taken in the order
// U_{K-1} (... (U_1 U_0)) of the reference's kron chain
__global__ void k_product_seed(double *__restrict__ X, int64_t N, int k, SeedArgs a, const int *__restrict__ idx) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * k) return;
    const int64_t c = t / N, p = t % N;
    int64_t rem = p;
    double v = 1.0;
    for (int ax = 0; ax < a.nd; ++ax) {
        const int i = (int)(rem % a.dims[ax]);
        rem /= a.dims[ax];
        const int j = idx[c * a.nd + ax];
        const double u = a.U[ax] ? a.U[ax][i + (int64_t)a.dims[ax] * j] : (i == j ? 1.0 : 0.0);
        v = u * v;
    }
    X[c * N + p] = v;
}

struct Cand {
    double sum;
    int64_t flat;
    std::vector<int> rank;
};

}  // namespace

// The k lowest product states' per-axis indices (k x nd, row c = state c), ordered by
// (separable energy, column-major index).  Best-first search over the lattice of per-axis
// ranks: every state's lattice predecessors have energies <= its own, so popping until the
// heap's smallest energy exceeds the k-th popped one visits every state that can rank <= k.
static std::vector<int> lowest_product_states(kf_op *op, int k) {
    auto &S = op->sep;
    const int nd = (int)op->dims.size();
    std::vector<std::vector<int>> ord(nd);
    std::vector<int> off(nd);
    int acc = 0;
    for (int a = 0; a < nd; ++a) {
        const int d = (int)op->dims[a];
        off[a] = acc;
        acc += d;
        ord[a].resize(d);
        std::iota(ord[a].begin(), ord[a].end(), 0);
        const double *lam = S.lam.data() + off[a];
        std::stable_sort(ord[a].begin(), ord[a].end(), [&](int x, int y) { return lam[x] < lam[y]; });
    }
    auto make = [&](const std::vector<int> &rank) {
        Cand c;
        c.rank = rank;
        c.sum = 0;
        c.flat = 0;
        int64_t stride = 1;
        for (int a = 0; a < nd; ++a) {
            const int i = ord[a][rank[a]];
            c.sum = (a == 0) ? S.lam[off[a] + i] : c.sum + S.lam[off[a] + i];
            c.flat += stride * i;
            stride *= op->dims[a];
        }
        return c;
    };
    auto worse = [](const Cand &x, const Cand &y) { return x.sum > y.sum || (x.sum == y.sum && x.flat > y.flat); };
    std::priority_queue<Cand, std::vector<Cand>, decltype(worse)> heap(worse);
    std::set<std::vector<int>> seen;
    std::vector<int> r0(nd, 0);
    heap.push(make(r0));
    seen.insert(r0);
    std::vector<Cand> got;
    double kth = INFINITY;
    while (!heap.empty()) {
        if ((int)got.size() >= k && heap.top().sum > kth) break;
        Cand c = heap.top();
        heap.pop();
        got.push_back(c);
        if ((int)got.size() == k) kth = c.sum;
        for (int a = 0; a < nd; ++a) {
            if (c.rank[a] + 1 >= (int)op->dims[a]) continue;
            std::vector<int> r = c.rank;
            ++r[a];
            if (seen.insert(r).second) heap.push(make(r));
        }
    }
    std::sort(got.begin(), got.end(), [&](const Cand &x, const Cand &y) { return worse(y, x); });
    std::vector<int> idx((size_t)k * nd);
    for (int c = 0; c < k; ++c)
        for (int a = 0; a < nd; ++a) idx[(size_t)c * nd + a] = ord[a][got[c].rank[a]];
    return idx;
}

void product_seed_device(kf_op *op, int k, double *X, cudaStream_t s) {
    const int64_t N = op->N;
    KF_REQUIRE(k >= 1 && k <= N, KF_EINVAL,
               "product_seed: k must lie in 1:" + std::to_string(N) + " (the operator's dimension), got " +
                   std::to_string(k));
    KF_REQUIRE(!op->sep.M.empty(), KF_EINVAL, "product_seed: the per-axis sums of this operator are too large");
    sep_prepare(op);
    auto &S = op->sep;
    const int nd = (int)op->dims.size();
    KF_CUDA(cudaMemsetAsync(X, 0, sizeof(double) * (size_t)N * k, s));
    bool all_ident = true;
    for (int a = 0; a < nd; ++a) all_ident = all_ident && S.ident[a];
    if (all_ident) {
        // unit vectors of the k smallest entries of the full diagonal (ties by index)
        std::vector<int64_t> ix(N);
        std::iota(ix.begin(), ix.end(), 0);
        const double *D = op->h_fulldiag.data();
        std::partial_sort(ix.begin(), ix.begin() + k, ix.end(),
                          [&](int64_t x, int64_t y) { return D[x] < D[y] || (D[x] == D[y] && x < y); });
        const double one = 1.0;
        for (int j = 0; j < k; ++j)
            KF_CUDA(cudaMemcpyAsync(X + (size_t)N * j + ix[j], &one, sizeof(double), cudaMemcpyHostToDevice, s));
        KF_CUDA(cudaStreamSynchronize(s));   // `one` is on this stack frame
        return;
    }
    const std::vector<int> idx = lowest_product_states(op, k);
    int *didx = nullptr;
    KF_CUDA(cudaMallocAsync((void **)&didx, idx.size() * sizeof(int), s));
    KF_CUDA(cudaMemcpyAsync(didx, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    SeedArgs a;
    a.nd = nd;
    for (int ax = 0; ax < MAXDIMS; ++ax) {
        a.dims[ax] = ax < nd ? (int)op->dims[ax] : 1;
        a.U[ax] = (ax < nd && !S.ident[ax]) ? S.dU64[ax] : nullptr;
    }
    const int64_t tot = N * k;
    k_product_seed<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(X, N, k, a, didx);
    KF_LAUNCH_CHECK();
    KF_CUDA(cudaFreeAsync(didx, s));
    KF_CUDA(cudaStreamSynchronize(s));   // idx (host) stays valid until the copy is done
}

float *sep_apply(kf_op *op, float *W, float *s1, int k, const double *theta_dev, double eta, cudaStream_t s) {
    sep_prepare(op);
    auto &S = op->sep;
    const int nd = (int)op->dims.size();
    const int64_t N = op->N;
    float *cur = W, *other = s1;
    // tensor cores (BF16 operands, FP32 sums) where the axis fits the tcgen05 image, else SIMT FP32
    auto product = [&](int a, bool forward) {
        const TcMatrix &t = forward ? S.tUt[a] : S.tU[a];
        if (t.img)
            tc_mode_product(other, N, cur, N, t, op->strides[a], N, k, 1.0, 0.0, s);
        else
            mode_product<float>(other, N, cur, N, forward ? S.dUt[a] : S.dU[a], (int)op->dims[a], op->strides[a], N,
                                k, 1.0, 0.0, s);
        std::swap(cur, other);
    };
    for (int a = 0; a < nd; ++a)
        if (!S.ident[a]) product(a, true);
    sep_scale<float>(cur, N, N, k, nd, S.d_dims, S.d_lam, S.d_lam_off, theta_dev, eta, s, S.d_shl);
    for (int a = nd - 1; a >= 0; --a)
        if (!S.ident[a]) product(a, false);
    return cur;
}

}  // namespace kf

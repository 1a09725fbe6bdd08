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
    S.ready = true;
    const char *tr = std::getenv("KF_TRACE");
    if (tr && tr[0] && tr[0] != '0')
        std::fprintf(stderr, "kf separable preconditioner set-up (wait for the host job + uploads) %.4f s\n",
                     std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
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
    sep_scale<float>(cur, N, N, k, nd, S.d_dims, S.d_lam, S.d_lam_off, theta_dev, eta, s);
    for (int a = nd - 1; a >= 0; --a)
        if (!S.ident[a]) product(a, false);
    return cur;
}

}  // namespace kf

// The linear solve on the complement of a node's known states, on the GPU (src/resolvent.jl:146-252,
// _complement_solve): X[:, j] solves Q (H - s_j) Q x = Q B[:, j] with x orthogonal to the known
// basis, Q = 1 - basis basis', by a conjugate gradient on all n columns in lockstep, each with its own
// scalars, preconditioned by the Jacobi diagonal 1 / hypot(D - s_j, eta) (D = diagonal(H)).  The
// Sternheimer solves of the reference's derivatives run through it.
//
// Per iteration, in FP64 on the device: AP = H P (the fused apply), AP -= s o P, AP = Q AP (a Gram
// basis' AP and an update), kappa = <P, AP>, alpha = rho / kappa on the active columns, X += alpha P,
// R -= alpha AP, ||R||, Z = Q (Minv o R) with Minv formed once per solve, rho' = <R, Z>.  One host wait brings kappa, ||R|| and rho'
// back; the host applies the reference's column rules -- the positivity check, the per-column
// target tol ||Q B_j||, the round-off cap 1000 eps scale_j with true residuals recomputed (a fresh
// apply) for the columns below it and the five-check patience, the final true-residual acceptance --
// and sends beta and the active mask for P = Z + beta P.  Column reductions are two-stage (per-block
// partials, then a fixed-order sum), so results do not depend on scheduling.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "kf_internal.h"

namespace kf {

namespace {

constexpr int CG_THREADS = 256;
constexpr double CG_FLOOR_CAP = 1000.0;   // src/resolvent.jl:115
constexpr int CG_FLOOR_PATIENCE = 5;      // src/resolvent.jl:117

__device__ __forceinline__ double cg_block_sum(double v, double *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = v;
    __syncthreads();
    double t = 0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    }
    return t;
}

// Y[:, j] += a c[j] X[:, j]
__global__ void k_cg_axpy_cols(double *__restrict__ Y, const double *__restrict__ X, const double *__restrict__ c,
                               double a, int64_t N, int n) {
    const int64_t tot = N * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(i / N);
        Y[i] += a * c[j] * X[i];
    }
}

// partials[j * nblk + blk] = sum over the block's rows of A[r, j] B[r, j]
__global__ void k_cg_coldot(const double *__restrict__ A, const double *__restrict__ B, int64_t N, int64_t rows_per,
                            double *__restrict__ partials) {
    __shared__ double red[32];
    const int j = blockIdx.y;
    const int64_t r0 = (int64_t)blockIdx.x * rows_per, r1 = r0 + rows_per < N ? r0 + rows_per : N;
    const double *a = A + (int64_t)j * N, *b = B + (int64_t)j * N;
    double s = 0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) s += a[r] * b[r];
    const double t = cg_block_sum(s, red);
    if (threadIdx.x == 0) partials[(size_t)j * gridDim.x + blockIdx.x] = t;
}

// X += alpha_j P; R -= alpha_j AP; partials of ||R_j||^2
__global__ void k_cg_step(double *__restrict__ X, double *__restrict__ R, const double *__restrict__ P,
                          const double *__restrict__ AP, const double *__restrict__ alpha, int64_t N, int64_t rows_per,
                          double *__restrict__ partials) {
    __shared__ double red[32];
    const int j = blockIdx.y;
    const double al = alpha[j];
    const int64_t r0 = (int64_t)blockIdx.x * rows_per, r1 = r0 + rows_per < N ? r0 + rows_per : N;
    const int64_t o = (int64_t)j * N;
    double s = 0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        X[o + r] += al * P[o + r];
        const double v = R[o + r] - al * AP[o + r];
        R[o + r] = v;
        s += v * v;
    }
    const double t = cg_block_sum(s, red);
    if (threadIdx.x == 0) partials[(size_t)j * gridDim.x + blockIdx.x] = t;
}

__global__ void k_cg_reduce(const double *__restrict__ partials, int nblk, int n, double *__restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double s = 0;
    for (int b = 0; b < nblk; ++b) s += partials[(size_t)j * nblk + b];
    out[j] = s;
}

// Minv[:, j] = 1 / hypot(D - s_j, eta), once per solve (src/resolvent.jl:156, `Minv = 1 ./ hypot.(D .- S,
// eta)`): the FP64 hypot is costly on this GPU's FP64 pipe, the per-iteration step is then a product
__global__ void k_cg_minv(double *__restrict__ Minv, const double *__restrict__ D, const double *__restrict__ s,
                          double eta, int64_t N, int n) {
    const int64_t tot = N * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(i / N);
        const int64_t r = i - (int64_t)j * N;
        Minv[i] = 1.0 / hypot(D[r] - s[j], eta);
    }
}

// Z = Minv o R
__global__ void k_cg_precond(double *__restrict__ Z, const double *__restrict__ R, const double *__restrict__ Minv,
                             int64_t tot) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x)
        Z[i] = Minv[i] * R[i];
}

// P = Z + beta_j P
__global__ void k_cg_dir(double *__restrict__ P, const double *__restrict__ Z, const double *__restrict__ beta,
                         int64_t N, int n) {
    const int64_t tot = N * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(i / N);
        P[i] = Z[i] + beta[j] * P[i];
    }
}

// alpha_j = rho_j / kappa_j on the active columns with kappa_j > 0, else 0 (the host then decides
// between the round-off floor and the positivity error for an active column with kappa_j <= 0)
__global__ void k_cg_alpha(const double *__restrict__ rho, const double *__restrict__ kappa,
                           const double *__restrict__ active, double *__restrict__ alpha, int n) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    alpha[j] = (active[j] != 0.0 && kappa[j] > 0.0) ? rho[j] / kappa[j] : 0.0;
}

unsigned ew_grid(int64_t tot) { return (unsigned)std::min<int64_t>((tot + CG_THREADS - 1) / CG_THREADS, 152 * 16); }

struct CgRed {
    int64_t rows_per;
    int nblk;
};

CgRed cg_red(int64_t N, int n) {
    int64_t nblk = (304 + n - 1) / n;
    if (nblk < 1) nblk = 1;
    int64_t rp = (N + nblk - 1) / nblk;
    if (rp < 1024) rp = 1024;
    return {rp, (int)((N + rp - 1) / rp)};
}

}  // namespace

void complement_solve(kf_op *op, const double *basis, int64_t ldbs, int nb, const double *B, int64_t ldb, int n,
                      const double *shifts, const double *scale_in, double tol, int maxiter, double eta, double *X_out,
                      int64_t ldx, CgResult &res, cudaStream_t s) {
    const int64_t N = op->N;
    const size_t blk = (size_t)N * n * sizeof(double);
    double *QB, *X, *R, *Z, *P, *AP, *T, *Mi, *D, *sm, *part, *C;
    const CgRed rd = cg_red(N, n);
    const size_t part_bytes = std::max(gram_partials_size(std::max(nb, 1), n, N), (size_t)rd.nblk * n * sizeof(double));
    std::vector<void *> owned;
    auto dalloc = [&](double *&p, size_t bytes) {
        KF_CUDA(cudaMallocAsync((void **)&p, bytes, s));
        owned.push_back(p);
    };
    auto cleanup = [&]() {
        for (void *p : owned) cudaFreeAsync(p, s);
        owned.clear();
    };
    try {
        dalloc(QB, blk);
        dalloc(X, blk);
        dalloc(R, blk);
        dalloc(Z, blk);
        dalloc(P, blk);
        dalloc(AP, blk);
        dalloc(T, blk);
        dalloc(Mi, blk);
        dalloc(D, (size_t)N * sizeof(double));
        dalloc(sm, (size_t)8 * n * sizeof(double));   // s, alpha, beta, rho, active, kappa, rn2, rho'
        dalloc(part, part_bytes);
        dalloc(C, (size_t)std::max(nb, 1) * n * sizeof(double));
        double *d_s = sm, *d_alpha = sm + n, *d_beta = sm + 2 * n, *d_rho = sm + 3 * n, *d_active = sm + 4 * n;
        double *d_kappa = sm + 5 * n, *d_rn2 = sm + 6 * n, *d_rhon = sm + 7 * n;
        KF_CUDA(cudaMemcpyAsync(D, op->h_fulldiag.data(), (size_t)N * sizeof(double), cudaMemcpyHostToDevice, s));
        KF_CUDA(cudaMemcpyAsync(d_s, shifts, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s));
        k_cg_minv<<<ew_grid(N * n), CG_THREADS, 0, s>>>(Mi, D, d_s, eta, N, n);
        KF_LAUNCH_CHECK();
        KF_CUDA(cudaMemcpy2DAsync(QB, N * sizeof(double), B, ldb * sizeof(double), N * sizeof(double), n,
                                  cudaMemcpyDeviceToDevice, s));
        auto project = [&](double *Y) {
            if (nb <= 0) return;
            gram<double>(basis, ldbs, nb, Y, N, n, N, C, part, s);
            update<double>(Y, N, n, basis, ldbs, nb, C, nb, -1.0, 1.0, N, s);
        };
        auto coldot = [&](const double *A, const double *Bv, double *out) {
            k_cg_coldot<<<dim3(rd.nblk, n), CG_THREADS, 0, s>>>(A, Bv, N, rd.rows_per, part);
            KF_LAUNCH_CHECK();
            k_cg_reduce<<<(n + 127) / 128, 128, 0, s>>>(part, rd.nblk, n, out);
            KF_LAUNCH_CHECK();
        };
        std::vector<double> h(3 * n), ones(n, 1.0);
        auto fetch = [&](const double *d, double *hp, int cnt) {
            KF_CUDA(cudaMemcpyAsync(hp, d, (size_t)cnt * sizeof(double), cudaMemcpyDeviceToHost, s));
            KF_CUDA(cudaStreamSynchronize(s));
        };
        // the right-hand sides' scale (src/resolvent.jl:148-149) and their complement parts
        std::vector<double> scale(n), b(n), cap(n), goal(n);
        if (scale_in) {
            for (int j = 0; j < n; ++j) scale[j] = scale_in[j];
        } else {
            colnorms2<double>(QB, N, n, N, d_rn2, part, s);
            fetch(d_rn2, scale.data(), n);
            for (double &v : scale) v = std::sqrt(v);
        }
        project(QB);
        colnorms2<double>(QB, N, n, N, d_rn2, part, s);
        fetch(d_rn2, b.data(), n);
        std::vector<char> met(n, 0), atfloor(n, 0), from_start(n, 0);
        const double eps = std::numeric_limits<double>::epsilon();
        for (int j = 0; j < n; ++j) {
            b[j] = std::sqrt(b[j]);
            cap[j] = CG_FLOOR_CAP * eps * scale[j];
            goal[j] = tol * b[j];
            if (b[j] <= cap[j]) from_start[j] = atfloor[j] = 1;
        }
        // x_j = 0 exactly for the columns converged from the start
        std::vector<double> keep(n);
        for (int j = 0; j < n; ++j) keep[j] = atfloor[j] ? 0.0 : 1.0;
        KF_CUDA(cudaMemcpyAsync(d_beta, keep.data(), (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s));
        scale_columns<double>(QB, N, n, N, d_beta, s);
        KF_CUDA(cudaMemsetAsync(X, 0, blk, s));
        KF_CUDA(cudaMemcpyAsync(R, QB, blk, cudaMemcpyDeviceToDevice, s));
        k_cg_precond<<<ew_grid(N * n), CG_THREADS, 0, s>>>(Z, R, Mi, N * n);
        KF_LAUNCH_CHECK();
        project(Z);
        KF_CUDA(cudaMemcpyAsync(P, Z, blk, cudaMemcpyDeviceToDevice, s));
        coldot(R, Z, d_rho);
        std::vector<double> rho(n), rn(b), anchor(n, INFINITY), hk(n), hr(n), hrn(n);
        std::vector<int> stalled(n, 0);
        fetch(d_rho, rho.data(), n);
        auto done = [&]() {
            for (int j = 0; j < n; ++j)
                if (!met[j] && !atfloor[j]) return false;
            return true;
        };
        // ||Q (H - s) X - Q B|| per column, with a fresh application of H
        auto true_residuals = [&](std::vector<double> &tr) {
            launch_apply(op, false, X, T, N, N, n, 1.0, 0.0, nullptr, 0, 0.0, s);
            k_cg_axpy_cols<<<ew_grid(N * n), CG_THREADS, 0, s>>>(T, X, d_s, -1.0, N, n);
            KF_LAUNCH_CHECK();
            project(T);
            KF_CUDA(cudaMemcpyAsync(d_beta, ones.data(), (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s));
            k_cg_axpy_cols<<<ew_grid(N * n), CG_THREADS, 0, s>>>(T, QB, d_beta, -1.0, N, n);
            KF_LAUNCH_CHECK();
            colnorms2<double>(T, N, n, N, d_rn2, part, s);
            tr.resize(n);
            fetch(d_rn2, tr.data(), n);
            for (double &v : tr) v = std::sqrt(v);
        };
        int it = 0;
        std::vector<double> act(n), tr;
        while (!done() && it < maxiter) {
            ++it;
            for (int j = 0; j < n; ++j) act[j] = (met[j] || atfloor[j]) ? 0.0 : 1.0;
            KF_CUDA(cudaMemcpyAsync(d_active, act.data(), (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s));
            KF_CUDA(cudaMemcpyAsync(d_rho, rho.data(), (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s));
            launch_apply(op, false, P, AP, N, N, n, 1.0, 0.0, nullptr, 0, 0.0, s);
            k_cg_axpy_cols<<<ew_grid(N * n), CG_THREADS, 0, s>>>(AP, P, d_s, -1.0, N, n);
            KF_LAUNCH_CHECK();
            project(AP);
            coldot(P, AP, d_kappa);
            k_cg_alpha<<<(n + 127) / 128, 128, 0, s>>>(d_rho, d_kappa, d_active, d_alpha, n);
            KF_LAUNCH_CHECK();
            k_cg_step<<<dim3(rd.nblk, n), CG_THREADS, 0, s>>>(X, R, P, AP, d_alpha, N, rd.rows_per, part);
            KF_LAUNCH_CHECK();
            k_cg_reduce<<<(n + 127) / 128, 128, 0, s>>>(part, rd.nblk, n, d_rn2);
            KF_LAUNCH_CHECK();
            k_cg_precond<<<ew_grid(N * n), CG_THREADS, 0, s>>>(Z, R, Mi, N * n);
            KF_LAUNCH_CHECK();
            project(Z);
            coldot(R, Z, d_rhon);
            // kappa, ||R||^2 and rho' in one wait (they sit next to each other)
            fetch(d_kappa, h.data(), 3 * n);
            for (int j = 0; j < n; ++j) {
                hk[j] = h[j];
                hrn[j] = h[n + j];
                hr[j] = h[2 * n + j];
            }
            // the positivity check (src/resolvent.jl:193-201), on the residual before this step
            for (int j = 0; j < n; ++j) {
                if (met[j] || atfloor[j] || hk[j] > 0) continue;
                if (rn[j] <= cap[j]) {
                    atfloor[j] = 1;   // alpha was 0 on the device: X and R are unchanged
                    continue;
                }
                throw Error(KF_EBREAKDOWN,
                            "the linear solve on the complement is not positive on the complement at column " +
                                std::to_string(j + 1) + " (<p, (H - s) p> = " + std::to_string(hk[j]) + " after " +
                                std::to_string(it) + " iterations)");
            }
            std::vector<char> active(n);
            for (int j = 0; j < n; ++j) active[j] = act[j] != 0.0 && !atfloor[j];
            for (int j = 0; j < n; ++j) rn[j] = std::sqrt(hrn[j]);
            bool any_near = false;
            for (int j = 0; j < n; ++j) {
                if (active[j] && rn[j] <= goal[j]) met[j] = 1;
                any_near |= !met[j] && !atfloor[j] && rn[j] <= cap[j];
            }
            if (any_near) {
                true_residuals(tr);
                for (int j = 0; j < n; ++j) {
                    if (met[j] || atfloor[j] || rn[j] > cap[j]) continue;
                    if (tr[j] < anchor[j] / 2) {
                        anchor[j] = tr[j];
                        stalled[j] = 0;
                    } else {
                        ++stalled[j];
                    }
                    if (stalled[j] >= CG_FLOOR_PATIENCE && tr[j] <= cap[j]) atfloor[j] = 1;
                }
            }
            if (done()) break;
            std::vector<double> beta(n);
            for (int j = 0; j < n; ++j) beta[j] = (met[j] || atfloor[j]) ? 0.0 : hr[j] / rho[j];
            KF_CUDA(cudaMemcpyAsync(d_beta, beta.data(), (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s));
            k_cg_dir<<<ew_grid(N * n), CG_THREADS, 0, s>>>(P, Z, d_beta, N, n);
            KF_LAUNCH_CHECK();
            rho = hr;
        }
        true_residuals(tr);
        for (int j = 0; j < n; ++j)
            if (!met[j] && !atfloor[j] && tr[j] <= cap[j]) atfloor[j] = 1;
        if (!done()) {
            int j = 0;
            while (met[j] || atfloor[j]) ++j;
            throw Error(KF_ENOCONV, "the linear solve on the complement did not converge at column " +
                                        std::to_string(j + 1) + ": residual " + std::to_string(rn[j] / b[j]) +
                                        " relative to its complement part after " + std::to_string(it) +
                                        " iterations (tolerance " + std::to_string(tol) + ", at most " +
                                        std::to_string(maxiter) + " iterations)");
        }
        std::vector<char> met0(met);
        for (int j = 0; j < n; ++j) {
            if (from_start[j]) continue;
            if (met[j] && tr[j] > 10 * goal[j]) {
                met[j] = 0;
                atfloor[j] = 1;   // the recurrence went below the true floor
            }
            if (atfloor[j] && tr[j] > cap[j])
                throw Error(KF_ENOCONV, std::string("the linear solve on the complement did not converge at column ") +
                                            std::to_string(j + 1) + ": " +
                                            (met0[j] ? "it met its tolerance by the recurrence, but its true residual "
                                                       "is above 10 x tol, and "
                                                     : "it stopped at the round-off floor, but ") +
                                            "its final true residual " + std::to_string(tr[j] / scale[j]) +
                                            " relative to the right-hand side is above the round-off cap");
        }
        res.iterations = it;
        res.state.assign(n, 0);
        res.residuals.assign(n, 0.0);
        res.floor_residuals.assign(n, 0.0);
        for (int j = 0; j < n; ++j) {
            if (from_start[j]) {
                res.state[j] = 1;
            } else if (atfloor[j]) {
                res.state[j] = 2;
                res.floor_residuals[j] = tr[j] / scale[j];
            } else {
                res.residuals[j] = tr[j] / b[j];
            }
        }
        KF_CUDA(cudaMemcpy2DAsync(X_out, ldx * sizeof(double), X, N * sizeof(double), N * sizeof(double), n,
                                  cudaMemcpyDeviceToDevice, s));
        KF_CUDA(cudaStreamSynchronize(s));
    } catch (...) {
        cleanup();
        throw;
    }
    cleanup();
}

}  // namespace kf

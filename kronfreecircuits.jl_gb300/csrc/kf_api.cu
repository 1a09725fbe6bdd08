// extern "C" entry points of libkfgpu.so (declared in include/kfgpu.h).  Each converts a
// kf::Error (or any C++ exception) into its status code and records the message for
// kf_last_error; nothing throws across the C boundary.
#include <cstring>
#include <limits>

#include <cmath>

#include "kf_internal.h"
#include "../../include/kfgpu_testing.h"

namespace kf {
void build_op(const kf_op_desc *desc, kf_op *op);
void free_op(kf_op *op);
void solve_dispatch(kf_op *op, const kf_solver_opts &o, int m, const double *X0, const double *seed, double *E_out,
                    double *V_out, kf_solve_stats &st);

std::atomic<uint64_t> g_launches{0};
static thread_local std::string g_last_error;
void set_last_error(const std::string &msg) { g_last_error = msg; }

template <typename F>
static int guarded(F &&f) {
    try {
        f();
        return KF_OK;
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::bad_alloc &) {
        set_last_error("host allocation failed");
        return KF_ENOMEM;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return KF_EINVAL;
    }
}
}  // namespace kf

using namespace kf;

extern "C" {

int kf_version(void) { return KFGPU_VERSION; }

int kf_launch_count(uint64_t *count) {
    if (!count) return KF_EINVAL;
    *count = g_launches.load(std::memory_order_relaxed);
    return KF_OK;
}

int kf_last_error(char *buf, size_t len) {
    if (!buf || len == 0) return KF_EINVAL;
    std::strncpy(buf, g_last_error.c_str(), len - 1);
    buf[len - 1] = '\0';
    return KF_OK;
}

int kf_op_create(const kf_op_desc *desc, kf_op **out) {
    return guarded([&] {
        KF_REQUIRE(out != nullptr, KF_EINVAL, "kf_op_create: out is NULL");
        *out = nullptr;
        kf_op *op = new kf_op();
        try {
            KF_CUDA(cudaGetDevice(&op->device));
            KF_CUDA(cudaStreamCreateWithFlags(&op->stream, cudaStreamNonBlocking));
            build_op(desc, op);   // also starts the preconditioner's host job
        } catch (...) {
            free_op(op);
            delete op;
            throw;
        }
        *out = op;
    });
}

int kf_op_product_seed(kf_op *op, int32_t k, double *X, int32_t flags) {
    return guarded([&] {
        KF_REQUIRE(op && X, KF_EINVAL, "kf_op_product_seed: NULL argument");
        if (flags & KF_HOST) {
            const size_t bytes = sizeof(double) * (size_t)op->N * (size_t)std::max(k, 0);
            KF_REQUIRE(k >= 1 && k <= op->N, KF_EINVAL,
                       "product_seed: k must lie in 1:" + std::to_string(op->N) + " (the operator's dimension), got " +
                           std::to_string(k));
            double *d = nullptr;
            KF_CUDA(cudaMallocAsync((void **)&d, bytes, op->stream));
            try {
                kf::product_seed_device(op, k, d, op->stream);
                KF_CUDA(cudaMemcpyAsync(X, d, bytes, cudaMemcpyDeviceToHost, op->stream));
                KF_CUDA(cudaStreamSynchronize(op->stream));
            } catch (...) {
                cudaFreeAsync(d, op->stream);
                throw;
            }
            KF_CUDA(cudaFreeAsync(d, op->stream));
        } else {
            kf::product_seed_device(op, k, X, op->stream);
        }
    });
}

int kf_op_destroy(kf_op *op) {
    return guarded([&] {
        if (!op) return;
        cudaStreamSynchronize(op->stream);
        free_op(op);
        delete op;
    });
}

int kf_op_size(const kf_op *op, int64_t *n) {
    return guarded([&] {
        KF_REQUIRE(op && n, KF_EINVAL, "kf_op_size: NULL argument");
        *n = op->N;
    });
}

static bool ranges_overlap(const void *a, size_t na, const void *b, size_t nb) {
    const char *pa = (const char *)a, *pb = (const char *)b;
    return pa < pb + nb && pb < pa + na;
}

int kf_op_apply(kf_op *op, const void *X, void *Y, int64_t ldx, int64_t ldy, int64_t b, int32_t flags) {
    return guarded([&] {
        KF_REQUIRE(op != nullptr, KF_EINVAL, "kf_op_apply: op is NULL");
        const int64_t N = op->N;
        KF_REQUIRE(b >= 0, KF_EDIM, "mul!: negative block width");
        KF_REQUIRE(ldx >= N && ldy >= N, KF_EDIM,
                   "KronFreeOperator of size (" + std::to_string(N) + ", " + std::to_string(N) +
                       ") applied to x with " + std::to_string(ldx) + " rows");
        if (b == 0) return;
        KF_REQUIRE(X && Y, KF_EINVAL, "kf_op_apply: NULL block");
        const size_t es = (flags & KF_F32) ? 4 : 8;
        const size_t bx = ((size_t)(b - 1) * ldx + N) * es, by = ((size_t)(b - 1) * ldy + N) * es;
        KF_REQUIRE(!ranges_overlap(X, bx, Y, by), KF_EALIAS, "mul!: y must not alias x");
        cudaStream_t s = op->stream;
        if (flags & KF_HOST) {
            void *dX = nullptr, *dY = nullptr;
            KF_CUDA(cudaMallocAsync(&dX, (size_t)N * b * es, s));
            KF_CUDA(cudaMallocAsync(&dY, (size_t)N * b * es, s));
            KF_CUDA(cudaMemcpy2DAsync(dX, N * es, X, ldx * es, N * es, b, cudaMemcpyHostToDevice, s));
            launch_apply(op, (flags & KF_F32) != 0, dX, dY, N, N, b, 1, 0, nullptr, 0, 0, s);
            KF_CUDA(cudaMemcpy2DAsync(Y, ldy * es, dY, N * es, N * es, b, cudaMemcpyDeviceToHost, s));
            KF_CUDA(cudaFreeAsync(dX, s));
            KF_CUDA(cudaFreeAsync(dY, s));
            KF_CUDA(cudaStreamSynchronize(s));
        } else {
            launch_apply(op, (flags & KF_F32) != 0, X, Y, ldx, ldy, b, 1, 0, nullptr, 0, 0, s);
        }
    });
}

int kf_op_apply_axpby(kf_op *op, const void *X, void *Y, const void *Z, int64_t ld, int64_t b, double alpha,
                      double beta, double gamma, int32_t flags) {
    return guarded([&] {
        KF_REQUIRE(op != nullptr, KF_EINVAL, "kf_op_apply_axpby: op is NULL");
        KF_REQUIRE(!(flags & KF_HOST), KF_EINVAL, "kf_op_apply_axpby: device pointers only");
        KF_REQUIRE(ld >= op->N && b >= 0, KF_EDIM, "kf_op_apply_axpby: bad block shape");
        if (b == 0) return;
        const size_t es = (flags & KF_F32) ? 4 : 8;
        const size_t bx = ((size_t)(b - 1) * ld + op->N) * es;
        KF_REQUIRE(!ranges_overlap(X, bx, Y, bx), KF_EALIAS, "mul!: y must not alias x");
        KF_REQUIRE(Z == nullptr || !ranges_overlap(Z, bx, Y, bx), KF_EALIAS, "kf_op_apply_axpby: y must not alias z");
        launch_apply(op, (flags & KF_F32) != 0, X, Y, ld, ld, b, alpha, beta, Z, ld, Z ? gamma : 0.0, op->stream);
    });
}

int kf_drive_apply(kf_op *H0, double E0, int32_t nports, kf_op *const *ports, kf_op *const *ports_im,
                   const double *coef, const double *omega, double t, const void *X, int64_t ldx, void *Y, int64_t ldy,
                   int64_t m, int32_t flags) {
    return guarded([&] {
        KF_REQUIRE(H0 != nullptr, KF_EINVAL, "kf_drive_apply: H0 is NULL");
        KF_REQUIRE(!(flags & KF_F32), KF_EINVAL, "kf_drive_apply: time evolution runs in FP64");
        KF_REQUIRE(nports >= 0 && (nports == 0 || ((ports || ports_im) && coef)), KF_EINVAL,
                   "kf_drive_apply: bad port list");
        const int64_t N = H0->N;
        for (int k = 0; k < nports; ++k) {
            kf_op *re = ports ? ports[k] : nullptr, *im = ports_im ? ports_im[k] : nullptr;
            KF_REQUIRE(re != nullptr || im != nullptr, KF_EINVAL,
                       "kf_drive_apply: port operator " + std::to_string(k) + " has neither component");
            for (kf_op *o : {re, im})
                KF_REQUIRE(o == nullptr || (o->N == N && o->dims == H0->dims), KF_EDIM,
                           "drive_hamiltonian: port operator " + std::to_string(k) + " is not on H0's product basis");
            KF_REQUIRE(std::isfinite(coef[k]), KF_EINVAL, "kf_drive_apply: coefficient " + std::to_string(k) +
                                                              " is not finite");
        }
        KF_REQUIRE(m >= 0, KF_EDIM, "kf_drive_apply: negative block width");
        KF_REQUIRE(ldx >= N && ldy >= N, KF_EDIM, "kf_drive_apply: leading dimension below the operator's size");
        KF_REQUIRE(std::isfinite(E0) && std::isfinite(t), KF_EINVAL, "kf_drive_apply: E0 and t must be finite");
        if (m == 0 || N == 0) return;
        KF_REQUIRE(X && Y, KF_EINVAL, "kf_drive_apply: NULL block");
        const size_t bx = ((size_t)(2 * m - 1) * ldx + N) * 8, by = ((size_t)(2 * m - 1) * ldy + N) * 8;
        KF_REQUIRE(!ranges_overlap(X, bx, Y, by), KF_EALIAS, "kf_drive_apply: y must not alias x");
        cudaStream_t s = H0->stream;
        if (flags & KF_HOST) {
            double *dX = nullptr, *dY = nullptr, *dW = nullptr;
            KF_CUDA(cudaMallocAsync((void **)&dX, (size_t)N * 2 * m * 8, s));
            KF_CUDA(cudaMallocAsync((void **)&dY, (size_t)N * 2 * m * 8, s));
            if (omega) {
                KF_CUDA(cudaMallocAsync((void **)&dW, (size_t)N * 8, s));
                KF_CUDA(cudaMemcpyAsync(dW, omega, (size_t)N * 8, cudaMemcpyHostToDevice, s));
            }
            KF_CUDA(cudaMemcpy2DAsync(dX, N * 8, X, ldx * 8, N * 8, 2 * m, cudaMemcpyHostToDevice, s));
            kf::drive_apply(H0, E0, nports, ports, ports_im, coef, dW, t, dX, N, dY, N, m);
            KF_CUDA(cudaMemcpy2DAsync(Y, ldy * 8, dY, N * 8, N * 8, 2 * m, cudaMemcpyDeviceToHost, s));
            KF_CUDA(cudaFreeAsync(dX, s));
            KF_CUDA(cudaFreeAsync(dY, s));
            if (dW) KF_CUDA(cudaFreeAsync(dW, s));
            KF_CUDA(cudaStreamSynchronize(s));
        } else {
            kf::drive_apply(H0, E0, nports, ports, ports_im, coef, omega, t, (const double *)X, ldx, (double *)Y, ldy,
                            m);
        }
    });
}

int kf_to_lab(const double *omega, int64_t N, double t, void *X, int64_t ldx, int64_t m, int32_t flags) {
    return guarded([&] {
        KF_REQUIRE(!(flags & KF_F32), KF_EINVAL, "kf_to_lab: time evolution runs in FP64");
        KF_REQUIRE(N >= 0 && m >= 0 && ldx >= N, KF_EDIM, "to_lab: bad block shape");
        KF_REQUIRE(std::isfinite(t), KF_EINVAL, "kf_to_lab: t must be finite");
        if (N == 0 || m == 0) return;
        KF_REQUIRE(omega && X, KF_EINVAL, "kf_to_lab: NULL argument");
        cudaStream_t s = 0;
        if (flags & KF_HOST) {
            double *dX = nullptr, *dW = nullptr;
            KF_CUDA(cudaMalloc((void **)&dX, (size_t)N * 2 * m * 8));
            KF_CUDA(cudaMalloc((void **)&dW, (size_t)N * 8));
            KF_CUDA(cudaMemcpy(dW, omega, (size_t)N * 8, cudaMemcpyHostToDevice));
            KF_CUDA(cudaMemcpy2D(dX, N * 8, X, ldx * 8, N * 8, 2 * m, cudaMemcpyHostToDevice));
            kf::rotate_rows(dW, N, t, -1.0, dX, N, m, s);
            KF_CUDA(cudaMemcpy2D(X, ldx * 8, dX, N * 8, N * 8, 2 * m, cudaMemcpyDeviceToHost));
            cudaFree(dX);
            cudaFree(dW);
        } else {
            kf::rotate_rows(omega, N, t, -1.0, (double *)X, ldx, m, s);
            KF_CUDA(cudaStreamSynchronize(s));
        }
    });
}

int kf_op_sandwich(kf_op *op, const double *W, int64_t ldw, int32_t kw, const double *V, int64_t ldv, int32_t kv,
                   double *P_out, int32_t flags) {
    return guarded([&] {
        KF_REQUIRE(op && V && P_out, KF_EINVAL, "kf_op_sandwich: NULL argument");
        const int64_t N = op->N;
        if (W == nullptr) {
            W = V;
            ldw = ldv;
            kw = kv;
        }
        KF_REQUIRE(kv >= 1 && kw >= 1 && kv <= 4096 && kw <= 4096, KF_EINVAL,
                   "kf_op_sandwich: the blocks must have 1..4096 columns");
        KF_REQUIRE(ldv >= N && ldw >= N, KF_EDIM, "kf_op_sandwich: leading dimensions must be >= N");
        cudaStream_t s = op->stream;
        const bool host = (flags & KF_HOST) != 0;
        double *dV = nullptr, *dW = nullptr, *dY = nullptr, *dG = nullptr, *dpart = nullptr;
        auto cleanup = [&]() {
            if (host) {
                cudaFreeAsync(dV, s);
                if (dW != dV) cudaFreeAsync(dW, s);
            }
            cudaFreeAsync(dY, s);
            cudaFreeAsync(dG, s);
            cudaFreeAsync(dpart, s);
        };
        try {
            const double *Vd = V, *Wd = W;
            int64_t lv = ldv, lw = ldw;
            if (host) {
                KF_CUDA(cudaMallocAsync((void **)&dV, (size_t)N * kv * 8, s));
                KF_CUDA(cudaMemcpy2DAsync(dV, N * 8, V, ldv * 8, N * 8, kv, cudaMemcpyHostToDevice, s));
                Vd = dV;
                lv = N;
                if (W == V) {
                    dW = dV;
                } else {
                    KF_CUDA(cudaMallocAsync((void **)&dW, (size_t)N * kw * 8, s));
                    KF_CUDA(cudaMemcpy2DAsync(dW, N * 8, W, ldw * 8, N * 8, kw, cudaMemcpyHostToDevice, s));
                }
                Wd = dW;
                lw = N;
            }
            KF_CUDA(cudaMallocAsync((void **)&dY, (size_t)N * kv * 8, s));
            KF_CUDA(cudaMallocAsync((void **)&dG, (size_t)kw * kv * 8, s));
            KF_CUDA(cudaMallocAsync((void **)&dpart, kf::gram_partials_size(kw, kv, N), s));
            kf::launch_apply(op, false, Vd, dY, lv, N, kv, 1.0, 0.0, nullptr, 0, 0.0, s);
            kf::gram<double>(Wd, lw, kw, dY, N, kv, N, dG, dpart, s);
            KF_CUDA(cudaMemcpyAsync(P_out, dG, (size_t)kw * kv * 8, cudaMemcpyDeviceToHost, s));
            KF_CUDA(cudaStreamSynchronize(s));
        } catch (...) {
            cleanup();
            throw;
        }
        cleanup();
    });
}

int kf_test_check_word(int32_t *site, int32_t *check_build) {
    return guarded([&] {
        KF_REQUIRE(site && check_build, KF_EINVAL, "kf_test_check_word: NULL argument");
        KF_CUDA(cudaDeviceSynchronize());
        *site = kf::check_take_site();
#ifdef KF_CHECK
        *check_build = 1;
#else
        *check_build = 0;
#endif
    });
}

int kf_test_rr_eig(const double *G, int32_t ldg, int32_t packed, int32_t na, int32_t k, int32_t status, double *C_out,
                   double *theta_out) {
    return guarded([&] {
        KF_REQUIRE(G && C_out && theta_out && na >= 1 && k >= 0 && na + k <= 64, KF_EINVAL,
                   "kf_test_rr_eig: 1 <= na, na + k <= 64");
        const int ns = na + k;
        const size_t gn = packed ? (size_t)na * na + (size_t)na * k + (size_t)k * k : (size_t)ldg * ns;
        KF_REQUIRE(packed || ldg >= ns, KF_EDIM, "kf_test_rr_eig: ldg >= na + k");
        double *dG = nullptr, *dC = nullptr, *dth = nullptr;
        int *dst = nullptr;
        auto cleanup = [&]() {
            cudaFree(dG);
            cudaFree(dC);
            cudaFree(dth);
            cudaFree(dst);
        };
        try {
            KF_CUDA(cudaMalloc(&dG, gn * 8));
            KF_CUDA(cudaMalloc(&dC, (size_t)ns * 2 * na * 8));
            KF_CUDA(cudaMalloc(&dth, (size_t)na * 8));
            KF_CUDA(cudaMalloc(&dst, sizeof(int)));
            KF_CUDA(cudaMemcpy(dG, G, gn * 8, cudaMemcpyHostToDevice));
            KF_CUDA(cudaMemcpy(dst, &status, sizeof(int), cudaMemcpyHostToDevice));
            KF_CUDA(cudaMemcpy(dth, theta_out, (size_t)na * 8, cudaMemcpyHostToDevice));   // in / out
            KF_REQUIRE(kf::rr_eig_device(dG, ldg, packed != 0, na, k, dC, dth, dst, 0), KF_EINVAL, "rr_eig_device refused");
            KF_CUDA(cudaMemcpy(C_out, dC, (size_t)ns * 2 * na * 8, cudaMemcpyDeviceToHost));
            KF_CUDA(cudaMemcpy(theta_out, dth, (size_t)na * 8, cudaMemcpyDeviceToHost));
        } catch (...) {
            cleanup();
            throw;
        }
        cleanup();
    });
}

int kf_complement_solve(kf_op *op, const double *basis, int64_t ldbasis, int32_t nbasis, const double *B, int64_t ldb,
                        int32_t n, const double *shifts, const double *scale, double tol, int32_t maxiter, double eta,
                        double *X, int64_t ldx, int32_t *iterations, int32_t *state, double *residuals,
                        double *floor_residuals, int32_t flags) {
    return guarded([&] {
        KF_REQUIRE(op && B && shifts && X, KF_EINVAL, "kf_complement_solve: NULL argument");
        KF_REQUIRE(n >= 1 && n <= 4096, KF_EINVAL, "kf_complement_solve: 1..4096 right-hand sides");
        KF_REQUIRE(nbasis >= 0 && nbasis <= 4096 && (nbasis == 0 || basis), KF_EINVAL,
                   "kf_complement_solve: the basis must have 0..4096 columns");
        KF_REQUIRE(tol > 0 && maxiter >= 0 && eta >= 0, KF_EINVAL, "kf_complement_solve: tol > 0, maxiter >= 0, eta >= 0");
        const int64_t N = op->N;
        KF_REQUIRE(ldb >= N && ldx >= N && (nbasis == 0 || ldbasis >= N), KF_EDIM,
                   "kf_complement_solve: leading dimensions must be >= N");
        KF_REQUIRE(nbasis < N, KF_EDIM, "kf_complement_solve: the basis must leave a complement");
        cudaStream_t s = op->stream;
        const bool host = (flags & KF_HOST) != 0;
        double *dB = nullptr, *dV = nullptr, *dX = nullptr;
        auto cleanup = [&]() {
            cudaFreeAsync(dB, s);
            cudaFreeAsync(dV, s);
            cudaFreeAsync(dX, s);
        };
        kf::CgResult r;
        try {
            const double *Bd = B, *Vd = basis;
            double *Xd = X;
            int64_t lb = ldb, lv = ldbasis, lx = ldx;
            if (host) {
                KF_CUDA(cudaMallocAsync((void **)&dB, (size_t)N * n * 8, s));
                KF_CUDA(cudaMemcpy2DAsync(dB, N * 8, B, ldb * 8, N * 8, n, cudaMemcpyHostToDevice, s));
                Bd = dB;
                lb = N;
                if (nbasis > 0) {
                    KF_CUDA(cudaMallocAsync((void **)&dV, (size_t)N * nbasis * 8, s));
                    KF_CUDA(cudaMemcpy2DAsync(dV, N * 8, basis, ldbasis * 8, N * 8, nbasis, cudaMemcpyHostToDevice, s));
                    Vd = dV;
                    lv = N;
                }
                KF_CUDA(cudaMallocAsync((void **)&dX, (size_t)N * n * 8, s));
                Xd = dX;
                lx = N;
            }
            kf::complement_solve(op, Vd, lv, nbasis, Bd, lb, n, shifts, scale, tol, maxiter, eta, Xd, lx, r, s);
            if (host) {
                KF_CUDA(cudaMemcpy2DAsync(X, ldx * 8, dX, N * 8, N * 8, n, cudaMemcpyDeviceToHost, s));
                KF_CUDA(cudaStreamSynchronize(s));
            }
        } catch (...) {
            cleanup();
            throw;
        }
        cleanup();
        if (iterations) *iterations = r.iterations;
        for (int j = 0; j < n; ++j) {
            if (state) state[j] = r.state[j];
            if (residuals) residuals[j] = r.residuals[j];
            if (floor_residuals) floor_residuals[j] = r.floor_residuals[j];
        }
    });
}

int kf_op_diagonal(kf_op *op, double *out) {
    return guarded([&] {
        KF_REQUIRE(op && out, KF_EINVAL, "kf_op_diagonal: NULL argument");
        std::memcpy(out, op->h_fulldiag.data(), sizeof(double) * op->N);
    });
}

int kf_op_gershgorin(kf_op *op, double *out) {
    return guarded([&] {
        KF_REQUIRE(op && out, KF_EINVAL, "kf_op_gershgorin: NULL argument");
        *out = op->gershgorin;
    });
}

int kf_op_get_stream(kf_op *op, void **stream) {
    return guarded([&] {
        KF_REQUIRE(op && stream, KF_EINVAL, "kf_op_get_stream: NULL argument");
        *stream = (void *)op->stream;
    });
}

int kf_op_set_stream(kf_op *op, void *stream) {
    return guarded([&] {
        KF_REQUIRE(op != nullptr, KF_EINVAL, "kf_op_set_stream: op is NULL");
        KF_CUDA(cudaStreamSynchronize(op->stream));
        if (op->own_stream) KF_CUDA(cudaStreamDestroy(op->stream));
        op->stream = (cudaStream_t)stream;
        op->own_stream = false;
    });
}

int kf_op_sync(kf_op *op) {
    return guarded([&] {
        KF_REQUIRE(op != nullptr, KF_EINVAL, "kf_op_sync: op is NULL");
        KF_CUDA(cudaStreamSynchronize(op->stream));
    });
}

void kf_solver_opts_default(kf_solver_opts *o, int32_t kind) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->kind = kind;
    o->precision = KF_PREC_F64;
    o->tol = kind == KF_SOLVER_LANCZOS ? 1e-10 : 1e-8;
    o->maxiter = kind == KF_SOLVER_LOBPCG ? 1000 : kind == KF_SOLVER_CHEBYSHEV ? 50 : 1000;
    o->preconditioner = KF_PRECOND_RITZ;
    o->eta = 0.01;
    o->guard = 4;
    o->degree = 100;
    o->extra = 40;
    o->rescale_every = 20;
    o->ortho = KF_ORTHO_SVQB;
    o->bound = std::numeric_limits<double>::quiet_NaN();
    o->krylovdim = 0;
    o->rng_seed = 0x4b46;
    o->mixed_switch = 1e-6;   // measured: 1e-6 126.5, 1.5e-6 123.2, 2e-6 122.9, 5e-7 91.4 eigenpairs/s
    o->fallback_iters = 3;
    o->fallback_resid = 0.0;
    o->seed_kind = KF_SEED_PRODUCT;
    o->buffer = KF_BUFFER_AUTO;
}

int kf_solve(kf_op *op, const kf_solver_opts *opts, int32_t m, const double *X0, const double *seed, double *E_out,
             double *V_out, kf_solve_stats *stats) {
    return guarded([&] {
        KF_REQUIRE(op && opts, KF_EINVAL, "kf_solve: NULL argument");
        kf_solve_stats st;
        try {
            solve_dispatch(op, *opts, m, X0, seed, E_out, V_out, st);
        } catch (...) {
            if (stats) *stats = st;
            throw;
        }
        if (stats) *stats = st;
    });
}

// ---- test-only entry points (include/kfgpu_testing.h) ----------------------------------

int kf_test_mode_product(int path, const float *X, float *Y, const double *A, int d, int64_t left, int64_t N,
                         int64_t b, double alpha, double beta, void *stream) {
    return guarded([&] {
        KF_REQUIRE(X && Y && A, KF_EINVAL, "kf_test_mode_product: NULL argument");
        KF_REQUIRE(d >= 1 && left >= 1 && N % d == 0 && (N / d) % left == 0, KF_EDIM,
                   "kf_test_mode_product: N must be a multiple of d * left");
        cudaStream_t s = (cudaStream_t)stream;
        if (path == 1 || path == 2) {
            kf::TcMatrix m = kf::tc_matrix_create(A, d, false, path == 2);
            kf::tc_mode_product(Y, N, X, N, m, left, N, b, alpha, beta, s);
            const cudaError_t e = cudaStreamSynchronize(s);
            kf::tc_matrix_free(m);
            KF_CUDA(e);
            if (const int t = kf::tc_take_error()) throw kf::Error(t, "tensor-core mode product: device wait timed out");
        } else {
            std::vector<float> a32((size_t)d * d);
            for (size_t i = 0; i < a32.size(); ++i) a32[i] = (float)A[i];
            float *dA = nullptr;
            KF_CUDA(cudaMalloc(&dA, a32.size() * 4));
            KF_CUDA(cudaMemcpy(dA, a32.data(), a32.size() * 4, cudaMemcpyHostToDevice));
            kf::mode_product<float>(Y, N, X, N, dA, d, left, N, b, alpha, beta, s);
            const cudaError_t e = cudaStreamSynchronize(s);
            cudaFree(dA);
            KF_CUDA(e);
        }
    });
}

int kf_test_time_mode_product(int path, const float *X, float *Y, const double *A, int d, int64_t left, int64_t N,
                              int64_t b, int reps, void *stream, float *ms_per_launch) {
    return guarded([&] {
        KF_REQUIRE(X && Y && A && ms_per_launch && reps >= 1, KF_EINVAL, "kf_test_time_mode_product: bad argument");
        KF_REQUIRE(d >= 1 && left >= 1 && N % d == 0 && (N / d) % left == 0, KF_EDIM,
                   "kf_test_time_mode_product: N must be a multiple of d * left");
        cudaStream_t s = (cudaStream_t)stream;
        kf::TcMatrix m;
        float *dA = nullptr;
        if (path == 1 || path == 2) {
            m = kf::tc_matrix_create(A, d, false, path == 2);
        } else {
            std::vector<float> a32((size_t)d * d);
            for (size_t i = 0; i < a32.size(); ++i) a32[i] = (float)A[i];
            KF_CUDA(cudaMalloc(&dA, a32.size() * 4));
            KF_CUDA(cudaMemcpy(dA, a32.data(), a32.size() * 4, cudaMemcpyHostToDevice));
        }
        auto launch = [&] {
            if (path == 1 || path == 2) kf::tc_mode_product(Y, N, X, N, m, left, N, b, 1.0, 0.0, s);
            else kf::mode_product<float>(Y, N, X, N, dA, d, left, N, b, 1.0, 0.0, s);
        };
        cudaEvent_t e0, e1;
        KF_CUDA(cudaEventCreate(&e0));
        KF_CUDA(cudaEventCreate(&e1));
        launch();   // warm
        KF_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < reps; ++r) launch();
        KF_CUDA(cudaEventRecord(e1, s));
        KF_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        KF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (path == 1 || path == 2) kf::tc_matrix_free(m);
        else cudaFree(dA);
        if (const int t = kf::tc_take_error()) throw kf::Error(t, "tensor-core mode product: device wait timed out");
        *ms_per_launch = ms / reps;
    });
}

int kf_test_time_gram(int path, const float *A, int64_t lda, int ka, const float *B, int64_t ldb, int kb, int64_t N,
                      int reps, void *stream, float *ms_per_launch, double *G_out) {
    return guarded([&] {
        KF_REQUIRE(A && B && ms_per_launch && reps >= 1 && N >= 1, KF_EINVAL, "kf_test_time_gram: bad argument");
        KF_REQUIRE(lda >= N && ldb >= N, KF_EDIM, "kf_test_time_gram: leading dimensions must be >= N");
        cudaStream_t s = (cudaStream_t)stream;
        double *G = nullptr, *part = nullptr;
        KF_CUDA(cudaMalloc(&G, (size_t)ka * kb * sizeof(double)));
        KF_CUDA(cudaMalloc(&part, kf::gram_partials_size(ka, kb, N)));
        cudaEvent_t e0, e1;
        KF_CUDA(cudaEventCreate(&e0));
        KF_CUDA(cudaEventCreate(&e1));
        KF_REQUIRE(path == 0 || path == 1, KF_EINVAL, "kf_test_time_gram: path must be 0 or 1");
        kf::gram<float>(A, lda, ka, B, ldb, kb, N, G, part, s, path == 0);   // warm
        KF_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < reps; ++r) kf::gram<float>(A, lda, ka, B, ldb, kb, N, G, part, s, path == 0);
        KF_CUDA(cudaEventRecord(e1, s));
        KF_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        KF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (G_out) KF_CUDA(cudaMemcpy(G_out, G, (size_t)ka * kb * sizeof(double), cudaMemcpyDeviceToHost));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(G);
        cudaFree(part);
        *ms_per_launch = ms / reps;
    });
}

int kf_test_gram_tc(const float *const *srcs, const int64_t *lds, const int32_t *ks, int32_t nsrc, int32_t r0,
                    int32_t r1, int32_t c0, int32_t c1, int64_t N, int32_t reps, void *stream,
                    float *ms_per_launch, double *G_out) {
    return guarded([&] {
        KF_REQUIRE(srcs && lds && ks && ms_per_launch && reps >= 1 && N >= 1 && nsrc >= 1 && nsrc <= 4, KF_EINVAL,
                   "kf_test_gram_tc: bad argument");
        KF_REQUIRE(r0 >= 0 && r0 < r1 && r1 <= nsrc && c0 >= 0 && c0 < c1 && c1 <= nsrc, KF_EINVAL,
                   "kf_test_gram_tc: source ranges out of bounds");
        std::vector<kf::GramTcSrc> src(nsrc);
        for (int q = 0; q < nsrc; ++q) {
            KF_REQUIRE(srcs[q] && ks[q] >= 1 && lds[q] >= N, KF_EINVAL, "kf_test_gram_tc: bad source block");
            src[q] = {srcs[q], lds[q], ks[q]};
        }
        int nr = 0, nc = 0;
        for (int q = r0; q < r1; ++q) nr += ks[q];
        for (int q = c0; q < c1; ++q) nc += ks[q];
        cudaStream_t s = (cudaStream_t)stream;
        double *G = nullptr;
        void *part = nullptr;
        const size_t pb = kf::gram_tc_partials_size(nr, nc);
        KF_CUDA(cudaMalloc(&G, (size_t)nr * nc * sizeof(double)));
        KF_CUDA(cudaMalloc(&part, pb));
        auto run = [&] { return kf::gram_tc(src.data(), nsrc, r0, r1, c0, c1, N, G, part, pb, s); };
        bool ok = run();   // warm
        cudaEvent_t e0, e1;
        KF_CUDA(cudaEventCreate(&e0));
        KF_CUDA(cudaEventCreate(&e1));
        KF_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; ok && r < reps; ++r) run();
        KF_CUDA(cudaEventRecord(e1, s));
        KF_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        KF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ok && G_out) KF_CUDA(cudaMemcpy(G_out, G, (size_t)nr * nc * sizeof(double), cudaMemcpyDeviceToHost));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(G);
        cudaFree(part);
        if (const int e = kf::tc_take_error()) throw kf::Error(e, "kf_test_gram_tc: the tensor-core Gram timed out");
        KF_REQUIRE(ok, KF_EINVAL, "kf_test_gram_tc: the shapes do not fit the tensor-core Gram");
        *ms_per_launch = ms / reps;
    });
}

int kf_test_sym_eig(int n, const double *A, int lda, double *w, double *V, int ldv) {
    return guarded([&] {
        KF_REQUIRE(n >= 0 && (n == 0 || (A && w && V && lda >= n && ldv >= n)), KF_EINVAL,
                   "kf_test_sym_eig: bad argument");
        if (kf::sym_eig(n, A, lda, w, V, ldv) != 0)
            throw kf::Error(KF_EBREAKDOWN, "kf_test_sym_eig: the QR iteration did not converge");
    });
}

int kf_test_op_scratch_bytes(const kf_op *op, uint64_t *bytes) {
    return guarded([&] {
        KF_REQUIRE(op && bytes, KF_EINVAL, "kf_test_op_scratch_bytes: NULL argument");
        *bytes = (uint64_t)op->scratch_bytes;
    });
}

int kf_test_march_plan(const kf_op *op, int64_t b, int32_t f32, int32_t sms, int32_t *eligible, int32_t *geom) {
    return guarded([&] {
        KF_REQUIRE(op && eligible && b >= 1 && sms >= 0, KF_EINVAL, "kf_test_march_plan: bad argument");
        if (sms == 0) KF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, op->device));
        kf::MarchPlan mp;
        const size_t es = f32 ? 4 : 8;
        const bool ok = kf::march_plan(op, b, es, sms, mp);
        *eligible = ok ? 1 : 0;
        if (geom && ok) {
            const int32_t g[16] = {mp.P, mp.nm, mp.nouter, mp.H, mp.R, mp.TQ, mp.ntile, mp.grid, mp.NR, mp.SLX,
                                   mp.SLD, mp.nsm, mp.ms, mp.pt, mp.flat,
                                   (int32_t)kf::march_smem_bytes(mp, es, mp.wn, mp.ms)};
            for (int i = 0; i < 16; ++i) geom[i] = g[i];
        }
    });
}

int kf_test_chol2(const double *G, int wx, int r, double *C_out, int *status_out) {
    return guarded([&] {
        KF_REQUIRE(G && C_out && status_out && wx >= 0 && r >= 1 && r <= kf::CHOL2_MAX_R, KF_EINVAL,
                   "kf_test_chol2: bad argument");
        double *dG = nullptr, *dC = nullptr;
        int *dst = nullptr;
        const size_t ng = (size_t)(wx + r) * r, nc = (size_t)(r + wx) * r;
        KF_CUDA(cudaMalloc(&dG, ng * sizeof(double)));
        KF_CUDA(cudaMalloc(&dC, nc * sizeof(double)));
        KF_CUDA(cudaMalloc(&dst, sizeof(int)));
        KF_CUDA(cudaMemcpy(dG, G, ng * sizeof(double), cudaMemcpyHostToDevice));
        kf::chol2_coeffs(dG, wx, r, dC, dst, nullptr);
        KF_CUDA(cudaMemcpy(C_out, dC, nc * sizeof(double), cudaMemcpyDeviceToHost));
        KF_CUDA(cudaMemcpy(status_out, dst, sizeof(int), cudaMemcpyDeviceToHost));
        cudaFree(dG);
        cudaFree(dC);
        cudaFree(dst);
    });
}

int kf_test_update_split(int path, float *Y0, int ky0, float *Y1, int ky1, const float *X0, int kx0, const float *X1,
                         int kx1, const double *C, double alpha, double beta, int64_t N, int64_t ld) {
    return guarded([&] {
        KF_REQUIRE(Y0 && X0 && C && N >= 1 && ld >= N && ky0 >= 1 && ky1 >= 0 && kx0 >= 1 && kx1 >= 0 &&
                       (path == 0 || path == 1),
                   KF_EINVAL, "kf_test_update_split: bad argument");
        const int kx = kx0 + kx1, ky = ky0 + ky1;
        double *dC = nullptr;
        KF_CUDA(cudaMalloc(&dC, sizeof(double) * (size_t)kx * ky));
        KF_CUDA(cudaMemcpy(dC, C, sizeof(double) * (size_t)kx * ky, cudaMemcpyHostToDevice));
        bool ok = true;
        if (path == 1) {
            KF_REQUIRE(kf::update_tc_ok(kx, ky), KF_EINVAL, "kf_test_update_split: the shapes do not fit the kernel");
            kf::update_tc2(Y0, ld, ky0, Y1, ld, ky1, X0, ld, kx0, X1, ld, kx1, dC, kx, alpha, beta, N, nullptr, -1);
        } else {
            ok = kf::update_pipe(Y0, ld, ky0, Y1, ld, ky1, X0, ld, kx0, X1, ld, kx1, dC, kx, alpha, beta, N, nullptr);
        }
        KF_CUDA(cudaDeviceSynchronize());
        cudaFree(dC);
        KF_REQUIRE(ok, KF_EINVAL, "kf_test_update_split: the shapes do not fit the pipelined kernel");
    });
}

int kf_test_update_f64(int path, double *Y, const double *X, int kx, int ky, const double *C, int64_t N, int reps,
                       void *stream, float *ms_per_launch) {
    return guarded([&] {
        KF_REQUIRE(Y && X && C && ms_per_launch && reps >= 1 && N >= 1 && kx >= 1 && ky >= 1, KF_EINVAL,
                   "kf_test_update_f64: bad argument");
        KF_REQUIRE(path == 0 || (path == 1 && kx <= 32 && ky <= 32), KF_EINVAL, "kf_test_update_f64: bad path");
        cudaStream_t s = (cudaStream_t)stream;
        double *dC = nullptr;
        KF_CUDA(cudaMalloc(&dC, sizeof(double) * (size_t)kx * ky));
        KF_CUDA(cudaMemcpy(dC, C, sizeof(double) * (size_t)kx * ky, cudaMemcpyHostToDevice));
        auto launch = [&] {
            if (path == 1) (void)kf::update_f64_df(Y, N, ky, X, N, kx, dC, kx, N, s);
            else kf::update<double>(Y, N, ky, X, N, kx, dC, kx, 1.0, 0.0, N, s);
        };
        launch();
        cudaEvent_t e0, e1;
        KF_CUDA(cudaEventCreate(&e0));
        KF_CUDA(cudaEventCreate(&e1));
        KF_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < reps; ++r) launch();
        KF_CUDA(cudaEventRecord(e1, s));
        KF_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        KF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(dC);
        *ms_per_launch = ms / reps;
    });
}

int kf_test_update(int path, float *Y, int64_t ldy, int ky, const float *X0, int64_t ldx0, int kx0, const float *X1,
                   int64_t ldx1, int kx1, const double *C, int ldc, double alpha, double beta, int64_t N, int reps,
                   void *stream, float *ms_per_launch) {
    return guarded([&] {
        KF_REQUIRE(Y && X0 && C && ms_per_launch && reps >= 1 && N >= 1 && ky >= 1 && kx0 >= 1 && kx1 >= 0,
                   KF_EINVAL, "kf_test_update: bad argument");
        KF_REQUIRE(kx1 == 0 || X1, KF_EINVAL, "kf_test_update: X1 is NULL");
        KF_REQUIRE(path >= 0 && path <= 4, KF_EINVAL, "kf_test_update: bad path");
        cudaStream_t s = (cudaStream_t)stream;
        const int kx = kx0 + kx1;
        double *dC = nullptr;
        KF_CUDA(cudaMalloc(&dC, sizeof(double) * (size_t)ldc * ky));
        KF_CUDA(cudaMemcpy(dC, C, sizeof(double) * (size_t)ldc * ky, cudaMemcpyHostToDevice));
        auto launch = [&] {
            // paths 2-4: the tensor-core kernel with its producer mode forced (register gather, two- and
            // three-tile staging rings)
            if (path >= 1)
                kf::update_tc2(Y, ldy, ky, nullptr, 0, 0, X0, ldx0, kx0, X1, ldx1, kx1, dC, ldc, alpha, beta, N, s,
                               path == 1 ? -1 : path == 2 ? 0 : path - 1);
            else kf::update2<float>(Y, ldy, ky, X0, ldx0, kx0, kx1 ? X1 : X0, kx1 ? ldx1 : ldx0, kx1, dC, ldc, alpha,
                                    beta, N, s, false);
        };
        (void)kx;
        cudaEvent_t e0, e1;
        KF_CUDA(cudaEventCreate(&e0));
        KF_CUDA(cudaEventCreate(&e1));
        KF_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < reps; ++r) launch();
        KF_CUDA(cudaEventRecord(e1, s));
        KF_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        KF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(dC);
        if (const int t = kf::tc_take_error()) throw kf::Error(t, "tensor-core update: device wait timed out");
        *ms_per_launch = ms / reps;
    });
}

int kf_test_apply_variant(kf_op *op, int variant, const void *X, void *Y, int64_t ld, int64_t b, int32_t flags,
                          int reps, float *ms_per_launch) {
    return guarded([&] {
        KF_REQUIRE(op && X && Y && variant >= 0 && variant < kf::KF_APPLY_VARIANTS && reps >= 1, KF_EINVAL,
                   "kf_test_apply_variant: bad argument");
        KF_REQUIRE(!(flags & KF_HOST), KF_EINVAL, "kf_test_apply_variant: device blocks only");
        cudaEvent_t e0, e1;
        KF_CUDA(cudaEventCreate(&e0));
        KF_CUDA(cudaEventCreate(&e1));
        op->force_variant = variant;
        float ms = 0;
        try {
            kf::launch_apply(op, (flags & KF_F32) != 0, X, Y, ld, ld, b, 1.0, 0.0, nullptr, 0, 0.0, op->stream);
            KF_CUDA(cudaEventRecord(e0, op->stream));
            for (int r = 0; r < reps; ++r)
                kf::launch_apply(op, (flags & KF_F32) != 0, X, Y, ld, ld, b, 1.0, 0.0, nullptr, 0, 0.0, op->stream);
            KF_CUDA(cudaEventRecord(e1, op->stream));
            KF_CUDA(cudaEventSynchronize(e1));
            KF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        } catch (...) {
            op->force_variant = -1;
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            throw;
        }
        op->force_variant = -1;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (ms_per_launch) *ms_per_launch = ms / reps;
        if (const int t = kf::tc_take_error()) throw kf::Error(t, "plane-marching apply: device wait timed out");
    });
}

}  // extern "C"

/*
 * kfgpu.h -- C ABI of libkfgpu.so, the GB300 (sm_103a) Kronecker-free operator and
 * eigensolver library for KronFreeCircuits.jl.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, and returns an int
 * status (KF_OK = 0).  On failure, kf_last_error() gives the message of the calling thread's
 * last failed call.  Layout everywhere is the reference's: column-major state blocks, axis 1
 * fastest, the block (column) axis last, column j of a block at X + j*ld.
 *
 * Each declaration names the reference interface it replaces (paths within
 * KronFreeCircuits.jl).
 */
#ifndef KFGPU_H
#define KFGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KFGPU_VERSION 1

/* ---- status codes ------------------------------------------------------------------ */
#define KF_OK          0
#define KF_EINVAL      1   /* an argument is invalid (the reference's ArgumentError)           */
#define KF_EDIM        2   /* sizes disagree (DimensionMismatch)                                */
#define KF_EALIAS      3   /* output aliases input (src/apply.jl:412 "y must not alias x")      */
#define KF_ECUDA       4   /* a CUDA runtime call failed                                        */
#define KF_ENOCONV     5   /* an eigensolver did not converge (ErrorException)                  */
#define KF_EBREAKDOWN  6   /* orthogonalization broke down (rank-deficient block)               */
#define KF_ENOMEM      7   /* device allocation failed                                          */
#define KF_ETIMEOUT    8   /* a device-side iteration cap was reached (kernels never spin)      */
#define KF_ENOTFINITE  9   /* a block became non-finite                                         */

/* ---- flags of kf_op_apply ---------------------------------------------------------- */
#define KF_F64     0x0   /* X, Y hold double                                                  */
#define KF_F32     0x1   /* X, Y hold float (the mixed-precision bulk arithmetic)             */
#define KF_DEVICE  0x0   /* X, Y are device pointers; the call is asynchronous on the op's stream */
#define KF_HOST    0x2   /* X, Y are host pointers; copied in and out, the call returns when Y is written */

/* ---- factor structures (src/localops.jl:11-73) -------------------------------------- */
#define KF_DIAG    0   /* DiagonalOp(d):            Y[i] = d[i] X[i]                            */
#define KF_BANDED  1   /* BandedOp(n, offs, w):     Y[i] = sum_b w[b][i] X[i + offs[b]] (valid)  */
#define KF_SHIFT   2   /* ShiftOp(n, s, f):         Y[i + s] = f X[i] (valid)                    */
#define KF_DENSE   3   /* DenseOp(M):               Y[i] = sum_j M[i,j] X[j]                     */

/* One factor of a product term; axis is 0-based (the reference's axis minus one). */
typedef struct {
    int32_t axis;
    int32_t kind;            /* KF_DIAG / KF_BANDED / KF_SHIFT / KF_DENSE                    */
    int64_t n;               /* the axis length (dimension(op))                              */
    const double *data;      /* DIAG: n values.  BANDED: nbands*n weights, band-major
                                (data[b*n + i] = weights[b][i]).  DENSE: n*n, column-major.  */
    const int64_t *offsets;  /* BANDED: nbands offsets                                       */
    int32_t nbands;          /* BANDED                                                       */
    int64_t shift;           /* SHIFT: s                                                     */
    double factor;           /* SHIFT: the factor                                            */
} kf_factor;

/* AxisTerm(coeff, factors) (src/apply.jl:157-166): axes strictly increasing. */
typedef struct {
    double coeff;
    int32_t nfactors;
    const kf_factor *factors;
} kf_term;

/* KronFreeOperator(dims, terms; constant, block_capacity) (src/apply.jl:222-253).
 * Terms whose factors are all KF_DIAG are fused with `constant` into one state-sized diagonal,
 * as the reference's constructor does (src/apply.jl:238-241); `diag`, when not NULL, is an
 * already-fused N-vector added to it (the reference's H.diag, for a caller that holds one). */
typedef struct {
    int32_t ndims;
    const int64_t *dims;
    double constant;
    int32_t nterms;
    const kf_term *terms;
    const double *diag;      /* optional, N values, host memory                               */
    int64_t block_capacity;  /* scratch columns reserved for dense-factor chains (>= 1)       */
} kf_op_desc;

typedef struct kf_op kf_op;

/* Replaces KronFreeOperator(dims, terms; constant, block_capacity, on=CuArray)
 * (src/apply.jl:222-253) together with _on_storage (src/apply.jl:258-267): validates the
 * descriptor (KF_EINVAL / KF_EDIM with the reference's messages), fuses the diagonal terms,
 * and copies everything to the current device.  The op owns its device memory and stream. */
int kf_op_create(const kf_op_desc *desc, kf_op **out);

/* Frees the op's device memory and stream. */
int kf_op_destroy(kf_op *op);

/* size(H, 1) = prod(dims) (src/apply.jl:269). */
int kf_op_size(const kf_op *op, int64_t *n);

/* Replaces LinearAlgebra.mul!(Y, H, X) (src/apply.jl:416-432) for a block of b columns:
 * Y = H X.  ldx, ldy >= N.  Y must not alias X (KF_EALIAS, src/apply.jl:409-414).
 * flags: KF_F64 | KF_F32, KF_DEVICE | KF_HOST. */
int kf_op_apply(kf_op *op, const void *X, void *Y, int64_t ldx, int64_t ldy, int64_t b, int32_t flags);

/* mul! fused with the Chebyshev three-term recurrence (src/chebyshev.jl:25-29 and :42-43):
 * Y = alpha * (H X) + beta * X + gamma * Z, device pointers only.  Z may be NULL (gamma = 0). */
int kf_op_apply_axpby(kf_op *op, const void *X, void *Y, const void *Z, int64_t ld, int64_t b,
                      double alpha, double beta, double gamma, int32_t flags);

/* kf_op_apply for callers that must not allocate device memory (no counterpart in the
 * reference).  kf_op_apply allocates two N x b scratch blocks with cudaMalloc the first time it
 * applies a term with dense factors to a block that wide; a caller whose device memory is owned
 * by its own pool or arena (a Julia or PyTorch caching allocator, a fixed-size arena) must not
 * have memory allocated behind its back, and a tight solver loop cannot take the device
 * synchronisation of a cudaMalloc.  This entry point computes the same Y = H X (device pointers
 * only; KF_F64 or KF_F32) and allocates nothing: its scratch is a static device array of
 * KF_NOALLOC_SCRATCH_BYTES that each device holds from its first call until exit.  Blocks whose
 * dense-factor chains need more than that (2 N b elements) are rejected with KF_EINVAL.  All calls
 * on a device share the array, so calls that overlap on the GPU race.  The array is reserved when
 * the library's module holding it loads, at the first call on each device (CUDA loads modules
 * lazily), so a caller that must see no allocation later makes one set-up call per device first:
 * b = 0 on an operator with dense-factor terms reserves the array, and a b > 0 call also loads the
 * kernels.  Make the set-up call before any stream capture. */
#define KF_NOALLOC_SCRATCH_BYTES (8u << 20)
int kf_op_apply_noalloc(kf_op *op, const void *X, void *Y, int64_t ldx, int64_t ldy, int64_t b, int32_t flags);

/* The port matrix W' H V (kw x kv, column-major, FP64, caller-owned HOST memory) of an operator H
 * on a node's product basis, for column blocks V (N x kv) and W (N x kw; NULL: W = V), FP64, host
 * (KF_HOST) or device pointers with leading dimensions ldv, ldw.  Replaces the formation of ports
 * and joint ports on a node's kept vectors, V' (x)_a O_a V, in _assemble_node (src/materialize.jl:
 * 426-441 _apply_ops / _port_matrix, :463-467 _node_port, :490-495 _joint_port, :505-517
 * _real_sandwich): H is the port's one-term operator (port_operator, src/portoperator.jl:18-39) or,
 * for a real expansion's component, the sum of its terms with their coefficients; the caller keeps
 * the port's character (real, imaginary or both components) and phase fixing. */
int kf_op_sandwich(kf_op *op, const double *W, int64_t ldw, int32_t kw, const double *V, int64_t ldv, int32_t kv,
                   double *P_out, int32_t flags);

/* Matrix-free time evolution under port drives: the action of the drive Hamiltonian on a node's
 * product basis, which QuantumToolbox's sesolve applies (src/quantumtoolbox.jl:84-99,
 * drive_hamiltonian with basis = :free, batch = true: a QobjEvo around the KronFreeOperator H0 and
 * the port operators of src/portoperator.jl:18-39).  Y = H(t) X with
 *     H(t) = 2 pi [H0 - E0 + sum_k coef[k] O_k]     (rad/ns; coef[k] = f_k(t) in GHz),
 * X and Y complex blocks of m columns stored as 2m FP64 columns: the real parts, then the imaginary
 * parts (column j at X + j ldx, its imaginary part at X + (m + j) ldx).  omega != NULL: the
 * interaction frame, Y = e^{i Omega t} (H(t) - diag Omega) e^{-i Omega t} X with Omega = omega (N
 * values, rad/ns: the diagonal of 2 pi (H0 - E0), on the same side as X).  Port k is
 * ports[k] + i ports_im[k]: its real and imaginary components as real operators on H0's product
 * basis (KF_EDIM otherwise), either array or entry may be NULL (a real-character port has no
 * imaginary component), not both entries of one port; coef: host array.  H0 is a real operator.
 * flags: KF_F64 with KF_DEVICE (H0's stream, asynchronous) or KF_HOST (returns when done). */
int kf_drive_apply(kf_op *H0, double E0, int32_t nports, kf_op *const *ports, kf_op *const *ports_im,
                   const double *coef, const double *omega, double t, const void *X, int64_t ldx, void *Y, int64_t ldy,
                   int64_t m, int32_t flags);

/* to_lab (src/quantumtoolbox.jl:25-37): the lab-frame state e^{-i Omega t} psi of an
 * interaction-picture block, in place: X as in kf_drive_apply (2m FP64 columns), omega N values
 * (rad/ns) on the same side as X.  KF_DEVICE: runs on the default stream and returns when done. */
int kf_to_lab(const double *omega, int64_t N, double t, void *X, int64_t ldx, int64_t m, int32_t flags);

/* The linear solve on the complement of a node's known states (src/resolvent.jl:146-252,
 * _complement_solve; the Sternheimer solves of the reference's derivatives): X[:, j] solves
 * Q (H - shifts[j]) Q x = Q B[:, j] with x orthogonal to the nbasis orthonormal columns of basis,
 * Q = 1 - basis basis', by a conjugate gradient on all n columns in lockstep, each with its own
 * scalars, preconditioned by 1 / hypot(diagonal(H) - shifts[j], eta).  FP64.  basis (N x nbasis),
 * B (N x n) and X (N x n) are host (KF_HOST) or device pointers with leading dimensions >= N;
 * shifts (n) and scale (n, or NULL: the column norms of B) are host arrays.  Stopping rule, round-off
 * floor (1000 eps scale_j, five checks of the true residual without halving), positivity check and
 * final acceptance are the reference's.  Outputs (host, each may be NULL): iterations; per column
 * state (0 met its tolerance tol ||Q B_j||, 1 converged from the start with x = 0, 2 stopped at the
 * round-off floor), residuals (true residual / ||Q B_j|| for state 0) and floor_residuals (true
 * residual / scale_j for state 2).  KF_EBREAKDOWN: "not positive on the complement";
 * KF_ENOCONV: "did not converge". */
int kf_complement_solve(kf_op *op, const double *basis, int64_t ldbasis, int32_t nbasis, const double *B, int64_t ldb,
                        int32_t n, const double *shifts, const double *scale, double tol, int32_t maxiter, double eta,
                        double *X, int64_t ldx, int32_t *iterations, int32_t *state, double *residuals,
                        double *floor_residuals, int32_t flags);

/* diagonal(H) real part (src/apply.jl:455-478, _full_diagonal), N values into host memory. */
int kf_op_diagonal(kf_op *op, double *out);

/* gershgorin_bound(H) (src/apply.jl:586-593). */
int kf_op_gershgorin(kf_op *op, double *out);

/* The cudaStream_t the op launches on (as void*); set one to launch on a caller's stream. */
int kf_op_get_stream(kf_op *op, void **stream);
int kf_op_set_stream(kf_op *op, void *stream);

/* Blocks until the op's stream is idle. */
int kf_op_sync(kf_op *op);

/* product_seed(H, k) (src/apply.jl:655-685): the k lowest product states of the single-axis part
 * of H (the Kronecker products of the per-axis eigenbases of separable_eigenbases,
 * src/apply.jl:606-642, ordered by their separable energy, ties by column-major index), or, when
 * every axis' single-axis sum is diagonal, the unit vectors of the k smallest entries of the
 * diagonal.  X: N x k, column-major, leading dimension N; flags KF_HOST / KF_DEVICE for where X
 * lives (device: asynchronous on the op's stream).  KF_EINVAL unless 1 <= k <= N. */
int kf_op_product_seed(kf_op *op, int32_t k, double *X, int32_t flags);

/* ---- eigensolvers (src/solvers.jl:6-31 custom-solver contract) ---------------------- */
#define KF_SOLVER_LOBPCG     0   /* src/lobpcg.jl:217-301                                  */
#define KF_SOLVER_CHEBYSHEV  1   /* src/chebyshev.jl:310-406                               */
#define KF_SOLVER_LANCZOS    2   /* src/solvers.jl:85-106                                  */

#define KF_PREC_F64    0   /* plain: every step in FP64                                    */
#define KF_PREC_MIXED  1   /* FP32 bulk (applies, Gram, updates; FP64 accumulation across
                              blocks), FP64 Rayleigh-Ritz, then an FP64 refinement phase with
                              FP64 residuals                                                */

#define KF_PRECOND_RITZ    0
#define KF_PRECOND_JACOBI  1
#define KF_PRECOND_NONE    2
#define KF_PRECOND_SEPARABLE 3   /* U diag(1/hypot(S - theta_j, eta_s)) U' from the per-axis
                                    eigenbases of the single-axis terms (separable_eigenbases,
                                    src/apply.jl:606-642); eta_s = max(eta, 1e-3 ||H||)  */

#define KF_ORTHO_SVQB    0
#define KF_ORTHO_CHOLQR  1

/* Options: the fields of LOBPCG(...) (src/tree.jl:66-87), ChebyshevFilter(...)
 * (src/tree.jl:293-321) and Lanczos(...) (src/tree.jl:15-23), plus the precision mode and the
 * warm-start fallback.  Call kf_solver_opts_default first. */
typedef struct {
    int32_t kind;              /* KF_SOLVER_*                                                  */
    int32_t precision;         /* KF_PREC_*                                                    */
    double tol;                /* absolute residual tolerance ||H v - E v||, energy units      */
    int32_t maxiter;
    int32_t preconditioner;    /* LOBPCG: KF_PRECOND_*                                         */
    double eta;                /* LOBPCG :ritz regularization                                  */
    int32_t guard;             /* LOBPCG guard columns                                         */
    int32_t degree;            /* Chebyshev: degree (1..200)                                   */
    int32_t extra;             /* Chebyshev: extra columns (>= 2)                              */
    int32_t rescale_every;     /* Chebyshev                                                    */
    int32_t ortho;             /* Chebyshev: KF_ORTHO_*                                        */
    double bound;              /* Chebyshev: lambda_max; NaN = gershgorin_bound(H)            */
    int32_t krylovdim;         /* Lanczos: 0 = max(2m + 10, 40)                                */
    uint64_t rng_seed;         /* random columns (guards, refills, retries)                    */
    double mixed_switch;       /* MIXED: FP32 phase stops when every active residual is below
                                  mixed_switch * ||H|| (||H|| = gershgorin bound)              */
    int32_t fallback_iters;    /* warm start judge: after this many iterations ...             */
    double fallback_resid;     /* ... a largest residual of the m warm-start columns above this
                                  (absolute, energy units) restarts a warm-started solve from a
                                  random block (0 disables); the check on a learned warm start */
    int32_t seed_kind;         /* LOBPCG / Chebyshev `seed` (src/tree.jl:66-87, 293-321):
                                  KF_SEED_PRODUCT (default) or KF_SEED_RANDOM; used when
                                  kf_solve's seed argument is NULL                             */
    int32_t buffer;            /* LOBPCG: unchecked columns carried beyond the guards; they
                                  speed the convergence of the top guard when an eigenvalue
                                  just above the block is nearly degenerate with it, and
                                  never count toward convergence or the returned pairs.
                                  KF_BUFFER_AUTO (default): 2 for KF_PREC_MIXED, 0 for
                                  KF_PREC_F64 (the reference algorithm column for column)     */
} kf_solver_opts;

#define KF_BUFFER_AUTO (-1)

#define KF_SEED_PRODUCT 0   /* seed=:product, product_seed(H, w) built by the library         */
#define KF_SEED_RANDOM  1   /* seed=:random                                                    */

typedef struct {
    int32_t iterations;        /* total iterations (FP32 + FP64)                               */
    int32_t iterations_f64;    /* iterations of the FP64 (refinement) phase                    */
    int64_t n_matvec;          /* columns H was applied to (the reference's n_matvec)          */
    int32_t warm;              /* 1 when X0 was used                                           */
    int32_t fell_back;         /* 1 when the warm start was judged bad and replaced            */
    int32_t converged;         /* number of returned pairs with residual <= tol               */
    double max_residual;       /* largest FP64 true residual of the returned pairs             */
    double hnorm;              /* gershgorin_bound(H)                                          */
    double seconds;            /* wall time inside kf_solve                                    */
    double seconds_f64;        /* wall time of the FP64 phase                                  */
} kf_solve_stats;

void kf_solver_opts_default(kf_solver_opts *opts, int32_t kind);

/* Replaces solve(s, H, m; X0) for s::LOBPCG / ChebyshevFilter / Lanczos (src/lobpcg.jl:303,
 * src/chebyshev.jl:310, src/solvers.jl:81): the lowest m eigenpairs, E ascending (m values)
 * and V (N x m, column-major, orthonormal), both caller-owned HOST memory, like the reference
 * returning host arrays (src/lobpcg.jl:298-299).
 *   X0:   NULL or an N x m warm-start block (LOBPCG only; src/lobpcg.jl:226-233 checks).
 *   seed: NULL or a caller's seed block, N x w with w = m + guard (LOBPCG) or m + extra
 *         (Chebyshev).  NULL: opts->seed_kind decides -- KF_SEED_PRODUCT builds product_seed(H, w)
 *         on the device, as lobpcg_solve does for seed=:product (src/lobpcg.jl:247,
 *         src/apply.jl:655-685); KF_SEED_RANDOM draws a random block.
 * Every returned pair is checked with a fresh FP64 application of H (src/solvers.jl:65-69).
 * KF_ENOCONV when a pair is above tol, with the reference's message. */
int kf_solve(kf_op *op, const kf_solver_opts *opts, int32_t m, const double *X0, const double *seed,
             double *E_out, double *V_out, kf_solve_stats *stats);

/* ---- batched leaf solves (many small operators in one persistent launch) ------------ */

/* The lowest m[i] eigenpairs of each of `count` operators, in one persistent launch over all
 * of them (one CTA pair of work per operator), the batched form of `solve` over the leaves of a
 * parameter sweep or of sibling nodes (src/materialize.jl:713-731 solves them one by one).
 * Supported operators: one or more axes whose kept terms have only diagonal, banded and shift
 * factors, N <= 4096, m[i] + 4 <= 32.  E_out: sum(m) values; V_out: sum(N_i * m_i) values,
 * operator i's block at offset sum_{k<i} N_k m_k.  `tile` = 0 picks the tuned tile
 * (kf_batch_autotune), else threads per CTA (128, 256 or 512). */
int kf_batch_solve(const kf_op_desc *descs, int32_t count, const int32_t *m, double tol,
                   int32_t maxiter, int32_t tile, double *E_out, double *V_out, int32_t *iters_out,
                   double *resid_out);

/* Times kf_batch_solve's persistent kernel over the candidate tiles on the given batch and
 * stores the fastest for batches of this size class; returns it in *best_tile. */
int kf_batch_autotune(const kf_op_desc *descs, int32_t count, const int32_t *m, double tol,
                      int32_t maxiter, int32_t *best_tile);

/* ---- the learned warm start (a small MLP trained by this library's own kernels) ----- */
typedef struct kf_mlp kf_mlp;

/* A din -> hidden -> hidden -> dout MLP with SiLU, BF16 weights, FP32 accumulation and
 * FP32 master weights for Adam.  Weights are initialised from `seed`. */
int kf_mlp_create(int32_t din, int32_t hidden, int32_t dout, uint64_t seed, kf_mlp **out);
int kf_mlp_destroy(kf_mlp *mlp);

/* Input/output normalisation: x_n = (x - xmu) / xsd per input, y = y_n * ysd + ymu per output
 * (host arrays of din and dout values). */
int kf_mlp_set_scaling(kf_mlp *mlp, const float *xmu, const float *xsd, const float *ymu, const float *ysd);

/* Adam training on (X: n x din, Y: n x dout, row-major, host) for `epochs` passes of
 * mini-batches of `batch` rows (shuffled with `seed`); mean-squared error on the normalised
 * outputs.  losses_out (epochs values, may be NULL) receives each epoch's mean loss. */
int kf_mlp_train(kf_mlp *mlp, const float *X, const float *Y, int64_t n, int32_t epochs, int32_t batch,
                 float lr, uint64_t seed, float *losses_out);

/* Forward pass: Y (n x dout) = mlp(X (n x din)), row-major host arrays. */
int kf_mlp_forward(kf_mlp *mlp, const float *X, float *Y, int64_t n);

/* One training step's gradients on (X, Y) without updating: loss and the FP32 gradients of
 * W1 (din x hidden), b1, W2, b2, W3, b3 concatenated in that order into grad_out (host). */
int kf_mlp_gradients(kf_mlp *mlp, const float *X, const float *Y, int64_t n, float *loss_out, float *grad_out);

/* The parameters as FP32 (the BF16 weights widened), in the kf_mlp_gradients order. */
int kf_mlp_get_params(kf_mlp *mlp, float *out, int64_t *count);

/* ---- errors and info ---------------------------------------------------------------- */

/* The message of the calling thread's last failed call ("" if none), copied into buf. */
int kf_last_error(char *buf, size_t len);

/* KFGPU_VERSION. */
int kf_version(void);

/* The number of CUDA kernels this library has launched in this process (all ops and solves). */
int kf_launch_count(uint64_t *count);

#ifdef __cplusplus
}
#endif

#endif /* KFGPU_H */

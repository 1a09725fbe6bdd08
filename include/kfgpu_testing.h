/*
 * kfgpu_testing.h -- entry points of libkfgpu.so that exist for the test suite only.  They have
 * no counterpart in KronFreeCircuits.jl and no caller of the reference interface needs them.
 */
#ifndef KFGPU_TESTING_H
#define KFGPU_TESTING_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/*
 * One mode product Y = alpha (A along an axis) X + beta Y on device blocks of b FP32 columns of
 * length N (leading dimension N), the axis of length d with stride `left` (the product of the
 * lengths of the axes before it).  A: host, d x d, column-major, FP64.  path 0: the SIMT FP32
 * kernel; path 1: the tcgen05 tensor-core kernel with BF16 operands; path 2: the same with TF32
 * hi / lo operands (three MMAs per K step); FP32 accumulation in TMEM; d <= 256.
 * Synchronous on `stream` (a cudaStream_t, 0 for the default stream).  Returns a KF_* status.
 */
int kf_test_mode_product(int path, const float *X, float *Y, const double *A, int d, int64_t left, int64_t N,
                         int64_t b, double alpha, double beta, void *stream);

/*
 * The same product launched `reps` times on `stream` (the operator image built once, outside the
 * timed region; X and Y as above), timed with CUDA events around the launches: *ms_per_launch
 * receives the mean device time of one launch.  Returns a KF_* status.
 */
int kf_test_time_mode_product(int path, const float *X, float *Y, const double *A, int d, int64_t left, int64_t N,
                              int64_t b, int reps, void *stream, float *ms_per_launch);

/*
 * The FP32 Gram product G = A' B (A: N x ka, B: N x kb, device, column-major with leading
 * dimensions lda, ldb; ka, kb <= 128) launched `reps` times on `stream` and timed with CUDA events
 * around the launches (the Gram kernel and its fixed-order partial reduction together).  path 0:
 * the solvers' choice (the tensor cores when the shapes fit), path 1: the SIMT kernel;
 * *ms_per_launch receives the mean device time of one product, G_out (host, ka x kb column-major,
 * may be NULL) the last result.  Returns a KF_* status.
 */
int kf_test_time_gram(int path, const float *A, int64_t lda, int ka, const float *B, int64_t ldb, int kb, int64_t N,
                      int reps, void *stream, float *ms_per_launch, double *G_out);

/*
 * The tensor-core FP32 Gram (tcgen05, TF32 hi / lo operands) on a pool of nsrc (1..4) device
 * blocks: srcs[q] (N x ks[q], leading dimension lds[q]) stacked in order; G_out (host, nr x nc
 * column-major FP64, nr = sum of ks[r0 .. r1-1], nc = sum of ks[c0 .. c1-1]) receives
 * [srcs r0..r1-1]' [srcs c0..c1-1].  `reps` launches on `stream`, timed with CUDA events
 * (*ms_per_launch: mean device time, Gram and reduction).  Returns KF_EINVAL when the shapes do not
 * fit the kernel (the solvers then take the SIMT Gram), else a KF_* status.
 */
int kf_test_gram_tc(const float *const *srcs, const int64_t *lds, const int32_t *ks, int32_t nsrc, int32_t r0,
                    int32_t r1, int32_t c0, int32_t c1, int64_t N, int32_t reps, void *stream,
                    float *ms_per_launch, double *G_out);

/*
 * The host symmetric eigensolver of the small projected problems (Rayleigh-Ritz, SVQB, the per-axis
 * eigenbases of the separable preconditioner): eigenvalues w (ascending) and orthonormal
 * eigenvectors V (n x n, column-major, leading dimension ldv) of the symmetric A (n x n,
 * column-major, leading dimension lda; both triangles read as their average).  Host only, no GPU
 * call.  KF_EBREAKDOWN when the QR iteration does not converge.
 */
int kf_test_sym_eig(int n, const double *A, int lda, double *w, double *V, int ldv);

/*
 * The device second orthogonalisation pass's coefficients: from G ((wx + r) x r, host, FP64, column-
 * major: rows of X'Z then Z'Z), C_out ((r + wx) x r) = [R^-1 ; -(X'Z) R^-1] with R the Cholesky
 * factor of Z'Z - (X'Z)'(X'Z); *status_out 0, or 1 when a pivot is not finite or below 1e-4.
 * r <= 64.
 */
int kf_test_chol2(const double *G, int wx, int r, double *C_out, int *status_out);

/*
 * The FP32 update with its output split over two blocks: [Y0 Y1] = alpha [X0 X1] C + beta [Y0 Y1]
 * (device blocks, leading dimension ld; Y0: ky0 columns, Y1: ky1; X0: kx0, X1: kx1; C: host,
 * (kx0 + kx1) x (ky0 + ky1) column-major FP64): path 0 the pipelined SIMT kernel, path 1 the
 * tcgen05 kernel.  Returns KF_EINVAL when the shapes do not fit the kernel (path 0: more than 64
 * inputs or outputs, unaligned blocks; path 1: more than 64 inputs or 80 outputs).
 */
int kf_test_update_split(int path, float *Y0, int ky0, float *Y1, int ky1, const float *X0, int kx0, const float *X1,
                         int kx1, const double *C, double alpha, double beta, int64_t N, int64_t ld);

/*
 * The FP64 block update Y = X C (device blocks X: N x kx, Y: N x ky, leading dimension N; C: host,
 * kx x ky column-major FP64), `reps` times on `stream`: path 0 the FP64 kernel, path 1 double-float
 * arithmetic on the FP32 pipes (kx, ky <= 32).  *ms_per_launch: mean device time.
 */
int kf_test_update_f64(int path, double *Y, const double *X, int kx, int ky, const double *C, int64_t N, int reps,
                       void *stream, float *ms_per_launch);

/*
 * The FP32 block update Y = alpha [X0 X1] C + beta Y (device blocks: X0 N x kx0, X1 N x kx1 (kx1 may
 * be 0), Y N x ky; C: host, (kx0 + kx1) x ky, column-major FP64, leading dimension ldc), `reps`
 * times on `stream`, timed with CUDA events: path 0 the SIMT kernels, path 1 the tcgen05 kernel
 * (TF32 hi / lo operands; kx0 + kx1 <= 64, ky <= 80) with its producer mode picked by shape, paths
 * 2-4 the same with the mode forced: 2 register gather, 3 and 4 a staging ring of 2 and 3 tiles
 * (KF_EINVAL where it does not fit).  *ms_per_launch: mean device time.  With
 * beta != 0 every launch reads the Y the previous one wrote.
 */
int kf_test_update(int path, float *Y, int64_t ldy, int ky, const float *X0, int64_t ldx0, int kx0, const float *X1,
                   int64_t ldx1, int kx1, const double *C, int ldc, double alpha, double beta, int64_t N, int reps,
                   void *stream, float *ms_per_launch);

/*
 * kf_op_apply (device blocks, flags as there) with the fused-apply kernel variant forced instead of
 * the tuned one: 0-4 the point-per-thread kernel's shapes, 5 the plane-marching kernel (where its
 * geometry applies; otherwise variant 4 runs), 6 the point-per-thread kernel with 36 columns per
 * thread; `reps` launches timed with CUDA events on the op's
 * stream, *ms_per_launch (may be NULL) receives the mean.
 */
int kf_test_apply_variant(kf_op *op, int variant, const void *X, void *Y, int64_t ld, int64_t b, int32_t flags,
                          int reps, float *ms_per_launch);

/*
 * The bytes of chain scratch the operator has allocated for kf_op_apply so far (0 until a block
 * with dense-factor terms is applied through kf_op_apply).  Returns a KF_* status.
 */
int kf_test_op_scratch_bytes(const struct kf_op *op, uint64_t *bytes);

/*
 * Whether the plane-marching fused apply (forced-variant 5) applies to this operator for a block of
 * b columns (FP32 when f32 != 0, else FP64) on a device with `sms` multiprocessors (0: ask the
 * op's device); *eligible 1 or 0.  geom (may be NULL) receives 16 values: plane size P,
 * march-axis length, outer count, halo H, in-plane reach R, tile TQ, tiles per plane, persistent
 * CTAs, ring slots, slot X and diagonal lengths, shared entries, their register class (6, 8 or 16),
 * points per thread, 1 when every shared entry reads the current plane, the dynamic shared memory
 * bytes.  Returns a KF_* status.
 */
int kf_test_march_plan(const struct kf_op *op, int64_t b, int32_t f32, int32_t sms, int32_t *eligible,
                       int32_t *geom);

/* Bounds-recording builds (-DKF_CHECK): the site number of the first failed bounds check since the
 * last call (0: none; the word is reset), after a device synchronisation; check_build = 1 when the
 * library was compiled with KF_CHECK. */
int kf_test_check_word(int32_t *site, int32_t *check_build);

/* The device Rayleigh-Ritz eigensolver of the FP32 LOBPCG phase (FP32 Jacobi, one CTA): G on the
 * host in the merged (ldg x ldg, rows [X_a; Q], columns [H X_a, H Z]) or packed layout; writes
 * C (ns x 2 na: [C_x | [0; C_z]]) and the na lowest Ritz values into theta_out (in / out).  status
 * != 0 takes the path of a failed device Cholesky (C keeps X, drops P; theta_out comes back as given). */
int kf_test_rr_eig(const double *G, int32_t ldg, int32_t packed, int32_t na, int32_t k, int32_t status, double *C_out,
                   double *theta_out);

#ifdef __cplusplus
}
#endif

#endif

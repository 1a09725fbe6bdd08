// Internal declarations shared by the translation units of libkfgpu.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <future>
#include <map>
#include <vector>

#include "../../include/kfgpu.h"

namespace kf {

// An error carrying a status code; every extern "C" entry point converts it to its status and
// records the message for kf_last_error.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string &msg);

#define KF_CUDA(call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            throw ::kf::Error(e_ == cudaErrorMemoryAllocation ? KF_ENOMEM : KF_ECUDA,          \
                              std::string(#call) + ": " + cudaGetErrorString(e_));             \
    } while (0)

// Every kernel launch of the library is followed by this: it counts the launch (kf_launch_count)
// and turns a launch error into a kf::Error.
extern std::atomic<uint64_t> g_launches;
#define KF_LAUNCH_CHECK()                                                                      \
    do {                                                                                       \
        ::kf::g_launches.fetch_add(1, std::memory_order_relaxed);                              \
        KF_CUDA(cudaGetLastError());                                                           \
    } while (0)

// Bounds-recording builds (-DKF_CHECK, kfgpu.build.build_library(check=True)): a kernel tests an
// index before an access, writes the failing site's number into the second word of the host-mapped
// error allocation (tc_error_word() + 1) and skips the access; it never traps.  In normal builds the
// test is the constant true.
#ifdef KF_CHECK
#define KF_CHK(cond, err, site) ((cond) ? true : ((*(volatile int *)((err) + 1) = (site)), false))
#else
#define KF_CHK(cond, err, site) true
#endif

#define KF_REQUIRE(cond, code, msg)                                                            \
    do {                                                                                       \
        if (!(cond)) throw ::kf::Error((code), (msg));                                         \
    } while (0)

constexpr int MAXDIMS = 8;     // axes of a state tensor
constexpr int MAXB = 24;       // bands of one banded factor (a periodic order-8 stencil has 16)
// five (columns per thread, unroll) shapes of the point kernel, the plane-marching kernel (5), 36
// columns per thread (a 36-column block in one pass instead of 32 + 4)
constexpr int KF_APPLY_VARIANTS = 8;
constexpr int MAXE = 48;       // stencil entries (products of bands) over all fused terms

// The fused kernel's stencil entries.  Every term built only of diagonal, banded and shift
// factors on at most two axes is a product of banded factors; the cartesian product of its
// bands gives entries e with output  Y[p] += w_e(p) X[p + delta_e],  where
// w_e(p) = W[w0_e + i_{a0}(p) nb0_e] (* W[w1_e + i_{a1}(p) nb1_e]) and the entry is skipped when
// i_a + off_a leaves [0, n_a) on either axis.  The coefficient is folded into the weights.
struct Entry {
    int nf;            // 1 or 2 factors
    int a0, o0, n0, nb0, w0;
    int a1, o1, n1, nb1, w1;
    int delta;         // sum of off * stride over the factors
};

constexpr int MAXDIMS_F = 6;   // axes the fused kernel decodes (more: the chain path)

// Everything the fused apply kernel needs, passed by value as a kernel parameter.
struct ApplyPlan {
    int ndims;
    int dims[MAXDIMS_F];
    int N;
    int ne;
    Entry e[MAXE];
};

// A dense-containing term, applied as a chain of single-axis products through scratch.
struct ChainFactor {
    int axis;
    int kind;                  // KF_DENSE or KF_BANDED (diag and shift converted to banded)
    int n;
    int nb;
    int off[MAXB];
    size_t data_off;           // dense: n*n matrix (column-major); banded: n*nb weights
    int tc = -1;               // dense: index of its TF32-split tensor-core image in kf_op::chain_tc
};
struct ChainTerm {
    double coeff;
    std::vector<ChainFactor> f;
};

// Dense pairwise couplings on a three-axis basis (kf_pairs.cu): pairs (0,1), (0,2), (1,2), each
// g A (x) B with the factors' data at off[pair][0 / 1] in the chain pools
struct PairPlan {
    int ok;
    int d[3];
    int has[3];
    double g[3];
    size_t off[3][2];
    int share0, share1, share2;   // the axis-0 matrices of (0,1), (0,2) equal; axis 1 of (0,1), (1,2); axis 2 of (0,2), (1,2)
};

// tensor-core mode products (kf_tc.cu): a d x d operator (d <= 256) as a BF16 image in the
// tcgen05 K-major shared-memory layout, rows padded to Mp (128 or 256), columns to Kp
struct TcMatrix {
    void *img = nullptr;
    int d = 0, Mp = 0, Kp = 0;
    int split = 0;   // 0: BF16 operands; 1: TF32 hi / lo operands (three MMAs, FP32-accurate products)
};
int tc_mode_layout_ok(int d);
TcMatrix tc_matrix_create(const double *A, int d, bool transpose, bool split = false);
void tc_matrix_free(TcMatrix &m);
size_t tc_mode_smem(const TcMatrix &m);
bool tc_mode_fits(int d, bool split);
void tc_mode_product(float *Y, int64_t ldy, const float *X, int64_t ldx, const TcMatrix &A, int64_t left, int64_t N,
                     int64_t b, double alpha, double beta, cudaStream_t s);
int tc_take_error();
int *tc_error_word();  // the host-mapped word device-side waits report KF_ETIMEOUT in
int check_take_site(); // KF_CHECK builds: the first failed bounds-check site since the last call (0: none)
// FP32 block update on the tensor cores (kf_tcgemm.cu), TF32 hi / lo operands, kx <= 64, ky <= 80
bool update_tc_ok(int kx, int ky);
void update_tc(float *Y, int64_t ldy, int ky, const float *X0, int64_t ldx0, int kx0, const float *X1, int64_t ldx1,
               int kx1, const double *C, int ldc, double alpha, double beta, int64_t N, cudaStream_t s);
// the same with the outputs split over two blocks (columns [0, ky0) to Y0, the ky1 others to Y1);
// force_nstg >= 0 forces the producer mode (0 register gather, 2 or 3 staging tiles; KF_EINVAL when
// it does not fit), -1 picks the deepest staging ring that fits
void update_tc2(float *Y0, int64_t ldy0, int ky0, float *Y1, int64_t ldy1, int ky1, const float *X0, int64_t ldx0,
                int kx0, const float *X1, int64_t ldx1, int kx1, const double *C, int ldc, double alpha, double beta,
                int64_t N, cudaStream_t s, int force_nstg);
// whether the tensor-core update (with a staging ring) is the faster FP32 update for this shape: at
// least 40 inputs and 17 outputs on 65,536 rows or more, 16-byte aligned columns (X1 may be NULL);
// narrower updates are faster on the pipelined SIMT kernel
bool update_tc_prefer(int kx, int ky, int64_t N, const float *X0, int64_t ldx0, const float *X1, int64_t ldx1);   // a pending device-side timeout (KF_ETIMEOUT) of a tensor-core launch, cleared

}  // namespace kf

// The operator handle.
struct kf_op {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = true;
    kf::ApplyPlan plan{};
    std::map<int, int> apply_tuned;    // fused-apply variant per (precision, 4-column width class)
    int force_variant = -1;   // test-only: run this fused-apply variant instead of the tuned one
    int64_t N = 0;
    std::vector<int64_t> dims;
    std::vector<int64_t> strides;
    // fused diagonal on the device, FP64 and FP32
    double *d_diag64 = nullptr;
    float *d_diag32 = nullptr;
    // banded weight pool (fused terms), FP64 and FP32
    double *d_w64 = nullptr;
    float *d_w32 = nullptr;
    // dense-chain terms and their data (FP64 and FP32 copies)
    std::vector<kf::ChainTerm> chains;
    kf::PairPlan pairs{};                  // the chains as dense pairwise couplings, when they are
    std::vector<kf::TcMatrix> chain_tc;   // tensor-core images of dense chain factors (FP32 applies)
    double *d_chain64 = nullptr;
    float *d_chain32 = nullptr;
    // the plane-marching apply's weight tables (FP64, FP32), built on its first use
    void *d_march[2] = {nullptr, nullptr};
    // scratch for chains: two buffers of N * cap doubles
    int64_t cap = 0;
    void *d_scratch = nullptr;
    size_t scratch_bytes = 0;
    // scratch of the drive apply (kf_drive.cu): the rotated block and one port's product
    void *d_drive = nullptr;
    size_t drive_bytes = 0;
    // host copies of derived data
    std::vector<double> h_diag;           // fused diagonal (real)
    double gershgorin = 0;
    std::vector<double> h_fulldiag;       // full diagonal (fused + kept terms)
    // host-side term data for the diagonal and gershgorin
    struct HostFactor { int axis; int kind; int64_t n; std::vector<double> data; std::vector<int64_t> offs; int64_t shift; double factor; };
    struct HostTerm { double coeff; std::vector<HostFactor> f; };
    std::vector<HostTerm> kept;
    // separable part for the preconditioner: per axis the sum of the single-axis terms
    // (src/apply.jl:606-642), its eigendecomposition made on first use
    struct Separable {
        std::vector<std::vector<double>> M;   // host d_a x d_a sums (column-major)
        bool ready = false;
        std::vector<int> ident;               // axis whose sum is diagonal (U = I)
        std::vector<double> lam;              // concatenated per-axis eigenvalues
        std::vector<float *> dU, dUt;         // FP32 U and U' per axis (nullptr when ident)
        std::vector<double *> dU64;           // FP64 U per axis (nullptr when ident), for product_seed
        std::vector<kf::TcMatrix> tU, tUt;    // the same as tensor-core BF16 images (d <= 256)
        std::vector<std::vector<double>> Uh;  // host eigenbases per axis (empty when ident)
        bool host_ready = false;
        std::future<void> host_job;           // the host eigendecompositions, started at creation
        double *d_lam = nullptr;
        int *d_lam_off = nullptr, *d_dims = nullptr;
        float *d_shl = nullptr;               // per point: S(p) as FP32 hi, lo (interleaved, 2N)
    } sep;
};

namespace kf {

// plane-marching fused apply (kf_apply_march.cu): the slowest axis m with an offset is walked plane by
// plane; its neighbours come from a per-thread register window, in-plane neighbours from plane
// slices staged in shared memory by bulk copies
constexpr int MARCH_MAXW = 24;   // window entries (r = 0, no factor before m)
constexpr int MARCH_MAXC = 16;   // centre entries
constexpr int MARCH_MAXS = 16;   // shared-memory entries
struct MarchPlan {
    int m, P, nm, nouter, N, H, R;
    int nwin, win[MARCH_MAXW], wino[MARCH_MAXW];
    int ncen, cen[MARCH_MAXC];
    int nsm, nsm1, ms, sm[MARCH_MAXS], smr[MARCH_MAXS], smo[MARCH_MAXS], smpl[MARCH_MAXS];
    int TQ, ntile, nseg, L, NR, SLX, SLD, pt;
    int flat;       // every shared entry reads the current plane (o_e = 0)
    int grid;       // persistent CTAs
    int wn;         // the kernel's window length (2H + 1; a halo of 3 runs on the kernel for 4)
    int mcw;        // consumer warps (12, or 7 with twice the points per thread)
};
bool march_plan(const kf_op *op, int64_t b, size_t elem, int num_sms, MarchPlan &mp, int mcw = 12);
size_t march_smem_bytes(const MarchPlan &mp, size_t elem, int wn, int ms);
template <typename T>
void launch_apply_march(kf_op *op, const MarchPlan &mp, const T *D, const T *W, const T *X, T *Y, int64_t ldx,
                        int64_t ldy, int64_t b, T alpha, T beta, const T *Z, int64_t ldz, T gamma, int epi,
                        cudaStream_t s);

// dense pairwise couplings (kf_pairs.cu)
void pairs_plan(kf_op *op, const std::vector<std::vector<double>> &hdata);
size_t pairs_smem_bytes(const PairPlan &pp, size_t elem);
template <typename T>
void apply_pairs(const kf_op *op, const T *X, int64_t ldx, T *Y, int64_t ldy, int64_t b, const T *D, int accumulate,
                 T *scratch, cudaStream_t s);

// kernels of kf_op.cu
void launch_apply(kf_op *op, bool f32, const void *X, void *Y, int64_t ldx, int64_t ldy, int64_t b,
                  double alpha, double beta, const void *Z, int64_t ldz, double gamma, cudaStream_t s);

// the Rayleigh-Ritz eigenproblem of an FP32 LOBPCG iteration on the device (kf_rr.cu): from the
// Gram blocks G (merged ld x ld layout, or packed [X_a'HX_a | X_a'HZ | Q'HZ]), writes the update
// coefficients C (ns x 2 na, column-major) and the na lowest Ritz values to theta; false (nothing
// launched) when na + k > 64.  `status`: the device Cholesky's word; nonzero -> C keeps X, drops P
bool rr_eig_device(const double *G, int ldg, bool packed, int na, int k, double *C, double *theta, const int *status,
                   cudaStream_t s);

// time evolution under port drives (kf_drive.cu; src/quantumtoolbox.jl drive_hamiltonian with
// basis = :free): Y = H(t) X, H(t) = 2 pi [H0 - E0 + sum_k coef_k O_k] (rad/ns), X a complex block of m
// columns stored as 2m FP64 columns (real parts, then imaginary parts); omega != nullptr: the
// interaction frame e^{i Omega t} (H(t) - diag Omega) e^{-i Omega t}.  Device pointers, H0's stream.
// ports_im (may be NULL): the imaginary components of ports of complex character (entries may be NULL)
void drive_apply(kf_op *H0, double E0, int nports, kf_op *const *ports, kf_op *const *ports_im, const double *coef,
                 const double *omega, double t, const double *X, int64_t ldx, double *Y, int64_t ldy, int64_t m);
// X <- e^{sign i Omega t} X in place (complex block of m columns as above)
void rotate_rows(const double *omega, int64_t N, double t, double sign, double *X, int64_t ldx, int64_t m,
                 cudaStream_t s);

// the linear solve on the complement of known states (kf_cg.cu; src/resolvent.jl:146-252): per
// column, state 0 met its tolerance, 1 converged from the start (x = 0), 2 stopped at the round-off
// floor; residuals[j] the true residual relative to ||Q B_j|| (state 0), floor_residuals[j] relative
// to scale_j (state 2)
struct CgResult {
    int iterations = 0;
    std::vector<int> state;
    std::vector<double> residuals, floor_residuals;
};
void complement_solve(kf_op *op, const double *basis, int64_t ldbs, int nb, const double *B, int64_t ldb, int n,
                      const double *shifts, const double *scale, double tol, int maxiter, double eta, double *X_out,
                      int64_t ldx, CgResult &res, cudaStream_t s);

// run the fused apply's tuner now for every width class up to maxb columns not yet tuned for this
// operator's stencil shape (X, Y: N x maxb device blocks, leading dimension ld, contents unused)
void pretune_apply(kf_op *op, bool f32, const void *X, void *Y, int64_t ld, int maxb, cudaStream_t s);

// dense linear algebra on tall-skinny blocks (kf_blas.cu); T = float or double.
// Column-major blocks with leading dimension ld.
// G = A' B (ka x kb, column-major, FP64); FP32 blocks of N >= GRAM_TC_MIN_ROWS rows on the tensor
// cores when the shapes fit and allow_tc, else on the SIMT pipes
constexpr int64_t GRAM_TC_MIN_ROWS = 65536;
template <typename T>
void gram(const T *A, int64_t lda, int ka, const T *B, int64_t ldb, int kb, int64_t N, double *G_dev,
          double *partials, cudaStream_t s, bool allow_tc = true);
void perturb_block(double *X, int64_t N, int k, double delta, uint64_t key, double *R, double *nrm, double *partials,
                   cudaStream_t s);
// refinement phase: FP64 iterate, FP32 residual / directions
void residual_mixed(const double *X, const double *HX, int64_t ld, int k, int64_t N, const double *theta,
                    const double *thetap, const double *D, double eta, int mode, float *R, int64_t ldr, float *W,
                    int64_t ldw, double *norms2, double *partials, cudaStream_t s);
// FP32 Gram on the tensor cores: the sources are stacked as the rows of one pool (each at a multiple
// of 8 rows); G (nr x nc, column-major, ld nr) = [sources r0..r1-1]' [sources c0..c1-1], in FP64.
// Returns false, launching nothing, when the shapes do not fit the kernel (the row-only sources and
// the column sources over 128 rows, column sources over 64 columns, unaligned columns, too small a
// partial buffer).
struct GramTcSrc {
    const float *p;
    int64_t ld;
    int k;
};
bool gram_tc(const GramTcSrc *src, int nsrc, int r0, int r1, int c0, int c1, int64_t N, double *G, void *partials,
             size_t partial_bytes, cudaStream_t s);
size_t gram_tc_partials_size(int nr, int nc);
// a 2-D tensor map (a CUtensorMap, 64-byte aligned, 128 bytes) of an FP32 column block: N rows x k
// columns, leading dimension ld, boxes of 128 rows x k columns, unswizzled, rows past N read as zero
// and clipped on stores; false where the CUDA driver gives no encoder or k > 256 (the caller checks the
// base is 16-byte aligned and ld a multiple of 4); cached per (p, ld, N, k)
bool tensor_map_cols(const float *p, int64_t ld, int64_t N, int k, void *map);
// second orthogonalisation pass on the device: from G = [X Z]'Z, coefficients C ((r + wx) x r)
// with [Z X] C orthonormal and orthogonal to X (Cholesky of Z'Z - (X'Z)'(X'Z)); *status 1 on failure
constexpr int CHOL2_MAX_R = 64;
void chol2_coeffs(const double *G, int wx, int r, double *C, int *status, cudaStream_t s);
// Y[:, j] = d_j X[:, j] + (double) P[:, j] and Y32 = FP32(Y) (leading dimension N)
void scale_add(double *Y, const double *X, const double *d, const float *P, float *Y32, int k, int64_t N,
               cudaStream_t s);
void add_f32_into_f64(double *Y, int64_t ldy, const float *P, int64_t ldp, float *Y32, int64_t ld32, int k, int64_t N,
                      cudaStream_t s);
// G = [A0 A1]' [B0 B1] for FP32 column blocks (a block with 0 columns is skipped)
void gram32_sets(const float *A0, int64_t lda0, int ka0, const float *A1, int64_t lda1, int ka1, const float *B0,
                 int64_t ldb0, int kb0, const float *B1, int64_t ldb1, int kb1, int64_t N, double *G, double *partials,
                 cudaStream_t s, bool allow_tc = true);
// FP32 [Y0 Y1] = alpha [X0 X1] C + beta [Y0 Y1] (ky0 + ky1 <= 64 outputs, kx0 + kx1 <= 64 inputs,
// X blocks 16-byte aligned with ld % 4 == 0), a pipelined SIMT kernel; false when it does not apply
bool update_pipe(float *Y0, int64_t ldy0, int ky0, float *Y1, int64_t ldy1, int ky1, const float *X0, int64_t ldx0,
                 int kx0, const float *X1, int64_t ldx1, int kx1, const double *C, int ldc, double alpha, double beta,
                 int64_t N, cudaStream_t s);
// FP64 Y = X C (kx, ky <= 32) in double-float arithmetic on the FP32 pipes (relative error near
// 2^-46); false when it does not apply
bool update_f64_df(double *Y, int64_t ldy, int ky, const double *X, int64_t ldx, int kx, const double *C, int ldc,
                   int64_t N, cudaStream_t s);
// Y = alpha [X0 X1] C + beta Y
template <typename T>
void update2(T *Y, int64_t ldy, int ky, const T *X0, int64_t ldx0, int kx0, const T *X1, int64_t ldx1, int kx1,
             const double *C, int ldc, double alpha, double beta, int64_t N, cudaStream_t s, bool allow_tc = true);
size_t gram_partials_size(int ka, int kb, int64_t N);
template <typename T>
void update(T *Y, int64_t ldy, int ky, const T *X, int64_t ldx, int kx, const double *C_dev, int ldc,
            double alpha, double beta, int64_t N, cudaStream_t s);   // Y = alpha X C + beta Y
template <typename T>
void colnorms2(const T *X, int64_t ldx, int k, int64_t N, double *out_dev, double *partials, cudaStream_t s);
template <typename T>
void residual_precond(const T *X, const T *HX, int64_t ld, int k, int64_t N, const double *theta_dev,
                      const double *thetap_dev, const double *D_dev, double eta, int mode, T *R, int64_t ldr,
                      double *norms2_dev, double *partials, cudaStream_t s);
template <typename T>
void scale_columns(T *X, int64_t ld, int k, int64_t N, const double *scale_dev, cudaStream_t s);
template <typename T>
void fill_normal(T *X, int64_t ld, int k, int64_t N, uint64_t seed, uint64_t stream_id, cudaStream_t s);
template <typename Ts, typename Td>
void convert(const Ts *X, int64_t ldx, Td *Y, int64_t ldy, int k, int64_t N, cudaStream_t s);
template <typename T>
void copy_block(const T *X, int64_t ldx, T *Y, int64_t ldy, int k, int64_t N, cudaStream_t s);
template <typename T>
void residual_block(const T *X, const T *HX, int64_t ld, int k, int64_t N, const double *theta_dev, T *R,
                    int64_t ldr, cudaStream_t s);    // R = HX - X diag(theta)
void diag_expectation(const double *D, const double *X, int64_t ld, int k, int64_t N, double *theta_dev,
                      double *partials, cudaStream_t s);

// dense mode products and the separable preconditioner (kf_dense.cu, kf_precond.cu)
template <typename T>
void mode_product(T *Y, int64_t ldy, const T *X, int64_t ldx, const T *A, int d, int64_t left, int64_t N, int64_t b,
                  double alpha, double beta, cudaStream_t s);
// W[:, j] /= hypot(S(p) - theta_j, eta); shl (may be NULL): S(p) as FP32 hi / lo pairs from
// sep_spectrum, else S(p) is formed from the per-axis eigenvalues point by point
template <typename T>
void sep_scale(T *W, int64_t ld, int64_t N, int k, int ndims, const int *dims, const double *lam, const int *lam_off,
               const double *theta, double eta, cudaStream_t s, const float *shl = nullptr);
// shl[2p], shl[2p + 1] = S(p) = sum_a lam_a[i_a(p)] split into FP32 hi + lo (N points)
void sep_spectrum(float *shl, int64_t N, int ndims, const int *dims, const double *lam, const int *lam_off,
                  cudaStream_t s);
void sep_host_prepare(kf_op *op);   // host part only (no CUDA calls)
void sep_prepare(kf_op *op);
// product_seed(H, k) into the device block X (N x k, leading dimension N), on stream s
void product_seed_device(kf_op *op, int k, double *X, cudaStream_t s);
// W (N x k, FP32, leading dimension N) <- U diag(1 / hypot(S - theta_j, eta)) U' W; s1 is an
// N x k FP32 scratch.  Returns the block holding the result (W or s1).
float *sep_apply(kf_op *op, float *W, float *s1, int k, const double *theta_dev, double eta, cudaStream_t s);

// small dense FP64 routines on the host (kf_small.cpp); column-major.
int sym_eig(int n, const double *A, int lda, double *w, double *V, int ldv);   // ascending
bool cholesky_upper(int n, double *A, int lda);     // A = U'U in place (upper), false if not SPD
void tri_upper_inverse(int n, const double *U, int ldu, double *Ui, int ldi);

}  // namespace kf

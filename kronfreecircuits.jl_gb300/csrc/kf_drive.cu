// Matrix-free time evolution under port drives: the action of the reference's drive Hamiltonian on
// a node's product basis (src/quantumtoolbox.jl:84-99, drive_hamiltonian with basis = :free, the
// QobjEvo around KronFreeOperator and port_operator that QuantumToolbox's sesolve applies), and the
// frame rotation to_lab (src/quantumtoolbox.jl:25-37).
//
//   H(t) = 2 pi [H0 - E0 + sum_k f_k(t) O_k]        (rad/ns; f_k in GHz, E0 the node's lowest energy)
//   interaction frame: H_I(t) = e^{i Omega t} (H(t) - diag Omega) e^{-i Omega t},   psi_lab = e^{-i Omega t} psi_I
//
// H0 is a real operator (the real-by-structure circuits: every measured one), so on a complex block
// it acts on the real and the imaginary parts alike: the block of m complex columns is stored as 2m
// FP64 columns (real parts, then imaginary parts) and every product is one real apply of the
// existing kernels over 2m columns.  A port of complex character (e^{i phi}, e^{2 pi i n k}: the
// reference's real-character ports are the real ones) is given as its real and imaginary
// components, two real operators O = O_re + i O_im: i O_im psi is O_im applied to the same 2m
// columns with its halves exchanged and one negated.  The rotations and the accumulation of the
// port terms are elementwise kernels here.
#include "kf_internal.h"

namespace kf {

namespace {

// Y[:, j] += T[:, j] for j < w
__global__ void k_drive_acc(double *__restrict__ Y, int64_t ldy, const double *__restrict__ T, int64_t ldt, int64_t N,
                            int w) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= N || j >= w) return;
    Y[i + ldy * j] += T[i + ldt * j];
}

// Y = e^{sign i omega_r t} X, row r (complex columns j and m + j); Y may be X
__global__ void k_rotate(const double *X, int64_t ldx, double *Y, int64_t ldy, const double *__restrict__ omega,
                         double t, double sign, int64_t N, int m) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (r >= N || j >= m) return;
    double sn, cs;
    sincos(sign * omega[r] * t, &sn, &cs);
    const double a = X[r + ldx * j], b = X[r + ldx * (m + j)];
    Y[r + ldy * j] = a * cs - b * sn;
    Y[r + ldy * (m + j)] = a * sn + b * cs;
}

// Y += i T for complex blocks of m columns (real halves first): Y_re -= T_im, Y_im += T_re
__global__ void k_drive_acc_i(double *__restrict__ Y, int64_t ldy, const double *__restrict__ T, int64_t ldt,
                              int64_t N, int m) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= N || j >= m) return;
    const double tr = T[i + ldt * j], ti = T[i + ldt * (m + j)];
    Y[i + ldy * j] -= ti;
    Y[i + ldy * (m + j)] += tr;
}

// Y <- e^{i omega_r t} (Y - omega_r U), row r: the interaction frame's last step
__global__ void k_rotate_sub(double *__restrict__ Y, int64_t ldy, const double *__restrict__ U, int64_t ldu,
                             const double *__restrict__ omega, double t, int64_t N, int m) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (r >= N || j >= m) return;
    const double w = omega[r];
    double sn, cs;
    sincos(w * t, &sn, &cs);
    const double a = Y[r + ldy * j] - w * U[r + ldu * j], b = Y[r + ldy * (m + j)] - w * U[r + ldu * (m + j)];
    Y[r + ldy * j] = a * cs - b * sn;
    Y[r + ldy * (m + j)] = a * sn + b * cs;
}

constexpr double TWO_PI = 6.283185307179586476925286766559;

}  // namespace

void rotate_rows(const double *omega, int64_t N, double t, double sign, double *X, int64_t ldx, int64_t m,
                 cudaStream_t s) {
    if (N == 0 || m == 0) return;
    k_rotate<<<dim3((unsigned)((N + 255) / 256), (unsigned)m), 256, 0, s>>>(X, ldx, X, ldx, omega, t, sign, N, (int)m);
    KF_LAUNCH_CHECK();
}

void drive_apply(kf_op *H0, double E0, int nports, kf_op *const *ports, kf_op *const *ports_im, const double *coef,
                 const double *omega, double t, const double *X, int64_t ldx, double *Y, int64_t ldy, int64_t m) {
    const int64_t N = H0->N, w = 2 * m;
    cudaStream_t s = H0->stream;
    if (N == 0 || m == 0) return;
    int used = 0;
    for (int k = 0; k < nports; ++k) used += coef[k] != 0.0;
    // scratch: the rotated block U (interaction frame) and one port's product T, N x 2m each
    const size_t need = (size_t)N * w * sizeof(double) * ((omega ? 1 : 0) + (used ? 1 : 0));
    if (need > H0->drive_bytes) {
        KF_CUDA(cudaStreamSynchronize(s));
        if (H0->d_drive) KF_CUDA(cudaFree(H0->d_drive));
        H0->d_drive = nullptr;
        H0->drive_bytes = 0;
        KF_CUDA(cudaMalloc(&H0->d_drive, need));
        H0->drive_bytes = need;
    }
    double *U = omega ? (double *)H0->d_drive : nullptr;
    double *T = (double *)H0->d_drive + (omega ? (size_t)N * w : 0);
    const double *src = X;
    int64_t lds = ldx;
    const dim3 g((unsigned)((N + 255) / 256), (unsigned)m), g2((unsigned)((N + 255) / 256), (unsigned)w);
    if (omega) {
        k_rotate<<<g, 256, 0, s>>>(X, ldx, U, N, omega, t, -1.0, N, (int)m);   // e^{-i Omega t} X
        KF_LAUNCH_CHECK();
        src = U;
        lds = N;
    }
    // Y = 2 pi (H0 - E0) src
    launch_apply(H0, false, src, Y, lds, ldy, w, TWO_PI, -TWO_PI * E0, nullptr, 0, 0.0, s);
    for (int k = 0; k < nports; ++k) {
        if (coef[k] == 0.0) continue;
        // the port's products on H0's stream, then accumulated (the imaginary component times i)
        if (ports[k]) {
            launch_apply(ports[k], false, src, T, lds, N, w, TWO_PI * coef[k], 0.0, nullptr, 0, 0.0, s);
            k_drive_acc<<<g2, 256, 0, s>>>(Y, ldy, T, N, N, (int)w);
            KF_LAUNCH_CHECK();
        }
        if (ports_im && ports_im[k]) {
            launch_apply(ports_im[k], false, src, T, lds, N, w, TWO_PI * coef[k], 0.0, nullptr, 0, 0.0, s);
            k_drive_acc_i<<<g, 256, 0, s>>>(Y, ldy, T, N, N, (int)m);
            KF_LAUNCH_CHECK();
        }
    }
    if (omega) {
        k_rotate_sub<<<g, 256, 0, s>>>(Y, ldy, U, N, omega, t, N, (int)m);     // e^{i Omega t} (Y - Omega U)
        KF_LAUNCH_CHECK();
    }
}

}  // namespace kf

// The Rayleigh-Ritz eigenproblem of LOBPCG's FP32 phase on the device (the reference's RR inside
// LOBPCGEigensolver, called at src/lobpcg.jl:268): A = S' H S on S = [X_a Q] (ns <= 64) from the
// Gram blocks the tensor-core or SIMT Gram left on the device, its eigenpairs by cyclic Jacobi in
// FP32 on one CTA, and the update coefficients [C_x | C_p] and Ritz values written straight into the
// buffers the block updates and the next residual read.  So an FP32 iteration waits on the host
// once (residual norms with the first Gram), not twice.  Opt-in (KF_DEVICE_RR=1): measured on GB300
// the kernel costs more GPU time per iteration (~150-200 us on one SM) than the host round trip it
// removes (~65 us of idle GPU), 111.9 against 122.8 eigenpairs/s on the three-mode leaf.
//
// Why FP32 suffices here: the FP32 phase stops at residuals of 1e-6 ||H||; Jacobi in FP32 gives
// Ritz values to about 1e-7 of ||A|| <= ||H|| and eigenvectors orthonormal to about 1e-7, the
// precision of the FP32 blocks they rotate.  The FP64 refinement keeps its FP64 Rayleigh-Ritz.
//
// Jacobi: the round-robin ("chess tournament") ordering gives m / 2 disjoint pairs per round,
// m - 1 rounds per sweep (m = ns rounded up to even; an odd ns gets a padding row with a diagonal
// of 1e30 that sorts last); per round one thread per pair forms the rotation that zeroes A[p][q]
// (Golub & Van Loan, the symmetric Schur decomposition), then all rows, all columns and V are
// rotated with the block's threads.  Sweeps stop when the off-diagonal Frobenius norm is below
// 4 eps of the whole, when (below 1e-5 of it) a sweep no longer halves it, or after 10.  The
// retained vectors are then re-orthonormalised and their Ritz values taken as Rayleigh quotients of
// the original matrix (rotations orthogonal only to rounding scale the block by ~1e-5 over a few
// hundred rounds).
//
// When the device Cholesky of this iteration's second orthogonalisation pass failed (its status
// word), the kernel writes coefficients that leave X as it is and P zero, and keeps theta; the host
// reads the status at its next wait and takes the host orthogonalisation for that iteration.
#include <cfloat>

#include "kf_internal.h"

namespace kf {

namespace {

constexpr int RR_MAX = 64;
constexpr int RR_THREADS = 512;
constexpr int RR_MAX_SWEEPS = 10;

__global__ void __launch_bounds__(RR_THREADS) k_rr_jacobi(const double *__restrict__ G, int ldg, int packed, int na,
                                                          int k, double *__restrict__ C, double *__restrict__ theta,
                                                          const int *__restrict__ status) {
    __shared__ float A[RR_MAX][RR_MAX + 1];
    __shared__ float V[RR_MAX][RR_MAX + 1];
    __shared__ float cs[RR_MAX / 2], sn[RR_MAX / 2];
    __shared__ int pp[RR_MAX / 2], pq[RR_MAX / 2];
    __shared__ int perm[RR_MAX];
    __shared__ float red[2][RR_THREADS / 32];
    __shared__ int s_skip, s_done;
    __shared__ float s_prev_off;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ns = na + k, m = (ns + 1) & ~1, h = m / 2;
    if (tid == 0) {
        s_skip = *status != 0;
        s_prev_off = FLT_MAX;
    }
    __syncthreads();
    if (s_skip) {
        for (int e = tid; e < ns * 2 * na; e += blockDim.x) {
            const int i = e % ns, j = e / ns;
            C[e] = (j < na && i == j) ? 1.0 : 0.0;
        }
        return;
    }
    // A from the upper triangle of the Gram blocks (rows [X_a; Q], columns [H X_a, H Z])
    for (int e = tid; e < m * m; e += blockDim.x) {
        const int i = e % m, j = e / m;
        float v = 0.f;
        if (i < ns && j < ns) {
            const int a = min(i, j), b = max(i, j);
            double g;
            if (!packed) g = G[a + (size_t)ldg * b];
            else if (b < na) g = G[a + (size_t)na * b];
            else if (a < na) g = G[(size_t)na * na + a + (size_t)na * (b - na)];
            else g = G[(size_t)na * na + (size_t)na * k + (a - na) + (size_t)k * (b - na)];
            v = (float)g;
        } else if (i == j) {
            v = 1e30f;   // the padding row of an odd ns: decoupled, sorts last
        }
        A[i][j] = v;
        V[i][j] = i == j ? 1.f : 0.f;
    }
    __syncthreads();
    for (int sweep = 0; sweep < RR_MAX_SWEEPS; ++sweep) {
        for (int r = 0; r < m - 1; ++r) {
            if (tid < h) {
                // round r: player 0 fixed, the others rotated by r; pair positions tid and m - 1 - tid
                auto player = [&](int pos) { return pos == 0 ? 0 : 1 + (pos - 1 + r) % (m - 1); };
                int p = player(tid), q = player(m - 1 - tid);
                if (p > q) {
                    const int t = p;
                    p = q;
                    q = t;
                }
                const float app = A[p][p], aqq = A[q][q], apq = A[p][q];
                float c = 1.f, s = 0.f;
                if (apq != 0.f) {
                    const float tau = (aqq - app) / (2.f * apq);
                    const float t = copysignf(1.f, tau) / (fabsf(tau) + sqrtf(1.f + tau * tau));
                    c = 1.f / sqrtf(1.f + t * t);
                    s = t * c;
                }
                pp[tid] = p;
                pq[tid] = q;
                cs[tid] = c;
                sn[tid] = s;
            }
            __syncthreads();
            // rows p, q of A (A <- J' A)
            for (int e = tid; e < h * m; e += blockDim.x) {
                const int t = e / m, j = e % m;
                const int p = pp[t], q = pq[t];
                const float c = cs[t], s = sn[t];
                const float ap = A[p][j], aq = A[q][j];
                A[p][j] = c * ap - s * aq;
                A[q][j] = s * ap + c * aq;
            }
            __syncthreads();
            // columns p, q of A (A <- A J) and of V (V <- V J)
            for (int e = tid; e < h * m; e += blockDim.x) {
                const int t = e / m, i = e % m;
                const int p = pp[t], q = pq[t];
                const float c = cs[t], s = sn[t];
                const float ap = A[i][p], aq = A[i][q];
                A[i][p] = c * ap - s * aq;
                A[i][q] = s * ap + c * aq;
                const float vp = V[i][p], vq = V[i][q];
                V[i][p] = c * vp - s * vq;
                V[i][q] = s * vp + c * vq;
            }
            __syncthreads();
        }
        // off-diagonal and total Frobenius norms of the real block (the padding excluded)
        float off = 0.f, tot = 0.f;
        for (int e = tid; e < ns * ns; e += blockDim.x) {
            const int i = e % ns, j = e / ns;
            const float v = A[i][j] * A[i][j];
            tot += v;
            if (i != j) off += v;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            off += __shfl_down_sync(0xffffffffu, off, o);
            tot += __shfl_down_sync(0xffffffffu, tot, o);
        }
        if (lane == 0) {
            red[0][warp] = off;
            red[1][warp] = tot;
        }
        __syncthreads();
        if (tid == 0) {
            float o = 0.f, t = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
                o += red[0][w];
                t += red[1][w];
            }
            // off-diagonal below 4 eps of the whole (squared), or, once below 1e-5 of it, a sweep
            // that no longer halves it (the FP32 rounding floor)
            s_done = o <= 2.27e-13f * t || (o <= 1e-10f * t && o > 0.25f * s_prev_off);
            s_prev_off = o;
        }
        __syncthreads();
        if (s_done) break;
    }
    // ascending order of the Ritz values
    if (tid == 0) {
        for (int i = 0; i < m; ++i) perm[i] = i;
        for (int i = 1; i < m; ++i) {
            const int x = perm[i];
            const float v = A[x][x];
            int j = i - 1;
            while (j >= 0 && A[perm[j]][perm[j]] > v) {
                perm[j + 1] = perm[j];
                --j;
            }
            perm[j + 1] = x;
        }
    }
    __syncthreads();
    // the na retained vectors as the rows of U (A's storage is free now); rotations that are
    // orthogonal only to rounding scale the block a little over hundreds of rounds, so the vectors
    // are re-orthonormalised (classical Gram-Schmidt, twice) and the Ritz values taken as Rayleigh
    // quotients against the original matrix, read again from G
    float(*U)[RR_MAX + 1] = A;
    for (int e = tid; e < na * ns; e += blockDim.x) {
        const int j = e / ns, i = e % ns;
        U[j][i] = V[i][perm[j]];
    }
    __syncthreads();
    __shared__ float dots[RR_MAX];
    for (int j = 0; j < na; ++j) {
        for (int pass = 0; pass < 2; ++pass) {
            // d_i = <u_i, u_j> for i < j, one warp per i
            for (int i = warp; i < j; i += blockDim.x >> 5) {
                float d = 0.f;
                for (int a = lane; a < ns; a += 32) d += U[i][a] * U[j][a];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xffffffffu, d, o);
                if (lane == 0) dots[i] = d;
            }
            __syncthreads();
            for (int a = tid; a < ns; a += blockDim.x) {
                float v = U[j][a];
                for (int i = 0; i < j; ++i) v -= dots[i] * U[i][a];
                U[j][a] = v;
            }
            __syncthreads();
            if (warp == 0) {
                float d = 0.f;
                for (int a = lane; a < ns; a += 32) d += U[j][a] * U[j][a];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xffffffffu, d, o);
                d = __shfl_sync(0xffffffffu, d, 0);
                const float inv = 1.f / sqrtf(d);
                for (int a = lane; a < ns; a += 32) U[j][a] *= inv;
            }
            __syncthreads();
        }
    }
    // Rayleigh quotients u_j' A u_j against the Gram blocks (upper triangle), one warp per j
    auto gsym = [&](int a, int b) -> float {
        if (a > b) {
            const int t = a;
            a = b;
            b = t;
        }
        double g;
        if (!packed) g = G[a + (size_t)ldg * b];
        else if (b < na) g = G[a + (size_t)na * b];
        else if (a < na) g = G[(size_t)na * na + a + (size_t)na * (b - na)];
        else g = G[(size_t)na * na + (size_t)na * k + (a - na) + (size_t)k * (b - na)];
        return (float)g;
    };
    for (int j = warp; j < na; j += blockDim.x >> 5) {
        float q = 0.f;
        for (int a = lane; a < ns; a += 32) {
            float row = 0.f;
            for (int b = 0; b < ns; ++b) row += gsym(a, b) * U[j][b];
            q += U[j][a] * row;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) q += __shfl_down_sync(0xffffffffu, q, o);
        if (lane == 0) theta[j] = (double)q;
    }
    // [X_new P_new] = [X_a Q] [C_x | [0; C_z]]: C is ns x 2 na, column-major
    for (int e = tid; e < ns * 2 * na; e += blockDim.x) {
        const int i = e % ns, j = e / ns;
        const int col = j < na ? j : j - na;
        C[e] = (j >= na && i < na) ? 0.0 : (double)U[col][i];
    }
}

}  // namespace

bool rr_eig_device(const double *G, int ldg, bool packed, int na, int k, double *C, double *theta, const int *status,
                   cudaStream_t s) {
    if (na < 1 || k < 0 || na + k > RR_MAX) return false;
    k_rr_jacobi<<<1, RR_THREADS, 0, s>>>(G, ldg, packed ? 1 : 0, na, k, C, theta, status);
    KF_LAUNCH_CHECK();
    return true;
}

}  // namespace kf

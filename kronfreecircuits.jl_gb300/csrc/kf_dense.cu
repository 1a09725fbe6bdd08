// Mode-k products with a dense d x d matrix, Y[l, i, r] = alpha sum_j A[i, j] X[l, j, r] (+ beta Y),
// for blocks of columns (the column index folds into r), as one shared-memory-tiled GEMM:
//   rows m = (l, r) (l fastest, left = stride of axis k), columns i, reduction over j.
// Reference: the dense factor application of src/apply.jl:37-53 and 301-340 (which permutes a
// middle axis to the front through scratch; here the strided rows are gathered by the tile
// loader instead, so no permute passes).
//
// Tile: 64 rows x 64 columns x 16 reduction per step, 256 threads, a 4 x 4 register tile per
// thread.  The X tile loader walks l fastest when the axis stride is > 1 (coalesced along l) and
// j fastest when the axis is the leading one (coalesced along j).
#include <algorithm>

#include "kf_internal.h"

namespace kf {

constexpr int DM = 64, DN = 64, DK = 16;

template <typename T>
__global__ void __launch_bounds__(256) k_mode_product(T *__restrict__ Y, int64_t ldy, const T *__restrict__ X,
                                                      int64_t ldx, const T *__restrict__ A, int d, int64_t left,
                                                      int64_t rows_per_col, int64_t M, int64_t N, T alpha, T beta) {
    __shared__ T Xs[DK][DM + 1];
    __shared__ T As[DK][DN + 1];
    const int tid = threadIdx.x;
    const int64_t m0 = (int64_t)blockIdx.x * DM;
    const int i0 = blockIdx.y * DN;
    const int tr = (tid % 16) * 4, tc = (tid / 16) * 4;
    T acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = T(0);
    // base offset of row m: column c = m / rows_per_col of the block, within it (l, r) with
    // l = q % left, r = q / left, element (l, j, r) at l + left * (j + d * r)
    for (int j0 = 0; j0 < d; j0 += DK) {
        if (left == 1) {
            // j fastest: X[j + d * q] per column
            for (int e = tid; e < DM * DK; e += 256) {
                const int jj = e % DK, mm = e / DK;
                const int64_t m = m0 + mm;
                const int j = j0 + jj;
                T v = T(0);
                if (m < M && j < d) {
                    const int64_t c = m / rows_per_col, q = m % rows_per_col;
                    v = X[c * ldx + (int64_t)j + (int64_t)d * q];
                }
                Xs[jj][mm] = v;
            }
        } else {
            for (int e = tid; e < DM * DK; e += 256) {
                const int mm = e % DM, jj = e / DM;
                const int64_t m = m0 + mm;
                const int j = j0 + jj;
                T v = T(0);
                if (m < M && j < d) {
                    const int64_t c = m / rows_per_col, q = m % rows_per_col;
                    const int64_t l = q % left, r = q / left;
                    v = X[c * ldx + l + left * ((int64_t)j + (int64_t)d * r)];
                }
                Xs[jj][mm] = v;
            }
        }
        // A tile: As[jj][ii] = A[i, j] (A column-major, A[i + d * j])
        for (int e = tid; e < DN * DK; e += 256) {
            const int ii = e % DN, jj = e / DN;
            const int i = i0 + ii, j = j0 + jj;
            As[jj][ii] = (i < d && j < d) ? A[(int64_t)i + (int64_t)d * j] : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int jj = 0; jj < DK; ++jj) {
            T a[4], x[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) x[u] = Xs[jj][tr + u];
#pragma unroll
            for (int v = 0; v < 4; ++v) a[v] = As[jj][tc + v];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] += x[u] * a[v];
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int64_t m = m0 + tr + u;
        if (m >= M) continue;
        const int64_t c = m / rows_per_col, q = m % rows_per_col;
        const int64_t l = q % left, r = q / left;
        T *yrow = Y + c * ldy + l + left * ((int64_t)d * r);
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int i = i0 + tc + v;
            if (i >= d) continue;
            T *yp = yrow + left * (int64_t)i;
            *yp = (beta == T(0)) ? alpha * acc[u][v] : alpha * acc[u][v] + beta * *yp;
        }
    }
}

// Y = alpha (A along `axis` of X) + beta Y for a block of b columns of length N, the axis of
// length d with stride `left`.  A is d x d column-major on the device.
template <typename T>
void mode_product(T *Y, int64_t ldy, const T *X, int64_t ldx, const T *A, int d, int64_t left, int64_t N, int64_t b,
                  double alpha, double beta, cudaStream_t s) {
    if (b <= 0 || N <= 0) return;
    const int64_t rows_per_col = N / d;          // (l, r) pairs per column
    const int64_t M = rows_per_col * b;
    dim3 grid((unsigned)((M + DM - 1) / DM), (unsigned)((d + DN - 1) / DN));
    k_mode_product<T><<<grid, 256, 0, s>>>(Y, ldy, X, ldx, A, d, left, rows_per_col, M, N, (T)alpha, (T)beta);
    KF_LAUNCH_CHECK();
}

template void mode_product<float>(float *, int64_t, const float *, int64_t, const float *, int, int64_t, int64_t,
                                  int64_t, double, double, cudaStream_t);
template void mode_product<double>(double *, int64_t, const double *, int64_t, const double *, int, int64_t, int64_t,
                                   int64_t, double, double, cudaStream_t);

constexpr int SEP_SCALE_MAX_K = 256;   // columns per scale pass

// W[:, j] <- W[:, j] / hypot(S(p) - theta_j, eta) with S(p) = sum_a lam_a[i_a(p)] (the separable
// spectrum evaluated from per-axis eigenvalues, no N-sized table).  One thread per grid point: the
// point's indices and S(p) (FP64, one sum per point) serve every column.  S and theta are close
// where it matters, so both are split into FP32 hi + lo parts and S - theta = (S_hi - theta_hi) +
// (S_lo - theta_lo), the first difference exact there; the scale itself is FP32 -- it only steers
// the search directions, and GB300's FP64 rate would make a per-element FP64 pass FP64-bound.
// S(p) = sum_a lam_a[i_a(p)] in FP64 (one sum per point), split into FP32 hi + lo
__device__ __forceinline__ void sep_point(int64_t p, int ndims, const int *__restrict__ dims,
                                          const double *__restrict__ lam, const int *__restrict__ lam_off, float &hi,
                                          float &lo) {
    uint32_t rem = (uint32_t)p;
    double S = 0.0;
    for (int a = 0; a < ndims; ++a) {
        const uint32_t d = (uint32_t)dims[a];
        const uint32_t i = rem % d;
        rem /= d;
        S += lam[lam_off[a] + (int)i];
    }
    hi = (float)S;
    lo = (float)(S - (double)hi);
}

__global__ void k_sep_spectrum(float *__restrict__ shl, int64_t N, int ndims, const int *__restrict__ dims,
                               const double *__restrict__ lam, const int *__restrict__ lam_off) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (int64_t)gridDim.x * blockDim.x) {
        float hi, lo;
        sep_point(p, ndims, dims, lam, lam_off, hi, lo);
        reinterpret_cast<float2 *>(shl)[p] = make_float2(hi, lo);
    }
}

// W[:, j] <- W[:, j] / hypot(S(p) - theta_j, eta) with S(p) = sum_a lam_a[i_a(p)] (the separable
// spectrum evaluated from per-axis eigenvalues).  One thread per grid point: the point's S(p) serves
// every column, read from the operator's hi / lo table when there is one (it depends on the operator
// only), else formed from the per-axis eigenvalues (FP64, one sum per point).  S and theta are close
// where it matters, so both are split into FP32 hi + lo parts and S - theta = (S_hi - theta_hi) +
// (S_lo - theta_lo), the first difference exact there; the scale itself is FP32 -- it only steers
// the search directions, and GB300's FP64 rate would make a per-element FP64 pass FP64-bound.
template <typename T>
__global__ void k_sep_scale(T *__restrict__ W, int64_t ld, int64_t N, int k, int ndims, const int *__restrict__ dims,
                            const double *__restrict__ lam, const int *__restrict__ lam_off,
                            const double *__restrict__ theta, double eta, const float *__restrict__ shl) {
    __shared__ float th_hi[SEP_SCALE_MAX_K], th_lo[SEP_SCALE_MAX_K];
    for (int c = threadIdx.x; c < k; c += blockDim.x) {
        const float h = (float)theta[c];
        th_hi[c] = h;
        th_lo[c] = (float)(theta[c] - (double)h);
    }
    __syncthreads();
    const float eta2 = (float)(eta * eta);
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (int64_t)gridDim.x * blockDim.x) {
        float s_hi, s_lo;
        if (shl) {
            const float2 v = reinterpret_cast<const float2 *>(shl)[p];
            s_hi = v.x;
            s_lo = v.y;
        } else {
            sep_point(p, ndims, dims, lam, lam_off, s_hi, s_lo);
        }
        for (int c = 0; c < k; ++c) {
            const float dlt = (s_hi - th_hi[c]) + (s_lo - th_lo[c]);
            const float f = rsqrtf(fmaf(dlt, dlt, eta2));
            W[c * ld + p] = W[c * ld + p] * (T)f;
        }
    }
}

template <typename T>
void sep_scale(T *W, int64_t ld, int64_t N, int k, int ndims, const int *dims, const double *lam, const int *lam_off,
               const double *theta, double eta, cudaStream_t s, const float *shl) {
    if (k <= 0) return;
    KF_REQUIRE(k <= SEP_SCALE_MAX_K, KF_EINVAL, "sep_scale: too many columns");
    KF_REQUIRE(N < ((int64_t)1 << 32), KF_EINVAL, "sep_scale: operator dimension too large");
    const int64_t blocks = std::min<int64_t>((N + 255) / 256, 152 * 8);
    k_sep_scale<T><<<(unsigned)blocks, 256, 0, s>>>(W, ld, N, k, ndims, dims, lam, lam_off, theta, eta, shl);
    KF_LAUNCH_CHECK();
}

void sep_spectrum(float *shl, int64_t N, int ndims, const int *dims, const double *lam, const int *lam_off,
                  cudaStream_t s) {
    KF_REQUIRE(N < ((int64_t)1 << 32), KF_EINVAL, "sep_spectrum: operator dimension too large");
    const int64_t blocks = std::min<int64_t>((N + 255) / 256, 152 * 8);
    k_sep_spectrum<<<(unsigned)blocks, 256, 0, s>>>(shl, N, ndims, dims, lam, lam_off);
    KF_LAUNCH_CHECK();
}

template void sep_scale<float>(float *, int64_t, int64_t, int, int, const int *, const double *, const int *,
                               const double *, double, cudaStream_t, const float *);
template void sep_scale<double>(double *, int64_t, int64_t, int, int, const int *, const double *, const int *,
                                const double *, double, cudaStream_t, const float *);

}  // namespace kf

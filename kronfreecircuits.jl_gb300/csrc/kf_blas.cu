// Tall-skinny block linear algebra for the eigensolvers: Gram matrices, block updates, column
// norms, fused residual + preconditioner, random blocks, conversions.
//
// Reference call sites (KronFreeCircuits.jl): the Gram / Rayleigh-Ritz / projection gemms of
// src/chebyshev.jl:60,71,79,123,126,139-142 and inside LOBPCGEigensolver (called at
// src/lobpcg.jl:268); the residual of src/chebyshev.jl:147-150 and src/solvers.jl:65-69; the
// per-Ritz Jacobi division of src/lobpcg.jl:114-119; the diagonal expectation of
// ext/KronFreeCircuitsCUDAExt.jl:16-55.
//
// Blocks are column-major (N rows, k <= 128 columns, leading dimension ld).  Every reduction
// over N is split across CTAs into FP64 partials and summed in a fixed order by a second
// kernel, so results are deterministic run to run.  In a Gram product each thread accumulates its
// few rows in the block's precision, and the cross-thread sums are FP64.
#include "kf_internal.h"

namespace kf {

constexpr int GRAM_THREADS = 256;
constexpr int RED_THREADS = 256;

static int num_ctas_for(int64_t N, int64_t rows_per) {
    int64_t c = (N + rows_per - 1) / rows_per;
    if (c < 1) c = 1;
    if (c > 1216) c = 1216;               // 8 x 152 SMs
    return (int)c;
}

// rows per CTA so that all chunks together fill about four waves of 152 SMs, at least 256 rows
static int64_t gram_rows_per_cta(int64_t N, int chunks) {
    int64_t target = (608 + chunks - 1) / chunks;
    if (target < 1) target = 1;
    int64_t r = (N + target - 1) / target;
    if (r < 256) r = 256;
    return r;
}

size_t gram_partials_size(int ka, int kb, int64_t N) {
    // the largest CTA count over the chunkings used: one chunk gives the most row blocks
    const int nc = num_ctas_for(N, gram_rows_per_cta(N, 1));
    const size_t a = (size_t)nc * ka * kb;
    const size_t b = (size_t)1216 * 128;  // also enough for the column reductions
    return (a > b ? a : b) * sizeof(double);
}

// partial[cta][i + ka*j] = sum over this CTA's rows of A[r,i] B[r,j], for one RI x RJ chunk of
// the output (blockIdx.y).  Rows stream through the threads (consecutive threads read
// consecutive rows of a column: coalesced), each thread keeps its chunk's products in registers
// (FP32 blocks: FP32 over its few rows), and the CTA sums them in FP64 -- warp shuffles, then the
// warps in a fixed order through shared memory.
template <typename T, int RI, int RJ>
__global__ void __launch_bounds__(GRAM_THREADS) k_gram(const T *__restrict__ A, int64_t lda, int ka,
                                                       const T *__restrict__ B, int64_t ldb, int kb, int64_t N,
                                                       int64_t rows_per, double *__restrict__ partials) {
    __shared__ double red[GRAM_THREADS / 32][RI * RJ];
    const int cj_n = (kb + RJ - 1) / RJ;
    const int i0 = (blockIdx.y / cj_n) * RI, j0 = (blockIdx.y % cj_n) * RJ;
    const int ni = min(RI, ka - i0), nj = min(RJ, kb - j0);
    T acc[RI][RJ];
#pragma unroll
    for (int u = 0; u < RI; ++u)
#pragma unroll
        for (int v = 0; v < RJ; ++v) acc[u][v] = T(0);
    const int64_t r0 = (int64_t)blockIdx.x * rows_per;
    const int64_t r1 = (r0 + rows_per < N) ? r0 + rows_per : N;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += GRAM_THREADS) {
        T a[RI], bv[RJ];
#pragma unroll
        for (int u = 0; u < RI; ++u) a[u] = (u < ni) ? A[r + (int64_t)(i0 + u) * lda] : T(0);
#pragma unroll
        for (int v = 0; v < RJ; ++v) bv[v] = (v < nj) ? B[r + (int64_t)(j0 + v) * ldb] : T(0);
#pragma unroll
        for (int u = 0; u < RI; ++u)
#pragma unroll
            for (int v = 0; v < RJ; ++v) acc[u][v] += a[u] * bv[v];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int u = 0; u < RI; ++u)
#pragma unroll
        for (int v = 0; v < RJ; ++v) {
            double x = (double)acc[u][v];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) red[warp][u * RJ + v] = x;
        }
    __syncthreads();
    double *P = partials + (size_t)blockIdx.x * ka * kb;
    for (int e = threadIdx.x; e < RI * RJ; e += GRAM_THREADS) {
        const int u = e / RJ, v = e % RJ;
        if (u >= ni || v >= nj) continue;
        double s = 0;
        for (int w = 0; w < GRAM_THREADS / 32; ++w) s += red[w][e];
        P[(i0 + u) + (size_t)ka * (j0 + v)] = s;
    }
}

// out[e] = sum_c partials[c][e], e < n, in a fixed order
__global__ void k_reduce_partials(const double *__restrict__ partials, int nparts, int n, double *__restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    double s = 0;
    for (int c = 0; c < nparts; ++c) s += partials[(size_t)c * n + e];
    out[e] = s;
}

template <typename T>
void gram(const T *A, int64_t lda, int ka, const T *B, int64_t ldb, int kb, int64_t N, double *G, double *partials,
          cudaStream_t s) {
    KF_REQUIRE(ka >= 1 && kb >= 1 && ka <= 128 && kb <= 128, KF_EINVAL, "gram: block widths out of range");
    // output chunks of RI x RJ (FP64: 4 x 8, FP32: 8 x 8 accumulators per thread)
    constexpr int RI = sizeof(T) == 8 ? 4 : 8, RJ = 8;
    const int chunks = ((ka + RI - 1) / RI) * ((kb + RJ - 1) / RJ);
    const int64_t rp = gram_rows_per_cta(N, chunks);
    const int nc = num_ctas_for(N, rp);
    k_gram<T, RI, RJ><<<dim3(nc, chunks), GRAM_THREADS, 0, s>>>(A, lda, ka, B, ldb, kb, N, rp, partials);
    KF_LAUNCH_CHECK();
    const int n = ka * kb;
    k_reduce_partials<<<(n + 255) / 256, 256, 0, s>>>(partials, nc, n, G);
    KF_LAUNCH_CHECK();
}

// Y[r, j] = alpha * sum_i X[r, i] C[i, j] + beta * Y[r, j], one thread per row and a chunk of
// UC output columns; C (FP64, kx x ky) staged in shared memory in T.
template <typename T, int UC>
__global__ void k_update(T *__restrict__ Y, int64_t ldy, int ky, const T *__restrict__ X, int64_t ldx, int kx,
                         const double *__restrict__ C, int ldc, T alpha, T beta, int64_t N) {
    extern __shared__ unsigned char smem_raw[];
    T *Cs = reinterpret_cast<T *>(smem_raw);   // [kx][ky]
    for (int e = threadIdx.x; e < kx * ky; e += blockDim.x) {
        const int i = e % kx, j = e / kx;
        Cs[i * ky + j] = (T)C[i + (size_t)ldc * j];
    }
    __syncthreads();
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    for (int j0 = 0; j0 < ky; j0 += UC) {
        T acc[UC];
#pragma unroll
        for (int v = 0; v < UC; ++v) acc[v] = T(0);
        for (int i = 0; i < kx; ++i) {
            const T x = X[r + (int64_t)i * ldx];
            const T *cr = Cs + i * ky + j0;
#pragma unroll
            for (int v = 0; v < UC; ++v)
                if (j0 + v < ky) acc[v] += x * cr[v];
        }
#pragma unroll
        for (int v = 0; v < UC; ++v) {
            if (j0 + v < ky) {
                T *yp = Y + r + (int64_t)(j0 + v) * ldy;
                *yp = (beta == T(0)) ? alpha * acc[v] : alpha * acc[v] + beta * *yp;
            }
        }
    }
}

template <typename T>
void update(T *Y, int64_t ldy, int ky, const T *X, int64_t ldx, int kx, const double *C, int ldc, double alpha,
            double beta, int64_t N, cudaStream_t s) {
    if (ky <= 0 || N <= 0) return;
    if (kx <= 0) {
        // Y = beta Y
        KF_REQUIRE(beta == 0.0 || beta == 1.0, KF_EINVAL, "update: empty X with a general beta");
        if (beta == 0.0)
            for (int j = 0; j < ky; ++j) KF_CUDA(cudaMemsetAsync(Y + (int64_t)j * ldy, 0, N * sizeof(T), s));
        return;
    }
    const size_t sm = (size_t)kx * ky * sizeof(T);
    KF_REQUIRE(sm <= 200 * 1024, KF_EINVAL, "update: coefficient matrix too large");
    const unsigned grid = (unsigned)((N + 255) / 256);
    if (sm > 48 * 1024) {
        if (sizeof(T) == 8)
            KF_CUDA(cudaFuncSetAttribute(k_update<T, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        else
            KF_CUDA(cudaFuncSetAttribute(k_update<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    }
    if (sizeof(T) == 8)
        k_update<T, 8><<<grid, 256, sm, s>>>(Y, ldy, ky, X, ldx, kx, C, ldc, (T)alpha, (T)beta, N);
    else
        k_update<T, 16><<<grid, 256, sm, s>>>(Y, ldy, ky, X, ldx, kx, C, ldc, (T)alpha, (T)beta, N);
    KF_LAUNCH_CHECK();
}

// ---- column reductions -------------------------------------------------------------------

__device__ inline double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0)
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
    return s;
}

// partials[col * nblk + blk] = sum over the block's rows of X[r, col]^2
template <typename T>
__global__ void k_colnorm2(const T *__restrict__ X, int64_t ldx, int64_t N, int64_t rows_per,
                           double *__restrict__ partials) {
    __shared__ double red[32];
    const int col = blockIdx.y;
    const int64_t r0 = (int64_t)blockIdx.x * rows_per;
    const int64_t r1 = (r0 + rows_per < N) ? r0 + rows_per : N;
    const T *x = X + (int64_t)col * ldx;
    T s = 0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const T v = x[r];
        s += v * v;
    }
    const double t = block_sum((double)s, red);
    if (threadIdx.x == 0) partials[(size_t)col * gridDim.x + blockIdx.x] = t;
}

__global__ void k_reduce_cols(const double *__restrict__ partials, int nblk, int k, double *__restrict__ out) {
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= k) return;
    double s = 0;
    for (int b = 0; b < nblk; ++b) s += partials[(size_t)col * nblk + b];
    out[col] = s;
}

static int64_t red_rows_per(int64_t N, int k) {
    // about 2 x 152 CTAs in total over the k columns
    int64_t nblk = (304 + k - 1) / k;
    if (nblk < 1) nblk = 1;
    int64_t rp = (N + nblk - 1) / nblk;
    if (rp < 1024) rp = 1024;
    return rp;
}

template <typename T>
void colnorms2(const T *X, int64_t ldx, int k, int64_t N, double *out, double *partials, cudaStream_t s) {
    if (k <= 0) return;
    const int64_t rp = red_rows_per(N, k);
    const int nblk = (int)((N + rp - 1) / rp);
    dim3 grid(nblk, k);
    k_colnorm2<T><<<grid, RED_THREADS, 0, s>>>(X, ldx, N, rp, partials);
    KF_LAUNCH_CHECK();
    k_reduce_cols<<<(k + 127) / 128, 128, 0, s>>>(partials, nblk, k, out);
    KF_LAUNCH_CHECK();
}

// R[:, j] = HX[:, j] - theta_j X[:, j]; partial sums of R^2; then R[:, j] is preconditioned in
// place: mode 0 (per-Ritz Jacobi) R / hypot(D - thetap_j, eta); mode 1 (fixed Jacobi)
// R / (D - thetap_0); mode 2 none.  mode < 0 leaves R unpreconditioned.
template <typename T>
__global__ void k_residual_precond(const T *__restrict__ X, const T *__restrict__ HX, int64_t ld, int64_t N,
                                   int64_t rows_per, const double *__restrict__ theta,
                                   const double *__restrict__ thetap, const double *__restrict__ D, double eta,
                                   int mode, T *__restrict__ R, int64_t ldr, double *__restrict__ partials) {
    __shared__ double red[32];
    const int col = blockIdx.y;
    const int64_t r0 = (int64_t)blockIdx.x * rows_per;
    const int64_t r1 = (r0 + rows_per < N) ? r0 + rows_per : N;
    const T th = (T)theta[col];
    const double tp = (mode == 0) ? thetap[col] : (mode == 1 ? thetap[0] : 0.0);
    const T *x = X + (int64_t)col * ld;
    const T *hx = HX + (int64_t)col * ld;
    T *rr = R + (int64_t)col * ldr;
    double s = 0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const T v = hx[r] - th * x[r];
        s += (double)v * (double)v;
        T out = v;
        if (mode == 0) {
            out = (T)((double)v / hypot(D[r] - tp, eta));
        } else if (mode == 1) {
            out = (T)((double)v / (D[r] - tp));
        }
        rr[r] = out;
    }
    const double t = block_sum(s, red);
    if (threadIdx.x == 0) partials[(size_t)col * gridDim.x + blockIdx.x] = t;
}

template <typename T>
void residual_precond(const T *X, const T *HX, int64_t ld, int k, int64_t N, const double *theta,
                      const double *thetap, const double *D, double eta, int mode, T *R, int64_t ldr, double *norms2,
                      double *partials, cudaStream_t s) {
    if (k <= 0) return;
    const int64_t rp = red_rows_per(N, k);
    const int nblk = (int)((N + rp - 1) / rp);
    dim3 grid(nblk, k);
    k_residual_precond<T><<<grid, RED_THREADS, 0, s>>>(X, HX, ld, N, rp, theta, thetap, D, eta, mode, R, ldr, partials);
    KF_LAUNCH_CHECK();
    k_reduce_cols<<<(k + 127) / 128, 128, 0, s>>>(partials, nblk, k, norms2);
    KF_LAUNCH_CHECK();
}

// theta_j = sum_i D_i X_ij^2 / sum_i X_ij^2 (ext/KronFreeCircuitsCUDAExt.jl:16-44): two
// partial sums per column, weighted then plain.
__global__ void k_diag_expect(const double *__restrict__ D, const double *__restrict__ X, int64_t ld, int64_t N,
                              int64_t rows_per, double *__restrict__ partials) {
    __shared__ double red[32];
    const int col = blockIdx.y;
    const int64_t r0 = (int64_t)blockIdx.x * rows_per;
    const int64_t r1 = (r0 + rows_per < N) ? r0 + rows_per : N;
    const double *x = X + (int64_t)col * ld;
    double sw = 0, s = 0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const double a = x[r] * x[r];
        sw += D[r] * a;
        s += a;
    }
    const double tw = block_sum(sw, red);
    const double t = block_sum(s, red);
    if (threadIdx.x == 0) {
        partials[(size_t)(2 * col) * gridDim.x + blockIdx.x] = tw;
        partials[(size_t)(2 * col + 1) * gridDim.x + blockIdx.x] = t;
    }
}

__global__ void k_expect_finish(const double *__restrict__ sums, int k, double *__restrict__ theta) {
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col < k) theta[col] = sums[2 * col] / sums[2 * col + 1];
}

void diag_expectation(const double *D, const double *X, int64_t ld, int k, int64_t N, double *theta,
                      double *partials, cudaStream_t s) {
    if (k <= 0) return;
    const int64_t rp = red_rows_per(N, k);
    const int nblk = (int)((N + rp - 1) / rp);
    dim3 grid(nblk, k);
    k_diag_expect<<<grid, RED_THREADS, 0, s>>>(D, X, ld, N, rp, partials);
    KF_LAUNCH_CHECK();
    // reduce 2k rows of partials in place into the head of `partials` region after them
    double *sums = partials + (size_t)2 * k * nblk;
    k_reduce_cols<<<(2 * k + 127) / 128, 128, 0, s>>>(partials, nblk, 2 * k, sums);
    k_expect_finish<<<(k + 127) / 128, 128, 0, s>>>(sums, k, theta);
    KF_LAUNCH_CHECK();
}

// ---- elementwise ---------------------------------------------------------------------------

template <typename T>
__global__ void k_scale_cols(T *__restrict__ X, int64_t ld, int64_t N, int k, const double *__restrict__ sc) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * k) return;
    const int64_t c = t / N, r = t % N;
    X[c * ld + r] = (T)((double)X[c * ld + r] * sc[c]);
}

template <typename T>
void scale_columns(T *X, int64_t ld, int k, int64_t N, const double *sc, cudaStream_t s) {
    if (k <= 0) return;
    const int64_t tot = N * k;
    k_scale_cols<T><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(X, ld, N, k, sc);
    KF_LAUNCH_CHECK();
}

template <typename T>
__global__ void k_residual_block(const T *__restrict__ X, const T *__restrict__ HX, int64_t ld, int64_t N, int k,
                                 const double *__restrict__ theta, T *__restrict__ R, int64_t ldr) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * k) return;
    const int64_t c = t / N, r = t % N;
    R[c * ldr + r] = HX[c * ld + r] - (T)theta[c] * X[c * ld + r];
}

template <typename T>
void residual_block(const T *X, const T *HX, int64_t ld, int k, int64_t N, const double *theta, T *R, int64_t ldr,
                    cudaStream_t s) {
    if (k <= 0) return;
    const int64_t tot = N * k;
    k_residual_block<T><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(X, HX, ld, N, k, theta, R, ldr);
    KF_LAUNCH_CHECK();
}

// A counter-based normal generator: splitmix64 of (seed, stream, column, row) into two
// uniforms, Box-Muller.  Reproducible for a given seed whatever the launch shape.
__device__ inline uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

template <typename T>
__global__ void k_fill_normal(T *__restrict__ X, int64_t ld, int64_t N, int k, uint64_t seed, uint64_t sid) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * k) return;
    const int64_t c = t / N, r = t % N;
    const uint64_t h = mix64(mix64(mix64(seed) ^ (sid * 0x632be59bd9b4e019ull)) ^ ((uint64_t)c << 40) ^ (uint64_t)r);
    const uint64_t h2 = mix64(h);
    const double u1 = ((h >> 11) + 1) * (1.0 / 9007199254740993.0);   // (0, 1]
    const double u2 = (h2 >> 11) * (1.0 / 9007199254740992.0);         // [0, 1)
    X[c * ld + r] = (T)(sqrt(-2.0 * log(u1)) * cospi(2.0 * u2));
}

template <typename T>
void fill_normal(T *X, int64_t ld, int k, int64_t N, uint64_t seed, uint64_t sid, cudaStream_t s) {
    if (k <= 0) return;
    const int64_t tot = N * k;
    k_fill_normal<T><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(X, ld, N, k, seed, sid);
    KF_LAUNCH_CHECK();
}

template <typename Ts, typename Td>
__global__ void k_convert(const Ts *__restrict__ X, int64_t ldx, Td *__restrict__ Y, int64_t ldy, int64_t N, int k) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * k) return;
    const int64_t c = t / N, r = t % N;
    Y[c * ldy + r] = (Td)X[c * ldx + r];
}

template <typename Ts, typename Td>
void convert(const Ts *X, int64_t ldx, Td *Y, int64_t ldy, int k, int64_t N, cudaStream_t s) {
    if (k <= 0) return;
    const int64_t tot = N * k;
    k_convert<Ts, Td><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(X, ldx, Y, ldy, N, k);
    KF_LAUNCH_CHECK();
}

template <typename T>
void copy_block(const T *X, int64_t ldx, T *Y, int64_t ldy, int k, int64_t N, cudaStream_t s) {
    if (k <= 0) return;
    KF_CUDA(cudaMemcpy2DAsync(Y, ldy * sizeof(T), X, ldx * sizeof(T), N * sizeof(T), k, cudaMemcpyDeviceToDevice, s));
}

// explicit instantiations
#define KF_INST(T)                                                                                                   \
    template void gram<T>(const T *, int64_t, int, const T *, int64_t, int, int64_t, double *, double *, cudaStream_t); \
    template void update<T>(T *, int64_t, int, const T *, int64_t, int, const double *, int, double, double, int64_t, \
                            cudaStream_t);                                                                           \
    template void colnorms2<T>(const T *, int64_t, int, int64_t, double *, double *, cudaStream_t);                  \
    template void residual_precond<T>(const T *, const T *, int64_t, int, int64_t, const double *, const double *,   \
                                      const double *, double, int, T *, int64_t, double *, double *, cudaStream_t); \
    template void scale_columns<T>(T *, int64_t, int, int64_t, const double *, cudaStream_t);                        \
    template void fill_normal<T>(T *, int64_t, int, int64_t, uint64_t, uint64_t, cudaStream_t);                      \
    template void copy_block<T>(const T *, int64_t, T *, int64_t, int, int64_t, cudaStream_t);                       \
    template void residual_block<T>(const T *, const T *, int64_t, int, int64_t, const double *, T *, int64_t,       \
                                    cudaStream_t);
KF_INST(float)
KF_INST(double)
template void convert<float, double>(const float *, int64_t, double *, int64_t, int, int64_t, cudaStream_t);
template void convert<double, float>(const double *, int64_t, float *, int64_t, int, int64_t, cudaStream_t);

}  // namespace kf

// FP64 block update Y = X C (N x kx FP64 block X, kx x ky FP64 coefficients) computed in
// double-float arithmetic on the FP32 pipes: the refinement's X-part update when the Rayleigh-Ritz
// rotation inside X is large (the reference's X = [X W P] C of src/lobpcg.jl:268 in FP64).
//
// GB300 runs FP64 FMAs at about 1/64 of its FP32 rate, so the FP64 kernel is compute-bound far above
// the memory time.  Here x = x_hi + x_lo and c = c_hi + c_lo (FP32 parts); each product x_hi c_hi
// is formed exactly as an FP32 pair (p_hi = x_hi c_hi, p_lo = fma(x_hi, c_hi, -p_hi)), the running
// sum is an FP32 pair updated by an exact two-sum, and the cross terms x_hi c_lo and x_lo c_hi join
// the low part.  About 12 FP32 operations per term, relative error near 2^-46 per sum over the
// <= 32 terms of an update -- far below the FP64 refinement's 1e-8 residual target.
#include "kf_internal.h"

namespace kf {

namespace {

// KX: input columns held per thread (x_hi, x_lo in registers); UC: outputs per pass
template <int KX, int UC>
__global__ void __launch_bounds__(256) k_update_df(double *__restrict__ Y, int64_t ldy, int ky,
                                                   const double *__restrict__ X, int64_t ldx, int kx,
                                                   const double *__restrict__ C, int ldc, int64_t N) {
    __shared__ float2 Cs[KX * 32];   // [i][j]: (c_hi, c_lo), ky <= 32
    for (int e = threadIdx.x; e < kx * ky; e += blockDim.x) {
        const int i = e / ky, j = e % ky;
        const double c = C[i + (size_t)ldc * j];
        const float h = (float)c;
        Cs[i * 32 + j] = make_float2(h, (float)(c - (double)h));
    }
    __syncthreads();
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    float xh[KX], xl[KX];
#pragma unroll
    for (int i = 0; i < KX; ++i) {
        const double x = i < kx ? X[r + (int64_t)i * ldx] : 0.0;
        xh[i] = (float)x;
        xl[i] = (float)(x - (double)xh[i]);
    }
    for (int j0 = 0; j0 < ky; j0 += UC) {
        float sh[UC], sl[UC];
#pragma unroll
        for (int v = 0; v < UC; ++v) sh[v] = sl[v] = 0.f;
#pragma unroll
        for (int i = 0; i < KX; ++i) {
            if (i < kx) {
#pragma unroll
                for (int v = 0; v < UC; ++v) {
                    // the error-free steps use the _rn intrinsics, which the compiler never
                    // contracts into FMAs
                    const float2 c = Cs[i * 32 + ((j0 + v) & 31)];
                    const float ph = __fmul_rn(xh[i], c.x);
                    const float pl = fmaf(xh[i], c.x, -ph);          // x_hi c_hi = ph + pl exactly
                    const float t = __fadd_rn(sh[v], ph);             // two-sum of sh + ph
                    const float bv = __fsub_rn(t, sh[v]);
                    const float er = __fadd_rn(__fsub_rn(sh[v], __fsub_rn(t, bv)), __fsub_rn(ph, bv));
                    sh[v] = t;
                    sl[v] += er + pl;
                    sl[v] = fmaf(xh[i], c.y, sl[v]);
                    sl[v] = fmaf(xl[i], c.x, sl[v]);
                }
            }
        }
#pragma unroll
        for (int v = 0; v < UC; ++v)
            if (j0 + v < ky) Y[r + (int64_t)(j0 + v) * ldy] = (double)sh[v] + (double)sl[v];
    }
}

}  // namespace

bool update_f64_df(double *Y, int64_t ldy, int ky, const double *X, int64_t ldx, int kx, const double *C, int ldc,
                   int64_t N, cudaStream_t s) {
    if (N <= 0 || ky <= 0) return true;
    if (kx < 1 || kx > 32 || ky > 32) return false;
    const unsigned grid = (unsigned)((N + 255) / 256);
    // the smallest register row that holds kx; output passes of 6 when they divide ky exactly and 8
    // do not (18 outputs: three passes of 6 instead of 24 computed)
    const bool six = ky % 6 == 0 && ky % 8 != 0;
#define KF_DF(KXV)                                                                              \
    do {                                                                                        \
        if (six) k_update_df<KXV, 6><<<grid, 256, 0, s>>>(Y, ldy, ky, X, ldx, kx, C, ldc, N);   \
        else k_update_df<KXV, 8><<<grid, 256, 0, s>>>(Y, ldy, ky, X, ldx, kx, C, ldc, N);       \
    } while (0)
    if (kx <= 8) KF_DF(8);
    else if (kx <= 16) KF_DF(16);
    else if (kx <= 24) KF_DF(24);
    else KF_DF(32);
#undef KF_DF
    KF_LAUNCH_CHECK();
    return true;
}

}  // namespace kf

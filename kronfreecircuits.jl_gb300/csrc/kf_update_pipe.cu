// FP32 block updates [Y0 Y1] = alpha [X0 X1] C + beta [Y0 Y1] for LOBPCG's tall-skinny
// Rayleigh-Ritz and orthogonalisation updates (the reference's block products inside
// LOBPCGEigensolver, called at src/lobpcg.jl:268, and src/chebyshev.jl:60,79,126): N rows, at most
// 64 input and 64 output columns.
//
// Every element of X meets every column of C, so the product is FMA-bound unless the loads overlap
// the arithmetic.  A persistent CTA (two per SM, 256 threads) walks 128-row tiles of X: the tile is
// staged column-major in shared memory by 16-byte cp.async copies, double-buffered so that the next
// tile loads while this one is multiplied; C stays in shared memory as FP32.  Thread t owns row
// t % 128 of the tile and one half of the output columns (t / 128): per input column one
// conflict-free shared load of its X value and warp-uniform (broadcast) loads of the C row, then
// FMAs into registers.  The outputs may go to two blocks (columns [0, ky0) to Y0, the rest to Y1),
// so that X_new and P_new of a Rayleigh-Ritz step, which both read [X_a Q], take one pass.
#include <algorithm>

#include "kf_internal.h"

namespace kf {

namespace {

constexpr int UP_TR = 128;        // rows per tile
constexpr int UP_PAD = 4;         // column stride UP_TR + UP_PAD floats (16-byte multiple, conflict-free)
constexpr int UP_S = UP_TR + UP_PAD;
constexpr int UP_KX = 64;         // input columns
constexpr int UP_KY = 64;         // output columns

struct UpArgs {
    float *Y0, *Y1;
    const float *X0, *X1;
    const double *C;
    int64_t ldy0, ldy1, ldx0, ldx1, N;
    int ky0, ky, kx0, kx, ldc, kyp, h0;
    float alpha, beta;
};

__device__ __forceinline__ void up_cp16(float *dst, const float *src, int bytes) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(src), "r"(bytes) : "memory");
}

// stage rows [row0, row0 + UP_TR) of the kx input columns into dst (column c at dst + c UP_S)
__device__ __forceinline__ void up_stage(float *dst, const UpArgs &a, int64_t row0) {
    constexpr int PER = UP_TR / 4;   // 16-byte pieces per column
    for (int e = threadIdx.x; e < a.kx * PER; e += blockDim.x) {
        const int c = e / PER, q = e % PER;
        const int64_t r = row0 + 4 * q;
        const int64_t left = a.N - r;
        const int bytes = left >= 4 ? 16 : left > 0 ? (int)left * 4 : 0;
        const float *col = c < a.kx0 ? a.X0 + (int64_t)c * a.ldx0 : a.X1 + (int64_t)(c - a.kx0) * a.ldx1;
        up_cp16(dst + c * UP_S + 4 * q, col + (bytes > 0 ? r : 0), bytes);
    }
}

// H: output columns per thread (a multiple of 4 covering the thread's half)
template <int H>
__global__ void __launch_bounds__(256, 2) k_update_pipe(const UpArgs a) {
    extern __shared__ __align__(16) float up_smem[];
    float *Cs = up_smem;                            // [kx][kyp], FP32
    float *Xs = up_smem + (size_t)a.kx * a.kyp;     // two stages of [kx][UP_S]
    const int stage_floats = a.kx * UP_S;
    for (int e = threadIdx.x; e < a.kx * a.kyp; e += blockDim.x) {
        const int i = e / a.kyp, j = e % a.kyp;
        Cs[e] = j < a.ky ? (float)a.C[i + (size_t)a.ldc * j] : 0.f;
    }
    const int64_t ntiles = (a.N + UP_TR - 1) / UP_TR;
    const int r = threadIdx.x & (UP_TR - 1), g = threadIdx.x >> 7;
    const int jb = g == 0 ? 0 : a.h0, je = g == 0 ? a.h0 : a.ky;   // this thread's output columns
    int64_t t = blockIdx.x;
    if (t < ntiles) up_stage(Xs, a, t * UP_TR);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    for (int k = 0; t < ntiles; t += gridDim.x, ++k) {
        const int64_t tn = t + gridDim.x;
        if (tn < ntiles) up_stage(Xs + ((k + 1) & 1) * stage_floats, a, tn * UP_TR);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        __syncthreads();   // tile t (and C) visible to every thread
        const float *xs = Xs + (k & 1) * stage_floats + r;
        float acc[H];
#pragma unroll
        for (int v = 0; v < H; ++v) acc[v] = 0.f;
        // an empty half (ky small) skips the product: its jb need not be a multiple of 4; unrolled so
        // that the next inputs' shared loads are in flight while this one's FMAs issue
#pragma unroll 4
        for (int i = 0; jb < je && i < a.kx; ++i) {
            const float xv = xs[i * UP_S];
            const float *cr = Cs + i * a.kyp + jb;
#pragma unroll
            for (int v = 0; v < H; v += 4) {
                const float4 c4 = *reinterpret_cast<const float4 *>(cr + v);
                acc[v] = fmaf(xv, c4.x, acc[v]);
                acc[v + 1] = fmaf(xv, c4.y, acc[v + 1]);
                acc[v + 2] = fmaf(xv, c4.z, acc[v + 2]);
                acc[v + 3] = fmaf(xv, c4.w, acc[v + 3]);
            }
        }
        const int64_t row = t * UP_TR + r;
        if (row < a.N) {
#pragma unroll
            for (int v = 0; v < H; ++v) {
                const int j = jb + v;
                if (j >= je) break;
                float *yp = j < a.ky0 ? a.Y0 + row + (int64_t)j * a.ldy0 : a.Y1 + row + (int64_t)(j - a.ky0) * a.ldy1;
                *yp = a.beta == 0.f ? a.alpha * acc[v] : a.alpha * acc[v] + a.beta * *yp;
            }
        }
        __syncthreads();   // every thread is done with this stage before it is refilled
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

}  // namespace

bool update_pipe(float *Y0, int64_t ldy0, int ky0, float *Y1, int64_t ldy1, int ky1, const float *X0, int64_t ldx0,
                 int kx0, const float *X1, int64_t ldx1, int kx1, const double *C, int ldc, double alpha, double beta,
                 int64_t N, cudaStream_t s) {
    const int kx = kx0 + kx1, ky = ky0 + ky1;
    if (N <= 0 || ky <= 0) return true;
    if (kx < 1 || kx > UP_KX || ky > UP_KY || kx0 < 1) return false;
    auto al = [](const float *p, int64_t ld) { return (uintptr_t)p % 16 == 0 && ld % 4 == 0; };
    if (!al(X0, ldx0) || (kx1 > 0 && !al(X1, ldx1))) return false;
    UpArgs a;
    a.Y0 = Y0;
    a.Y1 = ky1 > 0 ? Y1 : Y0;
    a.X0 = X0;
    a.X1 = kx1 > 0 ? X1 : X0;
    a.C = C;
    a.ldy0 = ldy0;
    a.ldy1 = ky1 > 0 ? ldy1 : ldy0;
    a.ldx0 = ldx0;
    a.ldx1 = kx1 > 0 ? ldx1 : ldx0;
    a.N = N;
    a.ky0 = ky0;
    a.ky = ky;
    a.kx0 = kx0;
    a.kx = kx;
    a.ldc = ldc;
    // the two halves of the output columns, each a multiple of 4 wide (float4 loads of C)
    a.h0 = std::min(ky, (ky / 2 + 3) / 4 * 4);
    const int hmax = std::max(a.h0, ky - a.h0);
    // the larger half rounded up to a multiple of 4 (a wider H multiplies zeros and spills)
    const int H = std::max(4, (hmax + 3) / 4 * 4);
    a.kyp = a.h0 + (ky - a.h0 + 3) / 4 * 4 + H;   // room for the float4 reads past a half's end
    a.kyp = (a.kyp + 3) / 4 * 4;
    a.alpha = (float)alpha;
    a.beta = (float)beta;
    const size_t smem = ((size_t)kx * a.kyp + (size_t)2 * kx * UP_S) * sizeof(float);
    if (smem > 100 * 1024) return false;
    using Kern = void (*)(const UpArgs);
    static const Kern kerns[8] = {k_update_pipe<4>,  k_update_pipe<8>,  k_update_pipe<12>, k_update_pipe<16>,
                                  k_update_pipe<20>, k_update_pipe<24>, k_update_pipe<28>, k_update_pipe<32>};
    static int attr_dev_mask = 0;
    int dev = 0, sms = 152;
    KF_CUDA(cudaGetDevice(&dev));
    KF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (dev < 31 && !(attr_dev_mask & (1 << dev))) {
        for (Kern k : kerns) KF_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
        attr_dev_mask |= 1 << dev;
    }
    const int64_t ntiles = (N + UP_TR - 1) / UP_TR;
    const int grid = (int)std::min<int64_t>(ntiles, 2 * (int64_t)sms);
    kerns[H / 4 - 1]<<<grid, 256, smem, s>>>(a);
    KF_LAUNCH_CHECK();
    return true;
}

}  // namespace kf

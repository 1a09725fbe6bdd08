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
    return std::max((a > b ? a : b) * sizeof(double), gram_tc_partials_size(ka, kb));
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

// out[e] = sum_c partials[c][e], e < n, in a fixed order: one warp per entry, lane l summing
// c = l, l + 32, ... , then a fixed shuffle tree
__global__ void k_reduce_partials(const double *__restrict__ partials, int nparts, int n, double *__restrict__ out) {
    const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (e >= n) return;
    double s = 0;
    for (int c = lane; c < nparts; c += 32) s += partials[(size_t)c * n + e];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) out[e] = s;
}

static void reduce_partials(const double *partials, int nparts, int n, double *out, cudaStream_t s) {
    k_reduce_partials<<<(n + 7) / 8, 256, 0, s>>>(partials, nparts, n, out);
    KF_LAUNCH_CHECK();
}

// ---- FP32 Gram: rows staged through shared memory, one 8 x 8 output tile per warp ----------
//
// A CTA owns a contiguous range of rows and one "group" of output tiles (at most 8 tiles of
// 8 x 8, a rectangle gti x gtj of them).  Rows arrive in batches of `tr` (a multiple of 64, larger
// for narrow blocks so that about 24 KB per stage is in flight) through a three-stage cp.async
// pipeline, one column-major slab per operand in shared memory, so each element of A and B is
// read from memory once per group.  Warp w works on tile w / wpt over the batch rows congruent to
// its sub-index (wpt = warps per tile, when the group has fewer than 8 tiles); lane l takes every
// 32nd of those rows.  Per row a lane loads 8 + 8 operands from shared memory (consecutive lanes,
// consecutive rows: conflict-free) for 64 FMAs.  The lanes' FP32 sums meet in a butterfly
// reduce-scatter (62 shuffles for 64 values; lane l ends with entries 2l and 2l + 1), the
// sub-warps of a tile in FP64 in a fixed order, and the CTA's partial lands in
// partials[cta][i + ka j] for the final fixed-order FP64 reduction.
constexpr int G32_PAD = 4;          // column stride tr + G32_PAD floats (16-byte multiple)
constexpr int G32_STAGES = 3;
constexpr int G32_SMEM = 96 * 1024; // dynamic shared memory ceiling (two CTAs per SM)

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, int src_bytes) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem, int src_bytes) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sa), "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// A set of FP32 columns in up to two blocks: columns [0, n0) at p0 + c ld0, the rest at
// p1 + (c - n0) ld1 (so [X Z] needs no copy)
struct Cols2 {
    const float *p0, *p1;
    int64_t ld0, ld1;
    int n0;
    __device__ __forceinline__ const float *col(int c) const {
        return c < n0 ? p0 + (int64_t)c * ld0 : p1 + (int64_t)(c - n0) * ld1;
    }
};

struct Gram32Shape {
    int nti, ntj, gti, gtj, ngi, ngj;   // tiles per axis, group size in tiles, groups per axis
    int tr;                             // rows per batch
};

static Gram32Shape gram32_shape(int ka, int kb) {
    Gram32Shape g;
    g.nti = (ka + 7) / 8;
    g.ntj = (kb + 7) / 8;
    g.gtj = g.ntj < 8 ? g.ntj : 8;
    g.gti = 8 / g.gtj;
    if (g.gti > g.nti) g.gti = g.nti;
    g.ngi = (g.nti + g.gti - 1) / g.gti;
    g.ngj = (g.ntj + g.gtj - 1) / g.gtj;
    // ~24 KB of loads per stage, at most 512 rows, within the shared-memory ceiling
    const int cols = 8 * (g.gti + g.gtj);
    int tr = (24 * 1024 / (4 * cols)) / 64 * 64;
    if (tr < 64) tr = 64;
    if (tr > 512) tr = 512;
    while (tr > 64 && (size_t)G32_STAGES * cols * (tr + G32_PAD) * 4 > (size_t)G32_SMEM) tr -= 64;
    // the kernel is compiled for batch heights 64, 128, 256 and 384 (shared-memory offsets as
    // immediates); take the largest of them that fits
    g.tr = tr >= 384 ? 384 : tr >= 256 ? 256 : tr >= 128 ? 128 : 64;
    return g;
}

static size_t gram32_smem(const Gram32Shape &g) {
    return (size_t)G32_STAGES * 8 * (g.gti + g.gtj) * (g.tr + G32_PAD) * sizeof(float);
}

// stage rows [row0, row0 + tr) of columns c0 .. c0 + nc - 1 of the column set `src` into dst
// (column stride tr + G32_PAD); rows at or past `rend` are zero-filled
template <bool VEC, int TR>
__device__ __forceinline__ void g32_stage(float *dst, const Cols2 &src, int c0, int nc, int64_t row0, int64_t rend) {
    constexpr int tr = TR, S = TR + G32_PAD;
    if (VEC) {
        // warp w stages columns w, w + 8, ...: the column pointer is warp-uniform and computed once
        // per column, the lanes take consecutive 16-byte pieces; a batch wholly below rend (all
        // but a CTA's last) skips the bounds arithmetic
        constexpr int per = TR / 4;
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
        const bool full = row0 + tr <= rend;
        for (int c = warp; c < nc; c += nw) {
            const float *col = src.col(c0 + c) + row0;
            float *d = dst + c * S;
            if (full) {
#pragma unroll
                for (int q = lane; q < per; q += 32) cp_async16(d + 4 * q, col + 4 * q, 16);
            } else {
                for (int q = lane; q < per; q += 32) {
                    const int64_t left = rend - (row0 + 4 * q);
                    const int bytes = left >= 4 ? 16 : left > 0 ? (int)left * 4 : 0;
                    cp_async16(d + 4 * q, bytes > 0 ? col + 4 * q : col - row0, bytes);
                }
            }
        }
    } else {
        for (int e = threadIdx.x; e < nc * tr; e += blockDim.x) {
            const int c = e / tr, q = e % tr;
            const int64_t r = row0 + q;
            const bool ok = r < rend;
            cp_async4(dst + c * S + q, src.col(c0 + c) + (ok ? r : 0), ok ? 4 : 0);
        }
    }
}

// one reduce-scatter step: the lanes differing in bit O exchange halves of their first L values
template <int O, int L>
__device__ __forceinline__ void g32_butterfly(float *f, int lane) {
    const bool upper = (lane & O) != 0;
#pragma unroll
    for (int k = 0; k < L / 2; ++k) {
        const float send = upper ? f[k] : f[k + L / 2];
        const float keep = upper ? f[k + L / 2] : f[k];
        f[k] = keep + __shfl_xor_sync(0xffffffffu, send, O);
    }
}

template <bool VEC, int TR>
__global__ void __launch_bounds__(256, 2) k_gram32(const Cols2 A, int ka, const Cols2 B, int kb, int64_t N,
                                                   int64_t rows_per, Gram32Shape sh, double *__restrict__ partials) {
    extern __shared__ __align__(16) unsigned char g32_smem[];
    constexpr int tr = TR, S = TR + G32_PAD;
    const int gi = blockIdx.y / sh.ngj, gj = blockIdx.y % sh.ngj;
    const int ti0 = gi * sh.gti, tj0 = gj * sh.gtj;
    const int gti = min(sh.gti, sh.nti - ti0), gtj = min(sh.gtj, sh.ntj - tj0);
    const int ca0 = ti0 * 8, cb0 = tj0 * 8;
    const int nca = min(gti * 8, ka - ca0), ncb = min(gtj * 8, kb - cb0);   // valid columns staged
    const int sa = gti * 8, sb = gtj * 8;                                     // slab widths (padded)
    float *const buf0 = reinterpret_cast<float *>(g32_smem);
    const int bstride = (sa + sb) * S;   // stage t starts at buf0 + t * bstride
    // padding columns (A's [nca, sa), B's [ncb, sb)) stay zero in every stage; only they are written
    {
        const int pa = sa - nca, pb = sb - ncb, pw = (pa + pb) * S;
        for (int e = threadIdx.x; e < G32_STAGES * pw; e += blockDim.x) {
            const int t = e / pw, rem = e - t * pw, pc = rem / S, q = rem - pc * S;
            const int c = pc < pa ? nca + pc : sa + ncb + (pc - pa);
            buf0[t * bstride + c * S + q] = 0.f;
        }
    }
    const int ntile = gti * gtj;
    const int wpt = 8 / ntile;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = warp / wpt, sub = warp % wpt;
    const bool active = tile < ntile;
    const int ta = active ? (tile / gtj) * 8 : 0, tb = active ? (tile % gtj) * 8 : 0;

    const int64_t r0 = (int64_t)blockIdx.x * rows_per;
    const int64_t r1 = (r0 + rows_per < N) ? r0 + rows_per : N;
    const int nb = (int)((r1 - r0 + tr - 1) / tr);
    float acc[8][8];
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int v = 0; v < 8; ++v) acc[u][v] = 0.f;

    // prologue: stages 0 and 1 in flight (an empty commit group keeps the group count uniform)
    for (int t = 0; t < G32_STAGES - 1; ++t) {
        if (t < nb) {
            float *st = buf0 + t * bstride;
            const int64_t rn = r0 + (int64_t)t * tr;
            g32_stage<VEC, TR>(st, A, ca0, nca, rn, r1);
            g32_stage<VEC, TR>(st + sa * S, B, cb0, ncb, rn, r1);
        }
        cp_async_commit();
    }
    for (int b = 0; b < nb; ++b) {
        // issue batch b + 2 into the stage batch b - 1 used (freed by the barrier ending b - 1)
        const int bn = b + G32_STAGES - 1;
        if (bn < nb) {
            float *st = buf0 + (bn % G32_STAGES) * bstride;
            const int64_t rn = r0 + (int64_t)bn * tr;
            g32_stage<VEC, TR>(st, A, ca0, nca, rn, r1);
            g32_stage<VEC, TR>(st + sa * S, B, cb0, ncb, rn, r1);
        }
        cp_async_commit();
        cp_async_wait<G32_STAGES - 1>();   // batch b has landed (this thread's copies)
        __syncthreads();                    // ... and everyone's
        if (active) {
            const float *cur = buf0 + (b % G32_STAGES) * bstride;
            const float *As = cur + ta * S, *Bs = cur + (sa + tb) * S;
            for (int q = sub * 32 + lane; q < tr; q += 32 * wpt) {
                float a[8], bv[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) a[u] = As[u * S + q];
#pragma unroll
                for (int v = 0; v < 8; ++v) bv[v] = Bs[v * S + q];
#pragma unroll
                for (int u = 0; u < 8; ++u)
#pragma unroll
                    for (int v = 0; v < 8; ++v) acc[u][v] = fmaf(a[u], bv[v], acc[u][v]);
            }
        }
        __syncthreads();
    }
    cp_async_wait<0>();
    // butterfly reduce-scatter over the 32 lanes: lane l ends with flattened entries 2l, 2l + 1
    float *f = &acc[0][0];
    g32_butterfly<16, 64>(f, lane);
    g32_butterfly<8, 32>(f, lane);
    g32_butterfly<4, 16>(f, lane);
    g32_butterfly<2, 8>(f, lane);
    g32_butterfly<1, 4>(f, lane);
    double *red = reinterpret_cast<double *>(g32_smem);   // [warp][64], staging no longer needed
    if (active) {
        red[warp * 64 + 2 * lane] = (double)f[0];
        red[warp * 64 + 2 * lane + 1] = (double)f[1];
    }
    __syncthreads();
    double *P = partials + (size_t)blockIdx.x * ka * kb;
    for (int e = threadIdx.x; e < ntile * 64; e += blockDim.x) {
        const int t = e / 64, idx = e % 64, u = idx / 8, v = idx % 8;
        const int i = ca0 + (t / gtj) * 8 + u, j = cb0 + (t % gtj) * 8 + v;
        if (i >= ka || j >= kb) continue;
        double s = 0;
        for (int w = 0; w < wpt; ++w) s += red[(t * wpt + w) * 64 + idx];
        P[i + (size_t)ka * j] = s;
    }
}

// The tensor-core Gram for [A0 A1]' [B0 B1] when it fits: a B set that is A1 (the orthogonalisation's
// [X Z]'Z) or A0 (a self Gram) is loaded once; otherwise the pool is [A0 A1 B0 B1].
static bool gram32_try_tc(const float *A0, int64_t lda0, int ka0, const float *A1, int64_t lda1, int ka1,
                          const float *B0, int64_t ldb0, int kb0, const float *B1, int64_t ldb1, int kb1, int64_t N,
                          double *G, double *partials, cudaStream_t s) {
    if (N < GRAM_TC_MIN_ROWS) return false;
    // a tcgen05.mma (K = 8 rows) costs about the same whatever its width up to N = 128, so the
    // tensor-core Gram takes a near-constant time per row; the SIMT kernel's grows with the padded
    // output (measured on 671,744 rows: 16 x 32 SIMT 43 us vs 120 us, 32 x 32 71 vs 90, 24 x 40
    // 92 vs 116, 48 x 48 547 vs 127): the tensor cores from 24 8 x 8 output tiles on
    const int pa = (ka0 + ka1 + 7) / 8 * 8, pb = (kb0 + kb1 + 7) / 8 * 8;
    if (pa * pb < 1536) return false;
    const size_t cap = gram_partials_size(ka0 + ka1, kb0 + kb1, N);
    GramTcSrc src[4];
    int n = 0;
    src[n++] = {A0, lda0, ka0};
    if (ka1 > 0) src[n++] = {A1, lda1, ka1};
    const int na = n;
    if (kb1 == 0 && ka1 > 0 && B0 == A1 && ldb0 == lda1 && kb0 == ka1)
        return gram_tc(src, n, 0, na, na - 1, na, N, G, partials, cap, s);
    if (kb1 == 0 && ka1 == 0 && B0 == A0 && ldb0 == lda0 && kb0 == ka0)
        return gram_tc(src, n, 0, 1, 0, 1, N, G, partials, cap, s);
    src[n++] = {B0, ldb0, kb0};
    if (kb1 > 0) src[n++] = {B1, ldb1, kb1};
    return gram_tc(src, n, 0, na, na, n, N, G, partials, cap, s);
}

// G ((ka0 + ka1) x (kb0 + kb1), column-major, FP64) = [A0 A1]' [B0 B1] for FP32 column blocks; on
// the tensor cores when the shapes fit (allow_tc), else the SIMT kernel below
void gram32_sets(const float *A0, int64_t lda0, int ka0, const float *A1, int64_t lda1, int ka1, const float *B0,
                 int64_t ldb0, int kb0, const float *B1, int64_t ldb1, int kb1, int64_t N, double *G, double *partials,
                 cudaStream_t s, bool allow_tc) {
    const int ka = ka0 + ka1, kb = kb0 + kb1;
    KF_REQUIRE(ka >= 1 && kb >= 1 && ka <= 128 && kb <= 128, KF_EINVAL, "gram: block widths out of range");
    if (allow_tc && gram32_try_tc(A0, lda0, ka0, A1, lda1, ka1, B0, ldb0, kb0, B1, ldb1, kb1, N, G, partials, s))
        return;
    const Cols2 A{A0, ka1 > 0 ? A1 : A0, lda0, ka1 > 0 ? lda1 : lda0, ka0};
    const Cols2 B{B0, kb1 > 0 ? B1 : B0, ldb0, kb1 > 0 ? ldb1 : ldb0, kb0};
    const Gram32Shape sh = gram32_shape(ka, kb);
    const int groups = sh.ngi * sh.ngj;
    // about 2 CTAs per SM over all groups, whole batches per CTA, never more row blocks than
    // gram_partials_size provides for
    int64_t target = (304 + groups - 1) / groups;
    int64_t rp = (N + target - 1) / target;
    if (rp < 256) rp = 256;
    rp = (rp + sh.tr - 1) / sh.tr * sh.tr;
    const int nc = (int)((N + rp - 1) / rp);
    const size_t smem = gram32_smem(sh);
    auto al = [](const float *p, int64_t ld) { return ld % 4 == 0 && (uintptr_t)p % 16 == 0; };
    const bool vec = al(A.p0, A.ld0) && al(A.p1, A.ld1) && al(B.p0, B.ld0) && al(B.p1, B.ld1);
    using Kern = void (*)(const Cols2, int, const Cols2, int, int64_t, int64_t, Gram32Shape, double *);
    static const Kern kerns[2][4] = {
        {k_gram32<false, 64>, k_gram32<false, 128>, k_gram32<false, 256>, k_gram32<false, 384>},
        {k_gram32<true, 64>, k_gram32<true, 128>, k_gram32<true, 256>, k_gram32<true, 384>}};
    const int ti = sh.tr == 64 ? 0 : sh.tr == 128 ? 1 : sh.tr == 256 ? 2 : 3;
    static int attr_dev_mask = 0;   // devices whose kernel attributes are set
    int dev = 0;
    KF_CUDA(cudaGetDevice(&dev));
    if (dev < 31 && !(attr_dev_mask & (1 << dev))) {
        for (auto &row : kerns)
            for (Kern k : row) KF_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, G32_SMEM));
        attr_dev_mask |= 1 << dev;
    }
    kerns[vec ? 1 : 0][ti]<<<dim3(nc, groups), 256, smem, s>>>(A, ka, B, kb, N, rp, sh, partials);
    KF_LAUNCH_CHECK();
    reduce_partials(partials, nc, ka * kb, G, s);
}

template <typename T>
void gram(const T *A, int64_t lda, int ka, const T *B, int64_t ldb, int kb, int64_t N, double *G, double *partials,
          cudaStream_t s, bool allow_tc) {
    KF_REQUIRE(ka >= 1 && kb >= 1 && ka <= 128 && kb <= 128, KF_EINVAL, "gram: block widths out of range");
    if constexpr (sizeof(T) == 4) {
        gram32_sets((const float *)A, lda, ka, nullptr, 0, 0, (const float *)B, ldb, kb, nullptr, 0, 0, N, G, partials,
                    s, allow_tc);
        return;
    }
    // FP64: output chunks of 4 x 8 accumulators per thread
    constexpr int RI = 4, RJ = 8;
    const int chunks = ((ka + RI - 1) / RI) * ((kb + RJ - 1) / RJ);
    const int64_t rp = gram_rows_per_cta(N, chunks);
    const int nc = num_ctas_for(N, rp);
    k_gram<T, RI, RJ><<<dim3(nc, chunks), GRAM_THREADS, 0, s>>>(A, lda, ka, B, ldb, kb, N, rp, partials);
    KF_LAUNCH_CHECK();
    const int n = ka * kb;
    reduce_partials(partials, nc, n, G, s);
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

// The same product with the row's kx operands loaded into registers first (all loads in flight
// together) and C read from shared memory as UC-wide vectors (broadcast across the warp); C is
// padded to a multiple of UC columns with zeros.  For kx <= KX.
template <typename T, int KX, int UC>
__global__ void __launch_bounds__(256) k_update_reg(T *__restrict__ Y, int64_t ldy, int ky, const T *__restrict__ X,
                                                    int64_t ldx, int kx0, const T *__restrict__ X1, int64_t ldx1,
                                                    int kx, const double *__restrict__ C, int ldc, T alpha, T beta,
                                                    int64_t N) {
    extern __shared__ __align__(16) unsigned char smem_raw_reg[];
    T *Cs = reinterpret_cast<T *>(smem_raw_reg);   // [kx][kyp]
    const int kyp = (ky + UC - 1) / UC * UC;
    for (int e = threadIdx.x; e < kx * kyp; e += blockDim.x) {
        const int i = e / kyp, j = e % kyp;
        Cs[e] = j < ky ? (T)C[i + (size_t)ldc * j] : T(0);
    }
    __syncthreads();
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= N) return;
    // operand i of the row: X[:, i] for i < kx0, X1[:, i - kx0] after
    T x[KX];
#pragma unroll
    for (int i = 0; i < KX; ++i)
        x[i] = (i < kx0) ? X[r + (int64_t)i * ldx] : (i < kx) ? X1[r + (int64_t)(i - kx0) * ldx1] : T(0);
    for (int j0 = 0; j0 < ky; j0 += UC) {
        T acc[UC];
#pragma unroll
        for (int v = 0; v < UC; ++v) acc[v] = T(0);
#pragma unroll
        for (int i = 0; i < KX; ++i) {
            if (i < kx) {
                const T *cr = Cs + i * kyp + j0;
#pragma unroll
                for (int v = 0; v < UC; ++v) acc[v] = fma(x[i], cr[v], acc[v]);
            }
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
static void update_reg_launch(T *Y, int64_t ldy, int ky, const T *X0, int64_t ldx0, int kx0, const T *X1,
                              int64_t ldx1, int kx1, const double *C, int ldc, double alpha, double beta, int64_t N,
                              cudaStream_t s) {
    constexpr int UC = sizeof(T) == 8 ? 4 : 8;
    const int kx = kx0 + kx1;
    const int kyp = (ky + UC - 1) / UC * UC;
    const size_t smr = (size_t)kx * kyp * sizeof(T);
    const unsigned grid = (unsigned)((N + 255) / 256);
    const T a = (T)alpha, b = (T)beta;
    if (!X1) X1 = X0;
    if (kx <= 8)
        k_update_reg<T, 8, UC><<<grid, 256, smr, s>>>(Y, ldy, ky, X0, ldx0, kx0, X1, ldx1, kx, C, ldc, a, b, N);
    else if (kx <= 16)
        k_update_reg<T, 16, UC><<<grid, 256, smr, s>>>(Y, ldy, ky, X0, ldx0, kx0, X1, ldx1, kx, C, ldc, a, b, N);
    else if (kx <= 32)
        k_update_reg<T, 32, UC><<<grid, 256, smr, s>>>(Y, ldy, ky, X0, ldx0, kx0, X1, ldx1, kx, C, ldc, a, b, N);
    else
        k_update_reg<T, (sizeof(T) == 8 ? 32 : 64), UC><<<grid, 256, smr, s>>>(Y, ldy, ky, X0, ldx0, kx0, X1, ldx1, kx,
                                                                               C, ldc, a, b, N);
    KF_LAUNCH_CHECK();
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
    if constexpr (sizeof(T) == 4) {
        if (update_tc_prefer(kx, ky, N, (const float *)X, ldx, nullptr, 0)) {
            update_tc((float *)Y, ldy, ky, (const float *)X, ldx, kx, nullptr, 0, 0, C, ldc, alpha, beta, N, s);
            return;
        }
        if (N >= 4096 && update_pipe((float *)Y, ldy, ky, nullptr, 0, 0, (const float *)X, ldx, kx, nullptr, 0, 0, C,
                                     ldc, alpha, beta, N, s))
            return;
    }
    const unsigned grid = (unsigned)((N + 255) / 256);
    constexpr int UC = sizeof(T) == 8 ? 4 : 8;
    const int kyp = (ky + UC - 1) / UC * UC;
    const size_t smr = (size_t)kx * kyp * sizeof(T);
    const int kxmax = sizeof(T) == 8 ? 32 : 64;
    if (kx <= kxmax && smr <= 48 * 1024) {
        update_reg_launch<T>(Y, ldy, ky, X, ldx, kx, nullptr, 0, 0, C, ldc, alpha, beta, N, s);
        return;
    }
    const size_t sm = (size_t)kx * ky * sizeof(T);
    KF_REQUIRE(sm <= 200 * 1024, KF_EINVAL, "update: coefficient matrix too large");
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

// Y = alpha [X0 X1] C + beta Y: the operands of each row from two blocks (kx0 + kx1 columns), C
// ((kx0 + kx1) x ky, FP64, leading dimension ldc)
template <typename T>
void update2(T *Y, int64_t ldy, int ky, const T *X0, int64_t ldx0, int kx0, const T *X1, int64_t ldx1, int kx1,
             const double *C, int ldc, double alpha, double beta, int64_t N, cudaStream_t s, bool allow_tc) {
    if (ky <= 0 || N <= 0) return;
    if constexpr (sizeof(T) == 4) {
        // at least 40 inputs and 17 outputs: the tcgen05 kernel (TF32 hi / lo, staging ring), which
        // measured faster there (54 -> 36 columns: 99 us vs 126 us on 671,744 rows)
        if (allow_tc && kx0 > 0 &&
            update_tc_prefer(kx0 + kx1, ky, N, (const float *)X0, ldx0, kx1 > 0 ? (const float *)X1 : nullptr, ldx1)) {
            update_tc((float *)Y, ldy, ky, (const float *)X0, ldx0, kx0, (const float *)X1, ldx1, kx1, C, ldc, alpha,
                      beta, N, s);
            return;
        }
        // up to 64 x 64: the pipelined SIMT kernel (loads overlapped with the FMAs)
        if (N >= 4096 && kx0 > 0 &&
            update_pipe((float *)Y, ldy, ky, nullptr, 0, 0, (const float *)X0, ldx0, kx0, (const float *)X1, ldx1, kx1,
                        C, ldc, alpha, beta, N, s))
            return;
        // wider FP32 updates are FMA-bound on the SIMT pipes; the tcgen05 kernel (TF32 hi / lo)
        // measured faster there
        const int kx = kx0 + kx1;
        if (allow_tc && N >= 65536 && update_tc_ok(kx, ky) && kx * ky >= 1024) {
            update_tc((float *)Y, ldy, ky, (const float *)X0, ldx0, kx0, (const float *)X1, ldx1, kx1, C, ldc, alpha,
                      beta, N, s);
            return;
        }
    } else {
        (void)allow_tc;
    }
    constexpr int UC = sizeof(T) == 8 ? 4 : 8;
    const int kx = kx0 + kx1;
    const int kyp = (ky + UC - 1) / UC * UC;
    const int kxmax = sizeof(T) == 8 ? 32 : 64;
    if (kx0 > 0 && kx1 > 0 && kx <= kxmax && (size_t)kx * kyp * sizeof(T) <= 48 * 1024) {
        update_reg_launch<T>(Y, ldy, ky, X0, ldx0, kx0, X1, ldx1, kx1, C, ldc, alpha, beta, N, s);
        return;
    }
    update<T>(Y, ldy, ky, X0, ldx0, kx0, C, ldc, alpha, beta, N, s);
    update<T>(Y, ldy, ky, X1, ldx1, kx1, C + kx0, ldc, alpha, kx0 > 0 ? 1.0 : beta, N, s);
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

// Refinement-phase residual: R = HX - X theta from the FP64 iterate, its FP64 squared norms,
// and two FP32 blocks: R itself (for the Rayleigh-Ritz blocks) and, unless Wout is null, the
// preconditioned direction (mode 0: / hypot(D - theta, eta), mode 1: / (D - sigma)) computed in
// FP32 -- the preconditioner only steers the search directions.
__global__ void k_residual_mixed(const double *__restrict__ X, const double *__restrict__ HX, int64_t ld, int64_t N,
                                 int64_t rows_per, const double *__restrict__ theta,
                                 const double *__restrict__ thetap, const double *__restrict__ D, double eta, int mode,
                                 float *__restrict__ R, int64_t ldr, float *__restrict__ Wout, int64_t ldw,
                                 double *__restrict__ partials) {
    __shared__ double red[32];
    const int col = blockIdx.y;
    const int64_t r0 = (int64_t)blockIdx.x * rows_per;
    const int64_t r1 = (r0 + rows_per < N) ? r0 + rows_per : N;
    const double th = theta[col];
    const float tp = (float)((mode == 0) ? thetap[col] : (mode == 1 ? thetap[0] : 0.0));
    const float et = (float)eta;
    const double *x = X + (int64_t)col * ld;
    const double *hx = HX + (int64_t)col * ld;
    float *rr = R + (int64_t)col * ldr;
    float *ww = Wout ? Wout + (int64_t)col * ldw : nullptr;
    double s = 0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const double v = hx[r] - th * x[r];
        s += v * v;
        const float vf = (float)v;
        rr[r] = vf;
        if (ww) {
            const float d = (float)D[r] - tp;
            ww[r] = mode == 0 ? vf / hypotf(d, et) : mode == 1 ? vf / d : vf;
        }
    }
    const double t = block_sum(s, red);
    if (threadIdx.x == 0) partials[(size_t)col * gridDim.x + blockIdx.x] = t;
}

void residual_mixed(const double *X, const double *HX, int64_t ld, int k, int64_t N, const double *theta,
                    const double *thetap, const double *D, double eta, int mode, float *R, int64_t ldr, float *W,
                    int64_t ldw, double *norms2, double *partials, cudaStream_t s) {
    if (k <= 0) return;
    const int64_t rp = red_rows_per(N, k);
    const int nblk = (int)((N + rp - 1) / rp);
    k_residual_mixed<<<dim3(nblk, k), RED_THREADS, 0, s>>>(X, HX, ld, N, rp, theta, thetap, D, eta, mode, R, ldr, W,
                                                           ldw, partials);
    KF_LAUNCH_CHECK();
    k_reduce_cols<<<(k + 127) / 128, 128, 0, s>>>(partials, nblk, k, norms2);
    KF_LAUNCH_CHECK();
}

// Y64 += (double) P32 column by column; Y32 (optional) receives the FP32 rounding of the sum
__global__ void k_add_f32_into_f64(double *__restrict__ Y, int64_t ldy, const float *__restrict__ P, int64_t ldp,
                                   float *__restrict__ Y32, int64_t ld32, int64_t N, int64_t total) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int64_t c = t / N, r = t % N;
    const double v = Y[r + c * ldy] + (double)P[r + c * ldp];
    Y[r + c * ldy] = v;
    if (Y32) Y32[r + c * ld32] = (float)v;
}

void add_f32_into_f64(double *Y, int64_t ldy, const float *P, int64_t ldp, float *Y32, int64_t ld32, int k, int64_t N,
                      cudaStream_t s) {
    if (k <= 0 || N <= 0) return;
    const int64_t total = N * k;
    k_add_f32_into_f64<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(Y, ldy, P, ldp, Y32, ld32, N, total);
    KF_LAUNCH_CHECK();
}

// Y[:, j] = d_j X[:, j] + (double) P[:, j] (FP64, one FMA per element) and Y32 its FP32 rounding;
// all blocks with leading dimension N
__global__ void k_scale_add(double *__restrict__ Y, const double *__restrict__ X, const double *__restrict__ d,
                            const float *__restrict__ P, float *__restrict__ Y32, int64_t N, int64_t total) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int64_t c = t / N;
    const double v = fma(d[c], X[t], (double)P[t]);
    Y[t] = v;
    Y32[t] = (float)v;
}

void scale_add(double *Y, const double *X, const double *d, const float *P, float *Y32, int k, int64_t N,
               cudaStream_t s) {
    if (k <= 0 || N <= 0) return;
    const int64_t total = N * k;
    k_scale_add<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(Y, X, d, P, Y32, N, total);
    KF_LAUNCH_CHECK();
}

// Second orthogonalisation pass without the host: from G = [X Z]'Z ((wx + r) x r, FP64, the
// rows of X'Z first), S = Z'Z - (X'Z)'(X'Z) (the Gram of (I - XX')Z), its Cholesky factor
// S = R'R (R upper), and the coefficients C = [R^-1 ; -(X'Z) R^-1] ((r + wx) x r) with which
// [Z X] C = (I - XX') Z R^-1 is orthonormal.  One CTA; *status = 0, or 1 when a pivot is not
// finite or below 1e-4 (C is then not to be used).  r <= 64.
// The arithmetic is FP32: Z is an FP32 block that the first pass already orthonormalised, so S is
// near the identity (a pivot below 1e-4 goes to the host) and FP32 factors are as accurate as the
// FP32 update that applies them; GB300's FP64 rate made the FP64 version ~50 us.
// The kernel is latency-bound: G is staged in shared memory by one coalesced pass (no global
// load inside a dependent chain), and the factorisation and R^-1 run on warp 0 alone with warp
// synchronisation (lane l owns columns l and l + 32), so no CTA barrier sits inside the loops.
// column j of the trailing matrix minus row k's outer product: colj[i] -= rowk[i] skj, i = k+1..j
// (row k in its own buffer, so the loads need not wait for the stores)
__device__ __forceinline__ void chol2_col_update(float *__restrict__ colj, const float *__restrict__ rowk, int k,
                                                 int j, float skj) {
#pragma unroll 4
    for (int i = k + 1; i <= j; ++i) colj[i] = fmaf(-rowk[i], skj, colj[i]);
}

// column j of R^-1 by back substitution (R upper, r x r, column-major)
__device__ __forceinline__ void chol2_inv_col(const float *__restrict__ R, float *__restrict__ y, int r, int j) {
    y[j] = 1.f / R[j + r * j];
    for (int i = j - 1; i >= 0; --i) {
        float v = 0.f;
        for (int k = i + 1; k <= j; ++k) v = fmaf(R[i + r * k], y[k], v);
        y[i] = -v / R[i + r * i];
    }
}

__global__ void k_chol2_coeffs(const double *__restrict__ G, int wx, int r, double *__restrict__ C,
                               int *__restrict__ status) {
    extern __shared__ float cs[];
    const int ld = wx + r;
    float *Gs = cs;              // ld x r, G in FP32
    float *S = Gs + ld * r;      // r x r, column-major; becomes R (upper)
    float *Ri = S + r * r;       // r x r, R^-1
    float *rowk = Ri + r * r;    // r: row k of R during step k
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int e = tid; e < ld * r; e += nt) Gs[e] = (float)G[e];
    __syncthreads();
    for (int e = tid; e < r * r; e += nt) {
        const int i = e % r, j = e / r;
        float v = Gs[wx + i + ld * j];
        for (int q = 0; q < wx; ++q) v = fmaf(-Gs[q + ld * i], Gs[q + ld * j], v);
        S[e] = v;
        Ri[e] = 0.f;
    }
    __syncthreads();
    if (tid < 32) {
        const int lane = tid;
        bool bad = false;
        // right-looking Cholesky, upper factor: column k of R is row k of the trailing matrix
        for (int k = 0; k < r; ++k) {
            const float d = S[k + r * k];
            // S is the Gram of a block the first pass already orthonormalised (S ~ I): a pivot
            // below 1e-4 is a nearly dependent direction, left to the host's SVQB
            if (!(d > 1e-4f) || !isfinite(d)) bad = true;
            const float rkk = sqrtf(d > 0.f ? d : 1.f);
            __syncwarp();
            for (int j = lane; j < r; j += 32) {
                if (j == k) {
                    S[k + r * k] = rkk;
                } else if (j > k) {
                    const float v = S[k + r * j] / rkk;
                    S[k + r * j] = v;
                    rowk[j] = v;
                }
            }
            __syncwarp();
            for (int j = lane; j < r; j += 32)
                if (j > k) chol2_col_update(S + r * j, rowk, k, j, rowk[j]);
            __syncwarp();
        }
        // R^-1 column by column (back substitution), one lane per column
        for (int j = lane; j < r; j += 32) chol2_inv_col(S, Ri + r * j, r, j);
        if (lane == 0) *status = bad ? 1 : 0;
    }
    __syncthreads();
    const int lc = r + wx;
    for (int e = tid; e < lc * r; e += nt) {
        const int i = e % lc, j = e / lc;
        float v;
        if (i < r) {
            v = Ri[i + r * j];
        } else {
            const int q = i - r;
            v = 0.f;
            for (int t = 0; t <= j; ++t) v = fmaf(Gs[q + ld * t], Ri[t + r * j], v);
            v = -v;
        }
        C[i + (size_t)lc * j] = (double)v;
    }
}

void chol2_coeffs(const double *G, int wx, int r, double *C, int *status, cudaStream_t s) {
    KF_REQUIRE(r >= 1 && r <= CHOL2_MAX_R && wx >= 0 && wx <= 128, KF_EINVAL,
               "chol2_coeffs: block width out of range");
    const size_t smem = ((size_t)(wx + r) * r + (size_t)2 * r * r + r) * sizeof(float);
    static int attr_dev_mask = 0;
    int dev = 0;
    KF_CUDA(cudaGetDevice(&dev));
    if (dev < 31 && !(attr_dev_mask & (1 << dev))) {
        // up to (128 + 64) x 64 + 2 x 64 x 64 floats
        KF_CUDA(cudaFuncSetAttribute(k_chol2_coeffs, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
        attr_dev_mask |= 1 << dev;
    }
    k_chol2_coeffs<<<1, 256, smem, s>>>(G, wx, r, C, status);
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

// A counter-based normal generator: splitmix64 of (seed, stream, column, row) into two 24-bit
// uniforms, Box-Muller in FP32 (the draws are start and perturbation directions, where FP32
// normals truncated at 5.8 sigma serve as well as FP64 ones, and GB300's FP64 log / cos made the
// FP64 version ~1 ms per 13M draws).  Reproducible for a given seed whatever the launch shape.
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
    const float u1 = (float)((h >> 40) + 1) * (1.0f / 16777216.0f);   // (0, 1]
    const float u2 = (float)(h2 >> 40) * (1.0f / 16777216.0f);         // [0, 1)
    X[c * ld + r] = (T)(sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2));
}

template <typename T>
void fill_normal(T *X, int64_t ld, int k, int64_t N, uint64_t seed, uint64_t sid, cudaStream_t s) {
    if (k <= 0) return;
    const int64_t tot = N * k;
    k_fill_normal<T><<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(X, ld, N, k, seed, sid);
    KF_LAUNCH_CHECK();
}

// X[:, j] += delta * (||X_j|| / ||R_j||) R_j, the norms' squares in nrm[0..k) (X) and nrm[k..2k) (R).
// Column j = blockIdx.y; the factor is formed once per thread (FP64 square roots and divisions run
// on GB300's narrow FP64 pipe), then a grid-stride loop over the rows.
__global__ void k_perturb_add(double *__restrict__ X, const double *__restrict__ R, int64_t N, int k,
                              const double *__restrict__ nrm, double delta) {
    const int c = blockIdx.y;
    const double f = delta * sqrt(nrm[c]) / sqrt(nrm[k + c]);
    double *x = X + (int64_t)c * N;
    const double *rr = R + (int64_t)c * N;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x)
        x[r] += f * rr[r];
}

// Each column of X (N x k, leading dimension N) plus a vector of norm delta * ||column|| along a
// pseudo-random normal direction (keyed by `key`): the sqrt(eps) perturbation of the initial
// block (src/lobpcg.jl:182-190), drawn on the device.  R: N x k scratch; nrm: 2k doubles.
void perturb_block(double *X, int64_t N, int k, double delta, uint64_t key, double *R, double *nrm, double *partials,
                   cudaStream_t s) {
    if (k <= 0) return;
    fill_normal<double>(R, N, k, N, key, 0x50455254ull, s);
    colnorms2<double>(X, N, k, N, nrm, partials, s);
    colnorms2<double>(R, N, k, N, nrm + k, partials, s);
    const unsigned bx = (unsigned)std::min<int64_t>((N + 255) / 256, 1216);
    k_perturb_add<<<dim3(bx, (unsigned)k), 256, 0, s>>>(X, R, N, k, nrm, delta);
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
    template void gram<T>(const T *, int64_t, int, const T *, int64_t, int, int64_t, double *, double *, cudaStream_t, \
                          bool);                                                                                     \
    template void update2<T>(T *, int64_t, int, const T *, int64_t, int, const T *, int64_t, int, const double *, int,   \
                             double, double, int64_t, cudaStream_t, bool);                                          \
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

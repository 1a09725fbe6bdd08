// FP32 Gram products on the tensor cores (tcgen05), FP32-accurate: operands split into TF32
// hi / lo parts, hi*hi + hi*lo + lo*hi per K step, FP32 accumulation in TMEM, FP64 reduction
// across CTAs.
//
// The Gram products of LOBPCG's orthogonalisation and Rayleigh-Ritz (the reference's X' W, W' W,
// S' H S inside LOBPCGEigensolver, called at src/lobpcg.jl:268, and the Gram of SVQB at
// src/chebyshev.jl:68-81) are tall-skinny: N rows, a few dozen columns.  On the SIMT pipes they are
// FMA-bound (every element of A meets every column of B); here each element is read from memory
// once and the products run on the tensor cores, so the kernel is bound by HBM.
//
// The operand blocks (up to four sources, e.g. [X Z] for [X Z]'Z or [X_a Q HX_a HZ] for one merged
// Rayleigh-Ritz Gram) are stacked as the rows of one "pool" image in shared memory, each source
// starting at a multiple of 8 rows.  Per chunk of GT_KC data rows the image holds pool row m, data
// rows k (K-major, no swizzle: 8-row x 16-byte core matrices).  One MMA chain computes
//   D[m, n] += sum_k pool[m, k] pool[b_off + n, k]      (m < 128, n < Nb)
// i.e. every pool column against the contiguous range of B columns; the entries that the caller
// asked for are picked out of D at the end (rows of sources [r0, r1), columns of [c0, c1)).
//
// One persistent CTA per SM (or per chunk when there are fewer), warp-specialised:
//   warps 0-7   producers: 16-byte cp.async copies of their pieces of the chunk straight into the
//               core-matrix layout of stage t % S (S - 2 chunks in flight ahead),
//               then the split of their own pieces into hi (in place) and lo, arrive on full[s];
//   warp 8      issuer (one lane): waits full[s] and a drained accumulator slot, issues the chunk's
//               MMA chain into slot t % 2 (starting it afresh), commits to empty[s] and accf[t % 2];
//   warps 9-16  epilogue: TMEM lane = pool row (warp % 4 picks the lane quarter), (warp - 9) / 4
//               the half of the B columns; add slot t % 2 into FP32 registers (round to nearest),
//               arrive on acce[t % 2]; at the end write the CTA's FP32 partial sums.
// The tensor cores' FP32 accumulation rounds toward zero, a bias of about 2^-24 of the running sum
// per addition: over a CTA's ~4,400 rows (1,650 MMAs) that reached 1e-4 of a sum of squares.
// Chains of one chunk (12 MMAs) keep it near 1e-6, like the SIMT kernel's FP32 partial sums.
// Every wait is an mbarrier wait with a cycle budget; when one runs out the CTA records
// KF_ETIMEOUT in the host-mapped error word, every role leaves its loop at its next check, the
// issuer waits (bounded) for its MMAs in flight, and TMEM is freed.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "kf_internal.h"

namespace kf {

namespace {

constexpr int GT_PROD = 256;                          // producer threads (warps 0-7)
constexpr int GT_EPI = 256;                           // epilogue threads (warps 9-16)
constexpr int GT_THREADS = GT_PROD + 32 + GT_EPI;     // + the issuer warp
constexpr int GT_NBMAX = 128;                         // B columns (TMEM: two slots of Nb)
constexpr int GT_NBH = GT_NBMAX / 2;                  // B columns per epilogue thread
constexpr int GT_KC = 32;                             // data rows per chunk (MMA K per chunk)
constexpr int GT_ROWS = 144;                          // pool rows at most: the A window 128 + B overhang
constexpr int GT_SBO = (GT_KC / 4) * 128;             // bytes between 8-row groups

// Shared-memory plan for a pool of at most R rows: S stages of hi | lo images (R rows each), then a
// zeroed guard that the 128-row A window of the last images may reach past R (those rows only feed
// accumulator rows nobody reads).  Narrow pools get more stages: about 60 KB of loads in flight per
// SM whatever the pool.
template <int R, int S>
struct GtPlan {
    static constexpr int IMG = R * GT_KC * 4;
    static constexpr int STAGE = 2 * IMG;
    static constexpr int GUARD = R >= 128 ? 0 : (128 - R) * GT_KC * 4;
    static constexpr int PIECES = R * (GT_KC / 4);
    static constexpr int PPT = (PIECES + GT_PROD - 1) / GT_PROD;
    static constexpr int LA = S - 2;                   // chunks loading ahead of the one being split
    static constexpr size_t BARS = (size_t)S * STAGE + GUARD;
    static constexpr size_t SMEM = BARS + 8 * (2 * S + 6);
};
constexpr long long GT_WAIT_CYCLES = 4000000000LL;
constexpr int GT_MAX_SRC = 4;
constexpr int GRAM_TC_DEFAULT_ACCS = 4;

__device__ __forceinline__ uint32_t gsu32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t gt_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;   // descriptor version (tcgen05)
    return d;
}

__device__ __forceinline__ void gt_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void gt_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(gsu32(bar))
                 : "memory");
}

__device__ __forceinline__ void gt_bar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(gsu32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void gt_arrive(uint64_t *bar) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}\n" ::"r"(gsu32(bar))
        : "memory");
}

// completion number `n` (0-based) of the barrier's phases; false when the budget ran out or the
// CTA is aborting
__device__ __forceinline__ bool gt_wait(uint64_t *bar, uint32_t n, volatile int *abort) {
    const uint32_t parity = n & 1u;
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(gsu32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (*abort) return false;
        if (clock64() - t0 > GT_WAIT_CYCLES) return false;
    }
}

// 16-byte asynchronous copy, the bytes past `src_bytes` (0..16) zero-filled
__device__ __forceinline__ void gt_cp16(uint32_t dst, const void *src, int src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}

struct GtArgs {
    const float *p[GT_MAX_SRC];
    int64_t ld[GT_MAX_SRC];
    int off[GT_MAX_SRC], k[GT_MAX_SRC];
    int nsrc;
    int64_t N;
    int64_t nchunks;
    int b_off, Nb;                 // B operand: pool rows [b_off, b_off + Nb)
    int nr, nc;                    // output entries (nr x nc, column-major)
    uint8_t rinv[128];             // pool row -> output row (255: not wanted)
    uint8_t cinv[GT_ROWS];         // B column -> output column (255: not wanted)
    float *part;                   // [gridDim.x][nr * nc]
    int *err;
    uint32_t tcols;                // TMEM columns allocated: 2 x nacc accumulators of astride
    int nacc;                      // accumulators per chunk: MMA j of a chunk adds into j % nacc
    uint32_t astride;              // TMEM columns per accumulator (a power of two >= max(Nb, 32))
    int h0;                        // B columns [0, h0) to epilogue half 0, [h0, Nb) to half 1
};

template <int R, int S>
__global__ void __launch_bounds__(GT_THREADS, 1) k_gram_tc(const GtArgs a) {
    using P = GtPlan<R, S>;
    extern __shared__ __align__(1024) unsigned char gt_smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    unsigned char *stages = gt_smem;
    uint64_t *bars = reinterpret_cast<uint64_t *>(gt_smem + P::BARS);
    uint64_t *full = bars, *empty = bars + S, *accf = bars + 2 * S, *acce = accf + 2,
             *fin = acce + 2;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(fin + 1);
    __shared__ volatile int s_abort;

    // zero the images once: rows that no source fills (gaps, the A window past the pool) stay zero
    for (size_t o = (size_t)tid * 16; o < P::BARS; o += (size_t)GT_THREADS * 16)
        *reinterpret_cast<uint4 *>(stages + o) = make_uint4(0u, 0u, 0u, 0u);
    if (tid == 0) {
        for (int q = 0; q < S; ++q) {
            gt_bar_init(full + q, GT_PROD);
            gt_bar_init(empty + q, 1);
        }
        for (int q = 0; q < 2; ++q) {
            gt_bar_init(accf + q, 1);
            gt_bar_init(acce + q, GT_EPI);
        }
        gt_bar_init(fin, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        s_abort = 0;
    }
    if (warp == 8) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(gsu32(tslot)),
                     "r"(a.tcols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;
    int64_t my = 0;   // chunks of this CTA: blockIdx.x, + gridDim.x, ...
    if ((int64_t)blockIdx.x < a.nchunks) my = (a.nchunks - 1 - blockIdx.x) / gridDim.x + 1;

    if (warp < 8) {
        // ---- producers.  Piece e: pool row 8 (e / 64) + e % 8, data rows 4 ((e / 8) % 8) .. + 3 of
        // the chunk; a quarter-warp covers the 8 rows of one core matrix (conflict-free 16-byte
        // stores), a warp 8 pool columns x 16 data rows (64-byte runs per column).
        const float *gp[P::PPT];
        uint32_t soff[P::PPT];
        int k4[P::PPT];
#pragma unroll
        for (int j = 0; j < P::PPT; ++j) {
            const int e = tid + j * GT_PROD;
            gp[j] = nullptr;
            soff[j] = 0;
            k4[j] = 0;
            if (e < P::PIECES) {
                const int m = (e / 64) * 8 + (e & 7);
                k4[j] = (e >> 3) & 7;
                soff[j] = (uint32_t)((m >> 3) * GT_SBO + k4[j] * 128 + (m & 7) * 16);
                for (int q = 0; q < a.nsrc; ++q)
                    if (m >= a.off[q] && m < a.off[q] + a.k[q]) gp[j] = a.p[q] + (int64_t)(m - a.off[q]) * a.ld[q];
            }
        }
        const uint32_t sbase = gsu32(stages);
        auto issue = [&](int64_t t) {
            const int s = (int)(t % S);
            const int64_t row0 = ((int64_t)blockIdx.x + t * gridDim.x) * GT_KC;
            const uint32_t hi = sbase + (uint32_t)s * P::STAGE;
#pragma unroll
            for (int j = 0; j < P::PPT; ++j) {
                if (!gp[j]) continue;
                const int64_t r = row0 + 4 * k4[j];
                int64_t nb = (a.N - r) * 4;
                nb = nb < 0 ? 0 : nb > 16 ? 16 : nb;
                gt_cp16(hi + soff[j], nb > 0 ? (const void *)(gp[j] + r) : (const void *)gp[j], (int)nb);
            }
        };
        // P::LA chunks in flight ahead of the one being split; the slot refilled at step t held chunk
        // t - 2, whose MMAs had a whole step to retire (refilling t - 1's slot would wait on MMAs
        // issued a moment before and serialise the pipeline)
        for (int t = 0; t < P::LA; ++t) {
            if (t < my) issue(t);
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        }
        for (int64_t t = 0; t < my; ++t) {
            const int64_t tn = t + P::LA;
            if (tn < my) {
                // the slot's previous chunk (tn - S) must be consumed by the tensor cores
                if (tn >= S && !gt_wait(empty + tn % S, (uint32_t)(tn / S - 1), &s_abort)) {
                    s_abort = 1;
                    break;
                }
                issue(tn);
            }
            asm volatile("cp.async.commit_group;\n" ::: "memory");
            asm volatile("cp.async.wait_group %0;\n" ::"n"(P::LA) : "memory");
            // this thread's pieces of chunk t have landed: split them into hi (in place) and lo
            const int s = (int)(t % S);
            unsigned char *hi = stages + (size_t)s * P::STAGE, *lo = hi + P::IMG;
#pragma unroll
            for (int j = 0; j < P::PPT; ++j) {
                if (!gp[j]) continue;
                uint4 v = *reinterpret_cast<const uint4 *>(hi + soff[j]);
                uint32_t x[4] = {v.x, v.y, v.z, v.w}, h[4], l[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    h[q] = x[q] & 0xFFFFE000u;
                    l[q] = __float_as_uint(__uint_as_float(x[q]) - __uint_as_float(h[q]));
                }
                *reinterpret_cast<uint4 *>(hi + soff[j]) = make_uint4(h[0], h[1], h[2], h[3]);
                *reinterpret_cast<uint4 *>(lo + soff[j]) = make_uint4(l[0], l[1], l[2], l[3]);
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            gt_arrive(full + s);
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");
    } else if (warp == 8) {
        // ---- MMA issuer (one lane)
        if (lane == 0) {
            const uint32_t idesc =
                (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(a.Nb >> 3) << 17) | ((128u >> 4) << 24);
            const uint32_t sbase = gsu32(stages);
            const uint32_t boff = (uint32_t)(a.b_off >> 3) * GT_SBO;
            int64_t issued = 0;
            for (int64_t t = 0; t < my; ++t) {
                const int s = (int)(t % S), sl = (int)(t & 1);
                if (!gt_wait(full + s, (uint32_t)(t / S), &s_abort)) { s_abort = 1; break; }
                if (t >= 2 && !gt_wait(acce + sl, (uint32_t)(t / 2 - 1), &s_abort)) { s_abort = 1; break; }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t hi = sbase + (uint32_t)s * P::STAGE, lo = hi + P::IMG;
                const uint32_t d0 = tmem + (uint32_t)(sl * a.nacc) * a.astride;
                // the chunk's 12 MMAs (4 K steps x hi*hi, hi*lo, lo*hi) spread over nacc accumulators:
                // consecutive MMAs are independent, so the tensor pipe is not held by one chain
#pragma unroll
                for (int j = 0; j < 3 * (GT_KC / 8); ++j) {
                    const int ks = j / 3, part = j % 3;
                    const uint32_t o = (uint32_t)ks * 256;
                    const uint64_t da = gt_desc((part == 2 ? lo : hi) + o, 128, GT_SBO);
                    const uint64_t db = gt_desc((part == 1 ? lo : hi) + boff + o, 128, GT_SBO);
                    const int q = j % a.nacc;
                    gt_mma(d0 + (uint32_t)q * a.astride, da, db, idesc, j >= a.nacc ? 1u : 0u);
                }
                gt_commit(empty + s);
                gt_commit(accf + sl);
                ++issued;
            }
            // after an abort: no MMA left in flight before TMEM is freed (bounded)
            if (issued > 0 && s_abort) {
                gt_commit(fin);
                volatile int never = 0;
                (void)gt_wait(fin, 0, &never);
            }
        }
    } else {
        // ---- epilogue (warps 9-16): TMEM lane = pool row 32 (warp % 4) + lane, B columns
        // [cb, ce) of the half (warp - 9) / 4
        const int q = warp & 3, m = q * 32 + lane, h = (warp - 9) >> 2;
        const int cb = h == 0 ? 0 : a.h0, ce = h == 0 ? a.h0 : a.Nb;
        const uint32_t base = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)cb;
        float acc[GT_NBH];
#pragma unroll
        for (int c = 0; c < GT_NBH; ++c) acc[c] = 0.f;
        bool ok = true;
        for (int64_t t = 0; t < my; ++t) {
            const int sl = (int)(t & 1);
            ok = gt_wait(accf + sl, (uint32_t)(t / 2), &s_abort);
            ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld is warp-collective
            if (!ok) { s_abort = 1; break; }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            for (int qa = 0; qa < a.nacc; ++qa) {
                const uint32_t d = base + (uint32_t)(sl * a.nacc + qa) * a.astride;
#pragma unroll
                for (int c0 = 0; c0 < GT_NBH; c0 += 16) {
                    if (cb + c0 >= ce) break;
                    uint32_t r[16];
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
                        "%12, %13, %14, %15}, [%16];\n"
                        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                          "=r"(r[14]), "=r"(r[15])
                        : "r"(d + (uint32_t)c0));
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
                    for (int u = 0; u < 16; ++u) acc[c0 + u] += __uint_as_float(r[u]);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            gt_arrive(acce + sl);
        }
        const int i = a.rinv[m];
        if (ok && i != 255) {
            float *out = a.part + (size_t)blockIdx.x * a.nr * a.nc;
#pragma unroll
            for (int c = 0; c < GT_NBH; ++c) {
                if (cb + c >= ce) break;
                const int j = a.cinv[cb + c];
                if (j != 255) out[i + (size_t)a.nr * j] = acc[c];
            }
        }
    }
    if (s_abort && tid == 0) {
        *(volatile int *)a.err = KF_ETIMEOUT;
        __threadfence_system();
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 8) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(a.tcols));
}

// G[e] = sum over the CTAs' FP32 partials, in FP64, one warp per entry
__global__ void k_reduce_partials_f32(const float *__restrict__ part, int nparts, int n, double *__restrict__ G) {
    const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (e >= n) return;
    double s = 0;
    for (int c = lane; c < nparts; c += 32) s += (double)part[(size_t)c * n + e];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) G[e] = s;
}

// per device: SM count and, per plan, whether the kernel fits and its attribute is set
struct GtDevice {
    bool ready = false;
    int sms = 0;
    bool fits[3] = {false, false, false};
};
std::mutex g_gt_mu;
GtDevice g_gt_dev[32];

using GtKernel = void (*)(const GtArgs);
const GtKernel g_gt_kern[3] = {k_gram_tc<48, 14>, k_gram_tc<80, 8>, k_gram_tc<144, 5>};
const size_t g_gt_smem[3] = {GtPlan<48, 14>::SMEM, GtPlan<80, 8>::SMEM, GtPlan<144, 5>::SMEM};

const GtDevice &gt_device() {
    int dev = 0;
    KF_CUDA(cudaGetDevice(&dev));
    KF_REQUIRE(dev >= 0 && dev < 32, KF_EINVAL, "gram_tc: device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_gt_mu);
    GtDevice &d = g_gt_dev[dev];
    if (!d.ready) {
        int optin = 0;
        KF_CUDA(cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev));
        KF_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        for (int p = 0; p < 3; ++p) {
            cudaFuncAttributes fa;
            KF_CUDA(cudaFuncGetAttributes(&fa, g_gt_kern[p]));
            d.fits[p] = g_gt_smem[p] + fa.sharedSizeBytes <= (size_t)optin;
            if (d.fits[p])
                KF_CUDA(cudaFuncSetAttribute(g_gt_kern[p], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)g_gt_smem[p]));
        }
        d.ready = true;
    }
    return d;
}

}  // namespace

int gram_tc_sms() { return gt_device().sms; }

size_t gram_tc_partials_size(int nr, int nc) { return (size_t)256 * nr * nc * sizeof(float); }

bool gram_tc(const GramTcSrc *src, int nsrc, int r0, int r1, int c0, int c1, int64_t N, double *G, void *partials,
             size_t partial_bytes, cudaStream_t s, int accs) {
    if (nsrc < 1 || nsrc > GT_MAX_SRC || r0 < 0 || r1 > nsrc || r0 >= r1 || c0 < 0 || c1 > nsrc || c0 >= c1) return false;
    if (N < GT_KC) return false;
    GtArgs a;
    std::memset(&a, 0, sizeof a);
    int off = 0;
    for (int q = 0; q < nsrc; ++q) {
        const GramTcSrc &c = src[q];
        if (c.k < 1 || !c.p || c.ld % 4 != 0 || (uintptr_t)c.p % 16 != 0) return false;
        a.p[q] = c.p;
        a.ld[q] = c.ld;
        a.k[q] = c.k;
        a.off[q] = off;
        off = (off + c.k + 7) / 8 * 8;
    }
    if (off > GT_ROWS) return false;
    // rows of G: pool rows below 128 (the MMA's M); columns: the B window inside the image
    if (a.off[r1 - 1] + a.k[r1 - 1] > 128) return false;
    a.b_off = a.off[c0];
    const int bend = a.off[c1 - 1] + a.k[c1 - 1];
    a.Nb = (bend - a.b_off + 15) / 16 * 16;
    if (a.b_off + a.Nb > GT_ROWS || a.Nb > GT_NBMAX) return false;
    a.nsrc = nsrc;
    a.N = N;
    a.nchunks = (N + GT_KC - 1) / GT_KC;
    std::memset(a.rinv, 255, sizeof a.rinv);
    std::memset(a.cinv, 255, sizeof a.cinv);
    int nr = 0, nc = 0;
    for (int q = r0; q < r1; ++q)
        for (int c = 0; c < a.k[q]; ++c) a.rinv[a.off[q] + c] = (uint8_t)nr++;
    for (int q = c0; q < c1; ++q)
        for (int c = 0; c < a.k[q]; ++c) a.cinv[a.off[q] + c - a.b_off] = (uint8_t)nc++;
    if (nr > 254 || nc > 254) return false;
    a.nr = nr;
    a.nc = nc;
    const GtDevice &dv = gt_device();
    const int grid = (int)std::min<int64_t>(dv.sms, a.nchunks);
    if ((size_t)grid * nr * nc * sizeof(float) > partial_bytes) return false;
    a.part = (float *)partials;
    a.err = tc_error_word();
    // accumulators: two chunk slots x nacc, each a power of two >= max(Nb, 32) columns, within the
    // 512 TMEM columns of the SM
    uint32_t as = 32;
    while (as < (uint32_t)a.Nb) as <<= 1;
    const int amax = (int)(256 / as);
    int nacc = accs > 0 ? accs : GRAM_TC_DEFAULT_ACCS;
    nacc = std::min(nacc, std::min(amax, 12));
    a.nacc = nacc;
    a.astride = as;
    uint32_t tc = 32;
    while (tc < 2u * (uint32_t)nacc * as) tc <<= 1;
    a.tcols = tc;
    a.h0 = std::min(a.Nb, (a.Nb / 2 + 15) / 16 * 16);
    // the plan by pool rows (a multiple of 8): more stages for narrower pools
    const int plan = off <= 48 ? 0 : off <= 80 ? 1 : 2;
    if (!dv.fits[plan]) return false;
    g_gt_kern[plan]<<<grid, GT_THREADS, g_gt_smem[plan], s>>>(a);
    KF_LAUNCH_CHECK();
    const int n = nr * nc;
    k_reduce_partials_f32<<<(n + 7) / 8, 256, 0, s>>>((const float *)partials, grid, n, G);
    KF_LAUNCH_CHECK();
    return true;
}

}  // namespace kf

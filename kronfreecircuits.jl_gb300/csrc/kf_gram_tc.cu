// FP32 Gram products on the tensor cores (tcgen05), FP32-accurate: operands split into TF32
// hi / lo parts, hi*hi + hi*lo + lo*hi per K step, FP32 accumulation in TMEM, FP64 reduction
// across CTAs.
//
// The Gram products of LOBPCG's orthogonalisation and Rayleigh-Ritz (the reference's X' W, W' W,
// S' H S inside LOBPCGEigensolver, called at src/lobpcg.jl:268, and the Gram of SVQB at
// src/chebyshev.jl:68-81) are tall-skinny: N rows, a few dozen columns.  On the SIMT pipes they are
// FMA-bound and their cost grows with the output; here every element is read from memory once.
//
// A kind::tf32 MMA (M = 128, K = 8) costs 44.5 cycles at N = 16, 48 at N = 64 and 64 at N = 128
// (measured alone on GB300: the tensor core reads its operands at about 128 bytes per cycle), so
// one wide MMA that carries several of the split products is cheaper than several narrow ones, and
// the images are laid out for that:
//   the pool (up to four source blocks, each starting at a multiple of 8 rows) puts the sources
//   that only give rows of G first and the B sources (the columns of G) last, ending at row RB of
//   the hi image; the lo image follows it and starts with the B rows (then the others).  The B
//   operand "hi rows [b_off, RB) + lo rows [0, nbr)" is then one contiguous [B_hi; B_lo].
//   RB = 64 (pools up to 64 rows): the A operand "hi rows 0..63 + lo rows 0..63" is [A_hi; A_lo]
//     and ONE MMA per K step gives hi*hi | hi*lo (accumulator rows 0..63) and lo*hi | lo*lo
//     (rows 64..127; lo*lo is not used);
//   RB = 128: two MMAs per K step, A_hi x [B_hi; B_lo] and A_lo x [B_hi; B_lo] (whose lo*lo half
//     is not used either);
//   SPLIT (the row sources and the column sources disjoint, up to 64 rows each -- the Rayleigh-Ritz
//     Gram [X_a Q]'[HX_a HZ]): the stage's 256 rows hold A_hi | A_lo | B_hi | B_lo, so
//     [A_hi; A_lo] (M = 128) x [B_hi; B_lo] is again ONE MMA per K step, with the RB = 64
//     accumulator layout.
// The epilogue adds hi*hi + hi*lo on the lanes of the hi rows and lo*hi on the lanes of the lo
// rows into two FP32 partial sets per CTA; the reduction sums both.
//
// Two kernels share these layouts.  k_gram_tma (the default, below) loads with 2-D tensor copies
// of 128 rows x k columns per source; k_gram_tc, the fallback where the CUDA driver gives no tensor-map
// encoder, copies 16-byte pieces with cp.async.  What was measured on GB300 on the way there:
//   - a stream of tensor copies over the solve's 54 columns reaches 1.4-2.0 TB/s with 32-row boxes
//     (128-byte rows), 2.8 TB/s with 64-row, 5.0 TB/s with 128-row and 5.7 TB/s with 256-row boxes:
//     the copy engine pays per box row, so the rows must be long;
//   - a synchronisation per 32-row chunk (split -> issuer -> epilogue -> issuer) costs more than
//     the chunk's loads, split and 4 MMAs together: timing-only copies that dropped the loads, the
//     split, the MMAs or the epilogue's TMEM loads all stayed within 15% of the full kernel, and a
//     clock64 timeline showed each barrier hop taking a few hundred cycles.  So the 64-row pools
//     synchronise once per 4 chunks (two accumulator slots of 2 chunks each, double-buffered);
//   - the split loads its pieces for a chunk before storing any (the loads and stores go to
//     different buffers, which the compiler cannot tell apart).
// [X Z]'Z at block 18 (18 + 36 columns, N = 671,744) went 94.5 -> 53.4 us with these, the
// Rayleigh-Ritz pool (108 columns) 131.3 -> 106.7 us.
//
// k_gram_tc: one persistent CTA per SM (or per chunk when there are fewer), warp-specialised:
//   warps 0-7   producers: 16-byte cp.async copies of their pieces of the chunk straight into the
//               core-matrix layout of the hi image of stage t % S (S - R chunks in flight ahead),
//               then the split of their own pieces into hi (in place) and lo, arrive on full[s];
//   warp 8      issuer (one lane): waits full[s] and a drained accumulator slot, issues the chunk's
//               MMAs into slot t % 2 (starting it afresh), commits to empty[s] and accf[t % 2];
//   warps 9-16  epilogue: TMEM lane = accumulator row (warp % 4 picks the lane quarter), (warp - 9)
//               / 4 the half of the B columns; adds slot t % 2 into FP32 registers (round to
//               nearest), arrives on acce[t % 2]; at the end writes the CTA's FP32 partial sums.
// The tensor cores' FP32 accumulation rounds toward zero, a bias of about 2^-24 of the running sum
// per addition: accumulator chains of one or two chunks (4 or 8 MMAs per accumulator) keep it near
// 1e-7 or 2e-7 of an entry.
// Every wait is an mbarrier wait with a cycle budget; when one runs out the CTA records
// KF_ETIMEOUT in the host-mapped error word, every role leaves its loop at its next check, the
// issuer waits (bounded) for its MMAs in flight, and TMEM is freed.
// KF_CHECK builds test, in k_gram_tma, every raw-slot piece read (site 301), every operand-image
// store (302) and every tensor copy's box against its slot (303), and record a failure instead of
// the access.
#include <cuda.h>   // CUtensorMap and its enums (the encoder itself is taken from the CUDA driver at run time)

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "kf_internal.h"

namespace kf {

namespace {

constexpr int GT_PROD = 256;                          // producer threads (warps 0-7)
constexpr int GT_EPI = 256;                           // epilogue threads (warps 9-16)
constexpr int GT_THREADS = GT_PROD + 32 + GT_EPI;     // + the issuer warp
constexpr int GT_KC = 32;                             // data rows per chunk (4 MMA K steps)
constexpr int GT_SBO = (GT_KC / 4) * 128;             // bytes between 8-row groups of an image
constexpr int GT_NBR_MAX = 64;                        // B columns
constexpr int GT_NBH = GT_NBR_MAX / 2;                // B columns per epilogue thread
constexpr long long GT_WAIT_CYCLES = 4000000000LL;
constexpr int GT_MAX_SRC = 4;

constexpr int GT_MAX_SLOTS = 2;                       // accumulator slots

// Shared-memory plan for RB image rows: S stages of hi | lo images; the producers refill the stage
// of chunk t - R.
template <int RB, int S, int R>
struct GtPlan {
    static constexpr int IMG = RB * GT_KC * 4;
    static constexpr int STAGE = 2 * IMG;
    static constexpr int PIECES = RB * (GT_KC / 4);    // 16-byte pieces of one image
    static constexpr int PPT = PIECES / GT_PROD;       // pieces per producer thread
    static constexpr int LA = S - R;                   // chunks loading ahead of the one being split
    static constexpr size_t BARS = (size_t)S * STAGE;
    static constexpr size_t SMEM = BARS + 8 * (2 * S + 2 * GT_MAX_SLOTS + 2);
    static_assert(PIECES % GT_PROD == 0, "pieces per thread");
    static_assert(LA >= 2, "loads in flight");
};

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
// CTA is aborting.  The waiting thread is suspended inside try_wait until the phase completes (or
// for at most the hint, 1 ms), so idle roles take no issue slots and no shared-memory bandwidth
// from the ones working: with spinning waits, a wait on a barrier that had completed long before
// took the MMA issuer 350-430 cycles.
__device__ __forceinline__ bool gt_wait(uint64_t *bar, uint32_t n, volatile int *abort) {
    const uint32_t parity = n & 1u;
    {
        // a phase that has completed already: the non-blocking test answers without the try_wait
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(gsu32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    long long t0 = -1;
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(gsu32(bar)), "r"(parity), "r"(1000000u)
            : "memory");
        if (done) return true;
        if (*abort) return false;
        const long long now = clock64();
        if (t0 < 0) t0 = now;
        else if (now - t0 > GT_WAIT_CYCLES) return false;
    }
}

// 16-byte asynchronous copy, the bytes past `src_bytes` (0..16) zero-filled
__device__ __forceinline__ void gt_cp16(uint32_t dst, const void *src, int src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}

// 16 consecutive accumulator columns of this warp's 32 TMEM lanes
__device__ __forceinline__ void gt_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

struct GtArgs {
    CUtensorMap tm[GT_MAX_SRC];    // TMA variant: per source, boxes of 128 rows x k columns
    uint32_t roff[GT_MAX_SRC];     // TMA variant: byte offset of source q's box in a raw slot
    uint32_t rslot, tx_bytes;      // TMA variant: bytes of a raw slot (one group, all sources)
    int nraw;                      // TMA variant: raw slots
    const float *p[GT_MAX_SRC];
    int64_t ld[GT_MAX_SRC];
    int off[GT_MAX_SRC], k[GT_MAX_SRC];   // hi image rows [off, off + k) per source
    int nsrc;
    int64_t N;
    int64_t nchunks;
    int b_off, nbr;                // B rows: hi rows [b_off, RB) = lo rows [0, nbr); nbr % 8 == 0
                                   // (SPLIT: stage rows RB + [0, nbr) and RB + nbr + [0, nbr))
    int nr, nc;                    // output entries (nr x nc, column-major)
    uint8_t rinv_hi[128];          // hi image row -> output row (255: not wanted)
    uint8_t rinv_lo[128];          // lo image row -> output row
    uint8_t cinv[GT_NBR_MAX];      // B column -> output column (255: padding)
    float *part;                   // [gridDim.x][2][nr * nc]: hi-row sums, lo-row sums
    int *err;
};

template <int RB, int S, int R, bool SPLIT = false>
__global__ void __launch_bounds__(GT_THREADS, 1) k_gram_tc(const GtArgs a) {
    using P = GtPlan<RB, S, R>;
    static_assert(!SPLIT || RB == 128, "the split layout fills two 128-row images");
    constexpr bool ONE = RB == 64 || SPLIT;    // one MMA per K step ([A_hi; A_lo] x [B_hi; B_lo])
    // two accumulator slots at power-of-two column offsets (measured faster than packed slots);
    // RB = 128: the second MMA's accumulator 128 columns into the slot
    constexpr uint32_t SLOT = ONE ? 128 : 256;
    extern __shared__ __align__(1024) unsigned char gt_smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    unsigned char *stages = gt_smem;
    uint64_t *bars = reinterpret_cast<uint64_t *>(gt_smem + P::BARS);
    uint64_t *full = bars, *empty = bars + S, *accf = bars + 2 * S, *acce = accf + GT_MAX_SLOTS,
             *fin = acce + GT_MAX_SLOTS;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(fin + 1);
    __shared__ volatile int s_abort;

    // zero the images once: rows that no source fills (alignment gaps) stay zero
    for (size_t o = (size_t)tid * 16; o < P::BARS; o += (size_t)GT_THREADS * 16)
        *reinterpret_cast<uint4 *>(stages + o) = make_uint4(0u, 0u, 0u, 0u);
    if (tid == 0) {
        for (int q = 0; q < S; ++q) {
            gt_bar_init(full + q, GT_PROD);
            gt_bar_init(empty + q, 1);
        }
        for (int q = 0; q < GT_MAX_SLOTS; ++q) {
            gt_bar_init(accf + q, 1);
            gt_bar_init(acce + q, GT_EPI);
        }
        gt_bar_init(fin, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        s_abort = 0;
    }
    if (warp == 8) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(gsu32(tslot)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;
    // this CTA's chunks: a contiguous range [c0, c0 + my) (each column streamed in order rather
    // than in 128-byte pieces spread over the whole grid)
    const int64_t cper = a.nchunks / gridDim.x, crem = a.nchunks % gridDim.x;
    const int64_t my = cper + ((int64_t)blockIdx.x < crem ? 1 : 0);
    const int64_t cfirst = (int64_t)blockIdx.x * cper + ((int64_t)blockIdx.x < crem ? (int64_t)blockIdx.x : crem);

    if (warp < 8) {
        // ---- producers.  Piece e: pool row 8 (e / 64) + e % 8, data rows 4 ((e / 8) % 8) .. + 3 of
        // the chunk; a quarter-warp covers the 8 rows of one core matrix (conflict-free 16-byte
        // stores), a warp 8 pool columns x 16 data rows (64-byte runs per column).  Positions count
        // the stage's rows across both images (the lo image starts at row RB).  Pool row m sits at
        // hi row m and its lo part at lo row m - b_off (B rows) or m + nbr (the others); SPLIT: an A
        // row m at m and 64 + m, B row b_off + r at RB + r and RB + nbr + r.
        const float *gp[P::PPT];
        uint32_t soff[P::PPT], loff[P::PPT];
        int k4[P::PPT];
#pragma unroll
        for (int j = 0; j < P::PPT; ++j) {
            const int e = tid + j * GT_PROD;
            const int m = (e / 64) * 8 + (e & 7);
            int ph, pl;
            if (SPLIT) {
                ph = m < a.b_off ? m : RB + (m - a.b_off);
                pl = m < a.b_off ? 64 + m : RB + a.nbr + (m - a.b_off);
            } else {
                ph = m;
                pl = RB + (m >= a.b_off ? m - a.b_off : m + a.nbr);
            }
            k4[j] = (e >> 3) & 7;
            soff[j] = (uint32_t)((ph >> 3) * GT_SBO + k4[j] * 128 + (ph & 7) * 16);
            loff[j] = (uint32_t)((pl >> 3) * GT_SBO + k4[j] * 128 + (pl & 7) * 16);
            gp[j] = nullptr;
            for (int q = 0; q < a.nsrc; ++q)
                if (m >= a.off[q] && m < a.off[q] + a.k[q]) gp[j] = a.p[q] + (int64_t)(m - a.off[q]) * a.ld[q];
        }
        const uint32_t sbase = gsu32(stages);
        auto issue = [&](int64_t t) {
            const int s = (int)(t % S);
            const int64_t row0 = (cfirst + t) * GT_KC;
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
        // P::LA chunks in flight ahead of the one being split; the stage refilled at step t held chunk
        // t - R, whose MMAs had R - 1 steps to retire
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
            unsigned char *st = stages + (size_t)s * P::STAGE;
#pragma unroll
            for (int j = 0; j < P::PPT; ++j) {
                if (!gp[j]) continue;
                uint4 v = *reinterpret_cast<const uint4 *>(st + soff[j]);
                uint32_t x[4] = {v.x, v.y, v.z, v.w}, h[4], l[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    h[q] = x[q] & 0xFFFFE000u;
                    l[q] = __float_as_uint(__uint_as_float(x[q]) - __uint_as_float(h[q]));
                }
                *reinterpret_cast<uint4 *>(st + soff[j]) = make_uint4(h[0], h[1], h[2], h[3]);
                *reinterpret_cast<uint4 *>(st + loff[j]) = make_uint4(l[0], l[1], l[2], l[3]);
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            gt_arrive(full + s);
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");
    } else if (warp == 8) {
        // ---- MMA issuer (one lane)
        if (lane == 0) {
            const uint32_t n1 = (uint32_t)(2 * a.nbr);
            const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((n1 >> 3) << 17) | ((128u >> 4) << 24);
            const uint32_t sbase = gsu32(stages);
            const uint32_t boff = SPLIT ? (uint32_t)P::IMG : (uint32_t)(a.b_off >> 3) * GT_SBO;
            int64_t issued = 0;
            for (int64_t t = 0; t < my; ++t) {
                const int s = (int)(t % S), sl = (int)(t & 1);
                if (!gt_wait(full + s, (uint32_t)(t / S), &s_abort)) { s_abort = 1; break; }
                if (t >= 2 && !gt_wait(acce + sl, (uint32_t)(t / 2 - 1), &s_abort)) { s_abort = 1; break; }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t hi = sbase + (uint32_t)s * P::STAGE, lo = hi + P::IMG;
                const uint32_t d = tmem + (uint32_t)sl * SLOT;
#pragma unroll
                for (int ks = 0; ks < GT_KC / 8; ++ks) {
                    const uint32_t o = (uint32_t)ks * 256;
                    const uint64_t db = gt_desc(hi + boff + o, 128, GT_SBO);   // [B_hi; B_lo]
                    gt_mma(d, gt_desc(hi + o, 128, GT_SBO), db, idesc, ks > 0 ? 1u : 0u);
                    if (!ONE) gt_mma(d + 128, gt_desc(lo + o, 128, GT_SBO), db, idesc, ks > 0 ? 1u : 0u);
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
        // ---- epilogue (warps 9-16): TMEM lane = accumulator row 32 (warp % 4) + lane, B columns
        // [cb, ce) of the half (warp - 9) / 4.  ONE: lanes 0-63 are hi rows (hi*hi at column n,
        // hi*lo at nbr + n), lanes 64-127 lo rows (lo*hi at n).  Otherwise every lane has hi row m
        // (slot columns n, nbr + n) and lo row m (slot column 128 + n).
        const int q = warp & 3, m = q * 32 + lane, h = (warp - 9) >> 2;
        const int h0 = min(a.nbr, (a.nbr / 2 + 15) / 16 * 16);
        const int cb = h == 0 ? 0 : h0, ce = h == 0 ? h0 : a.nbr;
        const uint32_t lb = (uint32_t)(q * 32) << 16;
        const bool has_hi = !ONE || q < 2, has_lo = !ONE || q >= 2;
        float acc_hi[GT_NBH], acc_lo[GT_NBH];
#pragma unroll
        for (int c = 0; c < GT_NBH; ++c) acc_hi[c] = acc_lo[c] = 0.f;
        bool ok = true;
        for (int64_t t = 0; t < my; ++t) {
            const int sl = (int)(t & 1);
            ok = gt_wait(accf + sl, (uint32_t)(t / 2), &s_abort);
            ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld is warp-collective
            if (!ok) { s_abort = 1; break; }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t d = tmem + lb + (uint32_t)sl * SLOT;
#pragma unroll
            for (int c0 = 0; c0 < GT_NBH; c0 += 16) {
                if (cb + c0 >= ce) break;
                const uint32_t col = (uint32_t)(cb + c0);
                uint32_t r1[16];
                if (has_hi) {
                    gt_ld16(d + col, r1);
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
                    for (int u = 0; u < 16; ++u) acc_hi[c0 + u] += __uint_as_float(r1[u]);
                    gt_ld16(d + (uint32_t)a.nbr + col, r1);
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
                    for (int u = 0; u < 16; ++u) acc_hi[c0 + u] += __uint_as_float(r1[u]);
                }
                if (has_lo) {
                    gt_ld16(d + (ONE ? 0u : 128u) + col, r1);
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
                    for (int u = 0; u < 16; ++u) acc_lo[c0 + u] += __uint_as_float(r1[u]);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            gt_arrive(acce + sl);
        }
        if (ok) {
            const size_t E = (size_t)a.nr * a.nc;
            float *out = a.part + (size_t)blockIdx.x * 2 * E;
            const int ih = has_hi ? a.rinv_hi[m] : 255;
            const int il = has_lo ? a.rinv_lo[ONE ? m - 64 : m] : 255;
#pragma unroll
            for (int c = 0; c < GT_NBH; ++c) {
                if (cb + c >= ce) break;
                const int j = a.cinv[cb + c];
                if (j == 255) continue;
                if (ih != 255) out[ih + (size_t)a.nr * j] = acc_hi[c];
                if (il != 255) out[E + il + (size_t)a.nr * j] = acc_lo[c];
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
    if (warp == 8) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(512));
}

// ---- The TMA-fed variant (the default).  Same pool layouts, accumulator slots and epilogue as
// k_gram_tc; the loads are 2-D tensor copies of 128 rows x k columns per source (512-byte rows:
// measured on GB300, a stream of such boxes over the solve's 54 columns reaches 5.0 TB/s, one of
// 32-row boxes -- 128-byte rows -- only 1.4-2.0 TB/s, whatever the ring depth), into a raw ring of
// groups (per source, per column, 128 consecutive FP32 values).  Four 32-row chunks per group:
//   warp 0      producer (one lane): one box per source per group into raw slot g % R,
//               completing on rfull;
//   warps 1-4   split: per chunk, the 16-byte pieces of the chunk's pool rows from the raw slot
//               (eight threads read one column's 128 bytes) into hi and lo operand images of
//               stage t % SO, K-major in the 128-byte-swizzled layout (piece j of image row r at
//               position j ^ (r % 8), 8-row atoms 1024 bytes apart); one arrival per warp on
//               ofull, and on rempty once the group's four chunks are done;
//   warp 5      issuer, warps 6-13 epilogue: as in k_gram_tc (swizzled descriptors).
// Rows past N read as zero (the tensor copy's fill), so a group is always four chunks.
constexpr int GM_SPLITTERS = 128;                               // warps 1-4
constexpr int GM_THREADS = 32 + GM_SPLITTERS + 32 + GT_EPI;     // 448
constexpr int GM_GR = 128;                                      // data rows per group
constexpr int GM_CPG = GM_GR / GT_KC;                           // chunks per group
constexpr int GM_MAX_RAW = 8;                                   // raw slots at most

template <int RB, int SO, int CPS>
struct GmPlan {
    static constexpr int IMG = RB * GT_KC * 4;
    static constexpr int CHB = 2 * IMG;                         // hi + lo images of one chunk
    static constexpr int STAGE = CPS * CHB;                     // one synchronisation unit
    static constexpr int OPS = SO * STAGE;                      // operand stages
    static constexpr int PPT = RB * 8 / GM_SPLITTERS;           // 16-byte pieces of the pool rows per thread
    static constexpr int ASL = CPS == 4 ? 2 : 1;                // accumulator slots per unit
    static constexpr int CPA = CPS / ASL;                       // chunks accumulated per slot
    static constexpr size_t BARS = 8 * (2 * GM_MAX_RAW + 2 * SO + 2 * GT_MAX_SLOTS + 2);
    static_assert(IMG % 1024 == 0, "swizzle atoms");
    static_assert(CPS == 1 || CPS == 4, "chunks per unit");
};

// dynamic shared memory of a launch with R raw slots of `rslot` bytes
template <int RB, int SO, int CPS>
size_t gm_smem(int R, uint32_t rslot) {
    return 1024 + (size_t)GmPlan<RB, SO, CPS>::OPS + (size_t)R * rslot + GmPlan<RB, SO, CPS>::BARS;
}

// K-major operand in the 128-byte-swizzled layout: rows of 128 bytes, 8-row atoms 1024 bytes apart
__device__ __forceinline__ uint64_t gm_desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;                  // leading-dimension offset (unused for swizzled K-major)
    d |= (uint64_t)(1024u >> 4) << 32;       // stride between 8-row atoms
    d |= (uint64_t)1 << 46;                  // descriptor version (tcgen05)
    d |= (uint64_t)2 << 61;                  // 128-byte swizzle
    return d;
}

__device__ __forceinline__ void gm_expect(uint64_t *bar, uint32_t bytes) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}\n" ::"r"(gsu32(bar)),
        "r"(bytes)
        : "memory");
}

// one 2-D box of the tensor map (a kernel parameter) at element coordinates (x, y)
__device__ __forceinline__ void gm_tma2d(uint32_t dst, const CUtensorMap *tm, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];\n" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(gsu32(bar))
        : "memory");
}

template <int RB, int SO, bool SPLIT, int CPS>
__global__ void __launch_bounds__(GM_THREADS, 1) k_gram_tma(const __grid_constant__ GtArgs a) {
    using P = GmPlan<RB, SO, CPS>;
    static_assert(CPS == 1 || RB == 64 || SPLIT, "four chunks per unit need the one-MMA accumulator layout");
    constexpr int UPG = GM_CPG / CPS;          // units per group
    static_assert(!SPLIT || RB == 128, "the split layout fills two 128-row images");
    constexpr bool ONE = RB == 64 || SPLIT;
    constexpr uint32_t SLOT = ONE ? 128 : 256;
    extern __shared__ unsigned char gm_smem_raw[];
    unsigned char *ops = gm_smem_raw + ((1024u - (gsu32(gm_smem_raw) & 1023u)) & 1023u);
    const int R = a.nraw;
    unsigned char *raw = ops + P::OPS;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint64_t *bars = reinterpret_cast<uint64_t *>(raw + (size_t)R * a.rslot);
    uint64_t *rfull = bars, *rempty = bars + GM_MAX_RAW, *ofull = bars + 2 * GM_MAX_RAW, *oempty = ofull + SO,
             *accf = oempty + SO, *acce = accf + GT_MAX_SLOTS, *fin = acce + GT_MAX_SLOTS;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(fin + 1);
    __shared__ volatile int s_abort;

    // zero the operand images once: rows that no source fills (alignment gaps) stay zero
    for (size_t o = (size_t)tid * 16; o < (size_t)P::OPS; o += (size_t)GM_THREADS * 16)
        *reinterpret_cast<uint4 *>(ops + o) = make_uint4(0u, 0u, 0u, 0u);
    if (tid == 0) {
        for (int q = 0; q < R; ++q) {
            gt_bar_init(rfull + q, 1);
            gt_bar_init(rempty + q, GM_SPLITTERS / 32);
        }
        for (int q = 0; q < SO; ++q) {
            gt_bar_init(ofull + q, GM_SPLITTERS / 32);
            gt_bar_init(oempty + q, 1);
        }
        for (int q = 0; q < GT_MAX_SLOTS; ++q) {
            gt_bar_init(accf + q, 1);
            gt_bar_init(acce + q, GT_EPI / 32);
        }
        gt_bar_init(fin, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        s_abort = 0;
    }
    if (warp == 5) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(gsu32(tslot)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;
    // this CTA's groups: a contiguous range [gfirst, gfirst + myg)
    const int64_t ngroups = a.nchunks;
    const int64_t gper = ngroups / gridDim.x, grem = ngroups % gridDim.x;
    const int64_t myg = gper + ((int64_t)blockIdx.x < grem ? 1 : 0);
    const int64_t gfirst = (int64_t)blockIdx.x * gper + ((int64_t)blockIdx.x < grem ? (int64_t)blockIdx.x : grem);
    const int64_t myu = myg * UPG;     // synchronisation units
    const uint32_t obase = gsu32(ops), rbase = gsu32(raw);

    if (warp == 0) {
        // ---- producer (one lane)
        if (lane == 0) {
            int64_t issued = 0;
            for (int64_t g = 0; g < myg; ++g) {
                const int r = (int)(g % R);
                // the slot held group g - R: its four chunks must have been split
                if (g >= R && !gt_wait(rempty + r, (uint32_t)(g / R - 1), &s_abort)) { s_abort = 1; break; }
                gm_expect(rfull + r, a.tx_bytes);
                const int x = (int)((gfirst + g) * GM_GR);
                const uint32_t slot = rbase + (uint32_t)r * a.rslot;
                // KF_CHECK site 303: every source's box inside the raw slot
                for (int q = 0; q < a.nsrc; ++q)
                    if (KF_CHK(a.roff[q] + (uint32_t)a.k[q] * (GM_GR * 4) <= a.rslot, a.err, 303))
                        gm_tma2d(slot + a.roff[q], &a.tm[q], x, 0, rfull + r);
                ++issued;
            }
            if (s_abort) {
                // copies still in flight write this CTA's shared memory: wait (bounded) for them
                volatile int never = 0;
                for (int64_t g = issued > R ? issued - R : 0; g < issued; ++g)
                    (void)gt_wait(rfull + g % R, (uint32_t)(g / R), &never);
            }
        }
    } else if (warp <= 4) {
        // ---- split: piece e of a chunk's pool rows is row m = e / 8, K piece j = e % 8 (data rows
        // 4 j .. 4 j + 3 of the chunk); eight consecutive threads read one column's 128 bytes and
        // write one swizzled image row (conflict-free both ways)
        const int ct = tid - 32;
        uint32_t roff[P::PPT], hoff[P::PPT], loff[P::PPT];
        bool has[P::PPT];
#pragma unroll
        for (int j = 0; j < P::PPT; ++j) {
            const int e = ct + j * GM_SPLITTERS;
            const int m = e >> 3, pj = e & 7;
            int ph, pl;
            if (SPLIT) {
                ph = m < a.b_off ? m : RB + (m - a.b_off);
                pl = m < a.b_off ? 64 + m : RB + a.nbr + (m - a.b_off);
            } else {
                ph = m;
                pl = RB + (m >= a.b_off ? m - a.b_off : m + a.nbr);
            }
            hoff[j] = (uint32_t)(ph * 128 + ((pj ^ (ph & 7)) << 4));
            loff[j] = (uint32_t)(pl * 128 + ((pj ^ (pl & 7)) << 4));
            has[j] = false;
            roff[j] = 0;
            for (int q = 0; q < a.nsrc; ++q)
                if (m >= a.off[q] && m < a.off[q] + a.k[q]) {
                    has[j] = true;
                    roff[j] = a.roff[q] + (uint32_t)(m - a.off[q]) * (GM_GR * 4) + (uint32_t)pj * 16;
                }
        }
        bool ok = true;
        for (int64_t g = 0; g < myg && ok; ++g) {
            const int r = (int)(g % R);
            ok = __all_sync(0xffffffffu, gt_wait(rfull + r, (uint32_t)(g / R), &s_abort));
            if (!ok) break;
            const unsigned char *slot = raw + (size_t)r * a.rslot;
            for (int i = 0; i < UPG; ++i) {
                const int64_t u = g * UPG + i;
                const int o = (int)(u % SO);
                // the stage held unit u - SO: its MMAs must have retired
                if (u >= SO) {
                    ok = __all_sync(0xffffffffu, gt_wait(oempty + o, (uint32_t)(u / SO - 1), &s_abort));
                    if (!ok) break;
                }
                // the pieces of chunk cu + 1 are loaded before those of chunk cu are stored, so the
                // loads of a chunk are in flight together (a piece without a source reads the slot's
                // first bytes and is not stored)
                uint4 v[P::PPT], w[P::PPT];
                // KF_CHECK site 301: a piece's 16 bytes inside the raw slot
#pragma unroll
                for (int j = 0; j < P::PPT; ++j)
                    v[j] = KF_CHK(roff[j] + (uint32_t)(i * CPS) * 128u + 16u <= a.rslot, a.err, 301)
                               ? *reinterpret_cast<const uint4 *>(slot + roff[j] + (i * CPS) * 128)
                               : make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
                for (int cu = 0; cu < CPS; ++cu) {
                    if (cu + 1 < CPS) {
#pragma unroll
                        for (int j = 0; j < P::PPT; ++j)
                            w[j] = KF_CHK(roff[j] + (uint32_t)(i * CPS + cu + 1) * 128u + 16u <= a.rslot, a.err, 301)
                                       ? *reinterpret_cast<const uint4 *>(slot + roff[j] + (i * CPS + cu + 1) * 128)
                                       : make_uint4(0u, 0u, 0u, 0u);
                    }
                    unsigned char *st = ops + (size_t)o * P::STAGE + (size_t)cu * P::CHB;
#pragma unroll
                    for (int j = 0; j < P::PPT; ++j) {
                        // KF_CHECK site 302: the hi and lo pieces inside the chunk's images
                        if (!has[j] || !KF_CHK(hoff[j] + 16u <= (uint32_t)P::CHB && loff[j] + 16u <= (uint32_t)P::CHB,
                                               a.err, 302))
                            continue;
                        const uint32_t x[4] = {v[j].x, v[j].y, v[j].z, v[j].w};
                        uint32_t h[4], l[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            h[e] = x[e] & 0xFFFFE000u;
                            l[e] = __float_as_uint(__uint_as_float(x[e]) - __uint_as_float(h[e]));
                        }
                        *reinterpret_cast<uint4 *>(st + hoff[j]) = make_uint4(h[0], h[1], h[2], h[3]);
                        *reinterpret_cast<uint4 *>(st + loff[j]) = make_uint4(l[0], l[1], l[2], l[3]);
                    }
#pragma unroll
                    for (int j = 0; j < P::PPT; ++j) v[j] = w[j];
                }
                asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                __syncwarp();
                if (lane == 0) gt_arrive(ofull + o);
            }
            if (!ok) break;
            // the group's raw slot is free for the producer
            __syncwarp();
            if (lane == 0) gt_arrive(rempty + r);
        }
        if (!ok) s_abort = 1;
    } else if (warp == 5) {
        // ---- MMA issuer (one lane)
        if (lane == 0) {
            const uint32_t n1 = (uint32_t)(2 * a.nbr);
            const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((n1 >> 3) << 17) | ((128u >> 4) << 24);
            const uint32_t boff = SPLIT ? (uint32_t)P::IMG : (uint32_t)a.b_off * 128u;   // [B_hi; B_lo]
            int64_t issued = 0;
            for (int64_t u = 0; u < myu; ++u) {
                const int o = (int)(u % SO), sl = (int)(u & 1);
                if (!gt_wait(ofull + o, (uint32_t)(u / SO), &s_abort)) { s_abort = 1; break; }
                if (u >= 2 && !gt_wait(acce + sl, (uint32_t)(u / 2 - 1), &s_abort)) { s_abort = 1; break; }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
                for (int cu = 0; cu < CPS; ++cu) {
                    const uint32_t hi = obase + (uint32_t)o * P::STAGE + (uint32_t)cu * P::CHB, lo = hi + P::IMG;
                    // unit u's slots: sl * ASL .. + ASL - 1, CPA chunks accumulated in each
                    const uint32_t d = tmem + (uint32_t)(sl * P::ASL + cu / P::CPA) * SLOT;
#pragma unroll
                    for (int ks = 0; ks < GT_KC / 8; ++ks) {
                        const uint32_t kb = (uint32_t)ks * 32;   // 8 TF32 values of every image row
                        const uint32_t acc = (cu % P::CPA == 0 && ks == 0) ? 0u : 1u;
                        const uint64_t db = gm_desc_sw128(hi + boff + kb);
                        gt_mma(d, gm_desc_sw128(hi + kb), db, idesc, acc);
                        if (!ONE) gt_mma(d + 128, gm_desc_sw128(lo + kb), db, idesc, acc);
                    }
                }
                gt_commit(oempty + o);
                gt_commit(accf + sl);
                ++issued;
            }
            if (issued > 0 && s_abort) {
                gt_commit(fin);
                volatile int never = 0;
                (void)gt_wait(fin, 0, &never);
            }
        }
    } else {
        // ---- epilogue (warps 6-13), as in k_gram_tc
        const int q = warp & 3, m = q * 32 + lane, h = (warp - 6) >> 2;
        const int h0 = min(a.nbr, (a.nbr / 2 + 15) / 16 * 16);
        const int cb = h == 0 ? 0 : h0, ce = h == 0 ? h0 : a.nbr;
        const uint32_t lb = (uint32_t)(q * 32) << 16;
        const bool has_hi = !ONE || q < 2, has_lo = !ONE || q >= 2;
        float acc_hi[GT_NBH], acc_lo[GT_NBH];
#pragma unroll
        for (int c = 0; c < GT_NBH; ++c) acc_hi[c] = acc_lo[c] = 0.f;
        bool ok = true;
        for (int64_t u = 0; u < myu; ++u) {
            const int sl = (int)(u & 1);
            ok = gt_wait(accf + sl, (uint32_t)(u / 2), &s_abort);
            ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld is warp-collective
            if (!ok) { s_abort = 1; break; }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
            for (int as = 0; as < P::ASL; ++as) {
            const uint32_t d = tmem + lb + (uint32_t)(sl * P::ASL + as) * SLOT;
#pragma unroll
            for (int c0 = 0; c0 < GT_NBH; c0 += 16) {
                if (cb + c0 >= ce) break;
                const uint32_t col = (uint32_t)(cb + c0);
                uint32_t r1[16];
                if (has_hi) {
                    gt_ld16(d + col, r1);
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
                    for (int w = 0; w < 16; ++w) acc_hi[c0 + w] += __uint_as_float(r1[w]);
                    gt_ld16(d + (uint32_t)a.nbr + col, r1);
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
                    for (int w = 0; w < 16; ++w) acc_hi[c0 + w] += __uint_as_float(r1[w]);
                }
                if (has_lo) {
                    gt_ld16(d + (ONE ? 0u : 128u) + col, r1);
                    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
                    for (int w = 0; w < 16; ++w) acc_lo[c0 + w] += __uint_as_float(r1[w]);
                }
            }
            }
            // the warp's loads have completed (tcgen05.wait::ld): one arrival per warp
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) gt_arrive(acce + sl);
        }
        if (ok) {
            const size_t E = (size_t)a.nr * a.nc;
            float *out = a.part + (size_t)blockIdx.x * 2 * E;
            const int ih = has_hi ? a.rinv_hi[m] : 255;
            const int il = has_lo ? a.rinv_lo[ONE ? m - 64 : m] : 255;
#pragma unroll
            for (int c = 0; c < GT_NBH; ++c) {
                if (cb + c >= ce) break;
                const int j = a.cinv[cb + c];
                if (j == 255) continue;
                if (ih != 255) out[ih + (size_t)a.nr * j] = acc_hi[c];
                if (il != 255) out[E + il + (size_t)a.nr * j] = acc_lo[c];
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
    if (warp == 5) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(512));
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

std::mutex g_gt_mu;
using GtKernel = void (*)(const GtArgs);
// plans 0-2: the cp.async kernel (RB 64, RB 128, split); 3-5: the TMA kernel (same order, its raw
// ring sized per launch from what the device leaves after the operand stages)
const GtKernel g_gt_kern[6] = {k_gram_tc<64, 12, 2>,         k_gram_tc<128, 6, 2>,
                               k_gram_tc<128, 6, 2, true>,   k_gram_tma<64, 2, false, 4>,
                               k_gram_tma<128, 2, false, 1>, k_gram_tma<128, 2, true, 1>};
const size_t g_gt_smem[6] = {GtPlan<64, 12, 2>::SMEM,    GtPlan<128, 6, 2>::SMEM,       GtPlan<128, 6, 2>::SMEM,
                             gm_smem<64, 2, 4>(0, 0),    gm_smem<128, 2, 1>(0, 0),      gm_smem<128, 2, 1>(0, 0)};

// per device: SM count and, per plan, whether the kernel fits and the dynamic shared memory its
// attribute allows
struct GtDevice {
    bool ready = false;
    int sms = 0;
    bool fits[6] = {false, false, false, false, false, false};
    size_t dyn[6] = {0, 0, 0, 0, 0, 0};
};

// the CUDA driver's tensor-map encoder (cuTensorMapEncodeTiled), looked up once through the runtime;
// null when the CUDA driver does not provide it (the cp.async kernel is used then)
using TmEncode = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
TmEncode tm_encoder() {
    static std::once_flag once;
    static TmEncode fn = nullptr;
    std::call_once(once, [] {
        const char *e = std::getenv("KF_GRAM_TMA");
        if (e && e[0] == '0') return;   // the cp.async kernel only
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<TmEncode>(p);
        else
            (void)cudaGetLastError();
    });
    return fn;
}

// tensor maps of the column blocks the solvers pass (their workspaces are reused, so a small
// direct-mapped cache saves most encodes): N rows x k columns, leading dimension ld, boxes of
// 128 rows x k columns (unswizzled: per column 512 contiguous bytes), rows past N read as zero
struct TmEntry {
    const float *p = nullptr;
    int64_t ld = 0, N = 0;
    int k = 0;
    CUtensorMap m;
};
TmEntry g_tm_cache[64];

bool tm_for(const float *p, int64_t ld, int64_t N, int k, CUtensorMap *out) {
    const TmEncode enc = tm_encoder();
    if (!enc || N > ((int64_t)1 << 31) - GM_GR || k > 256) return false;
    const size_t h = (((uintptr_t)p >> 8) ^ (size_t)ld * 31 ^ (size_t)N * 7 ^ (size_t)k) & 63;
    std::lock_guard<std::mutex> lk(g_gt_mu);
    TmEntry &c = g_tm_cache[h];
    if (c.p != p || c.ld != ld || c.N != N || c.k != k) {
        const cuuint64_t dims[2] = {(cuuint64_t)N, (cuuint64_t)k};
        const cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(float)};
        const cuuint32_t box[2] = {(cuuint32_t)GM_GR, (cuuint32_t)k};
        const cuuint32_t es[2] = {1, 1};
        if (enc(&c.m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(p), dims, strides, box, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
            c.p = nullptr;
            return false;
        }
        c.p = p;
        c.ld = ld;
        c.N = N;
        c.k = k;
    }
    *out = c.m;
    return true;
}
GtDevice g_gt_dev[32];

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
        for (int p = 0; p < 6; ++p) {
            cudaFuncAttributes fa;
            KF_CUDA(cudaFuncGetAttributes(&fa, g_gt_kern[p]));
            d.fits[p] = g_gt_smem[p] + fa.sharedSizeBytes <= (size_t)optin;
            // the TMA plans take all the device allows (their raw ring grows into it)
            d.dyn[p] = p >= 3 ? (size_t)optin - fa.sharedSizeBytes : g_gt_smem[p];
            if (d.fits[p])
                KF_CUDA(cudaFuncSetAttribute(g_gt_kern[p], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)d.dyn[p]));
        }
        d.ready = true;
    }
    return d;
}

}  // namespace

bool tensor_map_cols(const float *p, int64_t ld, int64_t N, int k, void *map) {
    return tm_for(p, ld, N, k, reinterpret_cast<CUtensorMap *>(map));
}

size_t gram_tc_partials_size(int nr, int nc) { return (size_t)2 * 256 * nr * nc * sizeof(float); }

bool gram_tc(const GramTcSrc *src, int nsrc, int r0, int r1, int c0, int c1, int64_t N, double *G, void *partials,
             size_t partial_bytes, cudaStream_t s) {
    if (nsrc < 1 || nsrc > GT_MAX_SRC || r0 < 0 || r1 > nsrc || r0 >= r1 || c0 < 0 || c1 > nsrc || c0 >= c1) return false;
    if (N < GT_KC) return false;
    for (int q = 0; q < nsrc; ++q) {
        const GramTcSrc &c = src[q];
        if (c.k < 1 || !c.p || c.ld % 4 != 0 || (uintptr_t)c.p % 16 != 0) return false;
    }
    GtArgs a;
    std::memset(&a, 0, sizeof a);
    // the pool: the row-only sources first (8-aligned from row 0), the column sources last, ending
    // at row RB; `order` lists the pool's sources by their index in src
    std::vector<int> order;
    int aspan = 0, cspan = 0;
    for (int q = r0; q < r1; ++q)
        if (q < c0 || q >= c1) {
            a.off[order.size()] = aspan;
            aspan = (aspan + src[q].k + 7) / 8 * 8;
            order.push_back(q);
        }
    const int na = (int)order.size();
    int coff[GT_MAX_SRC];
    for (int q = c0; q < c1; ++q) {
        coff[q - c0] = cspan;
        cspan = (cspan + src[q].k + 7) / 8 * 8;
        order.push_back(q);
    }
    // B columns in whole 8-row groups (the MMA's N = 2 nbr stays a multiple of 16): [X Z]'Z at
    // block 18 (24 + 40 pool rows) then fits the one-MMA layout
    const int nbr = cspan;
    if (nbr > GT_NBR_MAX) return false;
    const int RB = aspan + nbr <= 64 ? 64 : aspan + nbr <= 128 ? 128 : 0;
    if (!RB) return false;
    // disjoint row and column sources of up to 64 rows each: the one-MMA split layout
    const bool split = RB == 128 && (r1 <= c0 || c1 <= r0) && aspan <= 64;
    a.nbr = nbr;
    a.b_off = RB - nbr;
    a.nsrc = (int)order.size();
    for (int i = 0; i < a.nsrc; ++i) {
        const int q = order[i];
        a.p[i] = src[q].p;
        a.ld[i] = src[q].ld;
        a.k[i] = src[q].k;
        if (i >= na) a.off[i] = a.b_off + coff[i - na];
    }
    a.N = N;
    a.nchunks = (N + GT_KC - 1) / GT_KC;
    std::memset(a.rinv_hi, 255, sizeof a.rinv_hi);
    std::memset(a.rinv_lo, 255, sizeof a.rinv_lo);
    std::memset(a.cinv, 255, sizeof a.cinv);
    // output rows: the sources r0..r1-1 in order, wherever they sit in the pool
    int nr = 0, nc = 0;
    for (int q = r0; q < r1; ++q) {
        const int i = (int)(std::find(order.begin(), order.end(), q) - order.begin());
        for (int c = 0; c < src[q].k; ++c) {
            const int m = a.off[i] + c;
            const int ml = split ? m : m >= a.b_off ? m - a.b_off : m + nbr;
            a.rinv_hi[m] = (uint8_t)nr;
            a.rinv_lo[ml] = (uint8_t)nr;
            ++nr;
        }
    }
    for (int q = c0; q < c1; ++q)
        for (int c = 0; c < src[q].k; ++c) a.cinv[coff[q - c0] + c] = (uint8_t)nc++;
    if (nr > 254 || nc > 254) return false;
    a.nr = nr;
    a.nc = nc;
    const GtDevice &dv = gt_device();
    int plan = RB == 64 ? 0 : split ? 2 : 1;
    size_t smem = g_gt_smem[plan];
    if (dv.fits[plan + 3]) {
        // the TMA kernel: one tensor map per source; a raw slot holds every source's 128 x k box
        bool tma = true;
        a.rslot = 0;
        for (int i = 0; i < a.nsrc && tma; ++i) {
            tma = tm_for(a.p[i], a.ld[i], N, a.k[i], &a.tm[i]);
            a.roff[i] = a.rslot;
            a.rslot += (uint32_t)a.k[i] * GM_GR * 4u;
        }
        a.tx_bytes = a.rslot;
        const size_t fixed = g_gt_smem[plan + 3];
        const int R = tma ? (int)std::min<size_t>(GM_MAX_RAW, (dv.dyn[plan + 3] - fixed) / a.rslot) : 0;
        if (R >= 2) {
            a.nraw = R;
            plan += 3;
            smem = fixed + (size_t)R * a.rslot;
            a.nchunks = (N + GM_GR - 1) / GM_GR;   // groups of four chunks
        }
    }
    if (!dv.fits[plan]) return false;
    const int grid = (int)std::min<int64_t>(dv.sms, a.nchunks);
    if ((size_t)2 * grid * nr * nc * sizeof(float) > partial_bytes) return false;
    a.part = (float *)partials;
    a.err = tc_error_word();

    g_gt_kern[plan]<<<grid, plan >= 3 ? GM_THREADS : GT_THREADS, smem, s>>>(a);
    KF_LAUNCH_CHECK();
    const int n = nr * nc;
    k_reduce_partials_f32<<<(n + 7) / 8, 256, 0, s>>>((const float *)partials, 2 * grid, n, G);
    KF_LAUNCH_CHECK();
    return true;
}

}  // namespace kf

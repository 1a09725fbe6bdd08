// Block updates Y = alpha [X0 X1] C + beta Y on the tensor cores (tcgen05), FP32 blocks with
// FP32-accurate products: X and C split into TF32 hi / lo parts, hi*hi + hi*lo + lo*hi per K step,
// in two MMAs (A_hi x [C_hi'; C_lo'], A_lo x C_hi').
//
// The tall-skinny product of LOBPCG's orthogonalisation and Rayleigh-Ritz updates (the reference's
// gemms inside LOBPCGEigensolver, called at src/lobpcg.jl:268, and src/chebyshev.jl:60,79,126): N
// rows, kx <= 64 inputs, ky <= 80 outputs.  GEMM view: D[128 rows, Np] += A[128 rows, K] B[K, Np]
// per 128-row tile, A = the tile of [X0 X1] (K-major after the gather), B = C' (K-major as C is
// stored), D in TMEM.
//
// One persistent CTA per SM, warp-specialised:
//   warps 0-7   producers: bring a tile of X into shared memory, split it into TF32 hi / lo, store
//               the K-major images (4 columns per 16-byte core-matrix row) into stage t % 2, arrive
//               on full[s].  Two ways in: a staging ring of NSTG column-major tiles filled by 16-byte
//               cp.async copies (4 consecutive rows of one column) issued NSTG - 1 tiles ahead, so the
//               loads of later tiles overlap this one's split; or, where the ring does not fit or X
//               is not 16-byte aligned, a register gather (NSTG = 0);
//   warp 8      issuer (one lane): waits full[s] and a free accumulator slot, issues the MMA
//               chain, commits to empty[s] (stage reusable) and accf[a] (accumulator ready);
//   warps 9-16  epilogue: wait accf[a], tcgen05.ld their 32 TMEM lanes (= tile rows), two warps per
//               lane quarter taking alternate 16-column blocks, write Y (consecutive lanes =
//               consecutive rows: coalesced), arrive on acce[a].  Output
//               columns [0, ky0) go to Y0 and the rest to Y1, so that X_new and P_new of a
//               Rayleigh-Ritz step, which both read [X_a Q], take one pass.
// Every wait is an mbarrier wait with a cycle budget; when one runs out the CTA records
// KF_ETIMEOUT in the host-mapped error word, every role leaves its loop at its next check, the
// issuer waits (bounded) for its MMAs in flight and TMEM is freed.  The only named barrier inside
// a loop is the producers' own, a reduction that also carries the abort decision, so that all 256
// producer threads leave at the same iteration and none is stranded.
#include <cuda.h>   // CUtensorMap (the maps themselves come from tensor_map_cols)

#include <cstring>
#include <mutex>

#include "kf_internal.h"

namespace kf {

namespace {

constexpr int UG_PROD = 256;                  // producer threads (warps 0-7)
constexpr int UG_EPI = 256;                   // epilogue threads (warps 9-16)
constexpr int UG_THREADS = UG_PROD + 32 + UG_EPI;
constexpr int UG_TM = 128;                    // rows per tile (MMA M)
constexpr int UG_SS = UG_TM + 4;              // staging column stride in floats (16-byte multiple, conflict-free)
constexpr long long UG_WAIT_CYCLES = 4000000000LL;

__device__ __forceinline__ uint32_t su32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t ug_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

__device__ __forceinline__ void ug_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void ug_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(su32(bar))
                 : "memory");
}

__device__ __forceinline__ void ug_bar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(su32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void ug_arrive(uint64_t *bar) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}\n" ::"r"(su32(bar))
        : "memory");
}

// completion number `n` (0-based) of the barrier's phases; false when the budget ran out or the
// CTA is aborting
__device__ __forceinline__ bool ug_wait(uint64_t *bar, uint32_t n, volatile int *abort) {
    const uint32_t parity = n & 1u;
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(su32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (*abort) return false;
        if (clock64() - t0 > UG_WAIT_CYCLES) return false;
    }
}

__device__ __forceinline__ void ug_split(float x, uint32_t &hi, uint32_t &lo) {
    hi = __float_as_uint(x) & 0xFFFFE000u;
    lo = __float_as_uint(x - __uint_as_float(hi));
}

// named barrier 1 over the 256 producer threads, returning the OR of their flags (uniform)
__device__ __forceinline__ bool ug_prod_sync_or(bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.b32 q, %1, 0;\n\tbar.red.or.pred p, 1, 256, q;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)v)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ void ug_cp16(void *dst, const float *src, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(su32(dst)), "l"(src), "r"(bytes) : "memory");
}

struct UgArgs {
    CUtensorMap ym[2];  // tstore: the output blocks Y0, Y1 as 128-row x k-column boxes
    int tstore;         // 1: the epilogue stages a tile's outputs in shared memory and stores them with
                        // 2-D tensor copies (beta = 0, aligned outputs); 0: per-element global stores
    float *Y, *Y1;
    const float *X0, *X1;
    const double *C;
    int *err;
    int64_t ldy, ldy1, ldx0, ldx1, N;
    int ky0, kx0, kx, ky, ldc, Kp, Np, ntiles;
    uint32_t tcols;     // TMEM columns allocated (two accumulator slots)
    float alpha, beta;
};

// NSTG: staging tiles of the cp.async ring (0: register gather)
// named barrier 2 over the 256 epilogue threads, returning the OR of their flags (uniform)
__device__ __forceinline__ bool ug_epi_sync_or(bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.b32 q, %1, 0;\n\tbar.red.or.pred p, 2, 256, q;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)v)
        : "memory");
    return r != 0;
}

template <int NSTG>
__global__ void __launch_bounds__(UG_THREADS, 1) k_update_tc(const __grid_constant__ UgArgs a) {
    extern __shared__ __align__(16) unsigned char ug_smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int Kp = a.Kp, Np = a.Np;
    const uint32_t sbo = (uint32_t)(Kp / 4) * 128;          // 8-row groups (rows of A, columns of C)
    const size_t aimg = (size_t)UG_TM * Kp * 4;             // one A image (hi or lo)
    const size_t bimg = (size_t)Np * Kp * 4;                // one B image
    unsigned char *Bsm = ug_smem;                           // B hi | B lo
    unsigned char *Asm = Bsm + 2 * bimg;                    // stage s: A hi | A lo at 2 s aimg
    float *Stg = reinterpret_cast<float *>(Asm + 4 * aimg);   // NSTG staging tiles of Kp x UG_SS floats
    // tstore: the output tile [ky][128] (column-major, 128-byte aligned for the tensor copies)
    unsigned char *Osm_raw = Asm + 4 * aimg + (size_t)NSTG * Kp * UG_SS * 4;
    float *Osm = reinterpret_cast<float *>(Osm_raw + ((128u - (su32(Osm_raw) & 127u)) & 127u));
    const size_t obytes = a.tstore ? (size_t)a.ky * UG_TM * 4 + 128 : 0;
    uint64_t *bars = reinterpret_cast<uint64_t *>(Osm_raw + obytes);
    uint64_t *full = bars, *empty = bars + 2, *accf = bars + 4, *acce = bars + 6, *fin = bars + 8;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 9);
    __shared__ volatile int s_abort;

    if (tid == 0) {
        for (int q = 0; q < 2; ++q) {
            ug_bar_init(full + q, UG_PROD);
            ug_bar_init(empty + q, 1);
            ug_bar_init(accf + q, 1);
            ug_bar_init(acce + q, UG_EPI);
        }
        ug_bar_init(fin, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        s_abort = 0;
    }
    if (warp == 8) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(su32(tslot)),
                     "r"(a.tcols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    // B = C' as TF32 hi / lo, K-major: entry (j, i) = C[i + ldc j], zero padding
    for (int e = tid; e < Np * (Kp / 4); e += UG_THREADS) {
        const int j = e / (Kp / 4), ig = e % (Kp / 4);
        uint32_t h[4], l[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int i = ig * 4 + t;
            const float v = (j < a.ky && i < a.kx) ? (float)a.C[i + (size_t)a.ldc * j] : 0.f;
            ug_split(v, h[t], l[t]);
        }
        const size_t at = (size_t)(j >> 3) * sbo + (size_t)ig * 128 + (j & 7) * 16;
        *reinterpret_cast<uint4 *>(Bsm + at) = make_uint4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<uint4 *>(Bsm + bimg + at) = make_uint4(l[0], l[1], l[2], l[3]);
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tslot;
    const uint32_t slot_cols = a.tcols / 2;
    int my = 0;   // tiles handled by this CTA
    for (int t = blockIdx.x; t < a.ntiles; t += gridDim.x) ++my;

    if (warp < 8 && NSTG > 0) {
        // ---- producers, cp.async staging ring.  Tile k goes into staging tile k % NSTG; the copies
        // of tile k + NSTG - 1 are issued after the barrier of iteration k, which every producer
        // reaches only after its split of tile k - 1 (the previous user of that staging tile).
        auto issue = [&](int k) {
            if (k < my) {
                const int64_t row0 = (int64_t)(blockIdx.x + (int64_t)k * gridDim.x) * UG_TM;
                float *dst = Stg + (size_t)(k % (NSTG > 0 ? NSTG : 1)) * Kp * UG_SS;
                for (int e = tid; e < a.kx * (UG_TM / 4); e += UG_PROD) {
                    const int c = e / (UG_TM / 4), q = e % (UG_TM / 4);
                    const int64_t r = row0 + 4 * q;
                    const int64_t left = a.N - r;
                    const int bytes = left >= 4 ? 16 : left > 0 ? (int)left * 4 : 0;
                    const float *col = c < a.kx0 ? a.X0 + (int64_t)c * a.ldx0 : a.X1 + (int64_t)(c - a.kx0) * a.ldx1;
                    ug_cp16(dst + c * UG_SS + 4 * q, col + (bytes > 0 ? r : 0), bytes);
                }
            }
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        };
        for (int j = 0; j < NSTG - 1; ++j) issue(j);
        const int items = UG_TM * (Kp / 4);
        for (int k = 0; k < my; ++k) {
            const int s = k & 1;
            asm volatile("cp.async.wait_group %0;\n" ::"n"(NSTG > 1 ? NSTG - 2 : 0) : "memory");
            const bool bad = k >= 2 && !ug_wait(empty + s, (uint32_t)(k / 2 - 1), &s_abort);
            if (ug_prod_sync_or(bad || s_abort)) { s_abort = 1; break; }
            issue(k + NSTG - 1);
            const float *src = Stg + (size_t)(k % (NSTG > 0 ? NSTG : 1)) * Kp * UG_SS;
            unsigned char *Ah = Asm + (size_t)s * 2 * aimg, *Al = Ah + aimg;
            // item e = (row e % 128, columns 4 (e / 128) .. + 3): conflict-free staging reads
            // (consecutive rows) and 128-byte core-matrix rows per quarter-warp on the stores
            for (int e = tid; e < items; e += UG_PROD) {
                const int r = e % UG_TM, ig = e / UG_TM;
                uint32_t h[4], l[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int i = ig * 4 + q;
                    ug_split(i < a.kx ? src[i * UG_SS + r] : 0.f, h[q], l[q]);
                }
                const size_t at = (size_t)(r >> 3) * sbo + (size_t)ig * 128 + (r & 7) * 16;
                *reinterpret_cast<uint4 *>(Ah + at) = make_uint4(h[0], h[1], h[2], h[3]);
                *reinterpret_cast<uint4 *>(Al + at) = make_uint4(l[0], l[1], l[2], l[3]);
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            ug_arrive(full + s);
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");
    } else if (warp < 8) {
        // ---- producers, register gather
        for (int k = 0; k < my; ++k) {
            const int s = k & 1;
            if (k >= 2 && !ug_wait(empty + s, (uint32_t)(k / 2 - 1), &s_abort)) { s_abort = 1; break; }
            const int64_t row0 = (int64_t)(blockIdx.x + (int64_t)k * gridDim.x) * UG_TM;
            unsigned char *Ah = Asm + (size_t)s * 2 * aimg, *Al = Ah + aimg;
            // all of this thread's loads first (up to 8 items x 4 columns in flight), then the
            // splits and stores: item e = (row e % 128, columns 4 (e / 128) .. + 3)
            const int items = UG_TM * (Kp / 4);
            constexpr int MAXIT = (UG_TM * 64 / 4) / UG_PROD;   // Kp <= 64
            float v[MAXIT][4];
#pragma unroll
            for (int it = 0; it < MAXIT; ++it) {
                const int e = tid + it * UG_PROD;
                const int r = e % UG_TM, ig = e / UG_TM;
                const int64_t row = row0 + r;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int i = ig * 4 + q;
                    v[it][q] = 0.f;
                    if (e < items && row < a.N && i < a.kx)
                        v[it][q] = i < a.kx0 ? __ldg(a.X0 + row + (int64_t)i * a.ldx0)
                                             : __ldg(a.X1 + row + (int64_t)(i - a.kx0) * a.ldx1);
                }
            }
#pragma unroll
            for (int it = 0; it < MAXIT; ++it) {
                const int e = tid + it * UG_PROD;
                if (e >= items) break;
                const int r = e % UG_TM, ig = e / UG_TM;
                uint32_t h[4], l[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) ug_split(v[it][q], h[q], l[q]);
                const size_t at = (size_t)(r >> 3) * sbo + (size_t)ig * 128 + (r & 7) * 16;
                *reinterpret_cast<uint4 *>(Ah + at) = make_uint4(h[0], h[1], h[2], h[3]);
                *reinterpret_cast<uint4 *>(Al + at) = make_uint4(l[0], l[1], l[2], l[3]);
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            ug_arrive(full + s);
        }
    } else if (warp == 8) {
        // ---- MMA issuer (one lane)
        if (lane == 0) {
            // the lo image of C' follows its hi image row for row, so [C_hi'; C_lo'] is one B operand of
            // 2 Np rows: A_hi x [C_hi'; C_lo'] gives hi*hi | hi*lo, A_lo x C_hi' gives lo*hi -- two MMAs
            // per K step (an MMA costs about the same whatever its N)
            const uint32_t id2 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(2 * Np >> 3) << 17) |
                                 ((uint32_t)(UG_TM >> 4) << 24);
            const uint32_t id1 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(Np >> 3) << 17) |
                                 ((uint32_t)(UG_TM >> 4) << 24);
            const uint32_t b0 = su32(Bsm);
            int issued = 0;
            for (int k = 0; k < my; ++k) {
                const int s = k & 1, sl = k & 1;
                if (!ug_wait(full + s, (uint32_t)(k / 2), &s_abort)) { s_abort = 1; break; }
                if (k >= 2 && !ug_wait(acce + sl, (uint32_t)(k / 2 - 1), &s_abort)) { s_abort = 1; break; }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t ah = su32(Asm + (size_t)s * 2 * aimg), al = ah + (uint32_t)aimg;
                const uint32_t d = tmem + (uint32_t)sl * slot_cols;
                for (int ks = 0; ks < Kp / 8; ++ks) {
                    const uint32_t o = (uint32_t)ks * 256;
                    const uint64_t dah = ug_desc(ah + o, 128, sbo), dal = ug_desc(al + o, 128, sbo);
                    const uint64_t dbh = ug_desc(b0 + o, 128, sbo);
                    ug_mma(d, dah, dbh, id2, ks > 0 ? 1u : 0u);                           // columns 0 .. 2 Np
                    ug_mma(d + (uint32_t)(2 * Np), dal, dbh, id1, ks > 0 ? 1u : 0u);      // columns 2 Np .. 3 Np
                }
                ug_commit(empty + s);
                ug_commit(accf + sl);
                ++issued;
            }
            // all MMAs retired before TMEM is freed (bounded)
            if (issued > 0) {
                ug_commit(fin);
                volatile int never = 0;
                (void)ug_wait(fin, 0, &never);
            }
        }
    } else {
        // ---- epilogue: warp w (9-16) reads TMEM lanes 32 (w % 4) .. + 31 and the 16-column blocks
        // of parity (w - 9) / 4; the three partial products of a block are loaded before one wait
        const int q = warp & 3, h = (warp - 9) >> 2;
        auto drain = [&](int k, int sl, auto &&put) {
            const uint32_t base = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)sl * slot_cols;
            for (int j0 = 16 * h; j0 < a.ky; j0 += 32) {
                // hi*hi (column j), hi*lo (Np + j), lo*hi (2 Np + j)
                uint32_t r[3][16];
#pragma unroll
                for (int part = 0; part < 3; ++part)
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
                        "%12, %13, %14, %15}, [%16];\n"
                        : "=r"(r[part][0]), "=r"(r[part][1]), "=r"(r[part][2]), "=r"(r[part][3]), "=r"(r[part][4]),
                          "=r"(r[part][5]), "=r"(r[part][6]), "=r"(r[part][7]), "=r"(r[part][8]), "=r"(r[part][9]),
                          "=r"(r[part][10]), "=r"(r[part][11]), "=r"(r[part][12]), "=r"(r[part][13]),
                          "=r"(r[part][14]), "=r"(r[part][15])
                        : "r"(base + (uint32_t)(part * Np + j0)));
                asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
                for (int t = 0; t < 16; ++t) {
                    const int j = j0 + t;
                    if (j < a.ky)
                        put(j, a.alpha * ((__uint_as_float(r[0][t]) + __uint_as_float(r[1][t])) +
                                          __uint_as_float(r[2][t])));
                }
            }
        };
        if (a.tstore) {
            // the tile's outputs go to shared memory ([j][row], conflict-free: consecutive lanes write
            // consecutive rows), the accumulator slot is released at once, and one thread stores the
            // tile with 2-D tensor copies (128 rows x ky0, x ky1 columns).  Before a tile writes the
            // buffer, the previous tile's copies must have read it.  A last tile that ends past N
            // is stored element by element: the copies' clipping at the tensor's end was seen to
            // write the row just past N (N = 100,003, a 16-byte chunk across the end).
            const int m = q * 32 + lane;
            const bool leader = warp == 9 && lane == 0;
            bool ok = true;
            for (int k = 0; k < my; ++k) {
                const int sl = k & 1;
                const bool bad = !ug_wait(accf + sl, (uint32_t)(k / 2), &s_abort);
                if (leader && k > 0) asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
                if (ug_epi_sync_or(bad || s_abort)) { ok = false; break; }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const int64_t row0 = (int64_t)(blockIdx.x + (int64_t)k * gridDim.x) * UG_TM;
                const bool whole = row0 + UG_TM <= a.N;   // the same for every thread of the tile
                if (whole) {
                    drain(k, sl, [&](int j, float v) { Osm[j * UG_TM + m] = v; });
                } else {
                    const int64_t row = row0 + m;
                    drain(k, sl, [&](int j, float v) {
                        if (row < a.N) {
                            float *yp = j < a.ky0 ? a.Y + row + (int64_t)j * a.ldy
                                                  : a.Y1 + row + (int64_t)(j - a.ky0) * a.ldy1;
                            *yp = v;
                        }
                    });
                }
                asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
                ug_arrive(acce + sl);
                asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                if (ug_epi_sync_or(false)) { ok = false; break; }
                if (leader && whole) {
                    const int x = (int)row0;
                    asm volatile(
                        "cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];\n" ::"l"(
                            reinterpret_cast<uint64_t>(&a.ym[0])),
                        "r"(x), "r"(0), "r"(su32(Osm))
                        : "memory");
                    if (a.ky0 < a.ky)
                        asm volatile(
                            "cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];\n" ::"l"(
                                reinterpret_cast<uint64_t>(&a.ym[1])),
                            "r"(x), "r"(0), "r"(su32(Osm + (size_t)a.ky0 * UG_TM))
                            : "memory");
                    asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
                }
            }
            if (!ok) s_abort = 1;
            // the copies must have completed before the CTA leaves
            if (leader) asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
        } else {
            for (int k = 0; k < my; ++k) {
                const int sl = k & 1;
                if (!ug_wait(accf + sl, (uint32_t)(k / 2), &s_abort)) { s_abort = 1; break; }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const int64_t row = (int64_t)(blockIdx.x + (int64_t)k * gridDim.x) * UG_TM + q * 32 + lane;
                drain(k, sl, [&](int j, float v) {
                    if (row < a.N) {
                        float *yp = j < a.ky0 ? a.Y + row + (int64_t)j * a.ldy
                                              : a.Y1 + row + (int64_t)(j - a.ky0) * a.ldy1;
                        *yp = a.beta == 0.f ? v : v + a.beta * *yp;
                    }
                });
                asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
                ug_arrive(acce + sl);
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

std::mutex g_ug_mu;
int g_ug_attr_mask = 0;   // kernels (bit = NSTG) whose shared-memory limit is set

}  // namespace

// ky <= 80: two slots of 3 Np accumulator columns within the 512 TMEM columns
bool update_tc_ok(int kx, int ky) { return kx >= 1 && kx <= 64 && ky >= 1 && ky <= 80; }

bool update_tc_prefer(int kx, int ky, int64_t N, const float *X0, int64_t ldx0, const float *X1, int64_t ldx1) {
    if (N < 65536 || kx < 40 || kx > 64 || ky < 17 || ky > 80) return false;
    auto al = [](const float *p, int64_t ld) { return (uintptr_t)p % 16 == 0 && ld % 4 == 0; };
    if (!al(X0, ldx0) || (X1 && !al(X1, ldx1))) return false;
    // a two-tile staging ring within the 227 KB a CTA may hold (1 KB left for static shared memory)
    const size_t Kp = (size_t)(kx + 7) / 8 * 8, Np = (size_t)(ky + 15) / 16 * 16;
    const size_t smem = 2 * Np * Kp * 4 + 4 * (size_t)UG_TM * Kp * 4 + 16 * 8 + 2 * Kp * UG_SS * 4;
    return smem <= 227 * 1024 - 1024;
}

void update_tc2(float *Y0, int64_t ldy0, int ky0, float *Y1, int64_t ldy1, int ky1, const float *X0, int64_t ldx0,
                int kx0, const float *X1, int64_t ldx1, int kx1, const double *C, int ldc, double alpha, double beta,
                int64_t N, cudaStream_t s, int force_nstg) {
    const int kx = kx0 + kx1, ky = ky0 + ky1;
    KF_REQUIRE(update_tc_ok(kx, ky) && ky0 >= 1 && ky1 >= 0, KF_EINVAL,
               "update_tc: kx must lie in 1:64 and ky in 1:80");
    if (N <= 0) return;
    UgArgs a;
    a.Y = Y0;
    a.Y1 = ky1 > 0 ? Y1 : Y0;
    a.X0 = X0;
    a.X1 = kx1 > 0 ? X1 : X0;
    a.C = C;
    a.err = tc_error_word();
    a.ldy = ldy0;
    a.ldy1 = ky1 > 0 ? ldy1 : ldy0;
    a.ldx0 = ldx0;
    a.ldx1 = kx1 > 0 ? ldx1 : ldx0;
    a.N = N;
    a.ky0 = ky1 > 0 ? ky0 : ky;
    a.kx0 = kx0;
    a.kx = kx;
    a.ky = ky;
    a.ldc = ldc;
    a.Kp = (kx + 7) / 8 * 8;
    a.Np = (ky + 15) / 16 * 16;
    uint32_t tc = 32;
    while (tc < (uint32_t)(6 * a.Np)) tc <<= 1;   // two slots of 3 Np columns
    a.tcols = tc;
    a.alpha = (float)alpha;
    a.beta = (float)beta;
    a.ntiles = (int)((N + UG_TM - 1) / UG_TM);
    const size_t base = (size_t)2 * a.Np * a.Kp * 4 + (size_t)4 * UG_TM * a.Kp * 4 + 16 * 8;
    const size_t stg = (size_t)a.Kp * UG_SS * 4;
    int sms = 152, dev = 0, optin = 0;
    KF_CUDA(cudaGetDevice(&dev));
    KF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    KF_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    using Kern = void (*)(const UgArgs);
    static const Kern kerns[4] = {k_update_tc<0>, nullptr, k_update_tc<2>, k_update_tc<3>};
    // the deepest staging ring that fits; the ring's 16-byte copies want 16-byte aligned columns
    auto al = [](const float *p, int64_t ld) { return (uintptr_t)p % 16 == 0 && ld % 4 == 0; };
    const bool aligned = al(a.X0, a.ldx0) && al(a.X1, a.ldx1);
    int nstg = 0;
    size_t dyn_max[4] = {0, 0, 0, 0};
    for (int q : {0, 2, 3}) {
        cudaFuncAttributes fa;
        KF_CUDA(cudaFuncGetAttributes(&fa, kerns[q]));
        dyn_max[q] = (size_t)optin - fa.sharedSizeBytes;
    }
    for (int q : {3, 2})
        if (aligned && base + q * stg <= dyn_max[q]) { nstg = q; break; }
    if (force_nstg >= 0) {
        KF_REQUIRE(force_nstg == 0 || (aligned && (force_nstg == 2 || force_nstg == 3) &&
                                       base + force_nstg * stg <= dyn_max[force_nstg]),
                   KF_EINVAL, "update_tc: the requested staging ring does not fit");
        nstg = force_nstg;
    }
    // outputs by 2-D tensor copies where beta = 0, the output blocks are 16-byte aligned with a
    // staging ring and the tile buffer [ky][128] fitting (the ring one tile shallower if need be)
    a.tstore = 0;
    const size_t obuf = (size_t)ky * UG_TM * 4 + 128;
    if (beta == 0.0 && nstg > 0 && al(Y0, ldy0) && (ky1 == 0 || al(Y1, ldy1)) &&
        tensor_map_cols(Y0, ldy0, N, a.ky0, &a.ym[0]) && (ky1 == 0 || tensor_map_cols(Y1, ldy1, N, ky1, &a.ym[1]))) {
        for (int q : {3, 2}) {
            if ((force_nstg < 0 || force_nstg == q) && base + q * stg + obuf <= dyn_max[q]) {
                nstg = q;
                a.tstore = 1;
                break;
            }
        }
    }
    const size_t smem = base + nstg * stg + (a.tstore ? obuf : 0);
    KF_REQUIRE(smem <= dyn_max[nstg], KF_EINVAL, "update_tc: shared-memory stages too large");
    {
        std::lock_guard<std::mutex> lk(g_ug_mu);
        if (!(g_ug_attr_mask & (1 << nstg))) {
            KF_CUDA(cudaFuncSetAttribute(kerns[nstg], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_max[nstg]));
            g_ug_attr_mask |= 1 << nstg;
        }
    }
    const int grid = a.ntiles < sms ? a.ntiles : sms;
    kerns[nstg]<<<grid, UG_THREADS, smem, s>>>(a);
    KF_LAUNCH_CHECK();
}

void update_tc(float *Y, int64_t ldy, int ky, const float *X0, int64_t ldx0, int kx0, const float *X1, int64_t ldx1,
               int kx1, const double *C, int ldc, double alpha, double beta, int64_t N, cudaStream_t s) {
    update_tc2(Y, ldy, ky, nullptr, 0, 0, X0, ldx0, kx0, X1, ldx1, kx1, C, ldc, alpha, beta, N, s, -1);
}

}  // namespace kf

// Mode-k products on the 5th-generation tensor cores (tcgen05, sm_103a):
//   Y[l, i, r] = alpha sum_j A[i, j] X[l, j, r] + beta Y[l, i, r]
// for a block of FP32 columns, A a d x d matrix held as a BF16 image in the tensor core's
// K-major shared-memory layout, FP32 accumulation in tensor memory (TMEM).
//
// Reference: the dense factor application of src/apply.jl:37-53 and 301-340 -- the same product
// the SIMT kernel of kf_dense.cu forms; here for the separable preconditioner's axis bases
// (src/apply.jl:606-642), which only steer LOBPCG's search directions, so BF16 operands (8-bit
// mantissa, FP32 sums) are accurate enough.
//
// GEMM view: D[i, q] = sum_j A[i, j] B[j, q], with q enumerating the (column, l, r) triples of the
// block.  One CTA (persistent, 256 threads) keeps A in shared memory and walks tiles of 128 q:
//   1. the 256 threads gather the tile's X[:, j] values (coalesced along l when the axis stride
//      is > 1, along j for the leading axis), round them to BF16 and store them as the B operand
//      (K-major core matrices: 8 rows x 16 bytes, LBO = 128 B between K-neighbours);
//   2. one thread issues the tcgen05.mma chain (M = 128 per A tile, N = 128, K = 16 per
//      instruction) and commits it to an mbarrier;
//   3. the first warpgroup waits (bounded), reads its TMEM lanes with tcgen05.ld, and writes Y
//      through a shared-memory transpose so that the global stores are coalesced.
// A wait that exceeds its cycle budget records KF_ETIMEOUT in host-mapped memory and the CTA
// leaves its loop; TMEM is always released.
#include <cuda_bf16.h>

#include <cstring>
#include <mutex>

#include "kf_internal.h"

namespace kf {

namespace {

constexpr int TC_THREADS = 256;
constexpr int TC_NT = 128;                        // q per tile (MMA N)
constexpr int TC_EP_STRIDE = 33;                  // epilogue transpose row stride (floats)
constexpr long long TC_WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: no swizzle, K-major, version 1 (tcgen05)
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// instruction descriptor: D FP32, A and B both K-major, M x N; A/B type 1 = BF16 (kind::f16),
// 2 = TF32 (kind::tf32)
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N, uint32_t ab) {
    return (1u << 4) | (ab << 7) | (ab << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

template <bool TF32>
__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    if constexpr (TF32)
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
    else
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

// TF32 split of an FP32 value: hi keeps the TF32 bits (10 explicit mantissa bits), lo = x - hi
// (exact in FP32); hi*hi + hi*lo + lo*hi carries ~21 bits
__device__ __forceinline__ void tf32_split(float x, uint32_t &hi, uint32_t &lo) {
    hi = __float_as_uint(x) & 0xFFFFE000u;
    lo = __float_as_uint(x - __uint_as_float(hi));
}

__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// bounded wait on one mbarrier phase; false when the cycle budget ran out
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > TC_WAIT_CYCLES) return false;
    return true;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int t = 0; t < 16; ++t) v[t] = __uint_as_float(r[t]);
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);   // .x = lo (lower address)
    return *reinterpret_cast<uint32_t *>(&h);
}

struct TcArgs {
    float *Y;
    const float *X;
    const uint4 *Aimg;      // BF16 image, Mp x Kp, K-major core matrices
    int *err;               // host-mapped error word
    int64_t ldy, ldx, left, rows_per_col, Q;
    int d, Mp, Kp, ntiles;
    float alpha, beta;
};

// SPLIT = false: BF16 operands, one MMA per K step; true: TF32 hi/lo operands, three MMAs per K
// step (FP32-accurate products for the operator apply)
template <bool SPLIT>
__global__ void __launch_bounds__(TC_THREADS, 1) k_mode_tc(const TcArgs a) {
    constexpr int EB = SPLIT ? 4 : 2;        // operand bytes
    constexpr int EPC = 16 / EB;             // K elements per 16-byte core-matrix row
    constexpr int NS = SPLIT ? 2 : 1;        // operand images (hi, lo)
    extern __shared__ __align__(16) unsigned char tc_smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int Kp = a.Kp, Mp = a.Mp;
    // shared layout: A image | B tile | epilogue transpose | q bases | barrier, TMEM slot
    const size_t aimg = (size_t)Mp * Kp * EB, bimg = (size_t)TC_NT * Kp * EB;   // one image each
    unsigned char *Asm = tc_smem;
    unsigned char *Bsm = Asm + NS * aimg;
    float *Ep = reinterpret_cast<float *>(Bsm + NS * bimg);
    int64_t *xbase = reinterpret_cast<int64_t *>(Ep + 128 * TC_EP_STRIDE);
    int64_t *ybase = xbase + TC_NT;
    uint64_t *bar = reinterpret_cast<uint64_t *>(ybase + TC_NT);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 1);
    __shared__ int s_abort;

    const uint32_t ncols = (uint32_t)(Mp / 128) * TC_NT;   // 128 or 256 FP32 columns
    if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        s_abort = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tslot)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    {
        const int n16 = (int)(NS * aimg / 16);
        uint4 *dst = reinterpret_cast<uint4 *>(Asm);
        for (int e = tid; e < n16; e += TC_THREADS) dst[e] = a.Aimg[e];
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t sbo_a = (uint32_t)(Kp / EPC) * 128, sbo_b = sbo_a;   // 8-row groups along M / N
    const uint32_t idesc = tc_idesc(128, TC_NT, SPLIT ? 2u : 1u);
    const int kg_n = Kp / EPC;
    uint32_t phase = 0;

    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        const int64_t q0 = (int64_t)tile * TC_NT;
        if (tid < TC_NT) {
            const int64_t q = q0 + tid;
            if (q < a.Q) {
                const int64_t c = q / a.rows_per_col, qq = q % a.rows_per_col;
                const int64_t l = qq % a.left, r = qq / a.left;
                const int64_t off = l + a.left * ((int64_t)a.d * r);
                xbase[tid] = c * a.ldx + off;
                ybase[tid] = c * a.ldy + off;
            } else {
                xbase[tid] = -1;
                ybase[tid] = -1;
            }
        }
        __syncthreads();
        // 1. gather into the K-major B tile: item (n, kg) = EPC consecutive j of row n, rounded to
        //    BF16, or split into TF32 hi / lo
        // BG items per batch: all their loads in flight together, then the packing and stores
        const int items = TC_NT * kg_n;
        constexpr int BG = SPLIT ? 4 : 1;   // BF16: 8 loads per item already; more costs occupancy
        for (int e0 = tid; e0 < items; e0 += BG * TC_THREADS) {
            float v[BG][EPC];
#pragma unroll
            for (int g = 0; g < BG; ++g) {
                const int e = e0 + g * TC_THREADS;
                int n, kg;
                if (a.left > 1) { n = e % TC_NT; kg = e / TC_NT; }   // consecutive threads: consecutive l
                else { kg = e % kg_n; n = e / kg_n; }                // leading axis: consecutive j
                const int64_t xb = e < items ? xbase[n] : -1;
#pragma unroll
                for (int t = 0; t < EPC; ++t) {
                    const int j = kg * EPC + t;
                    v[g][t] = (xb >= 0 && j < a.d) ? __ldg(a.X + xb + a.left * (int64_t)j) : 0.f;
                }
            }
#pragma unroll
            for (int g = 0; g < BG; ++g) {
                const int e = e0 + g * TC_THREADS;
                if (e >= items) break;
                int n, kg;
                if (a.left > 1) { n = e % TC_NT; kg = e / TC_NT; }
                else { kg = e % kg_n; n = e / kg_n; }
                const size_t at = (size_t)(n >> 3) * sbo_b + (size_t)kg * 128 + (n & 7) * 16;
                if constexpr (SPLIT) {
                    uint4 h, l;
                    tf32_split(v[g][0], h.x, l.x);
                    tf32_split(v[g][1], h.y, l.y);
                    tf32_split(v[g][2], h.z, l.z);
                    tf32_split(v[g][3], h.w, l.w);
                    *reinterpret_cast<uint4 *>(Bsm + at) = h;
                    *reinterpret_cast<uint4 *>(Bsm + bimg + at) = l;
                } else {
                    uint4 pk;
                    pk.x = pack_bf16x2(v[g][0], v[g][1]);
                    pk.y = pack_bf16x2(v[g][2], v[g][3]);
                    pk.z = pack_bf16x2(v[g][4], v[g][5]);
                    pk.w = pack_bf16x2(v[g][6], v[g][7]);
                    *reinterpret_cast<uint4 *>(Bsm + at) = pk;
                }
            }
        }
        fence_proxy_async();
        tc_fence_before();
        __syncthreads();
        // 2. one thread issues the MMA chain for every 128-row tile of A, commits it to the
        //    mbarrier and waits for it (bounded)
        if (tid == 0) {
            tc_fence_after();
            const uint32_t a0 = smem_u32(Asm), b0 = smem_u32(Bsm);
            const int nks = Kp * EB / 32;   // 32 bytes of K per instruction
            for (int mt = 0; mt < Mp / 128; ++mt) {
                for (int ks = 0; ks < nks; ++ks) {
                    const uint32_t ao = (uint32_t)mt * 16 * sbo_a + (uint32_t)ks * 256, bo = (uint32_t)ks * 256;
                    const uint64_t ad = tc_desc(a0 + ao, 128, sbo_a), bd = tc_desc(b0 + bo, 128, sbo_b);
                    tc_mma<SPLIT>(tmem + (uint32_t)mt * TC_NT, ad, bd, idesc, ks > 0 ? 1u : 0u);
                    if constexpr (SPLIT) {
                        const uint64_t al = tc_desc(a0 + (uint32_t)aimg + ao, 128, sbo_a);
                        const uint64_t bl = tc_desc(b0 + (uint32_t)bimg + bo, 128, sbo_b);
                        tc_mma<true>(tmem + (uint32_t)mt * TC_NT, ad, bl, idesc, 1u);   // hi * lo
                        tc_mma<true>(tmem + (uint32_t)mt * TC_NT, al, bd, idesc, 1u);   // lo * hi
                    }
                }
            }
            tc_commit(bar);
            if (!mbar_wait_bounded(bar, phase)) {
                *(volatile int *)a.err = KF_ETIMEOUT;
                __threadfence_system();
                s_abort = 1;
            }
        }
        __syncthreads();
        if (s_abort) break;
        tc_fence_after();
        // 3. epilogue by warps 0-3 (TMEM lanes 32 w .. 32 w + 31 = rows i of each A tile)
        if (warp < 4) {
            for (int mt = 0; mt < Mp / 128; ++mt) {
                const int i = mt * 128 + warp * 32 + lane;   // output row of this thread
                for (int n0 = 0; n0 < TC_NT; n0 += 32) {
                    float v[32];
                    const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(mt * TC_NT + n0);
                    tmem_ld16(ta, v);
                    tmem_ld16(ta + 16, v + 16);
                    if (a.left == 1) {
                        // leading axis: consecutive lanes = consecutive i = consecutive addresses
                        if (i < a.d) {
#pragma unroll
                            for (int t = 0; t < 32; ++t) {
                                const int64_t yb = ybase[n0 + t];
                                if (yb >= 0) {
                                    float *yp = a.Y + yb + i;
                                    *yp = (a.beta == 0.f) ? a.alpha * v[t] : a.alpha * v[t] + a.beta * *yp;
                                }
                            }
                        }
                    } else {
                        // transpose 128 rows x 32 q through shared memory, then store along q
                        float *row = Ep + (warp * 32 + lane) * TC_EP_STRIDE;
#pragma unroll
                        for (int t = 0; t < 32; ++t) row[t] = v[t];
                        asm volatile("bar.sync 1, 128;\n" ::: "memory");
                        for (int rr = warp; rr < 128; rr += 4) {
                            const int ii = mt * 128 + rr;
                            const int64_t yb = ybase[n0 + lane];
                            if (ii < a.d && yb >= 0) {
                                float *yp = a.Y + yb + a.left * (int64_t)ii;
                                const float val = Ep[rr * TC_EP_STRIDE + lane];
                                *yp = (a.beta == 0.f) ? a.alpha * val : a.alpha * val + a.beta * *yp;
                            }
                        }
                        asm volatile("bar.sync 1, 128;\n" ::: "memory");
                    }
                }
            }
        }
        phase ^= 1u;
        tc_fence_before();
        __syncthreads();
    }
    // after a timeout: one more bounded wait for the MMAs still in flight before TMEM is freed
    if (s_abort && tid == 0) (void)mbar_wait_bounded(bar, phase);
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(ncols));
}

// ---- the BF16 mode product, pipelined -------------------------------------------------------
//
// k_mode_tc runs each tile's gather -> MMA -> epilogue one after another, so one CTA per SM waits
// on global loads, then the tensor pipe, then the stores (0.25 of HBM on the three-mode leaf's
// 256-point axis).  Here the roles overlap across tiles (the A image stays in shared memory):
//   warps 0-7   gather tile t's B operand (TN columns q x Kp values of j, rounded to BF16) into
//               stage t % 2, fence, arrive on full[s];
//   warp 8      one lane issues the tile's MMA chain into TMEM slot t % 2, commits to empty[s]
//               (stage free) and accf[slot];
//   warps 9-16  read their 32 TMEM lanes (rows i of each 128-row A tile; two warps per lane quarter
//               share the tile's columns), transpose 32 x 32 blocks through a private
//               shared-memory tile and store Y coalesced along q, arrive on acce[slot].
// Column bases come from 32-bit index arithmetic (the host checks the sizes): 64-bit divisions per
// gathered item made the first version of this kernel gather-bound.
// TN = 64 columns per tile when the operator is 256 long (its 128 KB image leaves room for two
// 32 KB stages), 128 otherwise.  Every wait is a bounded mbarrier wait (~2 s); on expiry the CTA
// records KF_ETIMEOUT, every role leaves at its next check, the issuer waits (bounded) for its MMAs
// in flight and TMEM is freed.
constexpr int MP_PROD = 256;
constexpr int MP_EPI = 256;   // epilogue threads: 8 warps, two per TMEM lane quarter
constexpr int MP_THREADS = MP_PROD + 32 + MP_EPI;
constexpr int MP_EPS = 33;   // transpose tile row stride (floats)
constexpr int MP_BG = 4;     // gather items per thread in flight (within the 96 registers of 544 threads)

// the base offset of column q = (c, l, r) of a block: c ld + l + left d r (32-bit quotients)
__device__ __forceinline__ int64_t mp_base(uint32_t q, int64_t rows_per_col, int64_t left, int d, int64_t ld) {
    const uint32_t rpc = (uint32_t)rows_per_col, lf = (uint32_t)left;
    const uint32_t c = q / rpc, qq = q - c * rpc;
    const uint32_t r = qq / lf, l = qq - r * lf;
    return (int64_t)c * ld + (int64_t)l + (int64_t)lf * d * (int64_t)r;
}

__device__ __forceinline__ bool mp_wait(uint64_t *bar, uint32_t n, volatile int *abort) {
    const uint32_t parity = n & 1u;
    const long long t0 = clock64();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort) return false;
        if (clock64() - t0 > TC_WAIT_CYCLES) return false;
    }
}

__device__ __forceinline__ void mp_arrive(uint64_t *bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}\n" ::"r"(smem_u32(bar))
                 : "memory");
}

template <int TN>
__global__ void __launch_bounds__(MP_THREADS, 1) k_mode_pipe(const TcArgs a) {
    constexpr int EPC = 8;   // BF16 values per 16-byte core-matrix row
    extern __shared__ __align__(16) unsigned char mp_smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int Kp = a.Kp, Mp = a.Mp, kg_n = Kp / EPC;
    const size_t aimg = (size_t)Mp * Kp * 2, bimg = (size_t)TN * Kp * 2;
    unsigned char *Asm = mp_smem;
    unsigned char *Bsm = Asm + aimg;                                 // two stages
    float *Ep = reinterpret_cast<float *>(Bsm + 2 * bimg);          // 8 x [32][MP_EPS]
    uint64_t *bars = reinterpret_cast<uint64_t *>(Ep + 8 * 32 * MP_EPS);
    uint64_t *full = bars, *empty = bars + 2, *accf = bars + 4, *acce = bars + 6, *fin = bars + 8;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + 9);
    __shared__ volatile int s_abort;
    const int mtiles = Mp / 128;
    const uint32_t slot_cols = (uint32_t)(mtiles * TN);   // 128
    if (tid == 0) {
        for (int q = 0; q < 2; ++q) {
            mbar_init(full + q, MP_PROD);
            mbar_init(empty + q, 1);
            mbar_init(accf + q, 1);
            mbar_init(acce + q, MP_EPI);
        }
        mbar_init(fin, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        s_abort = 0;
    }
    if (warp == 8) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tslot)),
                     "r"(2u * slot_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    {
        const int n16 = (int)(aimg / 16);
        uint4 *dst = reinterpret_cast<uint4 *>(Asm);
        for (int e = tid; e < n16; e += MP_THREADS) dst[e] = a.Aimg[e];
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t sbo = (uint32_t)kg_n * 128;   // 8-row groups of both operands (K extent Kp)
    const int ntiles = (int)((a.Q + TN - 1) / TN);
    int my = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) ++my;

    if (warp < 8) {
        // ---- gather: item (n, kg) = EPC consecutive j of column q = q0 + n
        const int items = TN * kg_n;
        for (int k = 0; k < my; ++k) {
            const int s = k & 1;
            if (k >= 2 && !mp_wait(empty + s, (uint32_t)(k / 2 - 1), &s_abort)) { s_abort = 1; break; }
            const int64_t q0 = (int64_t)(blockIdx.x + (int64_t)k * gridDim.x) * TN;
            unsigned char *B = Bsm + (size_t)s * bimg;
            // MP_BG items per thread per batch: all their loads in flight together
            for (int e0 = tid; e0 < items; e0 += MP_BG * MP_PROD) {
                float v[MP_BG][EPC];
                int nn[MP_BG], kk[MP_BG];
#pragma unroll
                for (int g = 0; g < MP_BG; ++g) {
                    const int e = e0 + g * MP_PROD;
                    int n, kg;
                    if (a.left > 1) { n = e % TN; kg = e / TN; }        // consecutive threads: consecutive l
                    else { kg = e % kg_n; n = e / kg_n; }               // leading axis: consecutive j
                    nn[g] = n;
                    kk[g] = kg;
                    int64_t xb = -1;
                    const uint32_t q = (uint32_t)q0 + (uint32_t)n;
                    if (e < items && q < (uint32_t)a.Q) xb = mp_base(q, a.rows_per_col, a.left, a.d, a.ldx);
#pragma unroll
                    for (int t = 0; t < EPC; ++t) {
                        const int j = kg * EPC + t;
                        v[g][t] = (xb >= 0 && j < a.d) ? __ldg(a.X + xb + a.left * (int64_t)j) : 0.f;
                    }
                }
#pragma unroll
                for (int g = 0; g < MP_BG; ++g) {
                    if (e0 + g * MP_PROD >= items) break;
                    uint4 pk;
                    pk.x = pack_bf16x2(v[g][0], v[g][1]);
                    pk.y = pack_bf16x2(v[g][2], v[g][3]);
                    pk.z = pack_bf16x2(v[g][4], v[g][5]);
                    pk.w = pack_bf16x2(v[g][6], v[g][7]);
                    const size_t at = (size_t)(nn[g] >> 3) * sbo + (size_t)kk[g] * 128 + (nn[g] & 7) * 16;
                    *reinterpret_cast<uint4 *>(B + at) = pk;
                }
            }
            fence_proxy_async();
            mp_arrive(full + s);
        }
    } else if (warp == 8) {
        // ---- MMA issuer (one lane)
        if (lane == 0) {
            const uint32_t idesc = tc_idesc(128, TN, 1u);
            const uint32_t a0 = smem_u32(Asm), b0 = smem_u32(Bsm);
            const int nks = Kp / 16;
            int issued = 0;
            for (int k = 0; k < my; ++k) {
                const int s = k & 1, sl = k & 1;
                if (!mp_wait(full + s, (uint32_t)(k / 2), &s_abort)) { s_abort = 1; break; }
                if (k >= 2 && !mp_wait(acce + sl, (uint32_t)(k / 2 - 1), &s_abort)) { s_abort = 1; break; }
                tc_fence_after();
                const uint32_t bs = b0 + (uint32_t)(s * bimg);
                for (int mt = 0; mt < mtiles; ++mt)
                    for (int ks = 0; ks < nks; ++ks) {
                        // a K step of 16 BF16 values spans two core matrices (LBO = 128 bytes apart)
                        const uint64_t ad = tc_desc(a0 + (uint32_t)mt * 16 * sbo + (uint32_t)ks * 256, 128, sbo);
                        const uint64_t bd = tc_desc(bs + (uint32_t)ks * 256, 128, sbo);
                        tc_mma<false>(tmem + (uint32_t)sl * slot_cols + (uint32_t)(mt * TN), ad, bd, idesc,
                                      ks > 0 ? 1u : 0u);
                    }
                tc_commit(empty + s);
                tc_commit(accf + sl);
                ++issued;
            }
            if (issued > 0 && s_abort) {
                tc_commit(fin);
                (void)mbar_wait_bounded(fin, 0);
            }
        }
    } else {
        // ---- epilogue (warps 9-16): TMEM lanes 32 (warp % 4) .. + 31 = rows i of each A tile; the
        // two warps of a lane quarter take alternate 32-column chunks of the tile
        const int qw = warp & 3, half = (warp - 9) >> 2;
        float *T = Ep + (warp - 9) * 32 * MP_EPS;
        for (int k = 0; k < my; ++k) {
            const int sl = k & 1;
            bool ok = mp_wait(accf + sl, (uint32_t)(k / 2), &s_abort);
            ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld is warp-collective
            if (!ok) { s_abort = 1; break; }
            tc_fence_after();
            const int64_t q0 = (int64_t)(blockIdx.x + (int64_t)k * gridDim.x) * TN;
            for (int mt = 0; mt < mtiles; ++mt) {
                const int i0 = mt * 128 + qw * 32;   // this warp's first row i
                for (int n0 = half * 32; n0 < TN; n0 += 64) {
                    float v[32];
                    const uint32_t ta = tmem + ((uint32_t)(qw * 32) << 16) + (uint32_t)sl * slot_cols +
                                        (uint32_t)(mt * TN + n0);
                    tmem_ld16(ta, v);
                    tmem_ld16(ta + 16, v + 16);
                    // this lane's column q = q0 + n0 + lane and its output base
                    const uint32_t q = (uint32_t)q0 + (uint32_t)(n0 + lane);
                    const int64_t yb = q < (uint32_t)a.Q ? mp_base(q, a.rows_per_col, a.left, a.d, a.ldy) : -1;
                    if (a.left == 1) {
                        // leading axis: lanes = consecutive i = consecutive addresses, per column t
                        const int i = i0 + lane;
#pragma unroll
                        for (int t = 0; t < 32; ++t) {
                            const int64_t ybt = __shfl_sync(0xffffffffu, yb, t);
                            if (ybt >= 0 && i < a.d) {
                                float *yp = a.Y + ybt + i;
                                *yp = (a.beta == 0.f) ? a.alpha * v[t] : a.alpha * v[t] + a.beta * *yp;
                            }
                        }
                    } else {
                        // transpose 32 rows x 32 columns through this warp's tile, store along q
#pragma unroll
                        for (int t = 0; t < 32; ++t) T[lane * MP_EPS + t] = v[t];
                        __syncwarp();
                        for (int rr = 0; rr < 32; ++rr) {
                            const int i = i0 + rr;
                            if (yb >= 0 && i < a.d) {
                                float *yp = a.Y + yb + a.left * (int64_t)i;
                                const float val = T[rr * MP_EPS + lane];
                                *yp = (a.beta == 0.f) ? a.alpha * val : a.alpha * val + a.beta * *yp;
                            }
                        }
                        __syncwarp();
                    }
                }
            }
            tc_fence_before();
            mp_arrive(acce + sl);
        }
    }
    if (s_abort && tid == 0) {
        *(volatile int *)a.err = KF_ETIMEOUT;
        __threadfence_system();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 8)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(2u * slot_cols));
}

static size_t mode_pipe_smem(const TcMatrix &m, int tn) {
    return (size_t)m.Mp * m.Kp * 2 + (size_t)2 * tn * m.Kp * 2 + (size_t)8 * 32 * MP_EPS * 4 + 10 * 8 + 16;
}

// host-mapped error words shared by every tensor-core and bulk-copy launch: [0] a wait that ran out
// (KF_ETIMEOUT), [1] in KF_CHECK builds the site of the first failed bounds check
std::mutex g_tc_mu;
int *g_tc_err_host = nullptr;
int *g_tc_err_dev = nullptr;
bool g_tc_attr = false;
int g_mp_attr_mask = 0;   // devices whose pipelined-kernel attributes are set

int *tc_err_word() {
    std::lock_guard<std::mutex> lk(g_tc_mu);
    if (!g_tc_err_host) {
        KF_CUDA(cudaHostAlloc(&g_tc_err_host, 2 * sizeof(int), cudaHostAllocMapped));
        g_tc_err_host[0] = g_tc_err_host[1] = 0;
        KF_CUDA(cudaHostGetDevicePointer(&g_tc_err_dev, g_tc_err_host, 0));
    }
    return g_tc_err_dev;
}

// round-to-nearest-even FP32 -> BF16 bits (finite inputs)
uint16_t bf16_bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    const uint32_t lsb = (u >> 16) & 1u;
    u += 0x7FFFu + lsb;
    return (uint16_t)(u >> 16);
}

}  // namespace

int tc_mode_layout_ok(int d) { return d >= 1 && d <= 256; }

TcMatrix tc_matrix_create(const double *A, int d, bool transpose, bool split) {
    KF_REQUIRE(tc_mode_layout_ok(d), KF_EINVAL, "tensor-core mode product: axis length must be 1..256");
    TcMatrix m;
    m.d = d;
    m.split = split ? 1 : 0;
    m.Mp = d <= 128 ? 128 : 256;
    m.Kp = (d + 15) / 16 * 16;
    const int eb = split ? 4 : 2, epc = 16 / eb;
    const size_t sbo = (size_t)(m.Kp / epc) * 128, img_bytes = (size_t)m.Mp * m.Kp * eb;
    std::vector<unsigned char> img(img_bytes * (split ? 2 : 1), 0);
    for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) {
            // operator entry (i, j): A[i + d j], or A[j + d i] when transposed
            const double v = transpose ? A[j + (size_t)d * i] : A[i + (size_t)d * j];
            const size_t byte = (size_t)(i >> 3) * sbo + (size_t)(j / epc) * 128 + (size_t)(i & 7) * 16 +
                                (size_t)(j % epc) * eb;
            if (split) {
                float f = (float)v;
                uint32_t u;
                std::memcpy(&u, &f, 4);
                u &= 0xFFFFE000u;
                float hi;
                std::memcpy(&hi, &u, 4);
                const float lo = (float)(v - (double)hi);
                std::memcpy(&img[byte], &hi, 4);
                std::memcpy(&img[img_bytes + byte], &lo, 4);
            } else {
                const uint16_t b = bf16_bits((float)v);
                std::memcpy(&img[byte], &b, 2);
            }
        }
    KF_CUDA(cudaMalloc(&m.img, img.size()));
    KF_CUDA(cudaMemcpy(m.img, img.data(), img.size(), cudaMemcpyHostToDevice));
    return m;
}

void tc_matrix_free(TcMatrix &m) {
    if (m.img) cudaFree(m.img);
    m.img = nullptr;
}

// whether the kernel's shared-memory image of a d x d operator fits this device
// the pipelined BF16 kernel, one persistent CTA per SM; false when its shared-memory plan does not fit
static bool mode_pipe(float *Y, int64_t ldy, const float *X, int64_t ldx, const TcMatrix &A, int64_t left, int64_t N,
                      int64_t b, double alpha, double beta, cudaStream_t s) {
    const int tn = A.Mp > 128 ? 64 : 128;
    // 32-bit column indices (mp_base)
    if ((N / A.d) * b >= ((int64_t)1 << 31)) return false;
    const size_t smem = mode_pipe_smem(A, tn);
    int sms = 152, optin = 0, dev = 0;
    KF_CUDA(cudaGetDevice(&dev));
    KF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    KF_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa;
    if (tn == 64) KF_CUDA(cudaFuncGetAttributes(&fa, k_mode_pipe<64>));
    else KF_CUDA(cudaFuncGetAttributes(&fa, k_mode_pipe<128>));
    const size_t dyn_max = (size_t)optin - fa.sharedSizeBytes;
    if (smem > dyn_max) return false;
    {
        std::lock_guard<std::mutex> lk(g_tc_mu);
        if (dev < 31 && !(g_mp_attr_mask & (1 << dev))) {
            KF_CUDA(cudaFuncSetAttribute(k_mode_pipe<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_max));
            KF_CUDA(cudaFuncSetAttribute(k_mode_pipe<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_max));
            g_mp_attr_mask |= 1 << dev;
        }
    }
    TcArgs a;
    a.Y = Y;
    a.X = X;
    a.Aimg = reinterpret_cast<const uint4 *>(A.img);
    a.err = tc_err_word();
    a.ldy = ldy;
    a.ldx = ldx;
    a.left = left;
    a.rows_per_col = N / A.d;
    a.Q = a.rows_per_col * b;
    a.d = A.d;
    a.Mp = A.Mp;
    a.Kp = A.Kp;
    a.ntiles = (int)((a.Q + tn - 1) / tn);
    a.alpha = (float)alpha;
    a.beta = (float)beta;
    const int grid = a.ntiles < sms ? a.ntiles : sms;
    if (tn == 64) k_mode_pipe<64><<<grid, MP_THREADS, smem, s>>>(a);
    else k_mode_pipe<128><<<grid, MP_THREADS, smem, s>>>(a);
    KF_LAUNCH_CHECK();
    return true;
}

bool tc_mode_fits(int d, bool split) {
    if (!tc_mode_layout_ok(d)) return false;
    TcMatrix m;
    m.d = d;
    m.split = split ? 1 : 0;
    m.Mp = d <= 128 ? 128 : 256;
    m.Kp = (d + 15) / 16 * 16;
    int optin = 0, dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return false;
    return tc_mode_smem(m) + 1024 <= (size_t)optin;
}

size_t tc_mode_smem(const TcMatrix &m) {
    const size_t eb = m.split ? 4 : 2, ns = m.split ? 2 : 1;
    return ns * ((size_t)m.Mp * m.Kp * eb + (size_t)TC_NT * m.Kp * eb) + (size_t)128 * TC_EP_STRIDE * 4 +
           (size_t)2 * TC_NT * 8 + 16;
}

void tc_mode_product(float *Y, int64_t ldy, const float *X, int64_t ldx, const TcMatrix &A, int64_t left, int64_t N,
                     int64_t b, double alpha, double beta, cudaStream_t s) {
    if (b <= 0 || N <= 0) return;
    // operators longer than 128: the pipelined kernel (one CTA per SM, its 128 KB image); shorter
    // ones keep several serial CTAs per SM, which measured as fast (64-point axis: 49.5 us both)
    if (!A.split && A.Mp > 128 && mode_pipe(Y, ldy, X, ldx, A, left, N, b, alpha, beta, s)) return;
    const int64_t rows_per_col = N / A.d;
    TcArgs a;
    a.Y = Y;
    a.X = X;
    a.Aimg = reinterpret_cast<const uint4 *>(A.img);
    a.err = tc_err_word();
    a.ldy = ldy;
    a.ldx = ldx;
    a.left = left;
    a.rows_per_col = rows_per_col;
    a.Q = rows_per_col * b;
    a.d = A.d;
    a.Mp = A.Mp;
    a.Kp = A.Kp;
    a.ntiles = (int)((a.Q + TC_NT - 1) / TC_NT);
    a.alpha = (float)alpha;
    a.beta = (float)beta;
    const size_t smem = tc_mode_smem(A);
    int sms = 152, optin = 0, dev = 0;
    KF_CUDA(cudaGetDevice(&dev));
    KF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    KF_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa;
    if (A.split) KF_CUDA(cudaFuncGetAttributes(&fa, k_mode_tc<true>));
    else KF_CUDA(cudaFuncGetAttributes(&fa, k_mode_tc<false>));
    const size_t dyn_max = (size_t)optin - fa.sharedSizeBytes;
    KF_REQUIRE(smem <= dyn_max, KF_EINVAL, "tensor-core mode product: shared-memory image too large");
    {
        std::lock_guard<std::mutex> lk(g_tc_mu);
        if (!g_tc_attr) {
            KF_CUDA(cudaFuncSetAttribute(k_mode_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_max));
            KF_CUDA(cudaFuncSetAttribute(k_mode_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_max));
            g_tc_attr = true;
        }
    }
    // resident CTAs per SM: by shared memory and by TMEM columns (512 per SM), at most 4
    int per_sm = (int)(dyn_max / smem);
    const int by_tmem = 512 / ((A.Mp / 128) * TC_NT);
    if (per_sm > by_tmem) per_sm = by_tmem;
    if (per_sm > 4) per_sm = 4;
    if (per_sm < 1) per_sm = 1;
    const int grid = a.ntiles < sms * per_sm ? a.ntiles : sms * per_sm;
    if (A.split) k_mode_tc<true><<<grid, TC_THREADS, smem, s>>>(a);
    else k_mode_tc<false><<<grid, TC_THREADS, smem, s>>>(a);
    KF_LAUNCH_CHECK();
}

int *tc_error_word() { return tc_err_word(); }

int check_take_site() {
    tc_err_word();   // allocates the words on first use
    std::lock_guard<std::mutex> lk(g_tc_mu);
    const int s = *(volatile int *)(g_tc_err_host + 1);
    *(volatile int *)(g_tc_err_host + 1) = 0;
    return s;
}

int tc_take_error() {
    std::lock_guard<std::mutex> lk(g_tc_mu);
    if (!g_tc_err_host) return 0;
    const int e = *(volatile int *)g_tc_err_host;
    if (e) *(volatile int *)g_tc_err_host = 0;
    return e;
}

}  // namespace kf

// The fused stencil apply, plane-marching through shared memory with TMA bulk copies.
//
// Y = D X + sum_e w_e(p) X[p + delta_e] for the same entry table as k_apply_fused (the diagonal,
// banded and shift terms of src/apply.jl:370-432 fused into one pass), organised around the
// slowest axis m that carries an offset: the state index splits as
//   p = q + P (k + n_m o),   q in [0, P) (the axes before m), k in [0, n_m), o the axes after m,
// every entry's offset as delta_e = r_e + P o_me (|r_e| <= R, |o_me| <= H), and every entry's
// weight as w_e(p) = w_inner(q) w_plane(k) w_outer(o).
//
// A CTA owns a tile of T = 256 PT consecutive q (PT = 2), a run of L planes k and CB columns.  For each plane
// k' it needs, one thread copies the column slices X[q0 - R .. q0 + T + R) of plane k' into a ring
// of shared-memory slots with cp.async.bulk (one 1-D TMA copy per column, completion counted in
// bytes on the slot's mbarrier), 6 planes ahead of use.  The inner weights of a thread's PT points
// are computed once (registers) and reused for every plane and column; a plane's weights are one
// scalar per entry.  So each X element is read from HBM once per tile (plus the plane halo, from
// L2), and a point-column costs one shared-memory load and one FMA per entry.
//
// Waits on the ring are bounded; a thread whose wait ran out reports it through __syncthreads_or,
// so the whole CTA leaves the plane loop together and records KF_ETIMEOUT.
#include <cstring>

#include "kf_internal.h"

namespace kf {

namespace {

constexpr int TT_THREADS = 256;
constexpr int TT_PF = 6;                       // planes prefetched beyond the ones in use
constexpr long long TT_WAIT_CYCLES = 4000000000LL;

__device__ __forceinline__ uint32_t tsu32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tt_bar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(tsu32(bar)) : "memory");
}

__device__ __forceinline__ void tt_expect(uint64_t *bar, uint32_t bytes) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}\n" ::"r"(tsu32(bar)),
        "r"(bytes)
        : "memory");
}

__device__ __forceinline__ void tt_bulk(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(tsu32(dst)),
        "l"(src), "r"(bytes), "r"(tsu32(bar))
        : "memory");
}

__device__ __forceinline__ bool tt_wait(uint64_t *bar, uint32_t use) {
    const uint32_t parity = use & 1u;
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(tsu32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > TT_WAIT_CYCLES) return false;
    }
}

// three CTAs per SM where the entry table is small enough to fit the registers without spills
template <typename T, int CB, int PT, int ME>
__global__ void __launch_bounds__(TT_THREADS, (ME <= 8 ? 3 : 2)) k_apply_tiled(const ApplyPlan plan, TiledGeom g, const T *__restrict__ D,
                                                           const T *__restrict__ W, const T *__restrict__ X,
                                                           T *__restrict__ Y, int64_t ldx, int64_t ldy, int b,
                                                           T alpha, T beta, const T *__restrict__ Z, int64_t ldz,
                                                           T gamma, int epi, int *err) {
    extern __shared__ __align__(16) unsigned char tt_smem[];
    constexpr int G = 16 / (int)sizeof(T);           // elements per 16 bytes
    constexpr int TILE = TT_THREADS * PT;
    const int NR = 2 * g.H + 1 + TT_PF;              // ring slots
    const int SL = g.SL;                             // slot length per column (elements)
    T *ring = reinterpret_cast<T *>(tt_smem);        // [NR][CB][SL]
    uint64_t *bars = reinterpret_cast<uint64_t *>(ring + (size_t)NR * CB * SL);
    __shared__ int s_om[ME], s_re[ME], s_off[ME + 1];
    __shared__ T s_wout[ME], s_wk[ME];
    const int tid = threadIdx.x;

    const int tile = blockIdx.x;
    const int seg = blockIdx.y % g.nseg, outer = blockIdx.y / g.nseg;
    const int c0 = blockIdx.z * CB, nc = min(CB, b - c0);
    const int q0 = tile * TILE;
    const int kb = seg * g.L, ke = min(kb + g.L, g.nm);
    const int64_t obase = (int64_t)outer * g.P * g.nm;   // column-relative offset of this outer index

    for (int e = tid; e < NR * CB * SL; e += TT_THREADS) ring[e] = T(0);
    if (tid == 0) {
        for (int s = 0; s < NR; ++s) tt_bar_init(bars + s);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    // per-entry plane offset o_me, inner offset r_e, and the weight of the axes after m
    if (tid < ME) {
        const int e = tid;
        int o = 0, r = 0;
        T w = T(0);
        if (e < plan.ne) {
            const Entry &E = plan.e[e];
            if (E.a0 == g.m) o = E.o0;
            if (E.nf == 2 && E.a1 == g.m) o = E.o1;
            r = E.delta - o * g.P;
            int64_t rem = outer;
            w = T(1);
            for (int a = g.m + 1; a < plan.ndims; ++a) {
                const int i = (int)(rem % plan.dims[a]);
                rem /= plan.dims[a];
                if (E.a0 == a)
                    w = ((unsigned)(i + E.o0) < (unsigned)E.n0) ? w * __ldg(W + E.w0 + i * E.nb0) : T(0);
                if (E.nf == 2 && E.a1 == a)
                    w = ((unsigned)(i + E.o1) < (unsigned)E.n1) ? w * __ldg(W + E.w1 + i * E.nb1) : T(0);
            }
        }
        s_om[e] = o;
        s_re[e] = r;
        s_wout[e] = w;
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();

    // inner weights of this thread's PT points (axes before m), 0 for an invalid neighbour
    T win[PT][ME];
#pragma unroll
    for (int j = 0; j < PT; ++j) {
        const int q = q0 + tid + j * TT_THREADS;
        int idx[MAXDIMS_F];
        int rem = q < g.P ? q : 0;
#pragma unroll
        for (int a = 0; a < MAXDIMS_F; ++a) {
            idx[a] = 0;
            if (a < g.m) {
                idx[a] = rem % plan.dims[a];
                rem /= plan.dims[a];
            }
        }
#pragma unroll
        for (int e = 0; e < ME; ++e) {
            T w = T(0);
            if (e < plan.ne && q < g.P) {
                const Entry &E = plan.e[e];
                w = T(1);
                if (E.a0 < g.m) {
                    int i = idx[0];
#pragma unroll
                    for (int a = 1; a < MAXDIMS_F; ++a) i = (E.a0 == a) ? idx[a] : i;
                    w = ((unsigned)(i + E.o0) < (unsigned)E.n0) ? __ldg(W + E.w0 + i * E.nb0) : T(0);
                }
                if (E.nf == 2 && E.a1 < g.m) {
                    int i = idx[0];
#pragma unroll
                    for (int a = 1; a < MAXDIMS_F; ++a) i = (E.a1 == a) ? idx[a] : i;
                    w = ((unsigned)(i + E.o1) < (unsigned)E.n1) ? w * __ldg(W + E.w1 + i * E.nb1) : T(0);
                }
            }
            win[j][e] = w;
        }
    }

    // slice j (plane k' = j): the tile's column range with the halo, aligned to 16 bytes, clamped
    // to the column; held in slot (j - kfirst) % NR, as that slot's use (j - kfirst) / NR
    const int kfirst = kb - g.H, klast = ke - 1 + g.H;
    const int qhi = min(q0 + TILE, g.P);
    auto base_of = [&](int j) -> int64_t {   // aligned (floor) column index of the slot's element 0
        const int64_t x = obase + (int64_t)j * g.P + q0 - g.R;
        return x >= 0 ? x / G * G : -((-x + G - 1) / G * G);
    };
    int last_issued = kfirst - 1;            // thread 0's record of the copies in flight
    auto issue = [&](int j) {
        last_issued = j;
        if (tid != 0) return;
        const int s = (j - kfirst) % NR;
        uint64_t *bar = bars + s;
        const int64_t base = base_of(j);
        int64_t lo = base, hi = obase + (int64_t)j * g.P + qhi + g.R;
        hi = (hi + G - 1) / G * G;
        if (lo < 0) lo = 0;
        if (hi > g.N) hi = g.N;
        const bool ok = j >= 0 && j < g.nm && hi > lo;
        const uint32_t bytes = ok ? (uint32_t)((hi - lo) * (int64_t)sizeof(T)) : 0u;
        tt_expect(bar, bytes * (uint32_t)nc);
        if (ok)
            for (int c = 0; c < nc; ++c)
                tt_bulk(ring + ((size_t)s * CB + c) * SL + (lo - base), X + (int64_t)(c0 + c) * ldx + lo, bytes, bar);
    };
    for (int j = kfirst; j <= min(klast, kfirst + NR - 1); ++j) issue(j);

    bool failed = false;
    for (int k = kb; k < ke; ++k) {
        // the slices of planes k - H .. k + H have landed: thread 0 polls (bounded), the barrier
        // below releases the others
        bool bad = false;
        if (tid == 0)
            for (int j = k - g.H; j <= k + g.H; ++j)
                if (!tt_wait(bars + (j - kfirst) % NR, (uint32_t)((j - kfirst) / NR))) bad = true;
        // per-plane tables: each entry's weight at plane k and the ring offset of its neighbour
        // (slot, alignment shift, halo, inner offset); the centre's offset last
        if (tid <= ME) {
            const int e = tid;
            const int om = e < ME ? s_om[e] : 0;
            const int kp = k + om;
            const int sl = (kp - kfirst) % NR;
            const int mis = (int)(obase + (int64_t)kp * g.P + q0 - g.R - base_of(kp));
            if (e < ME) {
                T w = e < plan.ne ? s_wout[e] : T(0);
                if (e < plan.ne) {
                    const Entry &E = plan.e[e];
                    if (E.a0 == g.m)
                        w = ((unsigned)(k + E.o0) < (unsigned)E.n0) ? w * __ldg(W + E.w0 + k * E.nb0) : T(0);
                    if (E.nf == 2 && E.a1 == g.m)
                        w = ((unsigned)(k + E.o1) < (unsigned)E.n1) ? w * __ldg(W + E.w1 + k * E.nb1) : T(0);
                }
                s_wk[e] = w;
                s_off[e] = e < plan.ne ? sl * CB * SL + mis + g.R + s_re[e] : 0;
            } else {
                s_off[ME] = sl * CB * SL + mis + g.R;
            }
        }
        if (__syncthreads_or(bad)) { failed = true; break; }
        // this plane's tables in registers: ring offsets and plane weights of the entries
        int off[ME];
        T wk[ME];
#pragma unroll
        for (int e = 0; e < ME; ++e) {
            off[e] = s_off[e];
            wk[e] = s_wk[e];
        }
        const int offc = s_off[ME];
        const int64_t pbase = obase + (int64_t)k * g.P;
#pragma unroll
        for (int j = 0; j < PT; ++j) {
            const int q = q0 + tid + j * TT_THREADS;
            if (q >= g.P) continue;
            const int64_t p = pbase + q;
            const T dv = D[p];
            T w[ME];
#pragma unroll
            for (int e = 0; e < ME; ++e) w[e] = win[j][e] * wk[e];   // zero past plan.ne
            for (int c = 0; c < nc; ++c) {
                const T *col = ring + (size_t)c * SL + (q - q0);
                const T xcen = col[offc];
                T acc = dv * xcen;
#pragma unroll
                for (int e = 0; e < ME; ++e) acc += w[e] * col[off[e]];
                T r = acc;
                if (epi) {
                    r = alpha * acc + beta * xcen;
                    if (Z != nullptr) r += gamma * Z[(int64_t)(c0 + c) * ldz + p];
                }
                Y[(int64_t)(c0 + c) * ldy + p] = r;
            }
        }
        __syncthreads();                                   // everyone is done with slice k - H
        const int jn = k + g.H + TT_PF + 1;                // reuses slice k - H's slot
        if (jn <= klast) {
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            issue(jn);
        }
    }
    if (failed && tid == 0) {
        *(volatile int *)err = KF_ETIMEOUT;
        __threadfence_system();
    }
    // copies still in flight write this CTA's shared memory: thread 0 waits (bounded) for the
    // latest use of every slot before the CTA exits
    if (tid == 0)
        for (int j = max(kfirst, last_issued - NR + 1); j <= last_issued; ++j)
            (void)tt_wait(bars + (j - kfirst) % NR, (uint32_t)((j - kfirst) / NR));
    __syncthreads();
}

}  // namespace

// geometry of the plane-marching apply for this plan, or false when it does not apply
bool tiled_geometry(const kf_op *op, int64_t b, size_t elem, TiledGeom &g) {
    const ApplyPlan &P = op->plan;
    if (P.ne < 1 || P.ne > 16) return false;
    int m = -1;
    for (int e = 0; e < P.ne; ++e) {
        const Entry &E = P.e[e];
        if (E.o0 != 0) m = std::max(m, E.a0);
        if (E.nf == 2 && E.o1 != 0) m = std::max(m, E.a1);
    }
    if (m < 0) return false;
    int64_t stride = 1;
    for (int a = 0; a < m; ++a) stride *= P.dims[a];
    g.m = m;
    g.P = (int)stride;
    g.nm = P.dims[m];
    g.N = P.N;
    g.H = 0;
    g.R = 0;
    for (int e = 0; e < P.ne; ++e) {
        const Entry &E = P.e[e];
        int o = 0;
        if (E.a0 == m) o = E.o0;
        if (E.nf == 2 && E.a1 == m) o = E.o1;
        g.H = std::max(g.H, std::abs(o));
        g.R = std::max(g.R, std::abs(E.delta - o * g.P));
    }
    if (g.H > 3 || g.R > 1024) return false;
    const int G = 16 / (int)elem;
    if (P.N % G != 0) return false;
    const int tile = TT_THREADS * 2;   // points per CTA: 2 per thread
    g.SL = (tile + 2 * g.R + 2 * G + G - 1) / G * G;
    g.L = 16;
    g.nseg = (g.nm + g.L - 1) / g.L;
    g.ntile = (g.P + tile - 1) / tile;
    g.nouter = (int)(P.N / ((int64_t)g.P * g.nm));
    (void)b;
    return true;
}

template <typename T, int ME>
static void launch_tiled_me(const kf_op *op, const TiledGeom &g, const T *D, const T *W, const T *X, T *Y, int64_t ldx,
                            int64_t ldy, int64_t b, T alpha, T beta, const T *Z, int64_t ldz, T gamma, int epi,
                            cudaStream_t s) {
    constexpr int CB = sizeof(T) == 4 ? 2 : 1, PT = 2;
    const int NR = 2 * g.H + 1 + TT_PF;
    const size_t smem = (size_t)NR * CB * g.SL * sizeof(T) + (size_t)NR * 8;
    KF_REQUIRE(smem <= 200 * 1024, KF_EINVAL, "apply: plane ring too large");
    dim3 grid((unsigned)g.ntile, (unsigned)(g.nseg * g.nouter), (unsigned)((b + CB - 1) / CB));
    static bool attr = false;   // per instantiation
    if (!attr) {
        KF_CUDA(cudaFuncSetAttribute(k_apply_tiled<T, CB, PT, ME>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     200 * 1024));
        attr = true;
    }
    k_apply_tiled<T, CB, PT, ME><<<grid, TT_THREADS, smem, s>>>(op->plan, g, D, W, X, Y, ldx, ldy, (int)b, alpha, beta,
                                                                 Z, ldz, gamma, epi, tc_error_word());
    KF_LAUNCH_CHECK();
}

template <typename T>
void launch_apply_tiled(const kf_op *op, const TiledGeom &g, const T *D, const T *W, const T *X, T *Y, int64_t ldx,
                        int64_t ldy, int64_t b, T alpha, T beta, const T *Z, int64_t ldz, T gamma, int epi,
                        cudaStream_t s) {
    // the entry loop runs to the table size rounded up to 4 (extra entries carry weight 0)
    const int ne = op->plan.ne;
    if (ne <= 4) launch_tiled_me<T, 4>(op, g, D, W, X, Y, ldx, ldy, b, alpha, beta, Z, ldz, gamma, epi, s);
    else if (ne <= 8) launch_tiled_me<T, 8>(op, g, D, W, X, Y, ldx, ldy, b, alpha, beta, Z, ldz, gamma, epi, s);
    else if (ne <= 12) launch_tiled_me<T, 12>(op, g, D, W, X, Y, ldx, ldy, b, alpha, beta, Z, ldz, gamma, epi, s);
    else launch_tiled_me<T, 16>(op, g, D, W, X, Y, ldx, ldy, b, alpha, beta, Z, ldz, gamma, epi, s);
}

template void launch_apply_tiled<float>(const kf_op *, const TiledGeom &, const float *, const float *, const float *,
                                        float *, int64_t, int64_t, int64_t, float, float, const float *, int64_t,
                                        float, int, cudaStream_t);
template void launch_apply_tiled<double>(const kf_op *, const TiledGeom &, const double *, const double *,
                                         const double *, double *, int64_t, int64_t, int64_t, double, double,
                                         const double *, int64_t, double, int, cudaStream_t);

}  // namespace kf

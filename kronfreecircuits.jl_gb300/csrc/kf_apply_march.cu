// The fused stencil apply, marching along the slowest stencil axis with a register window.
//
// Y = D X + sum_e w_e(p) X[p + delta_e] for the entry table of k_apply_fused (the diagonal, banded
// and shift terms of src/apply.jl:370-432 fused into one pass), organised around the slowest axis m
// that carries an offset: the state index splits as
//     p = q + P (k + n_m o),   q in [0, P) (the axes before m), k in [0, n_m), o (the axes after m),
// every entry's offset as delta_e = r_e + P o_e (|r_e| <= R, |o_e| <= H), and every entry's weight as
// w_e(p) = w_in(q) w_plane(k) w_out(o).  The entries fall into three classes:
//   window   r_e = 0 and no factor on the axes before m: X[q, k + o_e] comes from a per-thread
//            register window of 2H + 1 planes, the weights summed per (plane, o) in a table;
//   centre   r_e = 0, o_e = 0, factors on the axes before m only: one per-thread weight on X[q, k];
//   shared   everything else: X[q + r_e, k + o_e] read from the shared-memory copy of plane k + o_e.
// So every X element is read from global memory once per tile (plus the in-plane halo, from L2),
// the slow axis' neighbours never leave registers, and only in-plane neighbours cost a
// shared-memory load.
//
// Weights.  They depend on the operator only, so a small kernel evaluates them once per operator and
// precision into a table in device memory: per outer index, the shared entries' and the centre's
// weights of every in-plane point (w_in w_out) and, per plane, the window weights summed per plane
// offset and the shared entries' plane weights (w_plane).  The march reads a thread's point weights
// with a few coalesced loads and copies its outer index's plane rows into shared memory.
//
// Work split.  The kernel is persistent: one CTA per SM.  A CTA owns one tile of TQ consecutive q
// (of one outer index) for its lifetime and marches a contiguous range of the tile's (column, plane)
// pairs, split evenly among the CTAs of the tile, column by column (each column's run with its plane
// halo).
//
// Pipeline.  A producer warp copies, for every plane the CTA touches, the column's slice
// X[q0 - R .. q0 + TQ + R) and the diagonal's slice D[q0 .. q0 + TQ) into the next slot of a ring
// in shared memory with cp.async.bulk (1-D bulk copies, completion counted in bytes on the slot's
// "full" mbarrier).  The 12 consumer warps wait on "full" for the plane entering their window and,
// when a plane leaves it (or a column's run ends), arrive on that slot's "empty" mbarrier, which the
// producer waits on before reusing the slot.  No CTA-wide barrier inside the march.
//
// KF_CHECK builds test every slice, ring, weight and output index first (sites 101-109: X slice fits
// its slot, diagonal slice fits, window reads, window reads on the fast path, shared-entry reads,
// diagonal reads, window weights, output stores, table reads) and record a failure instead of the
// access.
//
// Every wait is bounded (a clock64 budget of about two seconds): a role whose wait ran out records
// KF_ETIMEOUT in the host-mapped error word and raises the CTA's abort flag, which every other wait
// loop checks; the producer then waits (bounded) for its copies still in flight before the CTA exits.
#include <algorithm>
#include <cstring>

#include "kf_internal.h"

namespace kf {

namespace {

// consumer warps: 12 (4 FP32 / 2 FP64 points per thread at 128 registers), or 7 with more points
// per thread (8 FP32 / 4 FP64: with the producer, two warps per SM sub-partition, so up to 255
// registers; the per-plane work -- waits, weight loads, ring addresses, releases -- is spread over
// twice the points)
constexpr int MCW_STD = 12, MCW_WIDE = 7;
constexpr long long M_WAIT_CYCLES = 4000000000LL;
constexpr int M_SMEM_BUDGET = 200 * 1024;   // one CTA per SM

__device__ __forceinline__ uint32_t msu32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void m_bar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(msu32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void m_expect(uint64_t *bar, uint32_t bytes) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}\n" ::"r"(msu32(bar)),
        "r"(bytes)
        : "memory");
}

__device__ __forceinline__ void m_arrive(uint64_t *bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}\n" ::"r"(msu32(bar))
                 : "memory");
}

__device__ __forceinline__ void m_bulk(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(msu32(dst)),
        "l"(src), "r"(bytes), "r"(msu32(bar))
        : "memory");
}

// wait for the phase with the given parity to complete; false when the budget ran out or another
// role aborted
__device__ __forceinline__ bool m_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag) {
    {
        // the usual case, a plane that has landed already: one non-blocking test, no clock read
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(msu32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(msu32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (*abort_flag) return false;
        if (clock64() - t0 > M_WAIT_CYCLES) return false;
    }
}

// a load from shared memory at a 32-bit shared-window address (ordered after the mbarrier waits,
// which are volatile asm too)
template <typename T>
__device__ __forceinline__ T lds(uint32_t a);
template <>
__device__ __forceinline__ float lds<float>(uint32_t a) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];\n" : "=f"(v) : "r"(a));
    return v;
}
template <>
__device__ __forceinline__ double lds<double>(uint32_t a) {
    double v;
    asm volatile("ld.shared.f64 %0, [%1];\n" : "=d"(v) : "r"(a));
    return v;
}

__device__ __forceinline__ int64_t floor_to(int64_t x, int g) { return x >= 0 ? x / g * g : -((-x + g - 1) / g * g); }
__device__ __forceinline__ int64_t ceil_to(int64_t x, int g) { return (x + g - 1) / g * g; }

// one factor's weight at coordinate i (0 where the neighbour i + o leaves the axis)
template <typename T>
__device__ __forceinline__ T fac_w(const T *W, int w, int nb, int n, int o, int i) {
    return ((unsigned)(i + o) < (unsigned)n) ? __ldg(W + w + i * nb) : T(0);
}

// idx[a] for a runtime axis a, by a chain of selects (the array stays in registers)
__device__ __forceinline__ int coord(const int (&idx)[MAXDIMS_F], int a) {
    int v = idx[0];
#pragma unroll
    for (int k = 1; k < MAXDIMS_F; ++k) v = (a == k) ? idx[k] : v;
    return v;
}

// the part of entry E's weight from the factors on the axes of class `sel` (0: before m, 1: m,
// 2: after m); idx[a] is the coordinate on axis a
template <typename T>
__device__ __forceinline__ T entry_part(const Entry &E, const T *W, int m, const int (&idx)[MAXDIMS_F], int sel) {
    T w = T(1);
    {
        const int s = E.a0 < m ? 0 : (E.a0 == m ? 1 : 2);
        if (s == sel) w *= fac_w(W, E.w0, E.nb0, E.n0, E.o0, coord(idx, E.a0));
    }
    if (E.nf == 2) {
        const int s = E.a1 < m ? 0 : (E.a1 == m ? 1 : 2);
        if (s == sel) w *= fac_w(W, E.w1, E.nb1, E.n1, E.o1, coord(idx, E.a1));
    }
    return w;
}

// idx with axis a set to v (static indexing)
__device__ __forceinline__ void set_coord(int (&idx)[MAXDIMS_F], int a, int v) {
#pragma unroll
    for (int k = 0; k < MAXDIMS_F; ++k)
        if (a == k) idx[k] = v;
}

// this CTA's tile group and its range [f0, f1) of (column, plane) pairs f = col * n_m + k
struct Work {
    int tile, outer;
    int64_t f0, f1;
};
__device__ __forceinline__ Work cta_work(const MarchPlan &mp, int b) {
    const int G = mp.ntile * mp.nouter;
    const int g = blockIdx.x % G, r = blockIdx.x / G;
    const int ng = ((int)gridDim.x - g + G - 1) / G;       // CTAs of this group
    const int64_t tot = (int64_t)b * mp.nm;
    Work w;
    w.tile = g % mp.ntile;
    w.outer = g / mp.ntile;
    w.f0 = tot * r / ng;
    w.f1 = tot * (r + 1) / ng;
    return w;
}

// the end of the column run that starts at f: the column's last plane or the range's end
__device__ __forceinline__ int run_end(int64_t f, int k0, int64_t f1, int nm) {
    const int64_t e = k0 + (f1 - f);
    return e < (int64_t)nm ? (int)e : nm;
}

// The weight table of a march plan (layout per outer index o: [MS + 1][P] point weights -- the
// shared entries', then the centre's -- followed by [nm][wn + MS] plane rows -- the window weights
// per plane offset, then the shared entries' plane weights, 1 without a factor on axis m, 0 past
// nsm).  One thread per table element.
template <typename T>
__global__ void k_march_table(const ApplyPlan plan, const MarchPlan mp, const T *__restrict__ W, T *__restrict__ tab,
                              int64_t total) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int MS = mp.ms, WN = mp.wn, H = (mp.wn - 1) / 2;
    const int64_t per = (int64_t)(MS + 1) * mp.P + (int64_t)mp.nm * (WN + MS);
    const int o = (int)(t / per);
    const int64_t r = t % per;
    int idx[MAXDIMS_F];
    {
        int rem = o;
#pragma unroll
        for (int a = 0; a < MAXDIMS_F; ++a) {
            idx[a] = 0;
            if (a > mp.m && a < plan.ndims) {
                idx[a] = rem % plan.dims[a];
                rem /= plan.dims[a];
            }
        }
    }
    T v = T(0);
    if (r < (int64_t)(MS + 1) * mp.P) {
        const int e = (int)(r / mp.P), q = (int)(r % mp.P);
        int rem = q;
#pragma unroll
        for (int a = 0; a < MAXDIMS_F; ++a)
            if (a < mp.m) {
                idx[a] = rem % plan.dims[a];
                rem /= plan.dims[a];
            }
        if (e < mp.nsm) {
            const Entry &E = plan.e[mp.sm[e]];
            v = entry_part<T>(E, W, mp.m, idx, 0) * entry_part<T>(E, W, mp.m, idx, 2);
        } else if (e == MS) {
            for (int c = 0; c < mp.ncen; ++c) {
                const Entry &E = plan.e[mp.cen[c]];
                v += entry_part<T>(E, W, mp.m, idx, 0) * entry_part<T>(E, W, mp.m, idx, 2);
            }
        }
    } else {
        const int64_t r2 = r - (int64_t)(MS + 1) * mp.P;
        const int k = (int)(r2 / (WN + MS)), c = (int)(r2 % (WN + MS));
        set_coord(idx, mp.m, k);
        if (c < WN) {
            for (int q = 0; q < mp.nwin; ++q) {
                if (mp.wino[q] != c - H) continue;
                const Entry &E = plan.e[mp.win[q]];
                v += entry_part<T>(E, W, mp.m, idx, 1) * entry_part<T>(E, W, mp.m, idx, 2);
            }
        } else {
            const int e = c - WN;
            if (e < mp.nsm1) v = T(1);
            else if (e < mp.nsm) v = entry_part<T>(plan.e[mp.sm[e]], W, mp.m, idx, 1);
        }
    }
    tab[t] = v;
}

template <typename T, int H, int MS, int PT, bool EPI, int MCW>
__global__ void __launch_bounds__(MCW * 32 + 32, 1)
    k_apply_march(const ApplyPlan plan, const MarchPlan mp, const T *__restrict__ D, const T *__restrict__ W,
                  const T *__restrict__ X, T *__restrict__ Y, int64_t ldx, int64_t ldy, int b, T alpha, T beta,
                  const T *__restrict__ Z, int64_t ldz, T gamma, int epi, const T *__restrict__ tab, int *err) {
    constexpr int G = 16 / (int)sizeof(T);
    constexpr int WN = 2 * H + 1;
    constexpr int MCT = MCW * 32;               // consumer threads
    constexpr int MTHREADS = MCT + 32;          // + one producer warp
    extern __shared__ __align__(128) unsigned char m_smem[];
    const int SL = mp.SLX + mp.SLD;
    const int NR = mp.NR;
    T *ring = reinterpret_cast<T *>(m_smem);                      // [NR][SLX + SLD]
    T *wm = ring + (size_t)NR * SL;                              // [nm][WN] window weights per plane
    T *wp = wm + (size_t)mp.nm * WN;                             // [nm][MS] plane weights of the shared entries
    uint64_t *full = reinterpret_cast<uint64_t *>(
        ((uintptr_t)(wp + (size_t)mp.nm * MS + 2) + 7) & ~(uintptr_t)7);
    uint64_t *empty = full + NR;
    __shared__ int s_abort;

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const Work wk = cta_work(mp, b);
    const int q0 = wk.tile * mp.TQ, qn = min(mp.TQ, mp.P - q0);
    const int64_t obase = (int64_t)wk.outer * mp.P * mp.nm;
    // the plane size is a multiple of 16 bytes, so every plane's slice has the same alignment shift
    const int misx = (int)((obase + q0 - mp.R) - floor_to(obase + q0 - mp.R, G));
    const int misd = (int)((obase + q0) - floor_to(obase + q0, G));

    // coordinates of the outer index (axes after m)
    int idx_out[MAXDIMS_F];
    {
        int rem = wk.outer;
#pragma unroll
        for (int a = 0; a < MAXDIMS_F; ++a) {
            idx_out[a] = 0;
            if (a > mp.m && a < plan.ndims) {
                idx_out[a] = rem % plan.dims[a];
                rem /= plan.dims[a];
            }
        }
    }

    // the ring starts zeroed: a shared entry whose neighbour plane lies outside the axis reads a slot
    // no copy has filled yet, and its zero weight must meet a finite value there
    for (int e = tid; e < NR * SL; e += MTHREADS) ring[e] = T(0);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    if (tid == 0) {
        s_abort = 0;
        for (int s = 0; s < NR; ++s) {
            m_bar_init(full + s, 1);
            m_bar_init(empty + s, MCW);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();

    if (warp == MCW) {
        // ---- producer: lane 0 issues every plane's two bulk copies, in load order; a slice clamped at
        // an end of the column leaves part of its slot unwritten, which the warp zeroes first (the
        // slot may hold an earlier plane's values; zero keeps the halo of the column's end exact)
        int s = 0, use = 0, issued = 0;   // load t goes to slot t % NR, as use t / NR
        bool ok = true;
        for (int64_t f = wk.f0; f < wk.f1 && ok;) {
            const int col = (int)(f / mp.nm), k0 = (int)(f % mp.nm);
            const int k1 = run_end(f, k0, wk.f1, mp.nm);
            f += k1 - k0;
            const T *Xc = X + (int64_t)col * ldx;
            const int jfirst = max(0, k0 - H), jlast = min(mp.nm - 1, k1 - 1 + H);
            for (int j = jfirst; j <= jlast; ++j) {
                int good = 1;
                if (use > 0 && lane == 0) good = m_wait(empty + s, (uint32_t)((use - 1) & 1), &s_abort) ? 1 : 0;
                good = __shfl_sync(0xffffffffu, good, 0);
                if (!good) {
                    ok = false;
                    break;
                }
                T *slot = ring + (size_t)s * SL;
                const int64_t xs = obase + (int64_t)j * mp.P + q0 - mp.R, xb = xs - misx;
                const int64_t xend = ceil_to(xs + qn + 2 * mp.R, G);
                int64_t xlo = xb, xhi = xend;
                if (xlo < 0) xlo = 0;
                if (xhi > mp.N) xhi = mp.N;
                const bool xfit = KF_CHK(xend - xb <= mp.SLX && col < b, err, 101);
                if (!xfit) {
                    xlo = xb;
                    xhi = xb;   // nothing copied, nothing zeroed
                } else if (xlo > xb || xhi < xend) {
                    for (int e = lane; e < (int)(xlo - xb); e += 32) slot[e] = T(0);
                    for (int e = (int)(xhi - xb) + lane; e < (int)(xend - xb); e += 32) slot[e] = T(0);
                    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                }
                __syncwarp();
                if (lane == 0) {
                    const int64_t ds = obase + (int64_t)j * mp.P + q0, db = ds - misd;
                    int64_t dhi = ceil_to(ds + qn, G);
                    if (dhi > mp.N) dhi = mp.N;
                    const uint32_t bx = xhi > xlo ? (uint32_t)((xhi - xlo) * (int64_t)sizeof(T)) : 0u;
                    uint32_t bd = dhi > db ? (uint32_t)((dhi - db) * (int64_t)sizeof(T)) : 0u;
                    if (!KF_CHK(db >= 0 && mp.SLX + (dhi - db) <= SL, err, 102)) bd = 0u;
                    m_expect(full + s, bx + bd);
                    if (bx) m_bulk(slot + (xlo - xb), Xc + xlo, bx, full + s);
                    if (bd) m_bulk(slot + mp.SLX, D + db, bd, full + s);
                }
                ++issued;
                if (++s == NR) { s = 0; ++use; }
            }
        }
        if (!ok && lane == 0) {
            s_abort = 1;
            *(volatile int *)err = KF_ETIMEOUT;
            __threadfence_system();
            // copies still in flight write this CTA's shared memory: wait (bounded) for the latest
            // use of every slot before leaving
            volatile int never = 0;
            for (int t = max(0, issued - NR); t < issued; ++t)
                (void)m_wait(full + t % NR, (uint32_t)((t / NR) & 1), &never);
        }
    } else {
        // ---- consumers: this outer index's plane rows into shared memory, the points' weights into
        // registers, from the operator's weight table
        const T *tab_o = tab + (int64_t)wk.outer * ((int64_t)(MS + 1) * mp.P + (int64_t)mp.nm * (WN + MS));
        const T *rows = tab_o + (int64_t)(MS + 1) * mp.P;
        for (int t = tid; t < mp.nm * (WN + MS); t += MCT) {
            const int k = t / (WN + MS), c = t % (WN + MS);
            if (c < WN) wm[k * WN + c] = rows[t];
            else wp[k * MS + (c - WN)] = rows[t];
        }
        bool valid[PT];
        T wcen[PT];                   // centre weights (factors before m, times the outer ones)
        T wsm[PT][MS];                // weights of the shared entries on the axes before m and after m
#pragma unroll
        for (int j = 0; j < PT; ++j) {
            const int qi = tid + j * MCT;
            valid[j] = qi < qn;
            const T *pt = tab_o + q0 + qi;
#pragma unroll
            const bool tin = !valid[j] || KF_CHK(q0 + qi < mp.P, err, 109);
            for (int e = 0; e < MS; ++e) wsm[j][e] = (valid[j] && tin) ? __ldg(pt + (int64_t)e * mp.P) : T(0);
            wcen[j] = (valid[j] && tin) ? __ldg(pt + (int64_t)MS * mp.P) : T(0);
        }
        asm volatile("bar.sync 1, %0;\n" ::"r"(MCT) : "memory");   // the consumer warps only
        auto wrap = [&](int s) { return s >= NR ? s - NR : (s < 0 ? s + NR : s); };
        // offset, within a slot, of this thread's first point in the X slice
        const int xoff0 = mp.R + misx + tid;
        const bool plain_sm = mp.nsm1 == mp.nsm;
        const bool fast = plain_sm && mp.flat;
        const uint32_t ring_s = msu32(ring), wm_s = msu32(wm);
        int64_t t0 = 0;               // load index of the current run's first plane
        bool ok = true;
        for (int64_t f = wk.f0; f < wk.f1 && ok;) {
            const int col = (int)(f / mp.nm), k0 = (int)(f % mp.nm);
            const int k1 = run_end(f, k0, wk.f1, mp.nm);
            f += k1 - k0;
            const int jfirst = max(0, k0 - H), jlast = min(mp.nm - 1, k1 - 1 + H);
            T xw[PT][WN];
#pragma unroll
            for (int j = 0; j < PT; ++j)
#pragma unroll
                for (int o = 0; o < WN; ++o) xw[j][o] = T(0);
            // the window's first 2H planes
#pragma unroll
            for (int o = 0; o < 2 * H; ++o) {
                const int jj = k0 - H + o;
                if (!ok || jj < 0 || jj >= mp.nm) continue;
                const int64_t t = t0 + (jj - jfirst);
                if (!m_wait(full + (int)(t % NR), (uint32_t)((t / NR) & 1), &s_abort)) {
                    ok = false;
                    continue;
                }
                const T *sx = ring + (int)(t % NR) * SL + xoff0;
#pragma unroll
                for (int j = 0; j < PT; ++j) xw[j][o] = KF_CHK(xoff0 + j * MCT < mp.SLX, err, 103) ? sx[j * MCT] : T(0);
            }
            const int64_t tk0 = t0 + (k0 - jfirst);
            int sk = (int)(tk0 % NR);                    // slot of plane k
            int sn = (int)((tk0 + H) % NR);              // slot of plane k + H
            int usen = (int)((tk0 + H) / NR);            // and its use index
            T *ycol = Y + (int64_t)col * ldy + obase + q0 + tid;
            const T *zcol = Z != nullptr ? Z + (int64_t)col * ldz + obase + q0 + tid : nullptr;
            // the march, WN planes per block: at step r of a block, window position o (plane k - H + o)
            // lives in register xw[j][(o + r) % WN], so the window rotates without moves
            if (fast) {
                // every shared entry reads the current plane with in-plane weights only (the
                // three-mode leaf's stencil): 32-bit shared addresses, no per-entry plane weights
                for (int kb = k0; kb < k1 && ok; kb += WN) {
#pragma unroll
                    for (int r = 0; r < WN; ++r) {
                        const int k = kb + r;
                        if (k >= k1 || !ok) break;
                        if (k + H <= jlast) {
                            if (!m_wait(full + sn, (uint32_t)(usen & 1), &s_abort)) {
                                ok = false;
                                break;
                            }
                            const uint32_t ax = ring_s + (uint32_t)(sn * SL + xoff0) * (uint32_t)sizeof(T);
#pragma unroll
                            for (int j = 0; j < PT; ++j)
                                xw[j][(2 * H + r) % WN] = KF_CHK(sn < NR && xoff0 + j * MCT < mp.SLX, err, 104)
                                                              ? lds<T>(ax + (uint32_t)(j * MCT * sizeof(T)))
                                                              : T(0);
                        } else {
#pragma unroll
                            for (int j = 0; j < PT; ++j) xw[j][(2 * H + r) % WN] = T(0);
                        }
                        T wmk[WN];
                        const uint32_t aw = wm_s + (uint32_t)(k * WN) * (uint32_t)sizeof(T);
#pragma unroll
                        for (int o = 0; o < WN; ++o)
                            wmk[o] = KF_CHK(k * WN + o < mp.nm * WN, err, 107) ? lds<T>(aw + (uint32_t)(o * sizeof(T)))
                                                                               : T(0);
                        const uint32_t ab = ring_s + (uint32_t)(sk * SL + xoff0) * (uint32_t)sizeof(T);
                        uint32_t pa[MS];
#pragma unroll
                        for (int e = 0; e < MS; ++e) pa[e] = ab + (uint32_t)(mp.smr[e] * (int)sizeof(T));
                        const uint32_t ad = ring_s + (uint32_t)(sk * SL + mp.SLX + misd + tid) * (uint32_t)sizeof(T);
                        T *yk = ycol + (int64_t)k * mp.P;
#pragma unroll
                        for (int j = 0; j < PT; ++j) {
                            constexpr uint32_t JB = MCT * sizeof(T);
                            const T xc = xw[j][(H + r) % WN];
                            T a0 = (KF_CHK(mp.SLX + misd + tid + j * MCT < SL, err, 106) ? lds<T>(ad + j * JB) : T(0)) * xc;
                            a0 = fma(wcen[j], xc, a0);
                            T a1 = wmk[0] * xw[j][r % WN];
#pragma unroll
                            for (int o = 1; o < WN; ++o) a1 = fma(wmk[o], xw[j][(o + r) % WN], a1);
#pragma unroll
                            for (int e = 0; e < MS; e += 2) {
                                const bool in0 = KF_CHK(xoff0 + mp.smr[e] + j * MCT >= 0 &&
                                                            xoff0 + mp.smr[e] + j * MCT < mp.SLX, err, 105);
                                a0 = fma(wsm[j][e], in0 ? lds<T>(pa[e] + j * JB) : T(0), a0);
                                if (e + 1 < MS) {
                                    const bool in1 = KF_CHK(xoff0 + mp.smr[e + 1] + j * MCT >= 0 &&
                                                                xoff0 + mp.smr[e + 1] + j * MCT < mp.SLX, err, 105);
                                    a1 = fma(wsm[j][e + 1], in1 ? lds<T>(pa[e + 1] + j * JB) : T(0), a1);
                                }
                            }
                            T out = a0 + a1;
                            if (EPI) {
                                out = alpha * out + beta * xc;
                                if (zcol != nullptr && valid[j]) out += gamma * zcol[(int64_t)k * mp.P + j * MCT];
                            }
                            if (valid[j] && KF_CHK(obase + q0 + tid + j * MCT + (int64_t)k * mp.P < mp.N, err, 108))
                                yk[j * MCT] = out;
                        }
                        // plane k - H leaves the window: release its slot
                        __syncwarp();
                        if (k - H >= jfirst && lane == 0) m_arrive(empty + wrap(sk - H));
                        if (++sk == NR) sk = 0;
                        if (++sn == NR) { sn = 0; ++usen; }
                    }
                }
            } else {
            for (int kb = k0; kb < k1 && ok; kb += WN) {
#pragma unroll
            for (int r = 0; r < WN; ++r) {
                const int k = kb + r;
                if (k >= k1 || !ok) break;
                if (k + H <= jlast) {
                    if (!m_wait(full + sn, (uint32_t)(usen & 1), &s_abort)) {
                        ok = false;
                        break;
                    }
                    const T *sx = ring + sn * SL + xoff0;
#pragma unroll
                    for (int j = 0; j < PT; ++j)
                        xw[j][(2 * H + r) % WN] = KF_CHK(xoff0 + j * MCT < mp.SLX, err, 103) ? sx[j * MCT] : T(0);
                } else {
#pragma unroll
                    for (int j = 0; j < PT; ++j) xw[j][(2 * H + r) % WN] = T(0);
                }
                T wmk[WN];
#pragma unroll
                for (int o = 0; o < WN; ++o) wmk[o] = KF_CHK(k * WN + o < mp.nm * WN, err, 107) ? wm[k * WN + o] : T(0);
                // one ring offset per shared entry (its plane's slot, its in-plane offset); the
                // entries past nsm carry weight 0 and offset 0
                int pe[MS];
                const int base = sk * SL + xoff0;
                if (mp.flat) {
#pragma unroll
                    for (int e = 0; e < MS; ++e) pe[e] = base + mp.smr[e];
                } else {
#pragma unroll
                    for (int e = 0; e < MS; ++e) pe[e] = wrap(sk + mp.smo[e]) * SL + xoff0 + mp.smr[e];
                }
                const int sdi = base - xoff0 + mp.SLX + misd + tid;
                T *yk = ycol + (int64_t)k * mp.P;
                // a ring read, checked in KF_CHECK builds
                auto rd = [&](int idx, int site) -> T {
                    return KF_CHK(idx >= 0 && idx < NR * SL, err, site) ? ring[idx] : T(0);
                };
                if (plain_sm) {
#pragma unroll
                    for (int j = 0; j < PT; ++j) {
                        const T xc = xw[j][(H + r) % WN];
                        T a0 = rd(sdi + j * MCT, 106) * xc;
                        a0 = fma(wcen[j], xc, a0);
                        T a1 = wmk[0] * xw[j][r % WN];
#pragma unroll
                        for (int o = 1; o < WN; ++o) a1 = fma(wmk[o], xw[j][(o + r) % WN], a1);
#pragma unroll
                        for (int e = 0; e < MS; e += 2) {
                            a0 = fma(wsm[j][e], rd(pe[e] + j * MCT, 105), a0);
                            if (e + 1 < MS) a1 = fma(wsm[j][e + 1], rd(pe[e + 1] + j * MCT, 105), a1);
                        }
                        T out = a0 + a1;
                        if (EPI) {
                            out = alpha * out + beta * xc;
                            if (zcol != nullptr && valid[j]) out += gamma * zcol[(int64_t)k * mp.P + j * MCT];
                        }
                        if (valid[j] && KF_CHK(obase + q0 + tid + j * MCT + (int64_t)k * mp.P < mp.N, err, 108))
                            yk[j * MCT] = out;
                    }
                } else {
                    T wpk[MS];
#pragma unroll
                    for (int e = 0; e < MS; ++e) wpk[e] = wp[k * MS + e];
#pragma unroll
                    for (int j = 0; j < PT; ++j) {
                        const T xc = xw[j][(H + r) % WN];
                        T a0 = rd(sdi + j * MCT, 106) * xc;
                        a0 = fma(wcen[j], xc, a0);
                        T a1 = wmk[0] * xw[j][r % WN];
#pragma unroll
                        for (int o = 1; o < WN; ++o) a1 = fma(wmk[o], xw[j][(o + r) % WN], a1);
#pragma unroll
                        for (int e = 0; e < MS; e += 2) {
                            a0 = fma(wsm[j][e] * wpk[e], rd(pe[e] + j * MCT, 105), a0);
                            if (e + 1 < MS) a1 = fma(wsm[j][e + 1] * wpk[e + 1], rd(pe[e + 1] + j * MCT, 105), a1);
                        }
                        T out = a0 + a1;
                        if (EPI) {
                            out = alpha * out + beta * xc;
                            if (zcol != nullptr && valid[j]) out += gamma * zcol[(int64_t)k * mp.P + j * MCT];
                        }
                        if (valid[j] && KF_CHK(obase + q0 + tid + j * MCT + (int64_t)k * mp.P < mp.N, err, 108))
                            yk[j * MCT] = out;
                    }
                }
                // plane k - H leaves the window: release its slot
                __syncwarp();
                if (k - H >= jfirst && lane == 0) m_arrive(empty + wrap(sk - H));
                if (++sk == NR) sk = 0;
                if (++sn == NR) { sn = 0; ++usen; }
            }
            }
            }
            // the run ends: release its planes still in the window
            if (ok) {
                __syncwarp();
                if (lane == 0)
                    for (int jj = max(jfirst, k1 - H); jj <= jlast; ++jj)
                        m_arrive(empty + (int)((t0 + (jj - jfirst)) % NR));
            }
            t0 += jlast - jfirst + 1;
        }
        if (!ok && lane == 0) {
            s_abort = 1;
            *(volatile int *)err = KF_ETIMEOUT;
            __threadfence_system();
        }
    }
    __syncthreads();
}

template <typename T, int H, int MS, int PT, bool EPI, int MCW>
void launch_k(const kf_op *op, const MarchPlan &mp, const T *D, const T *W, const T *X, T *Y, int64_t ldx,
              int64_t ldy, int64_t b, T alpha, T beta, const T *Z, int64_t ldz, T gamma, int epi, const T *tab,
              cudaStream_t s) {
    const size_t smem = march_smem_bytes(mp, sizeof(T), 2 * H + 1, MS);
    static bool attr = false;   // per instantiation
    if (!attr) {
        KF_CUDA(cudaFuncSetAttribute(k_apply_march<T, H, MS, PT, EPI, MCW>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, M_SMEM_BUDGET + 16384));
        attr = true;
    }
    KF_REQUIRE(smem <= (size_t)M_SMEM_BUDGET + 16384, KF_EINVAL, "apply: plane ring too large");
    k_apply_march<T, H, MS, PT, EPI, MCW><<<mp.grid, MCW * 32 + 32, smem, s>>>(op->plan, mp, D, W, X, Y, ldx, ldy, (int)b, alpha,
                                                                beta, Z, ldz, gamma, epi, tab, tc_error_word());
    KF_LAUNCH_CHECK();
}

template <typename T, int H>
void launch_h(const kf_op *op, const MarchPlan &mp, const T *D, const T *W, const T *X, T *Y, int64_t ldx,
              int64_t ldy, int64_t b, T alpha, T beta, const T *Z, int64_t ldz, T gamma, int epi, const T *tab,
              cudaStream_t s) {
    // points per thread: what fits 128 registers without spilling (13 warps on one SM), or, with 7
    // consumer warps, 255 registers
    constexpr int P8 = sizeof(T) == 4 ? 4 : 2, P16 = sizeof(T) == 4 ? 2 : 1;
    constexpr int PW = sizeof(T) == 4 ? 8 : 4;
#define KF_MARCH(MS_, PT_, MCW_)                                                                                   \
    do {                                                                                                           \
        if (epi)                                                                                                   \
            launch_k<T, H, MS_, PT_, true, MCW_>(op, mp, D, W, X, Y, ldx, ldy, b, alpha, beta, Z, ldz, gamma, epi, tab, \
                                                 s);                                                               \
        else                                                                                                       \
            launch_k<T, H, MS_, PT_, false, MCW_>(op, mp, D, W, X, Y, ldx, ldy, b, alpha, beta, Z, ldz, gamma, epi, \
                                                  tab, s);                                                         \
    } while (0)
    if (mp.mcw == MCW_WIDE) {
        if (mp.ms == 6) KF_MARCH(6, PW, MCW_WIDE);
        else KF_MARCH(8, PW, MCW_WIDE);
    } else if (mp.ms == 6) KF_MARCH(6, P8, MCW_STD);
    else if (mp.ms == 8) KF_MARCH(8, P8, MCW_STD);
    else KF_MARCH(16, P16, MCW_STD);
#undef KF_MARCH
}

}  // namespace

size_t march_smem_bytes(const MarchPlan &mp, size_t elem, int wn, int ms) {
    size_t b = (size_t)mp.NR * (mp.SLX + mp.SLD) * elem + (size_t)mp.nm * (wn + ms) * elem + 2 * elem;
    b = (b + 7) / 8 * 8 + 8;
    return b + (size_t)2 * mp.NR * 8;
}

// The march plan of this operator for a block of b columns of element size `elem`, or false when
// the kernel does not apply (no axis with an offset beyond the first, a plane or column length that
// is not a multiple of 16 bytes, too wide a halo or too many shared entries).
bool march_plan(const kf_op *op, int64_t b, size_t elem, int num_sms, MarchPlan &mp, int mcw) {
    const ApplyPlan &P = op->plan;
    if (P.ne < 1 || P.ndims > MAXDIMS_F || b < 1) return false;
    std::memset(&mp, 0, sizeof(mp));
    int m = -1;
    for (int e = 0; e < P.ne; ++e) {
        const Entry &E = P.e[e];
        if (E.o0 != 0) m = std::max(m, E.a0);
        if (E.nf == 2 && E.o1 != 0) m = std::max(m, E.a1);
    }
    if (m < 1) return false;
    int64_t st = 1;
    for (int a = 0; a < m; ++a) st *= P.dims[a];
    mp.m = m;
    mp.P = (int)st;
    mp.nm = P.dims[m];
    mp.N = P.N;
    mp.nouter = (int)(P.N / ((int64_t)mp.P * mp.nm));
    if (mp.P < 128 || mp.nm < 4) return false;
    const int G = 16 / (int)elem;
    if (P.N % G != 0 || mp.P % G != 0) return false;
    mp.H = 0;
    mp.R = 0;
    for (int e = 0; e < P.ne; ++e) {
        const Entry &E = P.e[e];
        int o = 0;
        bool fin = false, fpl = false;
        auto cls = [&](int a, int off) {
            if (a == m) { o = off; fpl = true; }
            else if (a < m) fin = true;
        };
        cls(E.a0, E.o0);
        if (E.nf == 2) cls(E.a1, E.o1);
        const int r = E.delta - o * mp.P;
        mp.H = std::max(mp.H, std::abs(o));
        mp.R = std::max(mp.R, std::abs(r));
        if (r == 0 && !fin) {
            if (mp.nwin >= MARCH_MAXW) return false;
            mp.win[mp.nwin] = e;
            mp.wino[mp.nwin++] = o;
        } else if (r == 0 && o == 0 && !fpl) {
            if (mp.ncen >= MARCH_MAXC) return false;
            mp.cen[mp.ncen++] = e;
        } else {
            if (mp.nsm >= MARCH_MAXS) return false;
            mp.sm[mp.nsm] = e;
            mp.smr[mp.nsm] = r;
            mp.smo[mp.nsm] = o;
            mp.smpl[mp.nsm++] = fpl ? 1 : 0;
        }
    }
    if (mp.H < 1 || mp.H > 4 || mp.R > 1024) return false;
    // shared entries without a plane factor first; the entries past nsm stay 0 (offset 0, weight 0)
    {
        int ord[MARCH_MAXS], n1 = 0;
        for (int e = 0; e < mp.nsm; ++e) if (!mp.smpl[e]) ord[n1++] = e;
        mp.nsm1 = n1;
        for (int e = 0; e < mp.nsm; ++e) if (mp.smpl[e]) ord[n1++] = e;
        int sm[MARCH_MAXS], smr[MARCH_MAXS], smo[MARCH_MAXS], spl[MARCH_MAXS];
        for (int e = 0; e < mp.nsm; ++e) {
            sm[e] = mp.sm[ord[e]]; smr[e] = mp.smr[ord[e]]; smo[e] = mp.smo[ord[e]]; spl[e] = mp.smpl[ord[e]];
        }
        for (int e = 0; e < mp.nsm; ++e) {
            mp.sm[e] = sm[e]; mp.smr[e] = smr[e]; mp.smo[e] = smo[e]; mp.smpl[e] = spl[e];
        }
    }
    // register budget (128 per thread): up to 8 shared entries (padded to 6 or 8 with zero weights)
    // with 4 FP32 or 2 FP64 points per thread, up to 16 with half as many; with 7 consumer warps
    // (255 registers) 8 FP32 or 4 FP64 points, up to 8 shared entries
    mp.ms = mp.nsm <= 6 ? 6 : mp.nsm <= 8 ? 8 : 16;
    if (mcw != MCW_STD && (mcw != MCW_WIDE || mp.ms > 8)) return false;
    mp.mcw = mcw;
    const int pt = mcw == MCW_WIDE ? (elem == 4 ? 8 : 4) : (elem == 4 ? 4 : 2) / (mp.ms <= 8 ? 1 : 2);
    const int tqmax = 32 * mcw * pt;
    // tiles: at most tqmax points, balanced over the plane, a multiple of 16 bytes
    mp.ntile = (mp.P + tqmax - 1) / tqmax;
    mp.TQ = (mp.P + mp.ntile - 1) / mp.ntile;
    mp.TQ = (mp.TQ + G - 1) / G * G;
    if (mp.TQ > tqmax) { ++mp.ntile; mp.TQ = ((mp.P + mp.ntile - 1) / mp.ntile + G - 1) / G * G; }
    if (mp.TQ > tqmax) return false;
    // a slot spans every point a thread indexes (MCT pt, beyond TQ when the tiles are balanced
    // below it), so the loads of a thread's unused points stay inside the slot
    mp.pt = pt;
    mp.SLX = (tqmax + 2 * mp.R + 2 * G + G - 1) / G * G;
    mp.SLD = (tqmax + 2 * G + G - 1) / G * G;
    // persistent CTAs: one per SM, at least one per (tile, outer) group
    const int64_t groups = (int64_t)mp.ntile * mp.nouter;
    if (groups > (1 << 20)) return false;
    mp.grid = (int)std::max<int64_t>(groups, std::max(num_sms, 1));
    // ring slots within the budget (at least the window and one plane ahead)
    const size_t slot_b = (size_t)(mp.SLX + mp.SLD) * elem;
    const int hk = mp.H == 3 ? 4 : mp.H;      // the kernel's window half-width
    mp.wn = 2 * hk + 1;
    const size_t tab = (size_t)mp.nm * (2 * hk + 1 + mp.ms) * elem + 64;
    if (tab >= (size_t)M_SMEM_BUDGET) return false;
    int nr = (int)((M_SMEM_BUDGET - tab) / (slot_b + 16));
    nr = std::min(nr, 24);
    if (nr < 2 * 4 + 2) return false;        // a halo of 3 runs on the kernel for 4
    mp.NR = nr;
    mp.flat = 1;
    for (int e = 0; e < mp.nsm; ++e) mp.flat = mp.flat && mp.smo[e] == 0;
    mp.nseg = 1;
    mp.L = mp.nm;
    return true;
}

template <typename T>
void launch_apply_march(kf_op *op, const MarchPlan &mp, const T *D, const T *W, const T *X, T *Y, int64_t ldx,
                        int64_t ldy, int64_t b, T alpha, T beta, const T *Z, int64_t ldz, T gamma, int epi,
                        cudaStream_t s) {
    const int slot = sizeof(T) == 4 ? 1 : 0;
    if (op->d_march[slot] == nullptr) {
        const int64_t total = (int64_t)mp.nouter * ((int64_t)(mp.ms + 1) * mp.P + (int64_t)mp.nm * (mp.wn + mp.ms));
        void *p = nullptr;
        KF_CUDA(cudaMalloc(&p, (size_t)total * sizeof(T)));
        k_march_table<T><<<(unsigned)((total + 255) / 256), 256, 0, s>>>(op->plan, mp, W, (T *)p, total);
        KF_LAUNCH_CHECK();
        op->d_march[slot] = p;
    }
    const T *tab = (const T *)op->d_march[slot];
    switch (mp.wn) {
        case 3: launch_h<T, 1>(op, mp, D, W, X, Y, ldx, ldy, b, alpha, beta, Z, ldz, gamma, epi, tab, s); break;
        case 5: launch_h<T, 2>(op, mp, D, W, X, Y, ldx, ldy, b, alpha, beta, Z, ldz, gamma, epi, tab, s); break;
        default: launch_h<T, 4>(op, mp, D, W, X, Y, ldx, ldy, b, alpha, beta, Z, ldz, gamma, epi, tab, s); break;
    }
}

template void launch_apply_march<float>(kf_op *, const MarchPlan &, const float *, const float *, const float *,
                                        float *, int64_t, int64_t, int64_t, float, float, const float *, int64_t,
                                        float, int, cudaStream_t);
template void launch_apply_march<double>(kf_op *, const MarchPlan &, const double *, const double *,
                                         const double *, double *, int64_t, int64_t, int64_t, double, double,
                                         const double *, int64_t, double, int, cudaStream_t);

}  // namespace kf

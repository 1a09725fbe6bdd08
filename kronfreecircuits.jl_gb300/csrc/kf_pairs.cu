// Dense pairwise couplings on a three-axis product basis, in two passes instead of a chain per term.
//
// The parent-level operator of the reference's hierarchical method couples its children through
// their kept-basis port matrices: H = diag + sum over pairs g_ij A_i (x) B_j, every factor a dense
// d_a x d_a matrix (src/apply.jl:301-340 applies each term as a chain of mode products through
// scratch, then accumulates; src/apply.jl:370-393).  With the axes (a, b, c), X[a, b, c] column-major,
// and the pairs (01): g01 A0 (x) B1, (02): g02 C0 (x) E2, (12): g12 F1 (x) G2,
//     Y_c = D_c X_c + g01 A0 X_c B1' + g02 C0 (E2 x_c X)_c + g12 (G2 x_c X)_c F1'
// for every slab c (X_c the d0 x d1 matrix X[:, :, c]).  Pass 1 forms T = E2 x_c X (and G2 x_c X when
// G2 is another matrix) with the tiled mode-product kernel; pass 2 is one kernel over (slab, column)
// units: X_c and the T slabs are staged in shared memory with the coupling matrices (loaded once per
// persistent CTA), and the products run as register-blocked tiles (TM x TM outputs per thread,
// 16 x 16 threads).  When A0 = C0 the two axis-0 products merge: A0 (g01 X_c B1' + g02 T_c).  So X is
// read twice and Y written once, against the chain's 3 (2 reads + 1 write) passes per factor.
#include <algorithm>
#include <cstring>

#include "kf_internal.h"

namespace kf {

namespace {

constexpr int PT_THREADS = 256;

// out(i, j) += sum_k L(i, k) R(k, j) over a d x d tile owned by this thread (rows i0.., cols j0..);
// L column-major with leading dimension ldl; R(k, j) = R[k + ldr j] (RT = false) or R[j + ldr k]
// (RT = true: the transpose of a column-major matrix)
template <typename T, int TM, bool RT>
__device__ __forceinline__ void tile_gemm(T (&acc)[TM][TM], const T *L, int ldl, const T *R, int ldr, int kd, int i0,
                                          int j0) {
    for (int k = 0; k < kd; ++k) {
        T l[TM], r[TM];
#pragma unroll
        for (int u = 0; u < TM; ++u) l[u] = L[i0 + u + ldl * k];
#pragma unroll
        for (int v = 0; v < TM; ++v) r[v] = RT ? R[j0 + v + ldr * k] : R[k + ldr * (j0 + v)];
#pragma unroll
        for (int u = 0; u < TM; ++u)
#pragma unroll
            for (int v = 0; v < TM; ++v) acc[u][v] = fma(l[u], r[v], acc[u][v]);
    }
}

template <typename T, int TM>
__global__ void __launch_bounds__(PT_THREADS) k_pairs(const T *__restrict__ X, int64_t ldx, const T *__restrict__ TE,
                                                      const T *__restrict__ TG, int64_t ldt, T *__restrict__ Y,
                                                      int64_t ldy, const T *__restrict__ D, const T *__restrict__ mats,
                                                      PairPlan pp, int b, int accumulate) {
    extern __shared__ __align__(16) unsigned char p_smem[];
    const int d0 = pp.d[0], d1 = pp.d[1], d2 = pp.d[2];
    const int S = d0 * d1;                       // one slab
    T *sm = reinterpret_cast<T *>(p_smem);
    T *A0 = sm;                                  // d0 x d0
    T *C0 = A0 + d0 * d0;                        // d0 x d0 (A0 when shared)
    T *B1 = C0 + (pp.share0 ? 0 : d0 * d0);      // d1 x d1
    T *F1 = B1 + d1 * d1;                        // d1 x d1 (B1 when shared)
    T *Xs = F1 + (pp.share1 ? 0 : d1 * d1);      // slab of X
    T *Ts = Xs + S;                              // slab of E2 x_c X
    T *Us = Ts + S;                              // slab of G2 x_c X (Ts when shared)
    T *Ws = Us + (pp.share2 ? 0 : S);            // g01 X_c B1' + g02 T_c (merged case)
    if (pp.share0) C0 = A0;
    if (pp.share1) F1 = B1;
    if (pp.share2) Us = Ts;
    const int tid = threadIdx.x;
    const T *mA0 = mats + pp.off[0][0], *mB1 = mats + pp.off[0][1], *mC0 = mats + pp.off[1][0];
    const T *mF1 = mats + pp.off[2][0];
    for (int e = tid; e < d0 * d0; e += PT_THREADS) {
        if (pp.has[0]) A0[e] = mA0[e];
        if (pp.has[1] && !pp.share0) C0[e] = mC0[e];
        else if (pp.has[1] && !pp.has[0]) A0[e] = mC0[e];
    }
    for (int e = tid; e < d1 * d1; e += PT_THREADS) {
        if (pp.has[0]) B1[e] = mB1[e];
        if (pp.has[2] && !pp.share1) F1[e] = mF1[e];
        else if (pp.has[2] && !pp.has[0]) B1[e] = mF1[e];
    }
    const T g01 = (T)pp.g[0], g02 = (T)pp.g[1], g12 = (T)pp.g[2];
    const int i0 = TM * (tid % 16), j0 = TM * (tid / 16);
    const int units = d2 * b;
    for (int u = blockIdx.x; u < units; u += gridDim.x) {
        const int c = u % d2, col = u / d2;
        const int64_t so = (int64_t)c * S;
        __syncthreads();                         // the previous unit's slabs are no longer read
        for (int e = tid; e < S; e += PT_THREADS) {
            Xs[e] = X[(int64_t)col * ldx + so + e];
            if (pp.has[1] || pp.has[2]) Ts[e] = TE[(int64_t)col * ldt + so + e];
            if (pp.has[2] && !pp.share2) Us[e] = TG[(int64_t)col * ldt + so + e];
        }
        __syncthreads();
        T out[TM][TM];
#pragma unroll
        for (int u2 = 0; u2 < TM; ++u2)
#pragma unroll
            for (int v = 0; v < TM; ++v) out[u2][v] = T(0);
        const bool mine = i0 < d0 && j0 < d1;    // d0, d1 are multiples of TM
        // the axis-0 products: A0 (g01 X_c B1') (+ C0 g02 T_c)
        if (pp.has[0]) {
            T v1[TM][TM];
#pragma unroll
            for (int u2 = 0; u2 < TM; ++u2)
#pragma unroll
                for (int v = 0; v < TM; ++v) v1[u2][v] = T(0);
            if (mine) tile_gemm<T, TM, true>(v1, Xs, d0, B1, d1, d1, i0, j0);
            if (mine)
#pragma unroll
                for (int u2 = 0; u2 < TM; ++u2)
#pragma unroll
                    for (int v = 0; v < TM; ++v) {
                        const int i = i0 + u2, j = j0 + v;
                        T w = g01 * v1[u2][v];
                        if (pp.has[1] && pp.share0) w += g02 * Ts[i + d0 * j];
                        Ws[i + d0 * j] = w;
                    }
            __syncthreads();
            if (mine) tile_gemm<T, TM, false>(out, A0, d0, Ws, d0, d0, i0, j0);
        }
        if (pp.has[1] && !(pp.has[0] && pp.share0)) {
            T v1[TM][TM];
#pragma unroll
            for (int u2 = 0; u2 < TM; ++u2)
#pragma unroll
                for (int v = 0; v < TM; ++v) v1[u2][v] = T(0);
            if (mine) tile_gemm<T, TM, false>(v1, C0, d0, Ts, d0, d0, i0, j0);
#pragma unroll
            for (int u2 = 0; u2 < TM; ++u2)
#pragma unroll
                for (int v = 0; v < TM; ++v) out[u2][v] = fma(g02, v1[u2][v], out[u2][v]);
        }
        // the axis-1 product of the (12) pair: (G2 x_c X)_c F1'
        if (pp.has[2]) {
            T v1[TM][TM];
#pragma unroll
            for (int u2 = 0; u2 < TM; ++u2)
#pragma unroll
                for (int v = 0; v < TM; ++v) v1[u2][v] = T(0);
            if (mine) tile_gemm<T, TM, true>(v1, Us, d0, F1, d1, d1, i0, j0);
#pragma unroll
            for (int u2 = 0; u2 < TM; ++u2)
#pragma unroll
                for (int v = 0; v < TM; ++v) out[u2][v] = fma(g12, v1[u2][v], out[u2][v]);
        }
        if (mine) {
#pragma unroll
            for (int u2 = 0; u2 < TM; ++u2)
#pragma unroll
                for (int v = 0; v < TM; ++v) {
                    const int i = i0 + u2, j = j0 + v;
                    const int64_t p = so + i + (int64_t)d0 * j;
                    T r = out[u2][v];
                    if (D != nullptr) r = fma(D[p], Xs[i + d0 * j], r);
                    T *yp = Y + (int64_t)col * ldy + p;
                    *yp = accumulate ? *yp + r : r;
                }
        }
    }
}

}  // namespace

// the shared memory the pass-2 kernel needs for this plan (at most 200 KB applies)
size_t pairs_smem_bytes(const PairPlan &pp, size_t elem) {
    const size_t S = (size_t)pp.d[0] * pp.d[1];
    size_t n = (size_t)pp.d[0] * pp.d[0] * (pp.share0 ? 1 : 2) + (size_t)pp.d[1] * pp.d[1] * (pp.share1 ? 1 : 2);
    n += S * (pp.share2 ? 3 : 4);
    return n * elem;
}

// Y = (accumulate ? Y : 0) + (D ? D X : 0) + the pair terms, for b columns; scratch: 2 N b elements
template <typename T>
void apply_pairs(const kf_op *op, const T *X, int64_t ldx, T *Y, int64_t ldy, int64_t b, const T *D, int accumulate,
                 T *scratch, cudaStream_t s) {
    const PairPlan &pp = op->pairs;
    const int64_t N = op->N;
    const T *mats = sizeof(T) == 4 ? (const T *)op->d_chain32 : (const T *)op->d_chain64;
    const int64_t left = (int64_t)pp.d[0] * pp.d[1];
    T *TE = scratch, *TG = scratch + N * b;
    if (pp.has[1]) mode_product<T>(TE, N, X, ldx, mats + pp.off[1][1], pp.d[2], left, N, b, 1.0, 0.0, s);
    if (pp.has[2] && !pp.share2) mode_product<T>(TG, N, X, ldx, mats + pp.off[2][1], pp.d[2], left, N, b, 1.0, 0.0, s);
    if (pp.has[2] && pp.share2) TG = TE;
    if (pp.has[2] && !pp.has[1]) {
        mode_product<T>(TE, N, X, ldx, mats + pp.off[2][1], pp.d[2], left, N, b, 1.0, 0.0, s);
        TG = TE;
    }
    const size_t smem = pairs_smem_bytes(pp, sizeof(T));
    int sms = 0;
    KF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, op->device));
    const int64_t units = (int64_t)pp.d[2] * b;
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(units, (int64_t)sms * 2));
    const int dmax = std::max(pp.d[0], pp.d[1]);
    auto go = [&](auto kern) {
        KF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<grid, PT_THREADS, smem, s>>>(X, ldx, TE, TG, N, Y, ldy, D, mats, pp, (int)b, accumulate);
        KF_LAUNCH_CHECK();
    };
    if (dmax <= 32) go(k_pairs<T, 2>);
    else if (dmax <= 48) go(k_pairs<T, 3>);
    else go(k_pairs<T, 4>);
}

template void apply_pairs<float>(const kf_op *, const float *, int64_t, float *, int64_t, int64_t, const float *, int,
                                 float *, cudaStream_t);
template void apply_pairs<double>(const kf_op *, const double *, int64_t, double *, int64_t, int64_t, const double *,
                                  int, double *, cudaStream_t);

// The pair plan of an operator's dense-chain terms (PairPlan::ok = 0 when they are not all pairs of
// dense factors on distinct axes of a three-axis basis with d <= 64, one term per axis pair, each
// axis length a multiple of the register tile).  hdata: the host copies of the chain factors' data
// in chain order (to recognise shared matrices).
void pairs_plan(kf_op *op, const std::vector<std::vector<double>> &hdata) {
    PairPlan &pp = op->pairs;
    std::memset(&pp, 0, sizeof(pp));
    if (op->dims.size() != 3 || op->chains.empty()) return;
    for (int a = 0; a < 3; ++a) {
        pp.d[a] = (int)op->dims[a];
        if (pp.d[a] > 64) return;
    }
    const int dmax = std::max(pp.d[0], pp.d[1]);
    const int tm = dmax <= 32 ? 2 : dmax <= 48 ? 3 : 4;
    if (pp.d[0] % tm || pp.d[1] % tm || 16 * tm < dmax) return;
    std::vector<const std::vector<double> *> data[3][2];
    size_t q = 0;
    for (const ChainTerm &ct : op->chains) {
        if (ct.f.size() != 2 || ct.f[0].kind != KF_DENSE || ct.f[1].kind != KF_DENSE) return;
        const int a0 = ct.f[0].axis, a1 = ct.f[1].axis;
        const int pr = (a0 == 0 && a1 == 1) ? 0 : (a0 == 0 && a1 == 2) ? 1 : (a0 == 1 && a1 == 2) ? 2 : -1;
        if (pr < 0 || pp.has[pr]) return;
        pp.has[pr] = 1;
        pp.g[pr] = ct.coeff;
        pp.off[pr][0] = ct.f[0].data_off;
        pp.off[pr][1] = ct.f[1].data_off;
        data[pr][0].push_back(&hdata[q]);
        data[pr][1].push_back(&hdata[q + 1]);
        q += 2;
    }
    auto same = [&](int p1, int s1, int p2, int s2) {
        return pp.has[p1] && pp.has[p2] && *data[p1][s1][0] == *data[p2][s2][0];
    };
    pp.share0 = !(pp.has[0] && pp.has[1]) || same(0, 0, 1, 0);   // A0 = C0 (or only one of them)
    pp.share1 = !(pp.has[0] && pp.has[2]) || same(0, 1, 2, 0);   // B1 = F1
    pp.share2 = !(pp.has[1] && pp.has[2]) || same(1, 1, 2, 1);   // E2 = G2
    pp.ok = 1;
}

}  // namespace kf

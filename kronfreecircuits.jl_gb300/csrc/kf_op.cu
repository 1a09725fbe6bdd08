// The Kronecker-free operator: construction from the C descriptor and the apply kernels.
//
// Reference semantics (KronFreeCircuits.jl):
//   src/apply.jl:222-253   construction; all-diagonal terms fused with the constant into one diagonal
//   src/apply.jl:416-432   mul!(Y, H, X) = diag .* X + sum over kept terms of coeff * (chain of factors) X
//   src/apply.jl:66-79     banded factor:  Y[t] = sum_b W[i_k, b] X[t + off_b * stride_k] (valid rows)
//   src/apply.jl:111-118   shift factor:   Y[t] = f X[t - s * stride_k] (valid rows)
//   src/apply.jl:301-340   dense factor:   the mode-k product with a d_k x d_k matrix
//
// GB300 design.  Every non-dense factor is a banded operator (a diagonal is one band at offset
// 0, a shift one band at offset -s), so every term built only of such factors is a product of
// banded operators, and all of them are evaluated in ONE pass over X: each thread owns one state
// index p, decodes its axis indices once, and for a chunk of CB columns accumulates
//   D[p] X[p] + sum_terms sum_bands (prod_f w_f[i_f, b_f]) X[p + sum_f off_f stride_f]
// in registers, so X is read from HBM once and Y written once per apply (the neighbour reads hit
// L1/L2: along the slowest stencil axis the planes p +- k*stride are read by CTAs resident a few
// waves apart).  The reference's one-pass-per-factor-plus-one-accumulate-pass structure
// (1 + sum_t (f_t + 1) passes) collapses to one pass.  Terms with dense factors run as chains of
// single-axis kernels through two scratch blocks, the last factor accumulating into Y.
#include <algorithm>
#include <cstring>
#include <map>

#include <mutex>
#include <string>
#include "kf_internal.h"

namespace kf {

// ------------------------------------------------------------------------------------------
// kernels

// The per-axis index of the state point p: idx[a] for a < ndims (static indexing only).
__device__ __forceinline__ int pick(const int (&idx)[MAXDIMS_F], int a) {
    int v = idx[0];
#pragma unroll
    for (int k = 1; k < MAXDIMS_F; ++k) v = (a == k) ? idx[k] : v;
    return v;
}

// Y = D X + sum_entries w_e X[p + delta_e]  (then the epilogue Y = alpha Y + beta X + gamma Z).
// One thread per state point p and group of CPT columns (blockIdx.y); the point's entry weights
// and offsets are evaluated once into registers (ME >= ne, fully unrolled) and reused for its
// columns.  (CPT, U) is chosen per operator by timing the candidates on its first apply.
template <typename T, int CPT, int U, int ME>
__global__ void __launch_bounds__(256, 2) k_apply_fused(const ApplyPlan plan, const T *__restrict__ D,
                                                     const T *__restrict__ W, const T *__restrict__ X,
                                                     T *__restrict__ Y, int64_t ldx, int64_t ldy, int b,
                                                     T alpha, T beta, const T *__restrict__ Z, int64_t ldz,
                                                     T gamma, int epi) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= plan.N) return;
    int idx[MAXDIMS_F];
    {
        int rem = p;
#pragma unroll
        for (int a = 0; a < MAXDIMS_F; ++a) {
            if (a < plan.ndims) {
                idx[a] = rem % plan.dims[a];
                rem /= plan.dims[a];
            } else {
                idx[a] = 0;
            }
        }
    }
    T w[ME];
    int off[ME];
#pragma unroll
    for (int e = 0; e < ME; ++e) {
        w[e] = T(0);
        off[e] = 0;
        if (e < plan.ne) {
            const Entry &E = plan.e[e];
            const int i0 = pick(idx, E.a0);
            bool ok = (unsigned)(i0 + E.o0) < (unsigned)E.n0;
            T wv = ok ? __ldg(W + E.w0 + i0 * E.nb0) : T(0);
            if (E.nf == 2) {
                const int i1 = pick(idx, E.a1);
                const bool ok1 = (unsigned)(i1 + E.o1) < (unsigned)E.n1;
                wv = ok1 ? wv * __ldg(W + E.w1 + i1 * E.nb1) : T(0);
                ok = ok && ok1;
            }
            w[e] = ok ? wv : T(0);
            off[e] = ok ? E.delta : 0;
        }
    }
    const T dv = D[p];
    // this thread's columns [blockIdx.y * CPT, ... + CPT), U of them at a time: the U columns'
    // ne neighbour loads are independent and all in flight together
    const int cbeg = blockIdx.y * CPT;
    const int cend = min(b, cbeg + CPT);
    for (int c0 = cbeg; c0 < cend; c0 += U) {
        T v[U];
        const T *xc[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int c = (c0 + u < cend) ? c0 + u : c0;
            xc[u] = X + (int64_t)c * ldx + p;
            v[u] = dv * xc[u][0];
        }
        // unconditional loads: an invalid entry has weight 0 and offset 0 (a valid address)
#pragma unroll
        for (int e = 0; e < ME; ++e) {
            if (e < plan.ne) {
#pragma unroll
                for (int u = 0; u < U; ++u) v[u] += w[e] * __ldg(xc[u] + off[e]);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int c = c0 + u;
            if (c >= cend) break;
            T r = v[u];
            if (epi) {
                r = alpha * r + beta * xc[u][0];
                if (Z != nullptr) r += gamma * Z[(int64_t)c * ldz + p];
            }
            Y[(int64_t)c * ldy + p] = r;
        }
    }
}

// dst = alpha * (banded factor along an axis) src  (+ dst when acc); blocks of b columns with
// leading dimensions ldd, lds.
template <typename T>
__global__ void k_axis_banded(T *__restrict__ dst, int64_t ldd, const T *__restrict__ src, int64_t lds,
                              const T *__restrict__ W, ChainFactor f, int64_t stride, int64_t N, int64_t total,
                              T alpha, int acc) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int64_t c = t / N, p = t % N;
    const int i = (int)((p / stride) % f.n);
    const T *sp = src + c * lds + p;
    T s = 0;
    for (int bb = 0; bb < f.nb; ++bb) {
        const int j = i + f.off[bb];
        if (j < 0 || j >= f.n) continue;
        s += W[(int64_t)i * f.nb + bb] * sp[(int64_t)f.off[bb] * stride];
    }
    s *= alpha;
    T *dp = dst + c * ldd + p;
    *dp = acc ? *dp + s : s;
}

// dst[l, i, r] = alpha * sum_j A[i, j] src[l, j, r]  (+ dst when acc); A column-major n x n,
// `left` the stride of the axis; per column of the block (leading dimensions ldd, lds).
template <typename T>
__global__ void k_axis_dense(T *__restrict__ dst, int64_t ldd, const T *__restrict__ src, int64_t lds,
                             const T *__restrict__ A, int n, int64_t left, int64_t N, int64_t total, T alpha,
                             int acc) {
    extern __shared__ unsigned char smem_raw[];
    T *As = reinterpret_cast<T *>(smem_raw);
    const bool use_smem = (int64_t)n * n * sizeof(T) <= 48 * 1024;
    if (use_smem) {
        for (int k = threadIdx.x; k < n * n; k += blockDim.x) As[k] = A[k];
        __syncthreads();
    }
    const T *Ap = use_smem ? As : A;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int64_t c = t / N, p = t % N;
    const int64_t l = p % left;
    const int64_t q = p / left;
    const int i = (int)(q % n);
    const int64_t r = q / n;
    const T *sp = src + c * lds + l + left * ((int64_t)n * r);
    T s = 0;
    for (int j = 0; j < n; ++j) s += Ap[i + (int64_t)n * j] * sp[left * j];
    s *= alpha;
    T *dp = dst + c * ldd + p;
    *dp = acc ? *dp + s : s;
}

template <typename T>
__global__ void k_axpby_cols(T *__restrict__ Y, int64_t ldy, const T *__restrict__ X, int64_t ldx,
                             const T *__restrict__ Z, int64_t ldz, int64_t N, int b, T alpha, T beta, T gamma) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * b) return;
    const int64_t c = t / N, p = t % N;
    T v = alpha * Y[c * ldy + p] + beta * X[c * ldx + p];
    if (Z != nullptr) v += gamma * Z[c * ldz + p];
    Y[c * ldy + p] = v;
}

// ------------------------------------------------------------------------------------------
// host launch

// fused-apply variant chosen per (device, stencil shape, precision and width class)
static std::mutex g_tune_mu;
static std::map<std::string, int> g_tune;

static std::string tune_key(const kf_op *op, int width) {
    const ApplyPlan &P = op->plan;
    std::string k = std::to_string(op->device) + ":" + std::to_string(width) + ":" + std::to_string(P.N) + ":" +
                    std::to_string(P.ne);
    for (int a = 0; a < P.ndims; ++a) k += "," + std::to_string(P.dims[a]);
    for (int e = 0; e < P.ne; ++e) {
        const Entry &E = P.e[e];
        k += ";" + std::to_string(E.nf) + "/" + std::to_string(E.a0) + "/" + std::to_string(E.o0) + "/" +
             std::to_string(E.a1) + "/" + std::to_string(E.o1);
    }
    return k;
}

// the tuner's width class of a block of b columns (classes of four columns; widths above 64 share one)
static int tune_class(bool f32, int64_t b) { return (f32 ? 1 << 20 : 0) | (int)((std::min<int64_t>(b, 65) + 3) / 4); }

// streaming multiprocessors of a device (cached per device)
static int num_sms(int dev) {
    static std::mutex mu;
    static std::map<int, int> cache;
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    int v = 0;
    KF_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
    cache[dev] = v;
    return v;
}

template <typename T>
static void apply_t(kf_op *op, const T *X, T *Y, int64_t ldx, int64_t ldy, int64_t b, double alpha, double beta,
                    const T *Z, int64_t ldz, double gamma, cudaStream_t s) {
    const int64_t N = op->N;
    const bool f32 = sizeof(T) == 4;
    const T *D = f32 ? (const T *)op->d_diag32 : (const T *)op->d_diag64;
    const T *W = f32 ? (const T *)op->d_w32 : (const T *)op->d_w64;
    const bool chains = !op->chains.empty();
    const bool trivial_epi = alpha == 1.0 && beta == 0.0 && (Z == nullptr || gamma == 0.0);
    const int epi = (!chains && !trivial_epi) ? 1 : 0;
    // dense pairwise couplings: two passes (kf_pairs.cu) instead of the chains; without banded or
    // shift terms the pair kernel also forms D X, so the fused pass is skipped
    const bool pairs = chains && op->pairs.ok && pairs_smem_bytes(op->pairs, sizeof(T)) <= 200 * 1024;
    auto chain_scratch = [&]() -> T * {
        const size_t need = (size_t)2 * op->N * b * sizeof(T);
        if (op->scratch_bytes < need) {
            if (op->d_scratch) KF_CUDA(cudaFree(op->d_scratch));
            op->d_scratch = nullptr;
            op->scratch_bytes = 0;
            KF_CUDA(cudaMalloc(&op->d_scratch, need));
            op->scratch_bytes = need;
        }
        return (T *)op->d_scratch;
    };
    if (pairs && op->plan.ne == 0 && op->force_variant < 0) {
        apply_pairs<T>(op, X, ldx, Y, ldy, b, D, 0, chain_scratch(), s);
        if (!trivial_epi) {
            const unsigned g2 = (unsigned)((N * b + 255) / 256);
            k_axpby_cols<T><<<g2, 256, 0, s>>>(Y, ldy, X, ldx, Z, ldz, N, (int)b, (T)alpha, (T)beta, (T)gamma);
            KF_LAUNCH_CHECK();
        }
        return;
    }
    const int ne = op->plan.ne;
    // the plane-marching kernel where its geometry applies and X is 16-byte aligned: variant 5 with 12
    // consumer warps, variant 7 with 7 and twice the points per thread
    MarchPlan mp, mpw;
    const int G = 16 / (int)sizeof(T);
    const bool aligned = ldx % G == 0 && (uintptr_t)X % 16 == 0 && (uintptr_t)D % 16 == 0;
    const bool march_ok = aligned && march_plan(op, b, sizeof(T), num_sms(op->device), mp);
    const bool march_wide_ok = march_ok && march_plan(op, b, sizeof(T), num_sms(op->device), mpw, 7);
    auto run = [&](int variant) {
        if ((variant == 5 && march_ok) || (variant == 7 && march_wide_ok)) {
            launch_apply_march<T>(op, variant == 7 ? mpw : mp, D, W, X, Y, ldx, ldy, b, (T)alpha, (T)beta, Z, ldz,
                                  (T)gamma, epi, s);
            return;
        }
#define KF_FUSED(CPT, U, ME)                                                                                  \
    k_apply_fused<T, CPT, U, ME><<<dim3((unsigned)((N + 255) / 256), (unsigned)((b + CPT - 1) / CPT)), 256, 0, s>>>( \
        op->plan, D, W, X, Y, ldx, ldy, (int)b, (T)alpha, (T)beta, Z, ldz, (T)gamma, epi)
#define KF_VARIANTS(ME)                                  \
    switch (variant) {                                   \
        case 0: KF_FUSED(16, 1, ME); break;              \
        case 1: KF_FUSED(16, 2, ME); break;              \
        case 2: KF_FUSED(8, 2, ME); break;               \
        case 3: KF_FUSED(4, 4, ME); break;               \
        case 6: KF_FUSED(36, 1, ME); break;              \
        default: KF_FUSED(32, 1, ME); break;             \
    }
        if (ne <= 16) { KF_VARIANTS(16) } else if (ne <= 32) { KF_VARIANTS(32) } else { KF_VARIANTS(48) }
#undef KF_VARIANTS
#undef KF_FUSED
        KF_LAUNCH_CHECK();
    };
    // autotune: on the first apply of a block in this width class (per precision; classes of four
    // columns, widths above 64 share one), time every variant on the caller's own buffers (each
    // overwrites Y completely with the same result) and keep the fastest; each variant's time is the
    // best of three batches of four launches.  Classes rather than exact widths: locking shrinks
    // the active block one column at a time, and a tuning costs about 80 launches
    const int wkey = tune_class(f32, b);
    if (op->force_variant >= 0) {
        run(op->force_variant);
        goto chained;
    }
    {
        auto hit = op->apply_tuned.find(wkey);
        int chosen = hit != op->apply_tuned.end() ? hit->second : -1;
        if (chosen < 0) {
            // operators of the same stencil shape (a parameter sweep rebuilds the same structure
            // with new coefficients) share one tuning per process and device
            const std::string key = tune_key(op, wkey);
            {
                std::lock_guard<std::mutex> lk(g_tune_mu);
                auto it = g_tune.find(key);
                if (it != g_tune.end()) chosen = it->second;
            }
            if (chosen < 0) {
                cudaEvent_t e0, e1;
                KF_CUDA(cudaEventCreate(&e0));
                KF_CUDA(cudaEventCreate(&e1));
                float best = 1e30f;
                int bestv = 0;
                for (int v = 0; v < KF_APPLY_VARIANTS; ++v) {
                    if ((v == 5 && !march_ok) || (v == 7 && !march_wide_ok)) continue;
                    run(v);                                   // warm
                    float vbest = 1e30f;
                    for (int batch = 0; batch < 3; ++batch) {
                        KF_CUDA(cudaEventRecord(e0, s));
                        for (int r = 0; r < 4; ++r) run(v);
                        KF_CUDA(cudaEventRecord(e1, s));
                        KF_CUDA(cudaEventSynchronize(e1));
                        float ms = 0;
                        KF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                        vbest = std::min(vbest, ms);
                    }
                    if (vbest < best) { best = vbest; bestv = v; }
                }
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                chosen = bestv;
                std::lock_guard<std::mutex> lk(g_tune_mu);
                g_tune[key] = bestv;
            }
            op->apply_tuned[wkey] = chosen;
        }
        run(chosen);
    }
chained:
    if (!chains) return;
    if (pairs) {
        apply_pairs<T>(op, X, ldx, Y, ldy, b, nullptr, 1, chain_scratch(), s);
        if (!trivial_epi) {
            const unsigned g3 = (unsigned)((N * b + 255) / 256);
            k_axpby_cols<T><<<g3, 256, 0, s>>>(Y, ldy, X, ldx, Z, ldz, N, (int)b, (T)alpha, (T)beta, (T)gamma);
            KF_LAUNCH_CHECK();
        }
        return;
    }
    // dense-containing terms: chain through scratch, one contiguous (N x b) block per buffer
    T *sbuf = chain_scratch();
    T *buf[2] = {sbuf, sbuf + N * b};
    const T *cdata = f32 ? (const T *)op->d_chain32 : (const T *)op->d_chain64;
    const int64_t total = N * b;
    const unsigned g2 = (unsigned)((total + 255) / 256);
    for (const ChainTerm &ct : op->chains) {
        const T *src = X;
        int64_t lds = ldx;
        const int nf = (int)ct.f.size();
        for (int k = 0; k < nf; ++k) {
            const ChainFactor &f = ct.f[k];
            const bool last = k == nf - 1;
            T *dst = last ? Y : buf[k & 1];
            const int64_t ldd = last ? ldy : N;
            const T a = last ? (T)ct.coeff : T(1);
            const int acc = last ? 1 : 0;
            const int64_t stride = op->strides[f.axis];
            if (f.kind == KF_DENSE) {
                // the mode-k product (accumulating into Y for the last factor): on the tensor cores
                // for FP32 blocks when the factor has an image, else a SIMT tiled GEMM
                if constexpr (sizeof(T) == 4) {
                    if (f.tc >= 0) {
                        tc_mode_product((float *)dst, ldd, (const float *)src, lds, op->chain_tc[f.tc], stride, N, b,
                                        (double)a, acc ? 1.0 : 0.0, s);
                        src = dst;
                        lds = ldd;
                        continue;
                    }
                }
                mode_product<T>(dst, ldd, src, lds, cdata + f.data_off, f.n, stride, N, b, (double)a, acc ? 1.0 : 0.0,
                                s);
                src = dst;
                lds = ldd;
                continue;
            } else {
                k_axis_banded<T><<<g2, 256, 0, s>>>(dst, ldd, src, lds, cdata + f.data_off, f, stride, N, total, a, acc);
            }
            KF_LAUNCH_CHECK();
            src = dst;
            lds = ldd;
        }
    }
    if (!trivial_epi) {
        k_axpby_cols<T><<<g2, 256, 0, s>>>(Y, ldy, X, ldx, Z, ldz, N, (int)b, (T)alpha, (T)beta, (T)gamma);
        KF_LAUNCH_CHECK();
    }
}

// Y = H X with the chain scratch supplied by the caller (2 N b elements of T) instead of the op's
// lazily allocated buffer; the same kernels as apply_t, no epilogue.  Used by the allocation-free
// entry point (kf_noalloc.cu).
template <typename T>
void apply_given_scratch(kf_op *op, const T *X, T *Y, int64_t ldx, int64_t ldy, int64_t b, T *scratch,
                         cudaStream_t s) {
    const int64_t N = op->N;
    if (b <= 0 || N == 0) return;
    const bool f32 = sizeof(T) == 4;
    const T *D = f32 ? (const T *)op->d_diag32 : (const T *)op->d_diag64;
    const T *W = f32 ? (const T *)op->d_w32 : (const T *)op->d_w64;
    const dim3 grid((unsigned)((N + 255) / 256), (unsigned)((b + 15) / 16));
    const int ne = op->plan.ne;
#define KF_FUSED2(ME)                                                                                     \
    k_apply_fused<T, 16, 1, ME><<<grid, 256, 0, s>>>(op->plan, D, W, X, Y, ldx, ldy, (int)b, T(1), T(0), nullptr, \
                                                 (int64_t)0, T(0), 0)
    if (ne <= 16) KF_FUSED2(16); else if (ne <= 32) KF_FUSED2(32); else KF_FUSED2(48);
#undef KF_FUSED2
    KF_LAUNCH_CHECK();
    if (op->chains.empty()) return;
    T *buf[2] = {scratch, scratch + N * b};
    const T *cdata = f32 ? (const T *)op->d_chain32 : (const T *)op->d_chain64;
    const int64_t total = N * b;
    const unsigned g2 = (unsigned)((total + 255) / 256);
    for (const ChainTerm &ct : op->chains) {
        const T *src = X;
        int64_t lds = ldx;
        const int nf = (int)ct.f.size();
        for (int k = 0; k < nf; ++k) {
            const ChainFactor &f = ct.f[k];
            const bool last = k == nf - 1;
            T *dst = last ? Y : buf[k & 1];
            const int64_t ldd = last ? ldy : N;
            const T a = last ? (T)ct.coeff : T(1);
            const int acc = last ? 1 : 0;
            const int64_t stride = op->strides[f.axis];
            if (f.kind == KF_DENSE) {
                // the mode-k product as a tiled GEMM (accumulating into Y for the last factor)
                mode_product<T>(dst, ldd, src, lds, cdata + f.data_off, f.n, stride, N, b, (double)a, acc ? 1.0 : 0.0,
                                s);
                src = dst;
                lds = ldd;
                continue;
            } else {
                k_axis_banded<T><<<g2, 256, 0, s>>>(dst, ldd, src, lds, cdata + f.data_off, f, stride, N, total, a, acc);
            }
            KF_LAUNCH_CHECK();
            src = dst;
            lds = ldd;
        }
    }
}

template void apply_given_scratch<float>(kf_op *, const float *, float *, int64_t, int64_t, int64_t, float *,
                                         cudaStream_t);
template void apply_given_scratch<double>(kf_op *, const double *, double *, int64_t, int64_t, int64_t, double *,
                                          cudaStream_t);

void launch_apply(kf_op *op, bool f32, const void *X, void *Y, int64_t ldx, int64_t ldy, int64_t b, double alpha,
                  double beta, const void *Z, int64_t ldz, double gamma, cudaStream_t s) {
    if (b <= 0 || op->N == 0) return;
    KF_REQUIRE(b <= 65535, KF_EINVAL, "mul!: at most 65535 columns per call");
    if (f32)
        apply_t<float>(op, (const float *)X, (float *)Y, ldx, ldy, b, alpha, beta, (const float *)Z, ldz, gamma, s);
    else
        apply_t<double>(op, (const double *)X, (double *)Y, ldx, ldy, b, alpha, beta, (const double *)Z, ldz, gamma, s);
}

void pretune_apply(kf_op *op, bool f32, const void *X, void *Y, int64_t ld, int maxb, cudaStream_t s) {
    if (op->force_variant >= 0 || op->N == 0) return;
    const bool pairs = !op->chains.empty() && op->pairs.ok &&
                       pairs_smem_bytes(op->pairs, f32 ? 4 : 8) <= 200 * 1024;
    if (pairs && op->plan.ne == 0) return;   // the pair kernel is not tuned
    for (int b = 4; b < maxb + 4; b += 4) {
        const int bb = std::min(b, maxb);
        const int wkey = tune_class(f32, bb);
        if (op->apply_tuned.count(wkey)) continue;
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            auto it = g_tune.find(tune_key(op, wkey));
            if (it != g_tune.end()) {
                op->apply_tuned[wkey] = it->second;
                continue;
            }
        }
        launch_apply(op, f32, X, Y, ld, ld, bb, 1, 0, nullptr, 0, 0, s);
    }
}

// ------------------------------------------------------------------------------------------
// construction

namespace {

// A factor in banded form on the host: offsets and per-row weights w[i*nb + b], zero where the
// neighbour i + off leaves the axis.
struct HBand {
    int axis;
    int n;
    std::vector<int> off;
    std::vector<double> w;     // n * nb, row-major
    int nb() const { return (int)off.size(); }
};

HBand to_band(const kf_factor &f) {
    HBand h;
    h.axis = f.axis;
    h.n = (int)f.n;
    const int n = h.n;
    if (f.kind == KF_DIAG) {
        h.off = {0};
        h.w.assign(f.data, f.data + n);
    } else if (f.kind == KF_SHIFT) {
        // Y[i + s] = f X[i]  <=>  Y[i] = f X[i - s]: one band at offset -s
        h.off = {(int)(-f.shift)};
        h.w.assign(n, 0.0);
        for (int i = 0; i < n; ++i)
            if (i - f.shift >= 0 && i - f.shift < n) h.w[i] = f.factor;
    } else {  // banded
        const int nb = f.nbands;
        h.off.resize(nb);
        h.w.assign((size_t)n * nb, 0.0);
        for (int bb = 0; bb < nb; ++bb) {
            h.off[bb] = (int)f.offsets[bb];
            for (int i = 0; i < n; ++i) {
                const int64_t j = (int64_t)i + f.offsets[bb];
                if (j >= 0 && j < n) h.w[(size_t)i * nb + bb] = f.data[(size_t)bb * n + i];
            }
        }
    }
    return h;
}

// Sum two banded factors on the same axis into one (union of offsets).
HBand band_sum(const HBand &a, double ca, const HBand &b, double cb) {
    HBand r;
    r.axis = a.axis;
    r.n = a.n;
    r.off = a.off;
    for (int o : b.off)
        if (std::find(r.off.begin(), r.off.end(), o) == r.off.end()) r.off.push_back(o);
    std::sort(r.off.begin(), r.off.end());
    const int nb = r.nb();
    r.w.assign((size_t)r.n * nb, 0.0);
    auto add = [&](const HBand &h, double c) {
        for (int bb = 0; bb < h.nb(); ++bb) {
            const int k = (int)(std::find(r.off.begin(), r.off.end(), h.off[bb]) - r.off.begin());
            for (int i = 0; i < r.n; ++i) r.w[(size_t)i * nb + k] += c * h.w[(size_t)i * h.nb() + bb];
        }
    };
    add(a, ca);
    add(b, cb);
    return r;
}

bool same_band(const HBand &a, const HBand &b) { return a.axis == b.axis && a.off == b.off && a.w == b.w; }

struct HTerm {
    double coeff;
    std::vector<HBand> f;
};

// Merge fused terms: two terms on the same axes whose factors agree on every axis but one become
// one term, the differing axis summed (S+ (x) cos + S- (x) cos -> (S+ + S-) (x) cos).
void merge_terms(std::vector<HTerm> &ts) {
    bool changed = true;
    while (changed) {
        changed = false;
        for (size_t x = 0; x < ts.size() && !changed; ++x) {
            for (size_t y = x + 1; y < ts.size() && !changed; ++y) {
                HTerm &A = ts[x], &B = ts[y];
                if (A.f.size() != B.f.size()) continue;
                bool axes_eq = true;
                for (size_t k = 0; k < A.f.size(); ++k) axes_eq = axes_eq && A.f[k].axis == B.f[k].axis;
                if (!axes_eq) continue;
                int diff = -1, ndiff = 0;
                for (size_t k = 0; k < A.f.size(); ++k)
                    if (!same_band(A.f[k], B.f[k])) { diff = (int)k; ++ndiff; }
                if (ndiff > 1) continue;
                if (ndiff == 0) {
                    A.coeff += B.coeff;
                } else {
                    A.f[diff] = band_sum(A.f[diff], A.coeff, B.f[diff], B.coeff);
                    A.coeff = 1.0;
                }
                ts.erase(ts.begin() + y);
                changed = true;
            }
        }
    }
}

double band_infnorm(const kf_factor &f) {
    const int64_t n = f.n;
    double m = 0;
    if (f.kind == KF_DIAG) {
        for (int64_t i = 0; i < n; ++i) m = std::max(m, std::fabs(f.data[i]));
    } else if (f.kind == KF_SHIFT) {
        m = (std::llabs(f.shift) < n) ? std::fabs(f.factor) : 0.0;
    } else if (f.kind == KF_BANDED) {
        for (int64_t i = 0; i < n; ++i) {
            double r = 0;
            for (int bb = 0; bb < f.nbands; ++bb) {
                const int64_t j = i + f.offsets[bb];
                if (j >= 0 && j < n) r += std::fabs(f.data[(size_t)bb * n + i]);
            }
            m = std::max(m, r);
        }
    } else {
        for (int64_t i = 0; i < n; ++i) {
            double r = 0;
            for (int64_t j = 0; j < n; ++j) r += std::fabs(f.data[i + n * j]);
            m = std::max(m, r);
        }
    }
    return m;
}

std::vector<double> factor_diagonal(const kf_factor &f) {
    const int64_t n = f.n;
    std::vector<double> d(n, 0.0);
    if (f.kind == KF_DIAG) {
        d.assign(f.data, f.data + n);
    } else if (f.kind == KF_SHIFT) {
        if (f.shift == 0) d.assign(n, f.factor);
    } else if (f.kind == KF_BANDED) {
        for (int bb = 0; bb < f.nbands; ++bb)
            if (f.offsets[bb] == 0) { d.assign(f.data + (size_t)bb * n, f.data + (size_t)(bb + 1) * n); break; }
    } else {
        for (int64_t i = 0; i < n; ++i) d[i] = f.data[i + n * i];
    }
    return d;
}

// acc[p] += c * prod over factors of vec_f[i_axis(p)]
// acc[p] += c * prod_f v_f[i_{axis_f}(p)] over the grid (axis 0 fastest).  The factors before the
// first one on axis 0 are constant along a run of axis 0, so each run is one scalar times the rest:
// an inner loop the compiler vectorises, the odometer over the other axes stepping once per run.
// The product is formed in the factors' order, as a point-by-point evaluation would.
void add_separable(std::vector<double> &acc, const std::vector<int64_t> &dims, double c,
                   const std::vector<std::pair<int, std::vector<double>>> &vecs) {
    const int64_t N = (int64_t)acc.size();
    const int nd = (int)dims.size();
    const int64_t d0 = dims[0];
    const int nf = (int)vecs.size();
    std::vector<int64_t> idx(nd, 0);
    int f0 = nf;   // the first factor on axis 0
    for (int k = 0; k < nf; ++k)
        if (vecs[k].first == 0) { f0 = k; break; }
    double *out = acc.data();
    for (int64_t p0 = 0; p0 < N; p0 += d0) {
        double pre = c;
        for (int k = 0; k < f0; ++k) pre *= vecs[k].second[idx[vecs[k].first]];
        double *row = out + p0;
        if (f0 == nf) {
            for (int64_t i = 0; i < d0; ++i) row[i] += pre;
        } else if (f0 == nf - 1) {
            const double *v0 = vecs[f0].second.data();
            for (int64_t i = 0; i < d0; ++i) row[i] += pre * v0[i];
        } else {
            for (int64_t i = 0; i < d0; ++i) {
                double v = pre;
                for (int k = f0; k < nf; ++k) v *= vecs[k].second[vecs[k].first == 0 ? i : idx[vecs[k].first]];
                row[i] += v;
            }
        }
        for (int a = 1; a < nd; ++a) {
            if (++idx[a] < dims[a]) break;
            idx[a] = 0;
        }
    }
}

}  // namespace

void build_op(const kf_op_desc *desc, kf_op *op) {
    KF_REQUIRE(desc != nullptr, KF_EINVAL, "KronFreeOperator: descriptor is NULL");
    KF_REQUIRE(desc->ndims >= 1 && desc->ndims <= MAXDIMS, KF_EINVAL,
               "KronFreeOperator: ndims must lie in 1:" + std::to_string(MAXDIMS));
    op->dims.assign(desc->dims, desc->dims + desc->ndims);
    int64_t N = 1;
    for (int a = 0; a < desc->ndims; ++a) {
        KF_REQUIRE(op->dims[a] >= 1, KF_EINVAL, "KronFreeOperator: dims must be positive");
        N *= op->dims[a];
    }
    KF_REQUIRE(N < (int64_t(1) << 31), KF_EINVAL, "KronFreeOperator: prod(dims) must be below 2^31");
    KF_REQUIRE(desc->block_capacity >= 1, KF_EINVAL, "KronFreeOperator: block_capacity must be positive");
    KF_REQUIRE(desc->nterms >= 0 && (desc->nterms == 0 || desc->terms != nullptr), KF_EINVAL,
               "KronFreeOperator: terms is NULL");
    op->N = N;
    ApplyPlan &P = op->plan;
    std::memset(&P, 0, sizeof(P));
    P.ndims = desc->ndims;
    P.N = (int)N;
    int64_t st = 1;
    op->strides.assign(desc->ndims, 0);
    for (int a = 0; a < desc->ndims; ++a) {
        if (a < MAXDIMS_F) P.dims[a] = (int)op->dims[a];
        op->strides[a] = st;
        st *= op->dims[a];
    }
    const bool fusable_dims = desc->ndims <= MAXDIMS_F;
    // validate terms (src/apply.jl:226-231, src/apply.jl:160-163)
    for (int t = 0; t < desc->nterms; ++t) {
        const kf_term &T = desc->terms[t];
        KF_REQUIRE(T.nfactors >= 0 && T.nfactors <= desc->ndims && (T.nfactors == 0 || T.factors), KF_EINVAL,
                   "KronFreeOperator: term " + std::to_string(t + 1) + " has an invalid factor list");
        for (int k = 0; k < T.nfactors; ++k) {
            const kf_factor &f = T.factors[k];
            KF_REQUIRE(f.axis >= 0 && f.axis < desc->ndims, KF_EINVAL,
                       "KronFreeOperator: factor axis " + std::to_string(f.axis + 1) + " outside 1:" +
                           std::to_string(desc->ndims));
            KF_REQUIRE(k == 0 || f.axis > T.factors[k - 1].axis, KF_EINVAL,
                       "AxisTerm: factor axes must be strictly increasing");
            KF_REQUIRE(f.n == op->dims[f.axis], KF_EDIM,
                       "KronFreeOperator: factor on axis " + std::to_string(f.axis + 1) + " has dimension " +
                           std::to_string(f.n) + ", expected " + std::to_string(op->dims[f.axis]));
            KF_REQUIRE(f.kind >= KF_DIAG && f.kind <= KF_DENSE, KF_EINVAL, "KronFreeOperator: unknown factor kind");
            KF_REQUIRE(f.kind == KF_SHIFT || f.data != nullptr, KF_EINVAL, "KronFreeOperator: factor data is NULL");
            if (f.kind == KF_BANDED) {
                KF_REQUIRE(f.nbands >= 0 && f.nbands <= MAXB && (f.nbands == 0 || f.offsets), KF_EINVAL,
                           "KronFreeOperator: a banded factor needs 0.." + std::to_string(MAXB) + " bands");
            }
            if (f.kind == KF_DENSE) {
                KF_REQUIRE(f.n <= 4096, KF_EINVAL, "KronFreeOperator: dense factors are limited to 4096 x 4096");
            }
        }
        KF_REQUIRE(std::isfinite(T.coeff), KF_EINVAL, "KronFreeOperator: a coefficient is not finite");
    }
    // per-axis sums of the single-axis terms, for the separable preconditioner (the matrices of
    // src/apply.jl:606-622: kept and fused single-factor terms, the constant on axis 1)
    {
        size_t tot = 0;
        for (int64_t d : op->dims) tot += (size_t)d * d;
        op->sep.M.clear();
        if (tot <= ((size_t)1 << 26)) {
            op->sep.M.resize(desc->ndims);
            for (int a = 0; a < desc->ndims; ++a) op->sep.M[a].assign((size_t)op->dims[a] * op->dims[a], 0.0);
            const int64_t d0 = op->dims[0];
            for (int64_t i = 0; i < d0; ++i) op->sep.M[0][i + d0 * i] += desc->constant;
            for (int t = 0; t < desc->nterms; ++t) {
                const kf_term &T = desc->terms[t];
                if (T.nfactors == 0) {
                    for (int64_t i = 0; i < d0; ++i) op->sep.M[0][i + d0 * i] += T.coeff;
                    continue;
                }
                if (T.nfactors != 1) continue;
                const kf_factor &f = T.factors[0];
                std::vector<double> &M = op->sep.M[f.axis];
                const int64_t n = f.n;
                const double c = T.coeff;
                if (f.kind == KF_DIAG) {
                    for (int64_t i = 0; i < n; ++i) M[i + n * i] += c * f.data[i];
                } else if (f.kind == KF_SHIFT) {
                    for (int64_t i = 0; i < n; ++i)
                        if (i + f.shift >= 0 && i + f.shift < n) M[(i + f.shift) + n * i] += c * f.factor;
                } else if (f.kind == KF_BANDED) {
                    for (int bb = 0; bb < f.nbands; ++bb)
                        for (int64_t i = 0; i < n; ++i) {
                            const int64_t j = i + f.offsets[bb];
                            if (j >= 0 && j < n) M[i + n * j] += c * f.data[(size_t)bb * n + i];
                        }
                } else {
                    for (int64_t k = 0; k < n * n; ++k) M[k] += c * f.data[k];
                }
            }
        }
    }
    // the separable preconditioner's per-axis eigendecompositions (host only) start as soon as the
    // per-axis sums exist, on their own thread, overlapping the rest of the construction; the first
    // solve that needs them waits for the result (free_op waits for the job if construction fails)
    if (!op->sep.M.empty()) op->sep.host_job = std::async(std::launch::async, [op] { sep_host_prepare(op); });
    // fused diagonal (src/apply.jl:234-241, 438-447)
    std::vector<double> D(N, desc->constant);
    if (desc->diag) for (int64_t p = 0; p < N; ++p) D[p] += desc->diag[p];
    std::vector<HTerm> fused;
    std::vector<ChainTerm> chains_h;
    std::vector<std::vector<double>> chain_data;
    double off_norm = 0;
    op->kept.clear();
    for (int t = 0; t < desc->nterms; ++t) {
        const kf_term &T = desc->terms[t];
        bool alldiag = true, anydense = false;
        for (int k = 0; k < T.nfactors; ++k) {
            alldiag = alldiag && T.factors[k].kind == KF_DIAG;
            anydense = anydense || T.factors[k].kind == KF_DENSE;
        }
        if (alldiag) {
            std::vector<std::pair<int, std::vector<double>>> vecs;
            for (int k = 0; k < T.nfactors; ++k)
                vecs.push_back({T.factors[k].axis, std::vector<double>(T.factors[k].data, T.factors[k].data + T.factors[k].n)});
            add_separable(D, op->dims, T.coeff, vecs);
            continue;
        }
        // a kept term: record it for the diagonal and the Gershgorin bound
        kf_op::HostTerm ht;
        ht.coeff = T.coeff;
        double prod = 1;
        for (int k = 0; k < T.nfactors; ++k) {
            const kf_factor &f = T.factors[k];
            prod *= band_infnorm(f);
            kf_op::HostFactor hf{f.axis, f.kind, f.n, factor_diagonal(f), {}, f.shift, f.factor};
            ht.f.push_back(hf);
        }
        off_norm += std::fabs(T.coeff) * prod;
        op->kept.push_back(ht);
        if (T.coeff == 0.0) continue;
        HTerm h{T.coeff, {}};
        for (int k = 0; k < T.nfactors; ++k)
            if (T.factors[k].kind != KF_DENSE) h.f.push_back(to_band(T.factors[k]));
        if (!anydense && T.nfactors <= 2) {
            fused.push_back(h);
        } else {
            ChainTerm ct;
            ct.coeff = T.coeff;
            size_t bi = 0;
            for (int k = 0; k < T.nfactors; ++k) {
                const kf_factor &f = T.factors[k];
                ChainFactor cf{};
                cf.axis = f.axis;
                cf.n = (int)f.n;
                if (f.kind == KF_DENSE) {
                    cf.kind = KF_DENSE;
                    chain_data.push_back(std::vector<double>(f.data, f.data + (size_t)f.n * f.n));
                } else {
                    const HBand &hb = h.f[bi++];
                    cf.kind = KF_BANDED;
                    cf.nb = hb.nb();
                    for (int q = 0; q < cf.nb; ++q) cf.off[q] = hb.off[q];
                    chain_data.push_back(hb.w);
                }
                cf.data_off = 0;
                ct.f.push_back(cf);
            }
            chains_h.push_back(ct);
        }
    }
    // merge single-axis and structurally equal fused terms
    merge_terms(fused);
    // fused terms become stencil entries (the cartesian product of their bands); a term that
    // would overflow the entry table, or an operator with more axes than the fused kernel
    // decodes, runs as a chain instead
    int ne = 0;
    std::vector<double> pool;
    for (HTerm &h : fused) {
        int cnt = 1;
        for (auto &b : h.f) cnt *= std::max(b.nb(), 1);
        bool fits = fusable_dims && (int)h.f.size() >= 1 && (int)h.f.size() <= 2 && ne + cnt <= MAXE;
        for (auto &b : h.f) fits = fits && b.nb() <= MAXB;
        if (!fits) {
            ChainTerm ct;
            ct.coeff = h.coeff;
            for (auto &b : h.f) {
                ChainFactor cf{};
                cf.axis = b.axis;
                cf.n = b.n;
                cf.kind = KF_BANDED;
                cf.nb = b.nb();
                KF_REQUIRE(cf.nb <= MAXB, KF_EINVAL, "KronFreeOperator: too many bands in one factor");
                for (int q = 0; q < cf.nb; ++q) cf.off[q] = b.off[q];
                chain_data.push_back(b.w);
                ct.f.push_back(cf);
            }
            chains_h.push_back(ct);
            continue;
        }
        // weights of the term's factors in the pool, the coefficient folded into the first
        std::vector<int> woff(h.f.size());
        for (size_t k = 0; k < h.f.size(); ++k) {
            woff[k] = (int)pool.size();
            const double c = (k == 0) ? h.coeff : 1.0;
            for (double v : h.f[k].w) pool.push_back(c * v);
        }
        const HBand &f0 = h.f[0];
        for (int b0 = 0; b0 < f0.nb(); ++b0) {
            if (h.f.size() == 1) {
                Entry &E = P.e[ne++];
                E = Entry{};
                E.nf = 1;
                E.a0 = f0.axis; E.o0 = f0.off[b0]; E.n0 = f0.n; E.nb0 = f0.nb(); E.w0 = woff[0] + b0;
                E.delta = (int)(f0.off[b0] * op->strides[f0.axis]);
                continue;
            }
            const HBand &f1 = h.f[1];
            for (int b1 = 0; b1 < f1.nb(); ++b1) {
                Entry &E = P.e[ne++];
                E = Entry{};
                E.nf = 2;
                E.a0 = f0.axis; E.o0 = f0.off[b0]; E.n0 = f0.n; E.nb0 = f0.nb(); E.w0 = woff[0] + b0;
                E.a1 = f1.axis; E.o1 = f1.off[b1]; E.n1 = f1.n; E.nb1 = f1.nb(); E.w1 = woff[1] + b1;
                E.delta = (int)(f0.off[b0] * op->strides[f0.axis] + f1.off[b1] * op->strides[f1.axis]);
            }
        }
    }
    P.ne = ne;
    // lay out chain data
    std::vector<double> cpool;
    {
        size_t q = 0;
        for (ChainTerm &ct : chains_h)
            for (ChainFactor &cf : ct.f) {
                cf.data_off = cpool.size();
                cpool.insert(cpool.end(), chain_data[q].begin(), chain_data[q].end());
                ++q;
            }
    }
    op->chains = chains_h;
    // dense chain factors short enough for the tensor-core kernel's TF32-split image: FP32 applies
    // run them on tcgen05 (three MMAs per K step, FP32-accurate products)
    {
        size_t q = 0;
        for (ChainTerm &ct : op->chains)
            for (ChainFactor &cf : ct.f) {
                if (cf.kind == KF_DENSE && tc_mode_fits(cf.n, true)) {
                    op->chain_tc.push_back(tc_matrix_create(chain_data[q].data(), cf.n, false, true));
                    cf.tc = (int)op->chain_tc.size() - 1;
                }
                ++q;
            }
    }
    pairs_plan(op, chain_data);
    // host-side derived quantities
    op->h_diag = D;
    double dmax = -INFINITY;
    for (double v : D) dmax = std::max(dmax, v);
    op->gershgorin = dmax + off_norm;
    op->h_fulldiag = D;
    for (auto &ht : op->kept) {
        std::vector<std::pair<int, std::vector<double>>> vecs;
        for (auto &hf : ht.f) vecs.push_back({hf.axis, hf.data});
        add_separable(op->h_fulldiag, op->dims, ht.coeff, vecs);
    }
    // upload
    auto up64 = [&](const std::vector<double> &v, double **d) {
        if (v.empty()) { *d = nullptr; return; }
        KF_CUDA(cudaMalloc(d, v.size() * sizeof(double)));
        KF_CUDA(cudaMemcpyAsync(*d, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, op->stream));
    };
    auto up32 = [&](const std::vector<double> &v, float **d) {
        if (v.empty()) { *d = nullptr; return; }
        std::vector<float> f(v.begin(), v.end());
        KF_CUDA(cudaMalloc(d, f.size() * sizeof(float)));
        KF_CUDA(cudaMemcpyAsync(*d, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice, op->stream));
        KF_CUDA(cudaStreamSynchronize(op->stream));
    };
    up64(D, &op->d_diag64);
    up32(D, &op->d_diag32);
    up64(pool, &op->d_w64);
    up32(pool, &op->d_w32);
    up64(cpool, &op->d_chain64);
    up32(cpool, &op->d_chain32);
    op->cap = desc->block_capacity;
    KF_CUDA(cudaStreamSynchronize(op->stream));
}

void free_op(kf_op *op) {
    if (op->sep.host_job.valid()) op->sep.host_job.wait();
    cudaFree(op->d_diag64);
    cudaFree(op->d_diag32);
    cudaFree(op->d_w64);
    cudaFree(op->d_w32);
    cudaFree(op->d_chain64);
    cudaFree(op->d_chain32);
    cudaFree(op->d_scratch);
    cudaFree(op->d_drive);
    cudaFree(op->d_march[0]);
    cudaFree(op->d_march[1]);
    for (float *p : op->sep.dU) cudaFree(p);
    for (float *p : op->sep.dUt) cudaFree(p);
    for (double *p : op->sep.dU64) cudaFree(p);
    for (auto &m : op->chain_tc) kf::tc_matrix_free(m);
    for (auto &m : op->sep.tU) kf::tc_matrix_free(m);
    for (auto &m : op->sep.tUt) kf::tc_matrix_free(m);
    cudaFree(op->sep.d_lam);
    cudaFree(op->sep.d_lam_off);
    cudaFree(op->sep.d_dims);
    cudaFree(op->sep.d_shl);
    if (op->own_stream && op->stream) cudaStreamDestroy(op->stream);
}

}  // namespace kf

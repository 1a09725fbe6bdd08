// The learned warm start's network: a din -> hidden -> hidden -> dout MLP with SiLU activations,
// BF16 weights (the copies the forward pass reads), FP32 accumulation, FP32 master weights and
// hand-written Adam.  It maps the circuit parameters theta of a node to the coefficients of its
// initial LOBPCG block over a fixed POD basis; the training labels are the plain solver's own
// eigenvectors.  (The reference warm-starts only from a previous solution's vectors,
// src/materialize.jl:656-670; this network is the learned extension of that hook.)
//
// Kernels: one tiled GEMM with strided operands (for X W, dZ W' and X' dZ), fused bias and
// activation epilogue; a bias-gradient column sum; the SiLU derivative; MSE loss and its gradient;
// Adam with bias correction writing both the FP32 master and the BF16 copy.
#include <cuda_bf16.h>

#include <cstring>
#include <functional>
#include <random>
#include <vector>

#include "kf_internal.h"

struct kf_mlp {
    int din = 0, h = 0, dout = 0;
    // parameters: W1 din x h, b1 h, W2 h x h, b2 h, W3 h x dout, b3 dout (row-major W: [in][out])
    int64_t nparam = 0;
    float *master = nullptr;          // FP32 master copy of all parameters, in the order above
    __nv_bfloat16 *wbf = nullptr;     // BF16 copies of the weights (biases stay FP32)
    float *grad = nullptr, *m = nullptr, *v = nullptr;
    float *xmu = nullptr, *xsd = nullptr, *ymu = nullptr, *ysd = nullptr;
    int64_t step = 0;
    cudaStream_t s = nullptr;
    int64_t off_W1, off_b1, off_W2, off_b2, off_W3, off_b3;
};

namespace kf {
namespace {

constexpr int GM = 64, GN = 64, GK = 16;

__device__ __forceinline__ float to_f(float x) { return x; }
__device__ __forceinline__ float to_f(__nv_bfloat16 x) { return __bfloat162float(x); }

// C[m, n] = sum_k A(m, k) B(k, n) (+ bias[n]); A(m, k) = A[m*sam + k*sak], B(k, n) = B[k*sbk + n*sbn].
// act: 0 none, 1 SiLU.  Z (pre-activation) is stored when not NULL, Y = act(Z) when not NULL;
// accumulate: C += result (for weight gradients over several batches).
template <typename TB>
__global__ void __launch_bounds__(256) k_gemm(const float *__restrict__ A, int64_t sam, int64_t sak,
                                              const TB *__restrict__ B, int64_t sbk, int64_t sbn,
                                              const float *__restrict__ bias, float *__restrict__ Z,
                                              float *__restrict__ Y, int M, int N, int K, int act, int accumulate) {
    __shared__ float As[GK][GM + 1];
    __shared__ float Bs[GK][GN + 1];
    const int tid = threadIdx.x;
    const int m0 = blockIdx.x * GM, n0 = blockIdx.y * GN;
    const int tr = (tid % 16) * 4, tc = (tid / 16) * 4;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += GK) {
        for (int e = tid; e < GM * GK; e += 256) {
            const int mm = e / GK, kk = e % GK;
            const int mi = m0 + mm, ki = k0 + kk;
            As[kk][mm] = (mi < M && ki < K) ? A[(int64_t)mi * sam + (int64_t)ki * sak] : 0.f;
        }
        for (int e = tid; e < GN * GK; e += 256) {
            const int nn = e % GN, kk = e / GN;
            const int ni = n0 + nn, ki = k0 + kk;
            Bs[kk][nn] = (ni < N && ki < K) ? to_f(B[(int64_t)ki * sbk + (int64_t)ni * sbn]) : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) a[u] = As[kk][tr + u];
#pragma unroll
            for (int u = 0; u < 4; ++u) b[u] = Bs[kk][tc + u];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int w = 0; w < 4; ++w) acc[u][w] = fmaf(a[u], b[w], acc[u][w]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int mi = m0 + tr + u;
        if (mi >= M) continue;
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            const int ni = n0 + tc + w;
            if (ni >= N) continue;
            float z = acc[u][w] + (bias ? bias[ni] : 0.f);
            const int64_t o = (int64_t)mi * N + ni;
            if (accumulate) {
                Y[o] += z;
                continue;
            }
            if (Z) Z[o] = z;
            if (Y) Y[o] = act == 1 ? z / (1.f + __expf(-z)) : z;
        }
    }
}

template <typename TB>
void gemm(const float *A, int64_t sam, int64_t sak, const TB *B, int64_t sbk, int64_t sbn, const float *bias, float *Z,
          float *Y, int M, int N, int K, int act, int accumulate, cudaStream_t s) {
    dim3 grid((M + GM - 1) / GM, (N + GN - 1) / GN);
    k_gemm<TB><<<grid, 256, 0, s>>>(A, sam, sak, B, sbk, sbn, bias, Z, Y, M, N, K, act, accumulate);
    KF_LAUNCH_CHECK();
}

// dZ = dY * SiLU'(Z), SiLU'(z) = s (1 + z (1 - s)), s = sigmoid(z)
__global__ void k_silu_back(const float *__restrict__ Z, const float *__restrict__ dY, float *__restrict__ dZ,
                            int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float z = Z[i];
    const float sg = 1.f / (1.f + __expf(-z));
    dZ[i] = dY[i] * sg * (1.f + z * (1.f - sg));
}

// db[j] = sum_r dZ[r, j]
__global__ void k_colsum(const float *__restrict__ dZ, int rows, int cols, float *__restrict__ db) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= cols) return;
    float s = 0.f;
    for (int r = 0; r < rows; ++r) s += dZ[(int64_t)r * cols + j];
    db[j] = s;
}

// loss partials and dOut = 2 (out - y) / (rows * cols) for the mean squared error on normalised y
__global__ void k_mse(const float *__restrict__ out, const float *__restrict__ y, const float *__restrict__ ymu,
                      const float *__restrict__ ysd, int rows, int cols, float *__restrict__ dout,
                      float *__restrict__ loss_partial) {
    __shared__ float red[256];
    const int64_t n = (int64_t)rows * cols;
    float s = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(i % cols);
        const float t = (y[i] - ymu[j]) / ysd[j];
        const float d = out[i] - t;
        s += d * d;
        dout[i] = 2.f * d / (float)n;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss_partial[blockIdx.x] = red[0] / (float)n;
}

// x_n = (x - mu) / sd per column
__global__ void k_normalize(const float *__restrict__ x, const float *__restrict__ mu, const float *__restrict__ sd,
                            float *__restrict__ out, int64_t rows, int cols) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * cols) return;
    const int j = (int)(i % cols);
    out[i] = (x[i] - mu[j]) / sd[j];
}

__global__ void k_denormalize(float *__restrict__ y, const float *__restrict__ mu, const float *__restrict__ sd,
                              int64_t rows, int cols) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * cols) return;
    const int j = (int)(i % cols);
    y[i] = y[i] * sd[j] + mu[j];
}

// Adam with bias correction; weights (not biases) also written as BF16
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       __nv_bfloat16 *__restrict__ pb, const unsigned char *__restrict__ is_weight, int64_t n, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float upd = lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    const float np = p[i] - upd;
    p[i] = np;
    if (is_weight[i]) pb[i] = __float2bfloat16(np);
}

__global__ void k_to_bf16(const float *__restrict__ p, __nv_bfloat16 *__restrict__ pb, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pb[i] = __float2bfloat16(p[i]);
}

struct Acts {
    float *xn, *Z1, *A1, *Z2, *A2, *out, *dout, *dA2, *dZ2, *dA1, *dZ1, *lossp;
};

unsigned blocks(int64_t n) { return (unsigned)((n + 255) / 256); }

// forward on normalised inputs xn (rows x din); out = network output (normalised units)
void forward(kf_mlp *m, const Acts &a, int rows) {
    const int din = m->din, h = m->h, dout = m->dout;
    const __nv_bfloat16 *W1 = m->wbf + m->off_W1, *W2 = m->wbf + m->off_W2, *W3 = m->wbf + m->off_W3;
    const float *b1 = m->master + m->off_b1, *b2 = m->master + m->off_b2, *b3 = m->master + m->off_b3;
    gemm<__nv_bfloat16>(a.xn, din, 1, W1, h, 1, b1, a.Z1, a.A1, rows, h, din, 1, 0, m->s);
    gemm<__nv_bfloat16>(a.A1, h, 1, W2, h, 1, b2, a.Z2, a.A2, rows, h, h, 1, 0, m->s);
    gemm<__nv_bfloat16>(a.A2, h, 1, W3, dout, 1, b3, nullptr, a.out, rows, dout, h, 0, 0, m->s);
}

// backward from dout (rows x dout) into m->grad (FP32, parameter order)
void backward(kf_mlp *m, const Acts &a, int rows) {
    const int din = m->din, h = m->h, dout = m->dout;
    const __nv_bfloat16 *W2 = m->wbf + m->off_W2, *W3 = m->wbf + m->off_W3;
    float *g = m->grad;
    cudaStream_t s = m->s;
    // layer 3: dW3 = A2' dout (h x dout), db3 = colsum(dout), dA2 = dout W3'
    gemm<float>(a.A2, 1, h, a.dout, dout, 1, nullptr, nullptr, g + m->off_W3, h, dout, rows, 0, 0, s);
    k_colsum<<<blocks(dout), 256, 0, s>>>(a.dout, rows, dout, g + m->off_b3);
    KF_LAUNCH_CHECK();
    gemm<__nv_bfloat16>(a.dout, dout, 1, W3, 1, dout, nullptr, nullptr, a.dA2, rows, h, dout, 0, 0, s);
    k_silu_back<<<blocks((int64_t)rows * h), 256, 0, s>>>(a.Z2, a.dA2, a.dZ2, (int64_t)rows * h);
    KF_LAUNCH_CHECK();
    // layer 2
    gemm<float>(a.A1, 1, h, a.dZ2, h, 1, nullptr, nullptr, g + m->off_W2, h, h, rows, 0, 0, s);
    k_colsum<<<blocks(h), 256, 0, s>>>(a.dZ2, rows, h, g + m->off_b2);
    KF_LAUNCH_CHECK();
    gemm<__nv_bfloat16>(a.dZ2, h, 1, W2, 1, h, nullptr, nullptr, a.dA1, rows, h, h, 0, 0, s);
    k_silu_back<<<blocks((int64_t)rows * h), 256, 0, s>>>(a.Z1, a.dA1, a.dZ1, (int64_t)rows * h);
    KF_LAUNCH_CHECK();
    // layer 1
    gemm<float>(a.xn, 1, din, a.dZ1, h, 1, nullptr, nullptr, g + m->off_W1, din, h, rows, 0, 0, s);
    k_colsum<<<blocks(h), 256, 0, s>>>(a.dZ1, rows, h, g + m->off_b1);
    KF_LAUNCH_CHECK();
}

struct ActBuf {
    std::vector<void *> ptrs;
    Acts a{};
    ActBuf(kf_mlp *m, int rows) {
        auto al = [&](int64_t n) {
            void *p = nullptr;
            KF_CUDA(cudaMalloc(&p, (size_t)std::max<int64_t>(n, 1) * sizeof(float)));
            ptrs.push_back(p);
            return (float *)p;
        };
        a.xn = al((int64_t)rows * m->din);
        a.Z1 = al((int64_t)rows * m->h);
        a.A1 = al((int64_t)rows * m->h);
        a.Z2 = al((int64_t)rows * m->h);
        a.A2 = al((int64_t)rows * m->h);
        a.out = al((int64_t)rows * m->dout);
        a.dout = al((int64_t)rows * m->dout);
        a.dA2 = al((int64_t)rows * m->h);
        a.dZ2 = al((int64_t)rows * m->h);
        a.dA1 = al((int64_t)rows * m->h);
        a.dZ1 = al((int64_t)rows * m->h);
        a.lossp = al(1024);
    }
    ~ActBuf() {
        for (void *p : ptrs) cudaFree(p);
    }
};

float loss_and_grad_out(kf_mlp *m, const Acts &a, const float *y, int rows) {
    const int nb = 120;
    k_mse<<<nb, 256, 0, m->s>>>(a.out, y, m->ymu, m->ysd, rows, m->dout, a.dout, a.lossp);
    KF_LAUNCH_CHECK();
    std::vector<float> lp(nb);
    KF_CUDA(cudaMemcpyAsync(lp.data(), a.lossp, nb * sizeof(float), cudaMemcpyDeviceToHost, m->s));
    KF_CUDA(cudaStreamSynchronize(m->s));
    double s = 0;
    for (float v : lp) s += v;
    return (float)s;
}

}  // namespace
}  // namespace kf

using namespace kf;

extern "C" {

static int mlp_guard(const std::function<void()> &f) {
    try {
        f();
        return KF_OK;
    } catch (const Error &e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        set_last_error(e.what());
        return KF_EINVAL;
    }
}

int kf_mlp_create(int32_t din, int32_t hidden, int32_t dout, uint64_t seed, kf_mlp **out) {
    return mlp_guard([&] {
        KF_REQUIRE(out && din >= 1 && hidden >= 1 && dout >= 1, KF_EINVAL, "kf_mlp_create: bad sizes");
        kf_mlp *m = new kf_mlp();
        m->din = din;
        m->h = hidden;
        m->dout = dout;
        int64_t o = 0;
        m->off_W1 = o; o += (int64_t)din * hidden;
        m->off_b1 = o; o += hidden;
        m->off_W2 = o; o += (int64_t)hidden * hidden;
        m->off_b2 = o; o += hidden;
        m->off_W3 = o; o += (int64_t)hidden * dout;
        m->off_b3 = o; o += dout;
        m->nparam = o;
        // He-style initialisation for SiLU layers, small output layer; biases zero
        std::mt19937_64 rng(seed);
        std::normal_distribution<float> nd(0.f, 1.f);
        std::vector<float> p(o, 0.f);
        auto init = [&](int64_t off, int64_t fan_in, int64_t n, float gain) {
            const float sc = gain / std::sqrt((float)fan_in);
            for (int64_t i = 0; i < n; ++i) p[off + i] = sc * nd(rng);
        };
        init(m->off_W1, din, (int64_t)din * hidden, 1.4142f);
        init(m->off_W2, hidden, (int64_t)hidden * hidden, 1.4142f);
        init(m->off_W3, hidden, (int64_t)hidden * dout, 0.5f);
        KF_CUDA(cudaStreamCreateWithFlags(&m->s, cudaStreamNonBlocking));
        KF_CUDA(cudaMalloc(&m->master, o * sizeof(float)));
        KF_CUDA(cudaMalloc(&m->wbf, o * sizeof(__nv_bfloat16)));
        KF_CUDA(cudaMalloc(&m->grad, o * sizeof(float)));
        KF_CUDA(cudaMalloc(&m->m, o * sizeof(float)));
        KF_CUDA(cudaMalloc(&m->v, o * sizeof(float)));
        KF_CUDA(cudaMalloc(&m->xmu, din * sizeof(float)));
        KF_CUDA(cudaMalloc(&m->xsd, din * sizeof(float)));
        KF_CUDA(cudaMalloc(&m->ymu, dout * sizeof(float)));
        KF_CUDA(cudaMalloc(&m->ysd, dout * sizeof(float)));
        KF_CUDA(cudaMemcpy(m->master, p.data(), o * sizeof(float), cudaMemcpyHostToDevice));
        KF_CUDA(cudaMemset(m->m, 0, o * sizeof(float)));
        KF_CUDA(cudaMemset(m->v, 0, o * sizeof(float)));
        std::vector<float> zeros(std::max(din, dout), 0.f), ones(std::max(din, dout), 1.f);
        KF_CUDA(cudaMemcpy(m->xmu, zeros.data(), din * 4, cudaMemcpyHostToDevice));
        KF_CUDA(cudaMemcpy(m->xsd, ones.data(), din * 4, cudaMemcpyHostToDevice));
        KF_CUDA(cudaMemcpy(m->ymu, zeros.data(), dout * 4, cudaMemcpyHostToDevice));
        KF_CUDA(cudaMemcpy(m->ysd, ones.data(), dout * 4, cudaMemcpyHostToDevice));
        k_to_bf16<<<blocks(o), 256, 0, m->s>>>(m->master, m->wbf, o);
        KF_LAUNCH_CHECK();
        KF_CUDA(cudaStreamSynchronize(m->s));
        *out = m;
    });
}

int kf_mlp_destroy(kf_mlp *m) {
    return mlp_guard([&] {
        if (!m) return;
        for (void *p : {(void *)m->master, (void *)m->wbf, (void *)m->grad, (void *)m->m, (void *)m->v, (void *)m->xmu,
                        (void *)m->xsd, (void *)m->ymu, (void *)m->ysd})
            cudaFree(p);
        if (m->s) cudaStreamDestroy(m->s);
        delete m;
    });
}

int kf_mlp_set_scaling(kf_mlp *m, const float *xmu, const float *xsd, const float *ymu, const float *ysd) {
    return mlp_guard([&] {
        KF_REQUIRE(m && xmu && xsd && ymu && ysd, KF_EINVAL, "kf_mlp_set_scaling: NULL argument");
        for (int j = 0; j < m->din; ++j) KF_REQUIRE(xsd[j] > 0, KF_EINVAL, "kf_mlp_set_scaling: xsd must be positive");
        for (int j = 0; j < m->dout; ++j) KF_REQUIRE(ysd[j] > 0, KF_EINVAL, "kf_mlp_set_scaling: ysd must be positive");
        KF_CUDA(cudaMemcpy(m->xmu, xmu, m->din * 4, cudaMemcpyHostToDevice));
        KF_CUDA(cudaMemcpy(m->xsd, xsd, m->din * 4, cudaMemcpyHostToDevice));
        KF_CUDA(cudaMemcpy(m->ymu, ymu, m->dout * 4, cudaMemcpyHostToDevice));
        KF_CUDA(cudaMemcpy(m->ysd, ysd, m->dout * 4, cudaMemcpyHostToDevice));
    });
}

int kf_mlp_forward(kf_mlp *m, const float *X, float *Y, int64_t n) {
    return mlp_guard([&] {
        KF_REQUIRE(m && X && Y && n >= 1, KF_EINVAL, "kf_mlp_forward: bad arguments");
        const int chunk = 4096;
        ActBuf ab(m, chunk);
        float *dx = nullptr;
        KF_CUDA(cudaMalloc(&dx, (size_t)chunk * m->din * 4));
        for (int64_t r0 = 0; r0 < n; r0 += chunk) {
            const int rows = (int)std::min<int64_t>(chunk, n - r0);
            KF_CUDA(cudaMemcpyAsync(dx, X + r0 * m->din, (size_t)rows * m->din * 4, cudaMemcpyHostToDevice, m->s));
            k_normalize<<<blocks((int64_t)rows * m->din), 256, 0, m->s>>>(dx, m->xmu, m->xsd, ab.a.xn, rows, m->din);
            KF_LAUNCH_CHECK();
            forward(m, ab.a, rows);
            k_denormalize<<<blocks((int64_t)rows * m->dout), 256, 0, m->s>>>(ab.a.out, m->ymu, m->ysd, rows, m->dout);
            KF_LAUNCH_CHECK();
            KF_CUDA(cudaMemcpyAsync(Y + r0 * m->dout, ab.a.out, (size_t)rows * m->dout * 4, cudaMemcpyDeviceToHost, m->s));
        }
        KF_CUDA(cudaStreamSynchronize(m->s));
        cudaFree(dx);
    });
}

int kf_mlp_gradients(kf_mlp *m, const float *X, const float *Y, int64_t n, float *loss_out, float *grad_out) {
    return mlp_guard([&] {
        KF_REQUIRE(m && X && Y && n >= 1 && n <= 65536, KF_EINVAL, "kf_mlp_gradients: bad arguments");
        const int rows = (int)n;
        ActBuf ab(m, rows);
        float *dx = nullptr, *dy = nullptr;
        KF_CUDA(cudaMalloc(&dx, (size_t)rows * m->din * 4));
        KF_CUDA(cudaMalloc(&dy, (size_t)rows * m->dout * 4));
        KF_CUDA(cudaMemcpyAsync(dx, X, (size_t)rows * m->din * 4, cudaMemcpyHostToDevice, m->s));
        KF_CUDA(cudaMemcpyAsync(dy, Y, (size_t)rows * m->dout * 4, cudaMemcpyHostToDevice, m->s));
        k_normalize<<<blocks((int64_t)rows * m->din), 256, 0, m->s>>>(dx, m->xmu, m->xsd, ab.a.xn, rows, m->din);
        KF_LAUNCH_CHECK();
        forward(m, ab.a, rows);
        const float loss = loss_and_grad_out(m, ab.a, dy, rows);
        backward(m, ab.a, rows);
        if (loss_out) *loss_out = loss;
        if (grad_out)
            KF_CUDA(cudaMemcpyAsync(grad_out, m->grad, m->nparam * 4, cudaMemcpyDeviceToHost, m->s));
        KF_CUDA(cudaStreamSynchronize(m->s));
        cudaFree(dx);
        cudaFree(dy);
    });
}

int kf_mlp_train(kf_mlp *m, const float *X, const float *Y, int64_t n, int32_t epochs, int32_t batch, float lr,
                 uint64_t seed, float *losses_out) {
    return mlp_guard([&] {
        KF_REQUIRE(m && X && Y && n >= 1 && epochs >= 1 && batch >= 1 && lr > 0, KF_EINVAL, "kf_mlp_train: bad arguments");
        const int bs = (int)std::min<int64_t>(batch, n);
        ActBuf ab(m, bs);
        float *dX = nullptr, *dY = nullptr, *bx = nullptr, *by = nullptr;
        unsigned char *isw = nullptr;
        KF_CUDA(cudaMalloc(&dX, (size_t)n * m->din * 4));
        KF_CUDA(cudaMalloc(&dY, (size_t)n * m->dout * 4));
        KF_CUDA(cudaMalloc(&bx, (size_t)bs * m->din * 4));
        KF_CUDA(cudaMalloc(&by, (size_t)bs * m->dout * 4));
        KF_CUDA(cudaMalloc(&isw, m->nparam));
        std::vector<unsigned char> w(m->nparam, 0);
        std::fill(w.begin() + m->off_W1, w.begin() + m->off_b1, 1);
        std::fill(w.begin() + m->off_W2, w.begin() + m->off_b2, 1);
        std::fill(w.begin() + m->off_W3, w.begin() + m->off_b3, 1);
        KF_CUDA(cudaMemcpy(isw, w.data(), m->nparam, cudaMemcpyHostToDevice));
        // normalised inputs once; targets are normalised inside the loss
        std::vector<float> xn((size_t)n * m->din);
        {
            std::vector<float> mu(m->din), sd(m->din);
            KF_CUDA(cudaMemcpy(mu.data(), m->xmu, m->din * 4, cudaMemcpyDeviceToHost));
            KF_CUDA(cudaMemcpy(sd.data(), m->xsd, m->din * 4, cudaMemcpyDeviceToHost));
            for (int64_t r = 0; r < n; ++r)
                for (int j = 0; j < m->din; ++j) xn[r * m->din + j] = (X[r * m->din + j] - mu[j]) / sd[j];
        }
        KF_CUDA(cudaMemcpy(dX, xn.data(), (size_t)n * m->din * 4, cudaMemcpyHostToDevice));
        KF_CUDA(cudaMemcpy(dY, Y, (size_t)n * m->dout * 4, cudaMemcpyHostToDevice));
        std::mt19937_64 rng(seed);
        std::vector<int64_t> perm(n);
        for (int64_t i = 0; i < n; ++i) perm[i] = i;
        const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
        for (int ep = 0; ep < epochs; ++ep) {
            std::shuffle(perm.begin(), perm.end(), rng);
            double esum = 0;
            int nbt = 0;
            for (int64_t r0 = 0; r0 + bs <= n; r0 += bs) {
                // gather the batch rows (device to device copies of contiguous rows)
                for (int r = 0; r < bs; ++r) {
                    KF_CUDA(cudaMemcpyAsync(ab.a.xn + (int64_t)r * m->din, dX + perm[r0 + r] * m->din, m->din * 4,
                                            cudaMemcpyDeviceToDevice, m->s));
                    KF_CUDA(cudaMemcpyAsync(by + (int64_t)r * m->dout, dY + perm[r0 + r] * m->dout, m->dout * 4,
                                            cudaMemcpyDeviceToDevice, m->s));
                }
                forward(m, ab.a, bs);
                esum += loss_and_grad_out(m, ab.a, by, bs);
                ++nbt;
                backward(m, ab.a, bs);
                ++m->step;
                const float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
                k_adam<<<blocks(m->nparam), 256, 0, m->s>>>(m->master, m->grad, m->m, m->v, m->wbf, isw, m->nparam, lr,
                                                           b1, b2, eps, c1, c2);
                KF_LAUNCH_CHECK();
            }
            if (losses_out) losses_out[ep] = (float)(esum / std::max(nbt, 1));
        }
        KF_CUDA(cudaStreamSynchronize(m->s));
        cudaFree(dX);
        cudaFree(dY);
        cudaFree(bx);
        cudaFree(by);
        cudaFree(isw);
    });
}

int kf_mlp_get_params(kf_mlp *m, float *out, int64_t *count) {
    return mlp_guard([&] {
        KF_REQUIRE(m && count, KF_EINVAL, "kf_mlp_get_params: NULL argument");
        *count = m->nparam;
        if (!out) return;
        // the weights as the forward pass sees them (BF16 widened), biases FP32
        std::vector<__nv_bfloat16> wb(m->nparam);
        KF_CUDA(cudaMemcpy(out, m->master, m->nparam * 4, cudaMemcpyDeviceToHost));
        KF_CUDA(cudaMemcpy(wb.data(), m->wbf, m->nparam * 2, cudaMemcpyDeviceToHost));
        auto widen = [&](int64_t a, int64_t b) {
            for (int64_t i = a; i < b; ++i) out[i] = __bfloat162float(wb[i]);
        };
        widen(m->off_W1, m->off_b1);
        widen(m->off_W2, m->off_b2);
        widen(m->off_W3, m->off_b3);
    });
}

}  // extern "C"

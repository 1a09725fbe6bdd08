// kf_op_apply_noalloc: the operator application for callers that must not allocate device memory.
//
// Who needs it.  kf_op_apply applies a term with dense factors as a chain of single-axis passes
// through two scratch blocks of N x b elements, and allocates those blocks with cudaMalloc the
// first time a block that wide is applied.  Some callers cannot let a library do that: a host
// program whose device memory is owned and accounted by its own pool or arena (the caching
// allocators of Julia's CUDA.jl or of PyTorch, a fixed-size arena in an embedded service) must not
// see memory allocated behind its back, and a tight solver loop cannot take the implicit device
// synchronisation of a cudaMalloc/cudaFree in the middle of its work.  This entry point performs
// the same application with no allocation at all: its chain scratch is one fixed array in device
// global memory, declared here with static storage, sized KF_NOALLOC_SCRATCH_BYTES.
//
// Costs and rules.  Each device holds the array from its first call until the process exits.
// All calls on a device share the one array, and it keeps whatever the last call left in it
// (nothing here needs it zeroed: each chain pass writes its scratch block in full before any pass
// reads it); calls whose executions overlap on the GPU (different streams, or different host
// threads with no ordering between their streams) race on it and give wrong results.
//
// Set-up.  The array belongs to this file's device module, and with CUDA's lazy module loading
// (the default) the driver loads a module -- reserving its static arrays in device memory -- the
// first time it is used.  So the first call on each device, which looks up the array's device
// address (cudaGetSymbolAddress) with that device current, is where the array's 8 MiB are taken,
// and the first launch of each kernel the call uses loads that kernel's module too.  A caller that
// must see no device allocation once it runs makes one warm-up call per device at set-up: a call
// with b = 0 on an operator with dense-factor terms does the address lookup and loads this module;
// one with b > 0 also loads the kernels (make it with the precision the caller will use), and
// every later call allocates nothing.  Make the set-up call before any stream capture begins.
// After cudaDeviceReset the looked-up addresses (and every kf_op) are invalid: the library must
// not be used across a reset.
#include <mutex>

#include "kf_internal.h"

namespace kf {
template <typename T>
void apply_given_scratch(kf_op *op, const T *X, T *Y, int64_t ldx, int64_t ldy, int64_t b, T *scratch,
                         cudaStream_t s);
}

// The scratch array.  In host code its name is only a host-side stand-in: its device address is
// taken with cudaGetSymbolAddress per device and passed to the kernels.
static __device__ __align__(256) unsigned char g_noalloc_scratch[KF_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_dev_ptr[kMaxDevices] = {};

// The array's device address on the current device, looked up once per device.
void *scratch_address() {
    int dev = 0;
    KF_CUDA(cudaGetDevice(&dev));
    KF_REQUIRE(dev >= 0 && dev < kMaxDevices, KF_EINVAL, "kf_op_apply_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_mu);
    if (g_dev_ptr[dev] == nullptr) {
        void *p = nullptr;
        KF_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        KF_REQUIRE(p != nullptr, KF_ECUDA, "kf_op_apply_noalloc: no device address for the scratch array");
        g_dev_ptr[dev] = p;
    }
    return g_dev_ptr[dev];
}
}  // namespace

extern "C" int kf_op_apply_noalloc(kf_op *op, const void *X, void *Y, int64_t ldx, int64_t ldy, int64_t b,
                                   int32_t flags) {
    try {
        KF_REQUIRE(op != nullptr, KF_EINVAL, "kf_op_apply_noalloc: op is NULL");
        KF_REQUIRE(!(flags & KF_HOST), KF_EINVAL,
                   "kf_op_apply_noalloc: device pointers only (the host path needs staging buffers)");
        const int64_t N = op->N;
        KF_REQUIRE(b >= 0 && ldx >= N && ldy >= N, KF_EDIM, "kf_op_apply_noalloc: bad block shape");
        if (b == 0) {
            if (!op->chains.empty()) (void)scratch_address();   // the set-up call (see above)
            return KF_OK;
        }
        KF_REQUIRE(X && Y, KF_EINVAL, "kf_op_apply_noalloc: NULL block");
        const bool f32 = (flags & KF_F32) != 0;
        const size_t es = f32 ? 4 : 8;
        const char *px = (const char *)X, *py = (const char *)Y;
        const size_t bx = ((size_t)(b - 1) * ldx + N) * es, by = ((size_t)(b - 1) * ldy + N) * es;
        KF_REQUIRE(!(px < py + by && py < px + bx), KF_EALIAS, "mul!: y must not alias x");
        const size_t need = op->chains.empty() ? 0 : (size_t)2 * N * b * es;
        if (need > (size_t)KF_NOALLOC_SCRATCH_BYTES)
            throw kf::Error(KF_EINVAL,
                            "kf_op_apply_noalloc: this operator's dense-factor terms need " + std::to_string(need) +
                                " bytes of scratch for a block of " + std::to_string(b) +
                                " columns, above the fixed KF_NOALLOC_SCRATCH_BYTES = " +
                                std::to_string((size_t)KF_NOALLOC_SCRATCH_BYTES) +
                                "; apply fewer columns per call, or use kf_op_apply");
        void *scratch = need ? scratch_address() : nullptr;
        if (f32)
            kf::apply_given_scratch<float>(op, (const float *)X, (float *)Y, ldx, ldy, b, (float *)scratch, op->stream);
        else
            kf::apply_given_scratch<double>(op, (const double *)X, (double *)Y, ldx, ldy, b, (double *)scratch,
                                            op->stream);
        return KF_OK;
    } catch (const kf::Error &e) {
        kf::set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        kf::set_last_error(e.what());
        return KF_EINVAL;
    }
}

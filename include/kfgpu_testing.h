/*
 * kfgpu_testing.h -- entry points of libkfgpu.so that exist for the test suite only.  They have
 * no counterpart in KronFreeCircuits.jl and no caller of the reference interface needs them.
 */
#ifndef KFGPU_TESTING_H
#define KFGPU_TESTING_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/*
 * One mode product Y = alpha (A along an axis) X + beta Y on device blocks of b FP32 columns of
 * length N (leading dimension N), the axis of length d with stride `left` (the product of the
 * lengths of the axes before it).  A: host, d x d, column-major, FP64.  path 0: the SIMT FP32
 * kernel; path 1: the tcgen05 tensor-core kernel (BF16 operands, FP32 accumulation; d <= 256).
 * Synchronous on `stream` (a cudaStream_t, 0 for the default stream).  Returns a KF_* status.
 */
int kf_test_mode_product(int path, const float *X, float *Y, const double *A, int d, int64_t left, int64_t N,
                         int64_t b, double alpha, double beta, void *stream);

#ifdef __cplusplus
}
#endif

#endif

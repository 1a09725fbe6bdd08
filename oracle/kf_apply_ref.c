/*
 * C restatement of the reference's CPU operator application -- TEST INFRASTRUCTURE ONLY
 * (the oracle's fast path and the timed CPU baseline; never part of libkfgpu).
 *
 * Follows KronFreeCircuits.jl src/apply.jl:416-432 (mul!) term by term, pass by pass:
 *   y = diag .* x                                   (src/apply.jl:427)
 *   for each kept term: chain its factors through two scratch buffers, one full pass per
 *   factor (src/apply.jl:370-382), then one accumulate pass Y += coeff * src (src/apply.jl:386)
 * with the factor passes of src/apply.jl:60-63 (diagonal), 66-79 (banded), 111-118 (shift) and
 * 37-53 (dense, the reference public apply_axis!).  OpenMP threads over the flat index, as the
 * reference's threaded host path (src/apply.jl:342-361).
 *
 * Factors use the C ABI's encoding (include/kfgpu.h): kind 0 diagonal, 1 banded (weights
 * band-major, w[b*n + i]), 2 shift, 3 dense (column-major n x n).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int32_t axis, kind;
    int64_t n;
    const double *data;
    const int64_t *offsets;
    int32_t nbands;
    int64_t shift;
    double factor;
} ref_factor;

/* dst = factor applied along its axis of src; the block has total = N*b entries with column
 * stride N; stride = prod(dims[0..axis)). */
static void apply_factor(double *dst, const double *src, const ref_factor *f, int64_t stride, int64_t total) {
    const int64_t n = f->n;
    if (f->kind == 0) {
#pragma omp parallel for schedule(static)
        for (int64_t t = 0; t < total; ++t) dst[t] = f->data[(t / stride) % n] * src[t];
    } else if (f->kind == 1) {
#pragma omp parallel for schedule(static)
        for (int64_t t = 0; t < total; ++t) {
            const int64_t i = (t / stride) % n;
            double acc = 0.0;
            for (int b = 0; b < f->nbands; ++b) {
                const int64_t j = i + f->offsets[b];
                if (j >= 0 && j < n) acc += f->data[(int64_t)b * n + i] * src[t + f->offsets[b] * stride];
            }
            dst[t] = acc;
        }
    } else if (f->kind == 2) {
#pragma omp parallel for schedule(static)
        for (int64_t t = 0; t < total; ++t) {
            const int64_t i = (t / stride) % n;
            const int64_t j = i - f->shift;
            dst[t] = (j >= 0 && j < n) ? f->factor * src[t - f->shift * stride] : 0.0;
        }
    } else {
        /* Y[l, i, r] = sum_j M[i, j] X[l, j, r] */
#pragma omp parallel for schedule(static)
        for (int64_t t = 0; t < total; ++t) {
            const int64_t l = t % stride, q = t / stride, i = q % n, r = q / n;
            const double *xs = src + l + stride * n * r;
            double acc = 0.0;
            for (int64_t j = 0; j < n; ++j) acc += f->data[i + n * j] * xs[stride * j];
            dst[t] = acc;
        }
    }
}

/* y = diag .* x + sum_t coeff_t (chain of factors) x for a block of b columns (column stride N).
 * factors of term t: factors[first[t] .. first[t] + nf[t]).  scratch: 2 * N * b doubles. */
int kf_ref_apply(int ndims, const int64_t *dims, const double *diag, int nterms, const double *coeff,
                 const int32_t *first, const int32_t *nf, const ref_factor *factors, const double *x, double *y,
                 int64_t b, double *scratch) {
    int64_t N = 1, stride[16];
    if (ndims > 16) return 1;
    for (int a = 0; a < ndims; ++a) {
        stride[a] = N;
        N *= dims[a];
    }
    const int64_t total = N * b;
#pragma omp parallel for schedule(static)
    for (int64_t t = 0; t < total; ++t) y[t] = diag[t % N] * x[t];
    double *buf[2] = {scratch, scratch + total};
    for (int k = 0; k < nterms; ++k) {
        const double *src = x;
        for (int q = 0; q < nf[k]; ++q) {
            const ref_factor *f = &factors[first[k] + q];
            double *dst = buf[q & 1];
            apply_factor(dst, src, f, stride[f->axis], total);
            src = dst;
        }
        const double c = coeff[k];
#pragma omp parallel for schedule(static)
        for (int64_t t = 0; t < total; ++t) y[t] += c * src[t];
    }
    return 0;
}

/*
 * C restatement of the reference's CPU operator application -- TEST INFRASTRUCTURE ONLY
 * (the oracle's fast path and the timed CPU baseline; never part of libkfgpu).
 *
 * Follows KronFreeCircuits.jl src/apply.jl:416-432 (mul!) term by term, pass by pass:
 *   y = diag .* x                                   (src/apply.jl:427)
 *   for each kept term: chain its factors through two scratch buffers, one full pass per
 *   factor (src/apply.jl:370-382), then one accumulate pass Y += coeff * src (src/apply.jl:386)
 * with the factor passes of src/apply.jl:60-63 (diagonal), 66-79 (banded), 111-118 (shift) and
 * 37-53 (dense, the reference public apply_axis!).  OpenMP threads over the outer indices, as the
 * reference's threaded host path (src/apply.jl:342-361).  Each pass walks the block as
 * (l, i, r) loop nests -- l the axes before the factor's axis, i the axis, r the axes after and
 * the columns -- so no index is decoded by division per element.
 *
 * Factors use the C ABI's encoding (include/kfgpu.h): kind 0 diagonal, 1 banded (weights
 * band-major, w[b*n + i]), 2 shift, 3 dense (column-major n x n).
 *
 * Also the elementwise steps of the oracle's LOBPCG (oracle/solvers.py), threaded: residuals
 * R = HX - X diag(lam) with their squared column norms, and the per-Ritz Jacobi preconditioner
 * W = R / hypot(D - theta, eta) (src/lobpcg.jl:73-96).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int32_t axis, kind;
    int64_t n;
    const double *data;
    const int64_t *offsets;
    int32_t nbands;
    int64_t shift;
    double factor;
} ref_factor;

/* dst = factor applied along its axis of src; the block is (stride, n, nr) with nr = the axes
 * after the factor's axis times the columns (column stride N = stride * n * (axes after)). */
static void apply_factor(double *dst, const double *src, const ref_factor *f, int64_t stride, int64_t nr) {
    const int64_t n = f->n;
    const int64_t slab = stride * n;
    if (f->kind == 0) {
#pragma omp parallel for collapse(2) schedule(static)
        for (int64_t r = 0; r < nr; ++r)
            for (int64_t i = 0; i < n; ++i) {
                const double w = f->data[i];
                const double *s = src + r * slab + i * stride;
                double *d = dst + r * slab + i * stride;
                for (int64_t l = 0; l < stride; ++l) d[l] = w * s[l];
            }
    } else if (f->kind == 1) {
#pragma omp parallel for collapse(2) schedule(static)
        for (int64_t r = 0; r < nr; ++r)
            for (int64_t i = 0; i < n; ++i) {
                double *d = dst + r * slab + i * stride;
                for (int64_t l = 0; l < stride; ++l) d[l] = 0.0;
                for (int b = 0; b < f->nbands; ++b) {
                    const int64_t j = i + f->offsets[b];
                    if (j < 0 || j >= n) continue;
                    const double w = f->data[(int64_t)b * n + i];
                    const double *s = src + r * slab + j * stride;
                    for (int64_t l = 0; l < stride; ++l) d[l] += w * s[l];
                }
            }
    } else if (f->kind == 2) {
#pragma omp parallel for collapse(2) schedule(static)
        for (int64_t r = 0; r < nr; ++r)
            for (int64_t i = 0; i < n; ++i) {
                const int64_t j = i - f->shift;
                double *d = dst + r * slab + i * stride;
                if (j < 0 || j >= n) {
                    for (int64_t l = 0; l < stride; ++l) d[l] = 0.0;
                } else {
                    const double *s = src + r * slab + j * stride;
                    for (int64_t l = 0; l < stride; ++l) d[l] = f->factor * s[l];
                }
            }
    } else {
        /* Y[l, i, r] = sum_j M[i, j] X[l, j, r] */
#pragma omp parallel for collapse(2) schedule(static)
        for (int64_t r = 0; r < nr; ++r)
            for (int64_t i = 0; i < n; ++i) {
                double *d = dst + r * slab + i * stride;
                for (int64_t l = 0; l < stride; ++l) d[l] = 0.0;
                for (int64_t j = 0; j < n; ++j) {
                    const double w = f->data[i + n * j];
                    const double *s = src + r * slab + j * stride;
                    for (int64_t l = 0; l < stride; ++l) d[l] += w * s[l];
                }
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
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t c = 0; c < b; ++c)
        for (int64_t p = 0; p < N; ++p) y[c * N + p] = diag[p] * x[c * N + p];
    double *buf[2] = {scratch, scratch + total};
    for (int k = 0; k < nterms; ++k) {
        const double *src = x;
        for (int q = 0; q < nf[k]; ++q) {
            const ref_factor *f = &factors[first[k] + q];
            double *dst = buf[q & 1];
            const int64_t nr = total / (stride[f->axis] * f->n);
            apply_factor(dst, src, f, stride[f->axis], nr);
            src = dst;
        }
        const double c = coeff[k];
#pragma omp parallel for schedule(static)
        for (int64_t t = 0; t < total; ++t) y[t] += c * src[t];
    }
    return 0;
}

/* R = HX - X diag(lam) (column-major, leading dimensions ldx, ldh, ldr; k columns of N rows) and
 * norms2[j] = sum_p R[p, j]^2.  Rows are split into chunks; each column's squared norm is summed
 * per chunk and the chunks are added in a fixed order. */
int kf_ref_resid(int64_t N, int k, const double *X, int64_t ldx, const double *HX, int64_t ldh, const double *lam,
                 double *R, int64_t ldr, double *norms2) {
    enum { CH = 65536 };
    const int64_t nch = (N + CH - 1) / CH;
    double *part = (double *)calloc((size_t)nch * (size_t)(k > 0 ? k : 1), sizeof(double));
    if (!part) return 1;
#pragma omp parallel for collapse(2) schedule(static)
    for (int j = 0; j < k; ++j)
        for (int64_t ch = 0; ch < nch; ++ch) {
            const int64_t p0 = ch * CH, p1 = p0 + CH < N ? p0 + CH : N;
            const double *x = X + j * ldx, *hx = HX + j * ldh;
            double *r = R + j * ldr;
            const double l = lam[j];
            double s = 0.0;
            for (int64_t p = p0; p < p1; ++p) {
                const double v = hx[p] - x[p] * l;
                r[p] = v;
                s += v * v;
            }
            part[ch * k + j] = s;
        }
    for (int j = 0; j < k; ++j) {
        double s = 0.0;
        for (int64_t ch = 0; ch < nch; ++ch) s += part[ch * k + j];
        norms2[j] = s;
    }
    free(part);
    return 0;
}

/* W[:, j] = R[:, j] / hypot(S - thp[j], eta) (mode 0: the per-Ritz Jacobi preconditioner with S the
 * full diagonal, src/lobpcg.jl:73-96, or the separable preconditioner's spectral scaling with S the
 * per-point sum of per-axis eigenvalues) or R[:, j] / (S - thp[0]) (mode 1: fixed Jacobi, shift
 * thp[0]).  W may equal R. */
int kf_ref_scale(int64_t N, int k, const double *R, int64_t ldr, const double *S, const double *thp, double eta,
                 int mode, double *W, int64_t ldw) {
#pragma omp parallel for collapse(2) schedule(static)
    for (int j = 0; j < k; ++j)
        for (int64_t p = 0; p < N; ++p) {
            const double v = R[j * ldr + p];
            W[j * ldw + p] = mode == 0 ? v / hypot(S[p] - thp[j], eta) : v / (S[p] - thp[0]);
        }
    return 0;
}

/* G = A' B (ka x kb, column-major, leading dimension ka) for column-major blocks A (N x ka, lda),
 * B (N x kb, ldb), ka, kb <= 256.  Each thread sums a contiguous row range in packed 64-row
 * chunks (widths padded to multiples of 4 with zeros) with a 4 x 4 register tile per (i, j) block
 * into its own partial; the partials are added in thread order. */
int kf_ref_gram(int64_t N, int ka, const double *A, int64_t lda, int kb, const double *B, int64_t ldb, double *G) {
    enum { RB = 64, KM = 256 };
    if (ka > KM || kb > KM || ka < 0 || kb < 0) return 1;
    const int kap = (ka + 3) / 4 * 4, kbp = (kb + 3) / 4 * 4;
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    double *part = (double *)calloc((size_t)nt * (size_t)(kap * kbp > 0 ? kap * kbp : 1), sizeof(double));
    if (!part) return 1;
#pragma omp parallel num_threads(nt)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        const int64_t r0 = N * tid / nt, r1 = N * (tid + 1) / nt;
        double *acc = part + (size_t)tid * kap * kbp;
        double *a = (double *)calloc((size_t)RB * (kap > 0 ? kap : 1), sizeof(double));
        double *b = (double *)calloc((size_t)RB * (kbp > 0 ? kbp : 1), sizeof(double));
        for (int64_t p0 = r0; p0 < r1 && a && b; p0 += RB) {
            const int nr = (int)(r1 - p0 < RB ? r1 - p0 : RB);
            for (int i = 0; i < ka; ++i)
                for (int r = 0; r < nr; ++r) a[r * kap + i] = A[i * lda + p0 + r];
            for (int j = 0; j < kb; ++j)
                for (int r = 0; r < nr; ++r) b[r * kbp + j] = B[j * ldb + p0 + r];
            for (int i0 = 0; i0 < kap; i0 += 4)
                for (int j0 = 0; j0 < kbp; j0 += 4) {
                    double t[4][4] = {{0}};
                    for (int r = 0; r < nr; ++r) {
                        const double *ar = a + (size_t)r * kap + i0, *br = b + (size_t)r * kbp + j0;
                        for (int u = 0; u < 4; ++u)
                            for (int v = 0; v < 4; ++v) t[u][v] += ar[u] * br[v];
                    }
                    for (int u = 0; u < 4; ++u)
                        for (int v = 0; v < 4; ++v) acc[(size_t)(i0 + u) * kbp + j0 + v] += t[u][v];
                }
        }
        free(a);
        free(b);
    }
    for (int i = 0; i < ka; ++i)
        for (int j = 0; j < kb; ++j) {
            double s = 0.0;
            for (int t = 0; t < nt; ++t) s += part[(size_t)t * kap * kbp + (size_t)i * kbp + j];
            G[i + (size_t)ka * j] = s;
        }
    free(part);
    return 0;
}

/* Y = alpha X C + beta Y for column-major X (N x kx, ldx), C (kx x ky, column-major, ldc),
 * Y (N x ky, ldy); kx, ky <= 256; Y must not overlap X.  Threads over packed 64-row chunks; each
 * chunk's rows are formed 4 at a time against 4 output columns in a register tile. */
int kf_ref_update(int64_t N, int kx, const double *X, int64_t ldx, int ky, const double *Cm, int64_t ldc,
                  double alpha, double beta, double *Y, int64_t ldy) {
    enum { RB = 64, KM = 256 };
    if (kx > KM || ky > KM || kx < 0 || ky < 0) return 1;
    const int kyp = (ky + 3) / 4 * 4;
    double *Ct = (double *)calloc((size_t)(kx > 0 ? kx : 1) * (kyp > 0 ? kyp : 1), sizeof(double));
    if (!Ct) return 1;
    for (int i = 0; i < kx; ++i)
        for (int j = 0; j < ky; ++j) Ct[(size_t)i * kyp + j] = alpha * Cm[i + ldc * j];
    const int64_t nch = (N + RB - 1) / RB;
#pragma omp parallel
    {
        double *x = (double *)calloc((size_t)RB * (kx > 0 ? kx : 1), sizeof(double));
        double *y = (double *)calloc((size_t)RB * (kyp > 0 ? kyp : 1), sizeof(double));
#pragma omp for schedule(static)
        for (int64_t ch = 0; ch < nch; ++ch) {
            if (!x || !y) continue;
            const int64_t p0 = ch * RB;
            const int nr = (int)(N - p0 < RB ? N - p0 : RB);
            for (int i = 0; i < kx; ++i)
                for (int r = 0; r < nr; ++r) x[r * kx + i] = X[i * ldx + p0 + r];
            for (int r0 = 0; r0 < nr; r0 += 4)
                for (int j0 = 0; j0 < kyp; j0 += 4) {
                    double t[4][4] = {{0}};
                    const int nu = nr - r0 < 4 ? nr - r0 : 4;
                    for (int i = 0; i < kx; ++i) {
                        const double *cr = Ct + (size_t)i * kyp + j0;
                        for (int u = 0; u < 4; ++u) {
                            const double xv = u < nu ? x[(r0 + u) * kx + i] : 0.0;
                            for (int v = 0; v < 4; ++v) t[u][v] += xv * cr[v];
                        }
                    }
                    for (int u = 0; u < nu; ++u)
                        for (int v = 0; v < 4; ++v) y[(r0 + u) * kyp + j0 + v] = t[u][v];
                }
            for (int j = 0; j < ky; ++j) {
                double *yc = Y + j * ldy + p0;
                if (beta == 0.0)
                    for (int r = 0; r < nr; ++r) yc[r] = y[r * kyp + j];
                else
                    for (int r = 0; r < nr; ++r) yc[r] = beta * yc[r] + y[r * kyp + j];
            }
        }
        free(x);
        free(y);
    }
    free(Ct);
    return 0;
}

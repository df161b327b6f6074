/*
 * oracle/sparse_oracle.c -- TEST INFRASTRUCTURE ONLY (and the timed CPU
 * baseline of bench.py).
 *
 * CPU restatement (C + OpenMP) of the sparse kernels QuSpin 1.0.1 calls in
 * the un-vendored package parallel-sparse-tools==0.2.5 (pyproject.toml:9):
 *
 *   _wrapper_csr_trace      docs/modules/parallel_sparse_tools/
 *                           expm_multiply_parallel_core/expm_multiply_parallel_core.html:196-198
 *   _wrapper_csr_1_norm     same file :200-202
 *   _wrapper_expm_multiply  same file :347-359 (1-d v)
 *   _wrapper_expm_multiply_batch  same file :361-372 (2-d v)
 *   _matvec (csr)           docs/modules/parallel_sparse_tools/matvec/matvec_core.html:199-201
 *
 * The Taylor loop follows scipy's _expm_multiply_simple_core
 * (scipy/sparse/linalg/_expm_multiply.py, the function the reference's
 * scipy-parity tests compare against, test/test_expm_multiply_parallel.py:65-74)
 * with the shift folded into the product exactly as the reference's
 * matvec_p does (html :392-396): B <- a/(s(j+1)) * (A B - mu B).
 * The CSR SpMV partitions rows by equal nonzero counts, the load-balanced
 * scheme sphinx/source/tutorials/parallelization.rst:119 describes.
 *
 * Vectors are complex128 stored as interleaved doubles.  data is either
 * float64 (data_complex = 0) or complex128 (data_complex = 1).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int nthreads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int orc_num_threads(void) { return nthreads(); }

/* row boundaries giving each of nt parts about nnz/nt nonzeros */
static void nnz_partition(const int64_t *indptr, int64_t n, int nt, int64_t *bounds)
{
    int64_t nnz = indptr[n];
    bounds[0] = 0;
    for (int t = 1; t < nt; t++) {
        int64_t target = nnz * t / nt;
        int64_t lo = 0, hi = n;
        while (lo < hi) {
            int64_t mid = (lo + hi) / 2;
            if (indptr[mid] < target) lo = mid + 1; else hi = mid;
        }
        bounds[t] = lo < bounds[t - 1] ? bounds[t - 1] : lo;
    }
    bounds[nt] = n;
}

/* y (=|+=) a * A x ; x, y: [n, nvec] complex interleaved, C order. */
void orc_csr_matvec(const int64_t *indptr, const int32_t *indices, const double *data,
                    int data_complex, int64_t n, int64_t nvec,
                    double a_re, double a_im, const double *x, double *y, int overwrite)
{
    int nt = nthreads();
    int64_t *bounds = (int64_t *)malloc(sizeof(int64_t) * (nt + 1));
    nnz_partition(indptr, n, nt, bounds);
    #pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        int t = omp_get_thread_num();
#else
        int t = 0;
#endif
        double *acc = (double *)malloc(sizeof(double) * 2 * (nvec > 0 ? nvec : 1));
        for (int64_t r = bounds[t]; r < bounds[t + 1]; r++) {
            for (int64_t c = 0; c < nvec; c++) { acc[2 * c] = 0.0; acc[2 * c + 1] = 0.0; }
            for (int64_t k = indptr[r]; k < indptr[r + 1]; k++) {
                int64_t col = indices[k];
                double dr = data_complex ? data[2 * k] : data[k];
                double di = data_complex ? data[2 * k + 1] : 0.0;
                const double *xp = x + 2 * col * nvec;
                for (int64_t c = 0; c < nvec; c++) {
                    acc[2 * c] += dr * xp[2 * c] - di * xp[2 * c + 1];
                    acc[2 * c + 1] += dr * xp[2 * c + 1] + di * xp[2 * c];
                }
            }
            double *yp = y + 2 * r * nvec;
            for (int64_t c = 0; c < nvec; c++) {
                double vr = a_re * acc[2 * c] - a_im * acc[2 * c + 1];
                double vi = a_re * acc[2 * c + 1] + a_im * acc[2 * c];
                if (overwrite) { yp[2 * c] = vr; yp[2 * c + 1] = vi; }
                else { yp[2 * c] += vr; yp[2 * c + 1] += vi; }
            }
        }
        free(acc);
    }
    free(bounds);
}

/* trace of a CSR matrix (complex result written to out[0..1]) */
void orc_csr_trace(const int64_t *indptr, const int32_t *indices, const double *data,
                   int data_complex, int64_t n, double *out)
{
    double tr = 0.0, ti = 0.0;
    for (int64_t r = 0; r < n; r++)
        for (int64_t k = indptr[r]; k < indptr[r + 1]; k++)
            if (indices[k] == r) {
                tr += data_complex ? data[2 * k] : data[k];
                ti += data_complex ? data[2 * k + 1] : 0.0;
            }
    out[0] = tr; out[1] = ti;
}

/* max over columns of sum_r |A[r,c] + shift * delta_rc| */
double orc_csr_1_norm(const int64_t *indptr, const int32_t *indices, const double *data,
                      int data_complex, int64_t n, double shift_re, double shift_im)
{
    double *colsum = (double *)calloc(n > 0 ? n : 1, sizeof(double));
    char *hasdiag = (char *)calloc(n > 0 ? n : 1, 1);
    for (int64_t r = 0; r < n; r++)
        for (int64_t k = indptr[r]; k < indptr[r + 1]; k++) {
            int64_t c = indices[k];
            double vr = data_complex ? data[2 * k] : data[k];
            double vi = data_complex ? data[2 * k + 1] : 0.0;
            if (c == r) { vr += shift_re; vi += shift_im; hasdiag[r] = 1; }
            colsum[c] += hypot(vr, vi);
        }
    for (int64_t r = 0; r < n; r++) if (!hasdiag[r]) colsum[r] += hypot(shift_re, shift_im);
    double m = 0.0;
    for (int64_t c = 0; c < n; c++) if (colsum[c] > m) m = colsum[c];
    free(colsum); free(hasdiag);
    return m;
}

/* infinity norm of an [n, nvec] complex block: max_r sum_c |B[r,c]| */
static double inf_norm(const double *B, int64_t n, int64_t nvec)
{
    double m = 0.0;
    #pragma omp parallel for reduction(max:m)
    for (int64_t r = 0; r < n; r++) {
        double s = 0.0;
        for (int64_t c = 0; c < nvec; c++) s += hypot(B[2 * (r * nvec + c)], B[2 * (r * nvec + c) + 1]);
        if (s > m) m = s;
    }
    return m;
}

/*
 * Substep i of the s-substep truncated-Taylor evolution e^{aA} v
 * (_expm_multiply_simple_core, scipy _expm_multiply.py:280-306, with the
 * shift of expm_multiply_parallel_core.html:392-396): B = F, at most m_star
 * terms with coefficients a / (s (j + 1)), the infinity-norm stopping test,
 * then F = eta F.  F: [n, nvec] complex, updated in place; B, T: scratch of
 * the same size.  Returns the number of terms executed.
 */
static int64_t expm_substep(const int64_t *indptr, const int32_t *indices, const double *data, int data_complex,
                            int64_t n, int64_t nvec, const int64_t *bounds, int nt, int s, int m_star, double tol,
                            double mu_re, double mu_im, double a_re, double a_im, double eta_re, double eta_im,
                            double *F, double *B, double *T)
{
    int64_t len = 2 * n * nvec;
    memcpy(B, F, sizeof(double) * len);
    int64_t terms = 0;
    double c1 = inf_norm(B, n, nvec);
    for (int j = 0; j < m_star; j++) {
        double den = (double)s * (double)(j + 1);
        double cr = a_re / den, ci = a_im / den;
        double c2 = 0.0, fn = 0.0;
        #pragma omp parallel num_threads(nt) reduction(max:c2,fn)
        {
#ifdef _OPENMP
            int t = omp_get_thread_num();
#else
            int t = 0;
#endif
            double *acc = (double *)malloc(sizeof(double) * 2 * nvec);
            for (int64_t r = bounds[t]; r < bounds[t + 1]; r++) {
                for (int64_t c = 0; c < nvec; c++) { acc[2 * c] = 0.0; acc[2 * c + 1] = 0.0; }
                for (int64_t k = indptr[r]; k < indptr[r + 1]; k++) {
                    int64_t col = indices[k];
                    double dr = data_complex ? data[2 * k] : data[k];
                    double di = data_complex ? data[2 * k + 1] : 0.0;
                    const double *xp = B + 2 * col * nvec;
                    for (int64_t c = 0; c < nvec; c++) {
                        acc[2 * c] += dr * xp[2 * c] - di * xp[2 * c + 1];
                        acc[2 * c + 1] += dr * xp[2 * c + 1] + di * xp[2 * c];
                    }
                }
                double rs_b = 0.0, rs_f = 0.0;
                for (int64_t c = 0; c < nvec; c++) {
                    int64_t o = 2 * (r * nvec + c);
                    /* (A B - mu B) */
                    double wr = acc[2 * c] - (mu_re * B[o] - mu_im * B[o + 1]);
                    double wi = acc[2 * c + 1] - (mu_re * B[o + 1] + mu_im * B[o]);
                    double br = cr * wr - ci * wi;
                    double bi = cr * wi + ci * wr;
                    T[o] = br; T[o + 1] = bi;
                    F[o] += br; F[o + 1] += bi;
                    rs_b += hypot(br, bi);
                    rs_f += hypot(F[o], F[o + 1]);
                }
                if (rs_b > c2) c2 = rs_b;
                if (rs_f > fn) fn = rs_f;
            }
            free(acc);
        }
        double *sw = B; B = T; T = sw;
        terms++;
        if (c1 + c2 <= tol * fn) break;
        c1 = c2;
    }
    #pragma omp parallel for
    for (int64_t o = 0; o < len; o += 2) {
        double fr = F[o], fi = F[o + 1];
        F[o] = eta_re * fr - eta_im * fi;
        F[o + 1] = eta_re * fi + eta_im * fr;
    }
    return terms;
}

/*
 * In-place e^{aA} v (v: [n, nvec] complex), work: 2*n*nvec complex.
 * Returns the number of Taylor terms executed (for the error statement).
 */
int64_t orc_expm_multiply(const int64_t *indptr, const int32_t *indices, const double *data,
                          int data_complex, int64_t n, int64_t nvec,
                          int s, int m_star, double tol,
                          double mu_re, double mu_im, double a_re, double a_im,
                          double eta_re, double eta_im,
                          double *v, double *work)
{
    int nt = nthreads();
    int64_t *bounds = (int64_t *)malloc(sizeof(int64_t) * (nt + 1));
    nnz_partition(indptr, n, nt, bounds);
    int64_t len = 2 * n * nvec;
    int64_t terms = 0;
    for (int i = 0; i < s; i++)
        terms += expm_substep(indptr, indices, data, data_complex, n, nvec, bounds, nt, s, m_star, tol, mu_re, mu_im,
                              a_re, a_im, eta_re, eta_im, v, work, work + len);
    free(bounds);
    return terms;
}

/*
 * One substep of the s-substep evolution (the body of orc_expm_multiply's
 * loop) on v in place; work: 2*n*nvec complex.  Returns the terms executed.
 */
int64_t orc_expm_substep(const int64_t *indptr, const int32_t *indices, const double *data,
                         int data_complex, int64_t n, int64_t nvec,
                         int s, int m_star, double tol,
                         double mu_re, double mu_im, double a_re, double a_im,
                         double eta_re, double eta_im,
                         double *v, double *work)
{
    int nt = nthreads();
    int64_t *bounds = (int64_t *)malloc(sizeof(int64_t) * (nt + 1));
    nnz_partition(indptr, n, nt, bounds);
    int64_t len = 2 * n * nvec;
    int64_t terms = expm_substep(indptr, indices, data, data_complex, n, nvec, bounds, nt, s, m_star, tol, mu_re,
                                 mu_im, a_re, a_im, eta_re, eta_im, v, work, work + len);
    free(bounds);
    return terms;
}

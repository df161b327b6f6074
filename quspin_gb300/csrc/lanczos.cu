// Device-resident Lanczos recurrence.
//
// Replaces the numpy BLAS-1 steps of QuSpin 1.0.1's lanczos_full /
// lanczos_iter (src/quspin/tools/lanczos/_lanczos_utils.py:158-204 and
// :283-311) and lin_comb_Q_T (:366-425):
//   Q[i] = r / b[i-1];  r = A Q[i];  r -= b[i-1] Q[i-1];
//   a[i] = Re <Q[i], r>;  r -= a[i] Q[i];  b[i] = ||r||;  stop if b[i] < eps
// alpha / beta live in device arrays and the stopping test sets a device
// flag, so an m-step run needs no host synchronisation.  Reductions are
// two-stage and deterministic (per-block partials summed in a fixed order).
// Optional full reorthogonalisation (classical Gram-Schmidt applied twice
// against all previous Lanczos vectors, stored row-major in Q[m, n]) runs
// between the a[i] and b[i] steps.
#include "qs_common.cuh"

#define LZ_THREADS 256
#define LZ_BLOCKS_MAX 1024

struct LzCtl {
    int done;      // b[i] < eps was seen
    int m_eff;     // number of valid Lanczos vectors
};

extern "C" int qs_lanczos_ctl_bytes() { return (int)sizeof(LzCtl); }
extern "C" int qs_lanczos_scratch_doubles() { return 2 * LZ_BLOCKS_MAX; }

static int lz_blocks(int64_t n)
{
    int64_t b = (n + LZ_THREADS - 1) / LZ_THREADS;
    int cap = qs_num_sms() * 4;
    if (cap > LZ_BLOCKS_MAX) cap = LZ_BLOCKS_MAX;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

__device__ __forceinline__ double wsum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double sh[32];
    v = wsum(v);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    if (w == 0) {
        t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
        t = wsum(t);
    }
    return t;   // valid in thread 0
}

// q = r / b[i-1] (also the first step with b = norm of v0 when i == 0)
__global__ void lz_scale_kernel(int64_t n2, const double *__restrict__ r, const double *__restrict__ bptr,
                                double *__restrict__ q, const LzCtl *ctl)
{
    if (ctl && ctl->done) return;
    const double b = *bptr;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x)
        q[i] = r[i] / b;
}

// r -= b * v (if v) ; partial[blk] = sum Re(conj(q) r)
__global__ void lz_axpy_dot_kernel(int64_t n, int cplx, double *__restrict__ r, const double *__restrict__ v,
                                   const double *__restrict__ bptr, const double *__restrict__ q,
                                   double *__restrict__ partial, const LzCtl *ctl)
{
    if (ctl->done) return;
    const double b = v ? *bptr : 0.0;
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (cplx) {
            double rr = r[2 * i], ri = r[2 * i + 1];
            if (v) { rr -= b * v[2 * i]; ri -= b * v[2 * i + 1]; r[2 * i] = rr; r[2 * i + 1] = ri; }
            s += q[2 * i] * rr + q[2 * i + 1] * ri;
        } else {
            double rr = r[i];
            if (v) { rr -= b * v[i]; r[i] = rr; }
            s += q[i] * rr;
        }
    }
    s = block_sum(s);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// out = sum of partials (fixed order); mode 1: out = sqrt(sum); mode 2:
// b = sqrt(sum), and if b < eps set done / m_eff = i.
__global__ void lz_finish_kernel(int nb, const double *__restrict__ partial, double *__restrict__ out, int mode,
                                 double eps, int i, LzCtl *ctl)
{
    if (ctl->done) return;
    double s = 0.0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) s += partial[k];
    s = block_sum(s);
    if (threadIdx.x == 0) {
        if (mode == 0) *out = s;
        else {
            double b = sqrt(s);
            *out = b;
            if (mode == 2 && b < eps) { ctl->done = 1; ctl->m_eff = i; }
        }
    }
}

// r -= a * q ; partial[blk] = sum |r|^2
__global__ void lz_axpy_norm_kernel(int64_t n2, double *__restrict__ r, const double *__restrict__ aptr,
                                    const double *__restrict__ q, double *__restrict__ partial, const LzCtl *ctl,
                                    int do_axpy)
{
    if (ctl->done) return;
    const double a = do_axpy ? *aptr : 0.0;
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
        double x = r[i];
        if (do_axpy) { x -= a * q[i]; r[i] = x; }
        s += x * x;
    }
    s = block_sum(s);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// ---- full reorthogonalisation ---------------------------------------------
// h[k] = <Q[k], r> for k < nk: per-block partials part[blk * nk + k]
#define RO_ROWS 8
__global__ void lz_gemv_t_kernel(int64_t n, int cplx, int nk, const double *__restrict__ Q, int64_t ldq,
                                 const double *__restrict__ r, double *__restrict__ part, const LzCtl *ctl)
{
    if (ctl->done) return;
    __shared__ double sh[RO_ROWS][2][LZ_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k0 = 0; k0 < nk; k0 += RO_ROWS) {
        double sr[RO_ROWS], si[RO_ROWS];
#pragma unroll
        for (int t = 0; t < RO_ROWS; t++) { sr[t] = 0.0; si[t] = 0.0; }
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
            if (cplx) {
                double rr = r[2 * i], ri = r[2 * i + 1];
#pragma unroll
                for (int t = 0; t < RO_ROWS; t++) {
                    if (k0 + t < nk) {
                        const double *qk = Q + (int64_t)(k0 + t) * ldq;
                        double qr = qk[2 * i], qi = qk[2 * i + 1];
                        sr[t] += qr * rr + qi * ri;
                        si[t] += qr * ri - qi * rr;
                    }
                }
            } else {
                double rr = r[i];
#pragma unroll
                for (int t = 0; t < RO_ROWS; t++)
                    if (k0 + t < nk) sr[t] += Q[(int64_t)(k0 + t) * ldq + i] * rr;
            }
        }
#pragma unroll
        for (int t = 0; t < RO_ROWS; t++) {
            double a = wsum(sr[t]), b = wsum(si[t]);
            if (lane == 0) { sh[t][0][w] = a; sh[t][1][w] = b; }
        }
        __syncthreads();
        if (threadIdx.x < RO_ROWS && k0 + threadIdx.x < nk) {
            double a = 0.0, b = 0.0;
            for (int ww = 0; ww < LZ_THREADS / 32; ww++) { a += sh[threadIdx.x][0][ww]; b += sh[threadIdx.x][1][ww]; }
            int64_t o = ((int64_t)blockIdx.x * nk + k0 + threadIdx.x) * 2;
            part[o] = a;
            part[o + 1] = b;
        }
        __syncthreads();
    }
}

// h[k] = sum over blocks of part[blk * nk + k] (fixed order)
__global__ void lz_gemv_t_finish(int nb, int nk, const double *__restrict__ part, double *__restrict__ h,
                                 const LzCtl *ctl)
{
    if (ctl->done) return;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nk; k += gridDim.x * blockDim.x) {
        double a = 0.0, b = 0.0;
        for (int blk = 0; blk < nb; blk++) { a += part[((int64_t)blk * nk + k) * 2]; b += part[((int64_t)blk * nk + k) * 2 + 1]; }
        h[2 * k] = a;
        h[2 * k + 1] = b;
    }
}

// r -= sum_k h[k] Q[k]
__global__ void lz_gemv_n_kernel(int64_t n, int cplx, int nk, const double *__restrict__ Q, int64_t ldq,
                                 const double *__restrict__ h, double *__restrict__ r, const LzCtl *ctl)
{
    if (ctl->done) return;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (cplx) {
            double ar = 0.0, ai = 0.0;
            for (int k = 0; k < nk; k++) {
                const double *qk = Q + (int64_t)k * ldq;
                double qr = qk[2 * i], qi = qk[2 * i + 1], hr = h[2 * k], hi = h[2 * k + 1];
                ar += qr * hr - qi * hi;
                ai += qr * hi + qi * hr;
            }
            r[2 * i] -= ar;
            r[2 * i + 1] -= ai;
        } else {
            double a = 0.0;
            for (int k = 0; k < nk; k++) a += Q[(int64_t)k * ldq + i] * h[2 * k];
            r[i] -= a;
        }
    }
}

// q = r / b (b device scalar); skipped once the stopping test fired
extern "C" int qs_lanczos_scale(int64_t n2, const double *r, const double *bptr, double *q, const void *ctl,
                                void *stream)
{
    if (n2 < 0 || !r || !bptr || !q) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    lz_scale_kernel<<<lz_blocks(n2), LZ_THREADS, 0, st>>>(n2, r, bptr, q, (const LzCtl *)ctl);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// r -= b * v (v may be NULL); a_out = Re <q, r>
extern "C" int qs_lanczos_alpha(int64_t n, int cplx, double *r, const double *v, const double *bptr,
                                const double *q, double *a_out, double *scratch, void *ctl, void *stream)
{
    if (n < 0 || !r || !q || !a_out || !scratch || !ctl) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    int nb = lz_blocks(n);
    lz_axpy_dot_kernel<<<nb, LZ_THREADS, 0, st>>>(n, cplx, r, v, bptr, q, scratch, (const LzCtl *)ctl);
    lz_finish_kernel<<<1, LZ_THREADS, 0, st>>>(nb, scratch, a_out, 0, 0.0, 0, (LzCtl *)ctl);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// r -= a * q (if do_axpy); b_out = ||r||; if b_out < eps: done, m_eff = i
extern "C" int qs_lanczos_beta(int64_t n2, double *r, const double *aptr, const double *q, int do_axpy,
                               double *b_out, double eps, int i, double *scratch, void *ctl, void *stream)
{
    if (n2 < 0 || !r || !b_out || !scratch || !ctl) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    int nb = lz_blocks(n2);
    lz_axpy_norm_kernel<<<nb, LZ_THREADS, 0, st>>>(n2, r, aptr, q, scratch, (const LzCtl *)ctl, do_axpy);
    lz_finish_kernel<<<1, LZ_THREADS, 0, st>>>(nb, scratch, b_out, 2, eps, i, (LzCtl *)ctl);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

extern "C" int64_t qs_lanczos_reorth_scratch_doubles(int nk)
{
    return (int64_t)2 * LZ_BLOCKS_MAX * (nk > 0 ? nk : 1) + 2 * (int64_t)(nk > 0 ? nk : 1);
}

// Classical Gram-Schmidt, applied `passes` times: r -= Q[:nk]^T (conj(Q[:nk]) r).
// Q row-major [>= nk, ldq] (ldq in elements: doubles for real, complex
// numbers for complex vectors).
extern "C" int qs_lanczos_reorth(int64_t n, int cplx, int nk, const double *Q, int64_t ldq, double *r, int passes,
                                 double *scratch, void *ctl, void *stream)
{
    if (n < 0 || nk < 0 || !Q || !r || !scratch || !ctl) return QS_ERR_ARG;
    if (nk == 0) return QS_OK;
    cudaStream_t st = qs_stream(stream);
    int nb = lz_blocks(n);
    double *part = scratch;
    double *h = scratch + (int64_t)2 * LZ_BLOCKS_MAX * nk;
    for (int p = 0; p < passes; p++) {
        lz_gemv_t_kernel<<<nb, LZ_THREADS, 0, st>>>(n, cplx, nk, Q, cplx ? 2 * ldq : ldq, r, part, (const LzCtl *)ctl);
        lz_gemv_t_finish<<<(nk + 127) / 128, 128, 0, st>>>(nb, nk, part, h, (const LzCtl *)ctl);
        lz_gemv_n_kernel<<<nb, LZ_THREADS, 0, st>>>(n, cplx, nk, Q, cplx ? 2 * ldq : ldq, h, r, (const LzCtl *)ctl);
    }
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// out = sum_k c[k] Q[k]  (c real [nk] on the device; Q row-major)
__global__ void lz_lincomb_kernel(int64_t n2, int nk, const double *__restrict__ c, int cplx_c,
                                  const double *__restrict__ Q, int64_t ldq2, int cplx_q, double *__restrict__ out)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
        if (!cplx_c) {
            double a = 0.0;
            for (int k = 0; k < nk; k++) a += c[k] * Q[(int64_t)k * ldq2 + i];
            out[i] = a;
        } else {
            // complex coefficients: i indexes complex output elements
            double ar = 0.0, ai = 0.0;
            for (int k = 0; k < nk; k++) {
                double cr = c[2 * k], ci = c[2 * k + 1];
                if (cplx_q) {
                    double qr = Q[(int64_t)k * ldq2 + 2 * i], qi = Q[(int64_t)k * ldq2 + 2 * i + 1];
                    ar += cr * qr - ci * qi;
                    ai += cr * qi + ci * qr;
                } else {
                    double q = Q[(int64_t)k * ldq2 + i];
                    ar += cr * q;
                    ai += ci * q;
                }
            }
            out[2 * i] = ar;
            out[2 * i + 1] = ai;
        }
    }
}

// lin_comb_Q_T: out = sum_k c[k] Q[k].  n_el: elements per Lanczos vector;
// cplx_c / cplx_q: coefficient / vector complexity; ldq: row stride in
// elements of Q.
extern "C" int qs_lanczos_lincomb(int64_t n_el, int nk, const double *c, int cplx_c, const double *Q, int64_t ldq,
                                  int cplx_q, double *out, void *stream)
{
    if (n_el < 0 || nk < 0 || !c || !Q || !out) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    int64_t ldq2 = cplx_q ? 2 * ldq : ldq;
    int64_t work = cplx_c ? n_el : (cplx_q ? 2 * n_el : n_el);
    int64_t b = (work + 255) / 256, cap = (int64_t)qs_num_sms() * 8;
    lz_lincomb_kernel<<<(unsigned)(b > cap ? cap : (b < 1 ? 1 : b)), 256, 0, st>>>(work, nk, c, cplx_c, Q, ldq2, cplx_q, out);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

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
// h[k] = <Q[k], r> for k < nk.  Each thread keeps 16 FP64 accumulators: 16
// rows (real) or 8 rows x (re, im) (complex).  A warp reduces them with a
// reduce-scatter butterfly (16 adds per lane instead of 5 per accumulator),
// which matters here because the FP64 pipe, not HBM, bounds this kernel.
// Per-block partials go to part[a * nb + blk], a = k (real) or 2k + c
// (complex), so that the finish kernel reads them contiguously.
#define RO_ACC 16

// sum over the 32 lanes of v[0..15]; returns the full warp sum of
// accumulator lane >> 1 (the same value in lanes 2a and 2a + 1)
__device__ __forceinline__ double warp_reduce_scatter16(double (&v)[RO_ACC], int lane)
{
    double w[8], x[4], y[2];
    const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4, b1 = lane & 2;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const double send = b4 ? v[j] : v[j + 8], keep = b4 ? v[j + 8] : v[j];
        w[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const double send = b3 ? w[j] : w[j + 4], keep = b3 ? w[j + 4] : w[j];
        x[j] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
#pragma unroll
    for (int j = 0; j < 2; j++) {
        const double send = b2 ? x[j] : x[j + 2], keep = b2 ? x[j + 2] : x[j];
        y[j] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    const double send = b1 ? y[0] : y[1], keep = b1 ? y[1] : y[0];
    double z = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    return z + __shfl_xor_sync(0xffffffffu, z, 1);
}

template <bool CPLX>
__global__ void __launch_bounds__(LZ_THREADS, 4)
lz_gemv_t_kernel(int64_t n, int nk, const double *__restrict__ Q, int64_t ldq, const double *__restrict__ r,
                 double *__restrict__ part, const LzCtl *ctl, const double *skip)
{
    if (ctl->done || (skip && *skip != 0.0)) return;
    constexpr int R = CPLX ? RO_ACC / 2 : RO_ACC;   // rows per group
    __shared__ double sh[RO_ACC][LZ_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nb = gridDim.x;
    for (int k0 = 0; k0 < nk; k0 += R) {
        const int rows = nk - k0 < R ? nk - k0 : R;
        double acc[RO_ACC];
#pragma unroll
        for (int t = 0; t < RO_ACC; t++) acc[t] = 0.0;
        const double *q0 = Q + (int64_t)k0 * ldq;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
            if constexpr (CPLX) {
                const double rr = r[2 * i], ri = r[2 * i + 1];
#pragma unroll
                for (int t = 0; t < R; t++) {
                    if (t < rows) {
                        const double qr = q0[t * ldq + 2 * i], qi = q0[t * ldq + 2 * i + 1];
                        acc[2 * t] += qr * rr + qi * ri;
                        acc[2 * t + 1] += qr * ri - qi * rr;
                    }
                }
            } else {
                const double rr = r[i];
#pragma unroll
                for (int t = 0; t < R; t++)
                    if (t < rows) acc[t] += q0[t * ldq + i] * rr;
            }
        }
        const double s = warp_reduce_scatter16(acc, lane);
        if (!(lane & 1)) sh[lane >> 1][w] = s;
        __syncthreads();
        if (threadIdx.x < RO_ACC) {
            const int a = threadIdx.x;
            if ((CPLX ? a >> 1 : a) < rows) {
                double tot = 0.0;
                for (int ww = 0; ww < LZ_THREADS / 32; ww++) tot += sh[a][ww];
                part[((int64_t)(CPLX ? 2 * k0 : k0) + a) * nb + blockIdx.x] = tot;
            }
        }
        __syncthreads();
    }
}

// h[k] = sum over blocks of the partials (one warp per accumulator, fixed
// order: strided lane sums, then a butterfly); real: h[2k + 1] = 0
__global__ void lz_gemv_t_finish(int nb, int nk, int cplx, const double *__restrict__ part, double *__restrict__ h,
                                 const LzCtl *ctl, const double *skip)
{
    if (ctl->done || (skip && *skip != 0.0)) return;
    const int a = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (a >= (cplx ? 2 * nk : nk)) return;
    const double *p = part + (int64_t)a * nb;
    double s = 0.0;
    for (int b = lane; b < nb; b += 32) s += p[b];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        if (cplx) h[a] = s;
        else { h[2 * a] = s; h[2 * a + 1] = 0.0; }
    }
}

// r -= sum_k h[k] Q[k]
__global__ void lz_gemv_n_kernel(int64_t n, int cplx, int nk, const double *__restrict__ Q, int64_t ldq,
                                 const double *__restrict__ h, double *__restrict__ r, const LzCtl *ctl,
                                 const double *skip)
{
    if (ctl->done || (skip && *skip != 0.0)) return;
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

// Scratch: per-block partials of h (2 * LZ_BLOCKS_MAX * nk), h (2 nk), the
// pass-control state (2) and the norm partials (LZ_BLOCKS_MAX).
extern "C" int64_t qs_lanczos_reorth_scratch_doubles(int nk)
{
    const int64_t k = nk > 0 ? nk : 1;
    return (int64_t)2 * LZ_BLOCKS_MAX * k + 2 * k + 2 + LZ_BLOCKS_MAX;
}

// Pass control of the adaptive reorthogonalisation.  state[0]: squared norm
// of r before the last pass; state[1]: 1 once a pass kept at least 1/sqrt(2)
// of the norm (then r is orthogonal to the rows to working precision and
// the remaining passes return at once).  first: record the norm of the
// incoming r and clear the flag.
__global__ void lz_dgks_kernel(int nb, const double *__restrict__ partial, double *state, int first, const LzCtl *ctl)
{
    if (ctl->done) return;
    if (!first && state[1] != 0.0) return;
    double s = 0.0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) s += partial[k];
    s = block_sum(s);
    if (threadIdx.x == 0) {
        if (first) {
            state[0] = s;
            state[1] = 0.0;
        } else if (s >= 0.5 * state[0]) {
            state[1] = 1.0;
        } else {
            state[0] = s;
        }
    }
}

static void reorth_pass(cudaStream_t st, int nb, int64_t n, int cplx, int nk, const double *Q, int64_t ldq, double *r,
                        double *part, double *h, const LzCtl *ctl, const double *skip)
{
    if (cplx) lz_gemv_t_kernel<true><<<nb, LZ_THREADS, 0, st>>>(n, nk, Q, 2 * ldq, r, part, ctl, skip);
    else lz_gemv_t_kernel<false><<<nb, LZ_THREADS, 0, st>>>(n, nk, Q, ldq, r, part, ctl, skip);
    const int nacc = cplx ? 2 * nk : nk;
    lz_gemv_t_finish<<<(nacc + 7) / 8, 256, 0, st>>>(nb, nk, cplx, part, h, ctl, skip);
    lz_gemv_n_kernel<<<nb, LZ_THREADS, 0, st>>>(n, cplx, nk, Q, cplx ? 2 * ldq : ldq, h, r, ctl, skip);
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
    for (int p = 0; p < passes; p++) reorth_pass(st, nb, n, cplx, nk, Q, ldq, r, part, h, (const LzCtl *)ctl, nullptr);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// The same with the pass count decided on the device (the criterion of
// Daniel, Gragg, Kaufman and Stewart, Math. Comp. 30 (1976) 772, as ARPACK
// applies it): after each pass the norm of r is compared with its norm
// before the pass; if at least 1/sqrt(2) of it remains, r is orthogonal to
// the rows to working precision and no further pass runs; otherwise another
// pass follows, up to max_passes.  No host synchronisation.
extern "C" int qs_lanczos_reorth_adaptive(int64_t n, int cplx, int nk, const double *Q, int64_t ldq, double *r,
                                          int max_passes, double *scratch, void *ctl, void *stream)
{
    if (n < 0 || nk < 0 || max_passes < 1 || !Q || !r || !scratch || !ctl) return QS_ERR_ARG;
    if (nk == 0) return QS_OK;
    cudaStream_t st = qs_stream(stream);
    const int nb = lz_blocks(n);
    const int64_t n2 = cplx ? 2 * n : n;
    const int nbn = lz_blocks(n2);
    double *part = scratch;
    double *h = scratch + (int64_t)2 * LZ_BLOCKS_MAX * nk;
    double *state = h + 2 * (int64_t)nk;
    double *npart = state + 2;
    const LzCtl *c = (const LzCtl *)ctl;
    lz_axpy_norm_kernel<<<nbn, LZ_THREADS, 0, st>>>(n2, r, nullptr, nullptr, npart, c, 0);
    lz_dgks_kernel<<<1, LZ_THREADS, 0, st>>>(nbn, npart, state, 1, c);
    for (int p = 0; p < max_passes; p++) {
        reorth_pass(st, nb, n, cplx, nk, Q, ldq, r, part, h, c, p == 0 ? nullptr : state + 1);
        if (p + 1 < max_passes) {
            lz_axpy_norm_kernel<<<nbn, LZ_THREADS, 0, st>>>(n2, r, nullptr, nullptr, npart, c, 0);
            lz_dgks_kernel<<<1, LZ_THREADS, 0, st>>>(nbn, npart, state, 0, c);
        }
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

// Truncated-Taylor action of the matrix exponential, e^{aA} v, on the GPU.
//
// Replaces the native loop QuSpin 1.0.1 runs through
// parallel-sparse-tools==0.2.5 (_wrapper_expm_multiply and
// _wrapper_expm_multiply_batch, called at
// docs/modules/parallel_sparse_tools/expm_multiply_parallel_core/
// expm_multiply_parallel_core.html:347-372).  Its contract, which the
// reference's tests pin against scipy at 1e-15 (test/test_expm_multiply_parallel.py:65-74),
// is scipy's _expm_multiply_simple_core with the shift folded into the
// product (html :392-396):
//
//   F = v; B = v; eta = exp(a mu / s)
//   repeat s times:
//     c1 = ||B||_inf
//     for j < m*:  B = a/(s(j+1)) (A B - mu B);  c2 = ||B||_inf;  F += B
//                  stop if c1 + c2 <= tol ||F||_inf;  c1 = c2
//     F = eta F;  B = F
//
// One launch per Taylor term does the whole term: CSR apply, shift, scale,
// accumulate into F and both infinity norms (row sums of moduli over the k
// right-hand sides).  The last block of each launch evaluates the stopping
// test in a small device control block, so the host never synchronises;
// launches after the test has fired return immediately.  The kernels here do
// every product in IEEE double (the "ieee" form); csrc/expm_lp.cu holds the
// paired-single and complex64 forms of the same term, selected by btype.
#include "qs_common.cuh"
#include "expm_ctl.cuh"

extern "C" int qs_expm_ctl_bytes() { return (int)sizeof(ExpmCtl); }
extern "C" int qs_multi_ctl_bytes() { return (int)sizeof(MultiCtl); }
extern "C" int qs_max_sectors() { return QS_MAX_SECTORS; }

template <typename T> struct BLoad;
template <> struct BLoad<cdbl> {
    __device__ static cdbl ld(const cdbl *p, int64_t i) {
        double2 v = __ldg(reinterpret_cast<const double2 *>(p) + i);
        return cdbl{v.x, v.y};
    }
    __device__ static void st(cdbl *p, int64_t i, cdbl v) { p[i] = v; }
};
template <typename T> struct DLoad;
template <> struct DLoad<double> { __device__ static double ld(const double *p, int64_t i) { return __ldg(p + i); } };
template <> struct DLoad<cdbl> {
    __device__ static cdbl ld(const cdbl *p, int64_t i) {
        double2 v = __ldg(reinterpret_cast<const double2 *>(p) + i);
        return cdbl{v.x, v.y};
    }
};

__device__ __forceinline__ void madd(cdbl &acc, double d, cdbl x) { acc.x += d * x.x; acc.y += d * x.y; }
__device__ __forceinline__ void madd(cdbl &acc, cdbl d, cdbl x)
{
    acc.x += d.x * x.x - d.y * x.y;
    acc.y += d.x * x.y + d.y * x.x;
}

__device__ __forceinline__ double cabs_(cdbl v) { return hypot(v.x, v.y); }

// F and the new term are touched once per term: stream them (evict-first)
// so the gathered vector keeps its place in L2.
__device__ __forceinline__ cdbl ldF(const cdbl *p)
{
    double2 v = __ldcs(reinterpret_cast<const double2 *>(p));
    return cdbl{v.x, v.y};
}
__device__ __forceinline__ void stF(cdbl *p, cdbl v) { __stcs(reinterpret_cast<double2 *>(p), make_double2(v.x, v.y)); }
__device__ __forceinline__ void stB(cdbl *p, cdbl v) { __stcs(reinterpret_cast<double2 *>(p), make_double2(v.x, v.y)); }

template <typename T> __device__ __forceinline__ T st_ld(const T *p) { return __ldcs(p); }
template <> __device__ __forceinline__ cdbl st_ld<cdbl>(const cdbl *p)
{
    double2 v = __ldcs(reinterpret_cast<const double2 *>(p));
    return cdbl{v.x, v.y};
}
__device__ __forceinline__ double wid(double v) { return v; }
__device__ __forceinline__ cdbl wid(cdbl v) { return v; }
template <typename T> __device__ __forceinline__ T zro();
template <> __device__ __forceinline__ double zro<double>() { return 0.0; }
template <> __device__ __forceinline__ cdbl zro<cdbl>() { return cdbl{0.0, 0.0}; }

// G lanes per row, U independent entries per lane per step, NB right-hand
// sides per pass (see csrc/sparse.cu for the row hand-out rule).
template <typename DT, typename BT, typename IT, int G, int NB, int U>
__global__ void __launch_bounds__(256) taylor_term_kernel(int64_t n, const IT *__restrict__ indptr,
                                                          const int32_t *__restrict__ indices,
                                                          const DT *__restrict__ data, const BT *__restrict__ Bin,
                                                          BT *__restrict__ Bout, cdbl *__restrict__ F, int64_t nvec,
                                                          cdbl mu, const cdbl *__restrict__ coeff, int j,
                                                          double tol, ExpmCtl *ctl)
{
    if (*((volatile int *)&ctl->done)) return;
    const cdbl cf = coeff[j];
    // Rows are handed out per warp (32/G consecutive rows per warp and
    // iteration): the loop bound is warp-uniform, so every lane reaches the
    // full-mask shuffles; groups past the last row idle.
    constexpr int GPW = 32 / G;
    const int lane = threadIdx.x & (G - 1);
    const int gsub = (threadIdx.x & 31) / G;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double mb = 0.0, mf = 0.0;
    for (int64_t rb = warp * GPW; rb < n; rb += nwarps * GPW) {
        const int64_t r = rb + gsub;
        const bool valid = r < n;
        const IT k0 = valid ? indptr[r] : (IT)0, k1 = valid ? indptr[r + 1] : (IT)0;
        double rb_ = 0.0, rf = 0.0;
        // the row's own B and F entries do not depend on the gathers: load them
        // first so their latency overlaps the row's gather loop
        cdbl bo_pre{0.0, 0.0}, f_pre{0.0, 0.0};
        if (NB == 1 && valid && lane == 0) {
            bo_pre = BLoad<BT>::ld(Bin, r);
            f_pre = ldF(F + r);
        }
        for (int64_t c0 = 0; c0 < nvec; c0 += NB) {
            cdbl acc[NB];
#pragma unroll
            for (int b = 0; b < NB; b++) acc[b] = cdbl{0.0, 0.0};
            for (IT k = k0 + lane; k < k1; k += G * U) {
                int32_t col[U];
                DT d[U];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const IT kk = k + u * G;
                    const bool in = kk < k1;
                    col[u] = in ? st_ld(indices + kk) : 0;
                    d[u] = in ? st_ld(data + kk) : zro<DT>();
                }
#pragma unroll
                for (int u = 0; u < U; u++) {
                    if (k + u * G < k1) {
#pragma unroll
                        for (int b = 0; b < NB; b++)
                            if (c0 + b < nvec) madd(acc[b], wid(d[u]), BLoad<BT>::ld(Bin, (int64_t)col[u] * nvec + c0 + b));
                    }
                }
            }
#pragma unroll
            for (int b = 0; b < NB; b++) {
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) {
                    acc[b].x += __shfl_down_sync(0xffffffffu, acc[b].x, o, G);
                    acc[b].y += __shfl_down_sync(0xffffffffu, acc[b].y, o, G);
                }
            }
            if (valid && lane == 0) {
#pragma unroll
                for (int b = 0; b < NB; b++) {
                    if (c0 + b >= nvec) break;
                    const int64_t e = r * nvec + c0 + b;
                    const cdbl bo = (NB == 1) ? bo_pre : BLoad<BT>::ld(Bin, e);
                    // w = A B - mu B
                    const double wr = acc[b].x - (mu.x * bo.x - mu.y * bo.y);
                    const double wi = acc[b].y - (mu.x * bo.y + mu.y * bo.x);
                    cdbl bn{cf.x * wr - cf.y * wi, cf.x * wi + cf.y * wr};
                    stB(Bout + e, bn);
                    cdbl f = (NB == 1) ? f_pre : ldF(F + e);
                    f.x += bn.x; f.y += bn.y;
                    stF(F + e, f);
                    if (NB == 1) {
                        // one column: track squared moduli, take the square
                        // root once (same value: sqrt is monotonic)
                        rb_ = bn.x * bn.x + bn.y * bn.y;
                        rf = f.x * f.x + f.y * f.y;
                    } else {
                        rb_ += cabs_(bn);
                        rf += cabs_(f);
                    }
                }
            }
        }
        mb = fmax(mb, rb_);
        mf = fmax(mf, rf);
    }
    fold_max2(mb, mf, &ctl->c2, &ctl->fn);
    if (last_block(ctl) && threadIdx.x == 0) {
        volatile ExpmCtl *vc = ctl;
        double c2 = __longlong_as_double((long long)vc->c2);
        double fn = __longlong_as_double((long long)vc->fn);
        if (nvec == 1) { c2 = sqrt(c2); fn = sqrt(fn); }
        vc->terms = vc->terms + 1;
        if (vc->c1 + c2 <= tol * fn) vc->done = 1;
        else vc->c1 = c2;
        vc->c2 = 0ull;
        vc->fn = 0ull;
        __threadfence();
        vc->arrive = 0u;
    }
}

// F = eta F; B0 = F; ctl->c1 = ||F||_inf; ctl->done = 0.  At the end of a
// substep (substep_end) a stopping test that never fired is counted in
// ctl->nonconv.
template <typename BT>
__global__ void __launch_bounds__(256) taylor_rescale_kernel(int64_t n, int64_t nvec, cdbl *__restrict__ F,
                                                             BT *__restrict__ B0, const cdbl *__restrict__ eta_p,
                                                             ExpmCtl *ctl, int substep_end)
{
    const cdbl eta = *eta_p;
    const bool scale = !(eta.x == 1.0 && eta.y == 0.0);
    double m = 0.0;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        double rs = 0.0;
        for (int64_t c = 0; c < nvec; c++) {
            const int64_t e = r * nvec + c;
            cdbl f = F[e];
            if (scale) {
                cdbl g{eta.x * f.x - eta.y * f.y, eta.x * f.y + eta.y * f.x};
                f = g;
                F[e] = f;
            }
            BLoad<BT>::st(B0, e, f);
            rs += cabs_(f);
        }
        m = fmax(m, rs);
    }
    fold_max2(m, 0.0, &ctl->c2, nullptr);
    if (last_block(ctl) && threadIdx.x == 0) {
        volatile ExpmCtl *vc = ctl;
        vc->c1 = __longlong_as_double((long long)vc->c2);
        vc->c2 = 0ull;
        vc->fn = 0ull;
        if (substep_end && !vc->done) vc->nonconv = vc->nonconv + 1;
        vc->done = 0;
        __threadfence();
        vc->arrive = 0u;
    }
}

static int pick_group_e(int64_t n, int64_t nnz)
{
    double avg = n > 0 ? (double)nnz / (double)n : 1.0;
    int g = 2;
    while (g < 32 && g * 24 < avg) g <<= 1;
    return g;
}

static int grid_for(int64_t n, int G)
{
    int64_t gpb = 256 / G;   // rows per block per iteration
    int64_t b = (n + gpb - 1) / gpb;
    int64_t cap = (int64_t)qs_num_sms() * 16;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

template <typename DT, typename BT, typename IT, int NB, int U>
static int term_launch(int64_t n, const void *indptr, const int32_t *indices, const void *data, const void *Bin,
                       void *Bout, cdbl *F, int64_t nvec, cdbl mu, const cdbl *coeff, int j, double tol, ExpmCtl *ctl,
                       int G, cudaStream_t st)
{
    int blocks = grid_for(n, G);
#define L_(GG) taylor_term_kernel<DT, BT, IT, GG, NB, U><<<blocks, 256, 0, st>>>(n, (const IT *)indptr, indices, (const DT *)data, (const BT *)Bin, (BT *)Bout, F, nvec, mu, coeff, j, tol, ctl)
    switch (G) {
    case 2: L_(2); break;
    case 4: L_(4); break;
    case 8: L_(8); break;
    case 16: L_(16); break;
    default: L_(32); break;
    }
#undef L_
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

template <typename DT, typename BT, typename IT>
static int term_nb(int64_t n, const void *indptr, const int32_t *indices, const void *data, const void *Bin,
                   void *Bout, cdbl *F, int64_t nvec, cdbl mu, const cdbl *coeff, int j, double tol, ExpmCtl *ctl,
                   int G, int U, cudaStream_t st)
{
    if (nvec == 1) {
        if (U >= 4) return term_launch<DT, BT, IT, 1, 4>(n, indptr, indices, data, Bin, Bout, F, nvec, mu, coeff, j, tol, ctl, G, st);
        if (U == 2) return term_launch<DT, BT, IT, 1, 2>(n, indptr, indices, data, Bin, Bout, F, nvec, mu, coeff, j, tol, ctl, G, st);
        return term_launch<DT, BT, IT, 1, 1>(n, indptr, indices, data, Bin, Bout, F, nvec, mu, coeff, j, tol, ctl, G, st);
    }
    if (nvec == 2) return term_launch<DT, BT, IT, 2, 1>(n, indptr, indices, data, Bin, Bout, F, nvec, mu, coeff, j, tol, ctl, G, st);
    if (nvec <= 4) return term_launch<DT, BT, IT, 4, 1>(n, indptr, indices, data, Bin, Bout, F, nvec, mu, coeff, j, tol, ctl, G, st);
    return term_launch<DT, BT, IT, 8, 1>(n, indptr, indices, data, Bin, Bout, F, nvec, mu, coeff, j, tol, ctl, G, st);
}

template <typename DT, typename BT>
static int term_idx(int idx64, int64_t n, const void *indptr, const int32_t *indices, const void *data,
                    const void *Bin, void *Bout, cdbl *F, int64_t nvec, cdbl mu, const cdbl *coeff, int j, double tol,
                    ExpmCtl *ctl, int G, int U, cudaStream_t st)
{
    if (idx64) return term_nb<DT, BT, int64_t>(n, indptr, indices, data, Bin, Bout, F, nvec, mu, coeff, j, tol, ctl, G, 1, st);
    return term_nb<DT, BT, int32_t>(n, indptr, indices, data, Bin, Bout, F, nvec, mu, coeff, j, tol, ctl, G, U, st);
}

// One Taylor term (see file header).  btype: storage of B -- QS_C128 (IEEE
// double; dtype QS_F64 / QS_C128), QS_CPF (paired single; dtype QS_PF /
// QS_CPF, values split by qs_split_pairs) or QS_C64 (dtype QS_F32 / QS_C64);
// F is complex128 [n, nvec]; coeff: device complex128 table, term j uses coeff[j];
// ctl: device control block (qs_expm_ctl_bytes()).  group: launch shape,
// G | (U << 8) | (C << 16) (G lanes per row 2..32, U = 1, 2, 4 entries in flight
// per lane; C = 1 asks the float forms for the chunk-outer sweep, which takes
// effect only through qs_taylor_term_rows with a row-sum scratch; bit 17
// narrows its chunks from 8 to 4 vectors; bits 18-19 cap the registers of the
// single-vector float-pair shapes for 6 / 8 blocks per SM; bits 20-22 = 1..7
// select a single-vector kernel of csrc/expm_st.cu: 1..3 the 32-row kernel
// with 4, 2 or 8 lanes per row, 4..7 the persistent row-handout kernel with
// 2 or 4 lanes per row (bits 18-19 then cap registers for 6 / 5 blocks per
// SM; 6..7 read packed column words four per load) -- one vector, int32
// indices; the packed value forms 8 / 9 run only there; with several
// vectors, 1..3 select the vectors-across-lanes kernel of csrc/expm_vl.cu;
// 0 picks G from nnz/n and U = 2.
extern "C" int qs_taylor_term_rows(int64_t n, int64_t nnz, const void *indptr, int idx64, const int32_t *indices,
                                   const void *data, int dtype, const void *Bin, void *Bout, int btype, void *F,
                                   int64_t nvec, double mu_re, double mu_im, const void *coeff, int j, double tol,
                                   void *ctl, int group, void *rownorm, void *stream);

extern "C" int qs_taylor_term(int64_t n, int64_t nnz, const void *indptr, int idx64, const int32_t *indices,
                              const void *data, int dtype, const void *Bin, void *Bout, int btype, void *F,
                              int64_t nvec, double mu_re, double mu_im, const void *coeff, int j, double tol,
                              void *ctl, int group, void *stream)
{
    return qs_taylor_term_rows(n, nnz, indptr, idx64, indices, data, dtype, Bin, Bout, btype, F, nvec, mu_re, mu_im,
                               coeff, j, tol, ctl, group, nullptr, stream);
}

// qs_taylor_term with row-sum scratch: with rownorm (n double pairs) and the
// chunk bit of group set (1 << 16), the float forms sweep the rows once per
// vector chunk of 8 so the gathered slice of B can stay in L2.
extern "C" int qs_taylor_term_rows(int64_t n, int64_t nnz, const void *indptr, int idx64, const int32_t *indices,
                                   const void *data, int dtype, const void *Bin, void *Bout, int btype, void *F,
                                   int64_t nvec, double mu_re, double mu_im, const void *coeff, int j, double tol,
                                   void *ctl, int group, void *rownorm, void *stream)
{
    if (n < 1 || nvec < 1 || !indptr || !Bin || !Bout || !F || !coeff || !ctl || j < 0) return QS_ERR_ARG;
    int G = group > 0 ? (group & 0xff) : pick_group_e(n, nnz);
    int U = group > 0 ? ((group >> 8) & 0xff) : 2;
    if (U < 1) U = 1;
    if (G != 2 && G != 4 && G != 8 && G != 16 && G != 32) return QS_ERR_ARG;
    if (U != 1 && U != 2 && U != 4) return QS_ERR_ARG;
    cdbl mu{mu_re, mu_im};
    cudaStream_t st = qs_stream(stream);
    ExpmCtl *c = reinterpret_cast<ExpmCtl *>(ctl);
    const cdbl *cf = reinterpret_cast<const cdbl *>(coeff);
    cdbl *Fp = reinterpret_cast<cdbl *>(F);
    if (lp_btype(btype)) {
        const int co = group > 0 && ((group >> 16) & 1) && rownorm != nullptr;
        LpTerm a{n, indptr, idx64, indices, data, dtype, Bin, Bout, btype, Fp, nvec, mu, nullptr, nullptr, cf, j, tol,
                 ctl, G, U, co, co && ((group >> 17) & 1), rownorm, st};
        a.occ = group > 0 ? (group >> 18) & 3 : 0;
        a.nnz = nnz;
        a.staged = group > 0 ? (group >> 20) & 7 : 0;
        if (a.staged) return a.nvec == 1 ? st_taylor_term(a) : vl_taylor_term(a, false);
        return lp_taylor_term(a, false);
    }
    if (btype == QS_C128) {
        switch (dtype) {
        case QS_F64: return term_idx<double, cdbl>(idx64, n, indptr, indices, data, Bin, Bout, Fp, nvec, mu, cf, j, tol, c, G, U, st);
        case QS_C128: return term_idx<cdbl, cdbl>(idx64, n, indptr, indices, data, Bin, Bout, Fp, nvec, mu, cf, j, tol, c, G, U, st);
        default: return QS_ERR_ARG;
        }
    }
    return QS_ERR_ARG;
}

// F = eta F; B0 = F (scaled by 2^-bexp for QS_CPF / QS_C64 storage);
// c1 = ||F||_inf; done = 0 (eta: device complex128).
// With eta = 1 and substep_end = 0 this is the set-up before the first
// substep; with substep_end = 1 a substep whose stopping test never fired is
// counted in the control block.
extern "C" int qs_taylor_rescale(int64_t n, int64_t nvec, void *F, void *B0, int btype, const void *eta, void *ctl,
                                 int substep_end, void *stream)
{
    if (n < 1 || nvec < 1 || !F || !B0 || !eta || !ctl) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    if (lp_btype(btype))
        return lp_taylor_rescale(n, nvec, (cdbl *)F, B0, btype, (const cdbl *)eta, 1, nullptr, ctl, substep_end, false,
                                 st);
    if (btype != QS_C128) return QS_ERR_ARG;
    int64_t b = (n + 255) / 256, cap = (int64_t)qs_num_sms() * 8;
    int blocks = (int)(b > cap ? cap : b);
    taylor_rescale_kernel<cdbl><<<blocks, 256, 0, st>>>(n, nvec, (cdbl *)F, (cdbl *)B0, (const cdbl *)eta,
                                                       (ExpmCtl *)ctl, substep_end);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// Full e^{aA} v in place on F (complex128 [n, nvec]): s substeps of at most
// m_star terms.  work: two B buffers of n*nvec elements of btype; coeff:
// device complex128[max(m_star,1)] with coeff[j] = a / (s (j+1)); eta: device
// complex128 = exp(a mu / s); one: device complex128 = 1.  ctl zeroed by the
// caller before the first call.  No host synchronisation.
extern "C" int qs_expm_multiply_rows(int64_t n, int64_t nnz, const void *indptr, int idx64, const int32_t *indices,
                                     const void *data, int dtype, void *F, int64_t nvec, int s, int m_star,
                                     double tol, double mu_re, double mu_im, const void *coeff, const void *eta,
                                     const void *one, void *work, int btype, void *ctl, int group, void *rownorm,
                                     void *stream);

extern "C" int qs_expm_multiply(int64_t n, int64_t nnz, const void *indptr, int idx64, const int32_t *indices,
                                const void *data, int dtype, void *F, int64_t nvec, int s, int m_star, double tol,
                                double mu_re, double mu_im, const void *coeff, const void *eta, const void *one,
                                void *work, int btype, void *ctl, int group, void *stream)
{
    return qs_expm_multiply_rows(n, nnz, indptr, idx64, indices, data, dtype, F, nvec, s, m_star, tol, mu_re, mu_im,
                                 coeff, eta, one, work, btype, ctl, group, nullptr, stream);
}

// qs_expm_multiply with the row-sum scratch of qs_taylor_term_rows.
extern "C" int qs_expm_multiply_rows(int64_t n, int64_t nnz, const void *indptr, int idx64, const int32_t *indices,
                                     const void *data, int dtype, void *F, int64_t nvec, int s, int m_star,
                                     double tol, double mu_re, double mu_im, const void *coeff, const void *eta,
                                     const void *one, void *work, int btype, void *ctl, int group, void *rownorm,
                                     void *stream)
{
    if (n < 1 || nvec < 1 || s < 1 || m_star < 0 || !work || !ctl) return QS_ERR_ARG;
    if (btype != QS_C128 && btype != QS_C64 && btype != QS_CPF) return QS_ERR_ARG;
    size_t esz = btype == QS_C64 ? 8 : 16;
    char *b0 = reinterpret_cast<char *>(work);
    char *b1 = b0 + (size_t)n * nvec * esz;
    int rc = qs_taylor_rescale(n, nvec, F, b0, btype, one, ctl, 0, stream);
    if (rc) return rc;
    for (int i = 0; i < s; i++) {
        for (int j = 0; j < m_star; j++) {
            void *bin = (j & 1) ? b1 : b0;
            void *bout = (j & 1) ? b0 : b1;
            rc = qs_taylor_term_rows(n, nnz, indptr, idx64, indices, data, dtype, bin, bout, btype, F, nvec, mu_re,
                                     mu_im, coeff, j, tol, ctl, group, rownorm, stream);
            if (rc) return rc;
        }
        rc = qs_taylor_rescale(n, nvec, F, b0, btype, eta, ctl, m_star > 0 ? 1 : 0, stream);
        if (rc) return rc;
    }
    return QS_OK;
}

// ---------------------------------------------------------------------------
// Many symmetry sectors in one launch.
//
// The sectors' CSR matrices are stacked block-diagonally (rows of sector b
// are [sec_off[b], sec_off[b+1]), columns shifted the same way) and every
// sector evolves its own block of k states with the common schedule
// (s substeps, at most m* terms, coefficient a / (s (j+1))) but its own shift
// mu_b, its own factor eta_b = exp(a mu_b / s) and its own stopping test on
// the row sums of its block.  A sector whose test has fired is skipped by
// the following launches of the substep.

template <typename DT, typename BT, typename IT, int G, int NB, int U>
__global__ void __launch_bounds__(256) taylor_multi_kernel(int64_t n, const IT *__restrict__ indptr,
                                                           const int32_t *__restrict__ indices,
                                                           const DT *__restrict__ data, const BT *__restrict__ Bin,
                                                           BT *__restrict__ Bout, cdbl *__restrict__ F, int64_t nvec,
                                                           const int64_t *__restrict__ sec_off,
                                                           const cdbl *__restrict__ mu, const cdbl *__restrict__ coeff,
                                                           int j, double tol, MultiCtl *ctl)
{
    __shared__ int64_t soff[QS_MAX_SECTORS + 1];
    __shared__ int sdone[QS_MAX_SECTORS];
    __shared__ unsigned long long smb[QS_MAX_SECTORS], smf[QS_MAX_SECTORS];
    const int nsec = ctl->nsec;
    for (int b = threadIdx.x; b <= nsec; b += blockDim.x) soff[b] = sec_off[b];
    for (int b = threadIdx.x; b < nsec; b += blockDim.x) {
        sdone[b] = *((volatile int *)&ctl->done[b]);
        smb[b] = 0ull;
        smf[b] = 0ull;
    }
    __syncthreads();
    const cdbl cf = coeff[j];
    constexpr int GPW = 32 / G;
    const int lane = threadIdx.x & (G - 1);
    const int gsub = (threadIdx.x & 31) / G;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t rb = warp * GPW; rb < n; rb += nwarps * GPW) {
        const int64_t r = rb + gsub;
        const int b = r < n ? sector_of(soff, nsec, r) : 0;
        const bool valid = r < n && !sdone[b];
        const IT k0 = valid ? indptr[r] : (IT)0, k1 = valid ? indptr[r + 1] : (IT)0;
        double rb_ = 0.0, rf = 0.0;
        for (int64_t c0 = 0; c0 < nvec; c0 += NB) {
            cdbl acc[NB];
#pragma unroll
            for (int q = 0; q < NB; q++) acc[q] = cdbl{0.0, 0.0};
            for (IT k = k0 + lane; k < k1; k += G * U) {
                int32_t col[U];
                DT d[U];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const IT kk = k + u * G;
                    const bool in = kk < k1;
                    col[u] = in ? st_ld(indices + kk) : 0;
                    d[u] = in ? st_ld(data + kk) : zro<DT>();
                }
#pragma unroll
                for (int u = 0; u < U; u++) {
                    if (k + u * G < k1) {
#pragma unroll
                        for (int q = 0; q < NB; q++)
                            if (c0 + q < nvec) madd(acc[q], wid(d[u]), BLoad<BT>::ld(Bin, (int64_t)col[u] * nvec + c0 + q));
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < NB; q++) {
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) {
                    acc[q].x += __shfl_down_sync(0xffffffffu, acc[q].x, o, G);
                    acc[q].y += __shfl_down_sync(0xffffffffu, acc[q].y, o, G);
                }
            }
            if (valid && lane == 0) {
                const cdbl m = mu[b];
#pragma unroll
                for (int q = 0; q < NB; q++) {
                    if (c0 + q >= nvec) break;
                    const int64_t e = r * nvec + c0 + q;
                    const cdbl bo = BLoad<BT>::ld(Bin, e);
                    const double wr = acc[q].x - (m.x * bo.x - m.y * bo.y);
                    const double wi = acc[q].y - (m.x * bo.y + m.y * bo.x);
                    cdbl bn{cf.x * wr - cf.y * wi, cf.x * wi + cf.y * wr};
                    BLoad<BT>::st(Bout, e, bn);
                    cdbl f = F[e];
                    f.x += bn.x; f.y += bn.y;
                    F[e] = f;
                    rb_ += cabs_(bn);
                    rf += cabs_(f);
                }
            }
        }
        if (valid && lane == 0) {
            atomicMax(&smb[b], (unsigned long long)__double_as_longlong(rb_));
            atomicMax(&smf[b], (unsigned long long)__double_as_longlong(rf));
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nsec; b += blockDim.x) {
        if (smb[b]) atomicMax(&ctl->c2[b], smb[b]);
        if (smf[b]) atomicMax(&ctl->fn[b], smf[b]);
    }
    if (last_block_multi(ctl) && threadIdx.x == 0) {
        volatile MultiCtl *vc = ctl;
        long long active = 0;
        for (int b = 0; b < nsec; b++) {
            if (vc->done[b]) continue;
            active++;
            double c2 = __longlong_as_double((long long)vc->c2[b]);
            double fn = __longlong_as_double((long long)vc->fn[b]);
            if (vc->c1[b] + c2 <= tol * fn) vc->done[b] = 1;
            else vc->c1[b] = c2;
            vc->c2[b] = 0ull;
            vc->fn[b] = 0ull;
        }
        vc->terms = vc->terms + active;
        __threadfence();
        vc->arrive = 0u;
    }
}

// F = eta_b F; B0 = F; c1[b] = ||F_b||_inf; done[b] = 0.  use_eta = 0 for
// the set-up before the first substep (eta = 1).
template <typename BT>
__global__ void __launch_bounds__(256) taylor_multi_rescale_kernel(int64_t n, int64_t nvec, cdbl *__restrict__ F,
                                                                   BT *__restrict__ B0,
                                                                   const int64_t *__restrict__ sec_off,
                                                                   const cdbl *__restrict__ eta, int use_eta,
                                                                   MultiCtl *ctl)
{
    __shared__ int64_t soff[QS_MAX_SECTORS + 1];
    __shared__ unsigned long long sm[QS_MAX_SECTORS];
    const int nsec = ctl->nsec;
    for (int b = threadIdx.x; b <= nsec; b += blockDim.x) soff[b] = sec_off[b];
    for (int b = threadIdx.x; b < nsec; b += blockDim.x) sm[b] = 0ull;
    __syncthreads();
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const int b = sector_of(soff, nsec, r);
        const cdbl et = use_eta ? eta[b] : cdbl{1.0, 0.0};
        double rs = 0.0;
        for (int64_t c = 0; c < nvec; c++) {
            const int64_t e = r * nvec + c;
            cdbl f = F[e];
            if (use_eta) {
                cdbl g{et.x * f.x - et.y * f.y, et.x * f.y + et.y * f.x};
                f = g;
                F[e] = f;
            }
            BLoad<BT>::st(B0, e, f);
            rs += cabs_(f);
        }
        atomicMax(&sm[b], (unsigned long long)__double_as_longlong(rs));
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nsec; b += blockDim.x)
        if (sm[b]) atomicMax(&ctl->c2[b], sm[b]);
    if (last_block_multi(ctl) && threadIdx.x == 0) {
        volatile MultiCtl *vc = ctl;
        for (int b = 0; b < nsec; b++) {
            vc->c1[b] = __longlong_as_double((long long)vc->c2[b]);
            vc->c2[b] = 0ull;
            vc->fn[b] = 0ull;
            vc->done[b] = 0;
        }
        __threadfence();
        vc->arrive = 0u;
    }
}

template <typename DT, typename BT, int NB, int U>
static int multi_launch(int64_t n, const void *indptr, const int32_t *indices, const void *data, const void *Bin,
                        void *Bout, cdbl *F, int64_t nvec, const int64_t *soff, const cdbl *mu, const cdbl *coeff, int j,
                        double tol, MultiCtl *ctl, int G, cudaStream_t st)
{
    int blocks = grid_for(n, G);
#define L_(GG) taylor_multi_kernel<DT, BT, int32_t, GG, NB, U><<<blocks, 256, 0, st>>>(n, (const int32_t *)indptr, indices, (const DT *)data, (const BT *)Bin, (BT *)Bout, F, nvec, soff, mu, coeff, j, tol, ctl)
    switch (G) {
    case 2: L_(2); break;
    case 4: L_(4); break;
    case 8: L_(8); break;
    case 16: L_(16); break;
    default: L_(32); break;
    }
#undef L_
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

template <typename DT, typename BT>
static int multi_nb(int64_t n, const void *indptr, const int32_t *indices, const void *data, const void *Bin,
                    void *Bout, cdbl *F, int64_t nvec, const int64_t *soff, const cdbl *mu, const cdbl *coeff, int j,
                    double tol, MultiCtl *ctl, int G, int U, cudaStream_t st)
{
    if (nvec == 1) {
        if (U >= 2) return multi_launch<DT, BT, 1, 2>(n, indptr, indices, data, Bin, Bout, F, nvec, soff, mu, coeff, j, tol, ctl, G, st);
        return multi_launch<DT, BT, 1, 1>(n, indptr, indices, data, Bin, Bout, F, nvec, soff, mu, coeff, j, tol, ctl, G, st);
    }
    if (nvec == 2) return multi_launch<DT, BT, 2, 1>(n, indptr, indices, data, Bin, Bout, F, nvec, soff, mu, coeff, j, tol, ctl, G, st);
    if (nvec <= 4) return multi_launch<DT, BT, 4, 1>(n, indptr, indices, data, Bin, Bout, F, nvec, soff, mu, coeff, j, tol, ctl, G, st);
    return multi_launch<DT, BT, 8, 1>(n, indptr, indices, data, Bin, Bout, F, nvec, soff, mu, coeff, j, tol, ctl, G, st);
}

// One Taylor term for every sector of a block-diagonal stack (int32 indptr).
// sec_off: device int64[nsec+1] row offsets; mu: device complex128[nsec];
// coeff: device complex128 table; ctl: MultiCtl (qs_multi_ctl_bytes()) with
// nsec set.  btype / dtype pairs as for qs_taylor_term.  group as for
// qs_taylor_term.
extern "C" int qs_taylor_multi_term_rows(int64_t n, const void *indptr, const int32_t *indices, const void *data,
                                         int dtype, const void *Bin, void *Bout, int btype, void *F, int64_t nvec,
                                         const int64_t *sec_off, const void *mu, const void *coeff, int j, double tol,
                                         void *ctl, int group, void *rownorm, void *stream);

extern "C" int qs_taylor_multi_term(int64_t n, const void *indptr, const int32_t *indices, const void *data, int dtype,
                                    const void *Bin, void *Bout, int btype, void *F, int64_t nvec,
                                    const int64_t *sec_off, const void *mu, const void *coeff, int j, double tol,
                                    void *ctl, int group, void *stream)
{
    return qs_taylor_multi_term_rows(n, indptr, indices, data, dtype, Bin, Bout, btype, F, nvec, sec_off, mu, coeff, j,
                                     tol, ctl, group, nullptr, stream);
}

// qs_taylor_multi_term with the row-sum scratch of qs_taylor_term_rows.
extern "C" int qs_taylor_multi_term_rows(int64_t n, const void *indptr, const int32_t *indices, const void *data,
                                         int dtype, const void *Bin, void *Bout, int btype, void *F, int64_t nvec,
                                         const int64_t *sec_off, const void *mu, const void *coeff, int j, double tol,
                                         void *ctl, int group, void *rownorm, void *stream)
{
    if (n < 1 || nvec < 1 || !indptr || !Bin || !Bout || !F || !sec_off || !mu || !coeff || !ctl || j < 0)
        return QS_ERR_ARG;
    int G = group > 0 ? (group & 0xff) : 4;
    int U = group > 0 ? ((group >> 8) & 0xff) : 2;
    if (G != 2 && G != 4 && G != 8 && G != 16 && G != 32) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    MultiCtl *c = reinterpret_cast<MultiCtl *>(ctl);
    const cdbl *m = reinterpret_cast<const cdbl *>(mu);
    const cdbl *cf = reinterpret_cast<const cdbl *>(coeff);
    cdbl *Fp = reinterpret_cast<cdbl *>(F);
    if (lp_btype(btype)) {
        const int co = group > 0 && ((group >> 16) & 1) && rownorm != nullptr;
        LpTerm a{n, indptr, 0, indices, data, dtype, Bin, Bout, btype, Fp, nvec, cdbl{0.0, 0.0}, m, sec_off, cf, j, tol,
                 ctl, G, U, co, co && ((group >> 17) & 1), rownorm, st};
        a.occ = group > 0 ? (group >> 18) & 3 : 0;
        a.staged = group > 0 ? (group >> 20) & 7 : 0;
        if (a.staged && nvec > 1) return vl_taylor_term(a, true);
        return lp_taylor_term(a, true);
    }
    if (btype == QS_C128) {
        if (dtype == QS_F64) return multi_nb<double, cdbl>(n, indptr, indices, data, Bin, Bout, Fp, nvec, sec_off, m, cf, j, tol, c, G, U, st);
        if (dtype == QS_C128) return multi_nb<cdbl, cdbl>(n, indptr, indices, data, Bin, Bout, Fp, nvec, sec_off, m, cf, j, tol, c, G, U, st);
    }
    return QS_ERR_ARG;
}

extern "C" int qs_taylor_multi_rescale(int64_t n, int64_t nvec, void *F, void *B0, int btype, const int64_t *sec_off,
                                       const void *eta, int use_eta, void *ctl, void *stream)
{
    if (n < 1 || nvec < 1 || !F || !B0 || !sec_off || !ctl || (use_eta && !eta)) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    if (lp_btype(btype))
        return lp_taylor_rescale(n, nvec, (cdbl *)F, B0, btype, (const cdbl *)eta, use_eta, sec_off, ctl, 0, true, st);
    if (btype != QS_C128) return QS_ERR_ARG;
    int64_t b = (n + 255) / 256, cap = (int64_t)qs_num_sms() * 8;
    int blocks = (int)(b > cap ? cap : b);
    taylor_multi_rescale_kernel<cdbl><<<blocks, 256, 0, st>>>(n, nvec, (cdbl *)F, (cdbl *)B0, sec_off,
                                                             (const cdbl *)eta, use_eta, (MultiCtl *)ctl);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

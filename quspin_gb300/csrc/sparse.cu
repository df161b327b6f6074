// Sparse matrix-vector kernels and BLAS-1 reductions.
//
// Replaces, for the hot path, the OpenMP kernels of the un-vendored package
// parallel-sparse-tools==0.2.5 (QuSpin pyproject.toml:9):
//   _matvec (csr / dia)    docs/modules/parallel_sparse_tools/matvec/matvec_core.html:146-201,
//                          called by hamiltonian.dot (src/quspin/operators/hamiltonian_core.py:744-772)
//   _wrapper_csr_trace     expm_multiply_parallel_core.html:196-198
//   _wrapper_csr_1_norm    expm_multiply_parallel_core.html:200-202
// and the numpy BLAS-1 steps of the Lanczos recurrence
// (src/quspin/tools/lanczos/_lanczos_utils.py:186-204).
//
// The kernels here compute in IEEE double; csrc/spmv_lp.cu holds the
// paired-single form for float64 / complex128 vectors (qs_csr_matvec_pairs)
// and the FP32 form that qs_csr_matvec uses for float32 / complex64 vectors.
//
// CSR SpMV: a group of G lanes (2..32, a power of two) owns one row, reads the
// row's values and column indices with coalesced loads, gathers x through L2
// and reduces with warp shuffles.  For k right-hand sides (C order [n, k]) each
// lane keeps NB complex accumulators per row and x rows are read as
// contiguous NB-element segments.
#include "qs_common.cuh"

template <typename T> struct Num;
template <> struct Num<double> {
    using acc = double;
    __device__ static double ld(const double *p, int64_t i) { return __ldg(p + i); }
};
template <> struct Num<float> {
    using acc = double;
    __device__ static double ld(const float *p, int64_t i) { return (double)__ldg(p + i); }
};
template <> struct Num<cdbl> {
    using acc = cdbl;
    __device__ static cdbl ld(const cdbl *p, int64_t i) {
        double2 v = __ldg(reinterpret_cast<const double2 *>(p) + i);
        return cdbl{v.x, v.y};
    }
};
template <> struct Num<cflt> {
    using acc = cdbl;
    __device__ static cdbl ld(const cflt *p, int64_t i) {
        float2 v = __ldg(reinterpret_cast<const float2 *>(p) + i);
        return cdbl{(double)v.x, (double)v.y};
    }
};

// accumulator arithmetic: real or complex double
__device__ __forceinline__ void fma_acc(double &acc, double d, double x) { acc += d * x; }
__device__ __forceinline__ void fma_acc(cdbl &acc, double d, cdbl x) { acc.x += d * x.x; acc.y += d * x.y; }
__device__ __forceinline__ void fma_acc(cdbl &acc, cdbl d, cdbl x)
{
    acc.x += d.x * x.x - d.y * x.y;
    acc.y += d.x * x.y + d.y * x.x;
}
__device__ __forceinline__ void fma_acc(cdbl &acc, cdbl d, double x) { acc.x += d.x * x; acc.y += d.y * x; }

__device__ __forceinline__ double shfl_down(double v, int o, int w) { return __shfl_down_sync(0xffffffffu, v, o, w); }
__device__ __forceinline__ cdbl shfl_down(cdbl v, int o, int w)
{
    return cdbl{__shfl_down_sync(0xffffffffu, v.x, o, w), __shfl_down_sync(0xffffffffu, v.y, o, w)};
}
__device__ __forceinline__ void add_to(double &a, double b) { a += b; }
__device__ __forceinline__ void add_to(cdbl &a, cdbl b) { a.x += b.x; a.y += b.y; }
__device__ __forceinline__ void set_zero(double &a) { a = 0.0; }
__device__ __forceinline__ void set_zero(cdbl &a) { a = cdbl{0.0, 0.0}; }

// store a * acc (+ y) into the output element type
__device__ __forceinline__ void store_out(double *y, int64_t i, double acc, cdbl a, int overwrite)
{
    double v = a.x * acc;
    y[i] = overwrite ? v : y[i] + v;
}
__device__ __forceinline__ void store_out(float *y, int64_t i, double acc, cdbl a, int overwrite)
{
    double v = a.x * acc;
    y[i] = overwrite ? (float)v : (float)((double)y[i] + v);
}
__device__ __forceinline__ void store_out(cdbl *y, int64_t i, cdbl acc, cdbl a, int overwrite)
{
    double vr = a.x * acc.x - a.y * acc.y, vi = a.x * acc.y + a.y * acc.x;
    if (overwrite) y[i] = cdbl{vr, vi};
    else { cdbl o = y[i]; y[i] = cdbl{o.x + vr, o.y + vi}; }
}
__device__ __forceinline__ void store_out(cflt *y, int64_t i, cdbl acc, cdbl a, int overwrite)
{
    double vr = a.x * acc.x - a.y * acc.y, vi = a.x * acc.y + a.y * acc.x;
    if (overwrite) y[i] = cflt{(float)vr, (float)vi};
    else { cflt o = y[i]; y[i] = cflt{(float)((double)o.x + vr), (float)((double)o.y + vi)}; }
}

template <typename T> __device__ __forceinline__ T ld_stream(const T *p) { return __ldcs(p); }
template <> __device__ __forceinline__ cdbl ld_stream<cdbl>(const cdbl *p)
{
    double2 v = __ldcs(reinterpret_cast<const double2 *>(p));
    return cdbl{v.x, v.y};
}
template <> __device__ __forceinline__ cflt ld_stream<cflt>(const cflt *p)
{
    float2 v = __ldcs(reinterpret_cast<const float2 *>(p));
    return cflt{v.x, v.y};
}
__device__ __forceinline__ double widen(double v) { return v; }
__device__ __forceinline__ double widen(float v) { return (double)v; }
__device__ __forceinline__ cdbl widen(cdbl v) { return v; }
__device__ __forceinline__ cdbl widen(cflt v) { return cdbl{(double)v.x, (double)v.y}; }
template <typename T> __device__ __forceinline__ T zero_of();
template <> __device__ __forceinline__ double zero_of<double>() { return 0.0; }
template <> __device__ __forceinline__ float zero_of<float>() { return 0.0f; }
template <> __device__ __forceinline__ cdbl zero_of<cdbl>() { return cdbl{0.0, 0.0}; }
template <> __device__ __forceinline__ cflt zero_of<cflt>() { return cflt{0.0f, 0.0f}; }

// G lanes per row, U independent entries per lane per step (more loads in
// flight), NB right-hand sides per pass.  Rows are handed out per warp (32/G
// consecutive rows per warp and iteration) so the loop bound is uniform across
// the warp and every lane reaches the full-mask shuffles; groups past the last
// row idle.  Matrix streams are read with evict-first hints so the gathered
// vector keeps its place in L2.
template <typename DT, typename XT, typename IT, int G, int NB, int U>
__global__ void __launch_bounds__(256) csr_spmm_kernel(int64_t n, const IT *__restrict__ indptr,
                                                       const int32_t *__restrict__ indices,
                                                       const DT *__restrict__ data, const XT *__restrict__ x,
                                                       XT *__restrict__ y, int64_t nvec, cdbl a, int overwrite)
{
    using ACC = typename Num<XT>::acc;
    constexpr int GPW = 32 / G;
    const int lane = threadIdx.x & (G - 1);
    const int gsub = (threadIdx.x & 31) / G;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t rb = warp * GPW; rb < n; rb += nwarps * GPW) {
        const int64_t r = rb + gsub;
        const bool valid = r < n;
        const IT k0 = valid ? indptr[r] : (IT)0, k1 = valid ? indptr[r + 1] : (IT)0;
        for (int64_t c0 = 0; c0 < nvec; c0 += NB) {
            ACC acc[NB];
#pragma unroll
            for (int b = 0; b < NB; b++) set_zero(acc[b]);
            for (IT k = k0 + lane; k < k1; k += G * U) {
                int32_t col[U];
                DT d[U];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const IT kk = k + u * G;
                    const bool in = kk < k1;
                    col[u] = in ? ld_stream(indices + kk) : 0;
                    d[u] = in ? ld_stream(data + kk) : zero_of<DT>();
                }
#pragma unroll
                for (int u = 0; u < U; u++) {
                    if (k + u * G < k1) {
#pragma unroll
                        for (int b = 0; b < NB; b++)
                            if (c0 + b < nvec) fma_acc(acc[b], widen(d[u]), Num<XT>::ld(x, (int64_t)col[u] * nvec + c0 + b));
                    }
                }
            }
#pragma unroll
            for (int b = 0; b < NB; b++) {
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) add_to(acc[b], shfl_down(acc[b], o, G));
            }
            if (valid && lane == 0) {
#pragma unroll
                for (int b = 0; b < NB; b++)
                    if (c0 + b < nvec) store_out(y, r * nvec + c0 + b, acc[b], a, overwrite);
            }
        }
    }
}

// Lanes per row from the mean row length: about 12-24 entries per lane (random
// gathers favour few lanes per row; the tuner refines this).
static int pick_group(int64_t n, int64_t nnz)
{
    double avg = n > 0 ? (double)nnz / (double)n : 1.0;
    int g = 2;
    while (g < 32 && g * 24 < avg) g <<= 1;
    return g;
}

template <typename DT, typename XT, typename IT, int NB, int U>
static int spmm_launch_gu(int64_t n, const void *indptr, const int32_t *indices, const void *data, const void *x,
                          void *y, int64_t nvec, cdbl a, int overwrite, int G, cudaStream_t st)
{
    int threads = 256;
    int64_t groups_per_block = threads / G;
    int64_t blocks = (n + groups_per_block - 1) / groups_per_block;
    int64_t cap = (int64_t)qs_num_sms() * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
#define L_(GG) csr_spmm_kernel<DT, XT, IT, GG, NB, U><<<(unsigned)blocks, threads, 0, st>>>(n, (const IT *)indptr, indices, (const DT *)data, (const XT *)x, (XT *)y, nvec, a, overwrite)
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

template <typename DT, typename XT, typename IT>
static int spmm_launch(int64_t n, const void *indptr, const int32_t *indices, const void *data, const void *x,
                       void *y, int64_t nvec, cdbl a, int overwrite, int G, int U, cudaStream_t st)
{
    if (nvec == 1) {
        if (U >= 4) return spmm_launch_gu<DT, XT, IT, 1, 4>(n, indptr, indices, data, x, y, nvec, a, overwrite, G, st);
        if (U == 2) return spmm_launch_gu<DT, XT, IT, 1, 2>(n, indptr, indices, data, x, y, nvec, a, overwrite, G, st);
        return spmm_launch_gu<DT, XT, IT, 1, 1>(n, indptr, indices, data, x, y, nvec, a, overwrite, G, st);
    }
    if (nvec == 2) return spmm_launch_gu<DT, XT, IT, 2, 1>(n, indptr, indices, data, x, y, nvec, a, overwrite, G, st);
    if (nvec <= 4) return spmm_launch_gu<DT, XT, IT, 4, 1>(n, indptr, indices, data, x, y, nvec, a, overwrite, G, st);
    return spmm_launch_gu<DT, XT, IT, 8, 1>(n, indptr, indices, data, x, y, nvec, a, overwrite, G, st);
}

template <typename DT, typename XT>
static int spmm_idx(int idx64, int64_t n, const void *indptr, const int32_t *indices, const void *data, const void *x,
                    void *y, int64_t nvec, cdbl a, int overwrite, int G, int U, cudaStream_t st)
{
    if (idx64) return spmm_launch<DT, XT, int64_t>(n, indptr, indices, data, x, y, nvec, a, overwrite, G, 1, st);
    return spmm_launch<DT, XT, int32_t>(n, indptr, indices, data, x, y, nvec, a, overwrite, G, U, st);
}

// y = a * A x (overwrite) or y += a * A x, for a CSR matrix with int32/int64
// indptr (idx64), int32 indices, value type dtype and vector type xtype
// (QS_F32/F64/C64/C128).  x, y: [n, nvec] C order.  Supported pairs: the
// vector type is the result type (complex if either is complex; the value
// precision never exceeds the vector precision's partner).  group: launch
// shape, G | (U << 8) with G lanes per row (2..32) and U in-flight entries per
// lane (1, 2, 4); 0 picks G from nnz/n and U = 2.
int spmv_lp_single(int64_t n, const void *indptr, int idx64, const int32_t *indices, const void *data, int dtype,
                   const void *x, int xtype, void *y, int64_t nvec, cdbl a, int overwrite, int G, int U,
                   cudaStream_t st);

extern "C" int qs_csr_matvec(int64_t n, int64_t nnz, const void *indptr, int idx64, const int32_t *indices,
                             const void *data, int dtype, const void *x, int xtype, void *y, int64_t nvec,
                             double a_re, double a_im, int overwrite, int group, void *stream)
{
    if (n < 0 || nvec < 1 || (n > 0 && (!indptr || !x || !y))) return QS_ERR_ARG;
    if (n == 0) return QS_OK;
    cdbl a{a_re, a_im};
    int G = group > 0 ? (group & 0xff) : pick_group(n, nnz);
    int U = group > 0 ? ((group >> 8) & 0xff) : 2;
    if (U < 1) U = 1;
    if (G != 2 && G != 4 && G != 8 && G != 16 && G != 32) return QS_ERR_ARG;
    if (U != 1 && U != 2 && U != 4) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    bool xc = xtype == QS_C64 || xtype == QS_C128;
    if (!xc && a_im != 0.0) return QS_ERR_ARG;
    switch (xtype) {
    case QS_F64:
        if (dtype == QS_F64) return spmm_idx<double, double>(idx64, n, indptr, indices, data, x, y, nvec, a, overwrite, G, U, st);
        if (dtype == QS_F32) return spmm_idx<float, double>(idx64, n, indptr, indices, data, x, y, nvec, a, overwrite, G, U, st);
        return QS_ERR_ARG;
    case QS_F32:
        if (dtype == QS_F32)   // FP32 products and row sums (csrc/spmv_lp.cu)
            return spmv_lp_single(n, indptr, idx64, indices, data, dtype, x, xtype, y, nvec, a, overwrite, G, U, st);
        return QS_ERR_ARG;
    case QS_C128:
        if (dtype == QS_F64) return spmm_idx<double, cdbl>(idx64, n, indptr, indices, data, x, y, nvec, a, overwrite, G, U, st);
        if (dtype == QS_C128) return spmm_idx<cdbl, cdbl>(idx64, n, indptr, indices, data, x, y, nvec, a, overwrite, G, U, st);
        if (dtype == QS_F32) return spmm_idx<float, cdbl>(idx64, n, indptr, indices, data, x, y, nvec, a, overwrite, G, U, st);
        if (dtype == QS_C64) return spmm_idx<cflt, cdbl>(idx64, n, indptr, indices, data, x, y, nvec, a, overwrite, G, U, st);
        return QS_ERR_ARG;
    case QS_C64:
        if (dtype == QS_F32 || dtype == QS_C64)
            return spmv_lp_single(n, indptr, idx64, indices, data, dtype, x, xtype, y, nvec, a, overwrite, G, U, st);
        return QS_ERR_ARG;
    default:
        return QS_ERR_ARG;
    }
}

// ---------------------------------------------------------------------------
// DIA with offsets (scipy dia_matrix layout: data[d, col], y[r] += data[d, r+off] x[r+off])

template <typename DT, typename XT>
__global__ void dia_kernel(int64_t n, int ndiag, const int64_t *__restrict__ offsets, int64_t ldd,
                           const DT *__restrict__ data, const XT *__restrict__ x, XT *__restrict__ y, int64_t nvec,
                           cdbl a, int overwrite)
{
    using ACC = typename Num<XT>::acc;
    const int64_t total = n * nvec;
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < total; w += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = w / nvec, c = w - r * nvec;
        ACC acc;
        set_zero(acc);
        for (int d = 0; d < ndiag; d++) {
            int64_t col = r + offsets[d];
            if (col < 0 || col >= n || col >= ldd) continue;
            fma_acc(acc, Num<DT>::ld(data, (int64_t)d * ldd + col), Num<XT>::ld(x, col * nvec + c));
        }
        store_out(y, w, acc, a, overwrite);
    }
}

template <typename DT, typename XT>
static int dia_launch(int64_t n, int ndiag, const int64_t *offsets, int64_t ldd, const void *data, const void *x,
                      void *y, int64_t nvec, cdbl a, int overwrite, cudaStream_t st)
{
    int64_t total = n * nvec;
    int64_t blocks = (total + 255) / 256, cap = (int64_t)qs_num_sms() * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    dia_kernel<DT, XT><<<(unsigned)blocks, 256, 0, st>>>(n, ndiag, offsets, ldd, (const DT *)data, (const XT *)x,
                                                         (XT *)y, nvec, a, overwrite);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// y (=|+=) a * D x for a matrix in scipy DIA layout (offsets int64[ndiag],
// data [ndiag, ldd]).
extern "C" int qs_dia_matvec(int64_t n, int ndiag, const int64_t *offsets, int64_t ldd, const void *data, int dtype,
                             const void *x, int xtype, void *y, int64_t nvec, double a_re, double a_im, int overwrite,
                             void *stream)
{
    if (n < 0 || nvec < 1 || ndiag < 0) return QS_ERR_ARG;
    if (n == 0) return QS_OK;
    cdbl a{a_re, a_im};
    cudaStream_t st = qs_stream(stream);
    switch (xtype) {
    case QS_F64:
        if (dtype == QS_F64) return dia_launch<double, double>(n, ndiag, offsets, ldd, data, x, y, nvec, a, overwrite, st);
        if (dtype == QS_F32) return dia_launch<float, double>(n, ndiag, offsets, ldd, data, x, y, nvec, a, overwrite, st);
        return QS_ERR_ARG;
    case QS_F32:
        if (dtype == QS_F32) return dia_launch<float, float>(n, ndiag, offsets, ldd, data, x, y, nvec, a, overwrite, st);
        return QS_ERR_ARG;
    case QS_C128:
        if (dtype == QS_F64) return dia_launch<double, cdbl>(n, ndiag, offsets, ldd, data, x, y, nvec, a, overwrite, st);
        if (dtype == QS_C128) return dia_launch<cdbl, cdbl>(n, ndiag, offsets, ldd, data, x, y, nvec, a, overwrite, st);
        if (dtype == QS_F32) return dia_launch<float, cdbl>(n, ndiag, offsets, ldd, data, x, y, nvec, a, overwrite, st);
        if (dtype == QS_C64) return dia_launch<cflt, cdbl>(n, ndiag, offsets, ldd, data, x, y, nvec, a, overwrite, st);
        return QS_ERR_ARG;
    case QS_C64:
        if (dtype == QS_F32) return dia_launch<float, cflt>(n, ndiag, offsets, ldd, data, x, y, nvec, a, overwrite, st);
        if (dtype == QS_C64) return dia_launch<cflt, cflt>(n, ndiag, offsets, ldd, data, x, y, nvec, a, overwrite, st);
        return QS_ERR_ARG;
    default:
        return QS_ERR_ARG;
    }
}

// ---------------------------------------------------------------------------
// deterministic reductions: per-block partials then one block sums them in
// a fixed order.

#define RED_THREADS 256
#define RED_BLOCKS_MAX 1024

__device__ __forceinline__ double warp_sum(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// sums two doubles per thread across the block; result valid in thread 0
__device__ __forceinline__ void block_sum2(double &a, double &b)
{
    __shared__ double sa[32], sb[32];
    a = warp_sum(a); b = warp_sum(b);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { sa[w] = a; sb[w] = b; }
    __syncthreads();
    if (w == 0) {
        int nw = blockDim.x >> 5;
        a = lane < nw ? sa[lane] : 0.0;
        b = lane < nw ? sb[lane] : 0.0;
        a = warp_sum(a); b = warp_sum(b);
    }
    __syncthreads();
}

// partial[blk] = sum conj(x) y over this block's elements; complex (cplx=1)
// or real vectors of doubles
__global__ void vdot_partial(int64_t n, const double *__restrict__ x, const double *__restrict__ y, int cplx,
                             double *__restrict__ partial)
{
    double sr = 0.0, si = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (cplx) {
            double xr = x[2 * i], xi = x[2 * i + 1], yr = y[2 * i], yi = y[2 * i + 1];
            sr += xr * yr + xi * yi;
            si += xr * yi - xi * yr;
        } else {
            sr += x[i] * y[i];
        }
    }
    block_sum2(sr, si);
    if (threadIdx.x == 0) { partial[2 * blockIdx.x] = sr; partial[2 * blockIdx.x + 1] = si; }
}

__global__ void finish_sum2(int nb, const double *__restrict__ partial, double *__restrict__ out, int mode)
{
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) { a += partial[2 * i]; b += partial[2 * i + 1]; }
    block_sum2(a, b);
    if (threadIdx.x == 0) {
        if (mode == 1) { out[0] = sqrt(a); out[1] = 0.0; }
        else { out[0] = a; out[1] = b; }
    }
}

static int red_blocks(int64_t n)
{
    int64_t b = (n + RED_THREADS - 1) / RED_THREADS;
    int cap = qs_num_sms() * 4;
    if (cap > RED_BLOCKS_MAX) cap = RED_BLOCKS_MAX;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

extern "C" int qs_reduce_scratch_doubles() { return 2 * RED_BLOCKS_MAX; }

// out[0..1] = sum_i conj(x_i) y_i (double / complex128 vectors, n elements).
// scratch: qs_reduce_scratch_doubles() doubles.  Result stays on the device.
extern "C" int qs_vdot(int64_t n, const void *x, const void *y, int cplx, double *out, double *scratch, void *stream)
{
    if (n < 0 || !out || !scratch) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    int nb = red_blocks(n);
    vdot_partial<<<nb, RED_THREADS, 0, st>>>(n, (const double *)x, (const double *)y, cplx, scratch);
    finish_sum2<<<1, RED_THREADS, 0, st>>>(nb, scratch, out, 0);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

__global__ void nrm2_partial(int64_t n2, const double *__restrict__ x, double *__restrict__ partial)
{
    double s = 0.0, z = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x)
        s += x[i] * x[i];
    block_sum2(s, z);
    if (threadIdx.x == 0) { partial[2 * blockIdx.x] = s; partial[2 * blockIdx.x + 1] = 0.0; }
}

// out[0] = ||x||_2 over n2 doubles (2n for complex vectors).
extern "C" int qs_nrm2(int64_t n2, const void *x, double *out, double *scratch, void *stream)
{
    if (n2 < 0 || !out || !scratch) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    int nb = red_blocks(n2);
    nrm2_partial<<<nb, RED_THREADS, 0, st>>>(n2, (const double *)x, scratch);
    finish_sum2<<<1, RED_THREADS, 0, st>>>(nb, scratch, out, 1);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// ---------------------------------------------------------------------------
// trace and 1-norm of a CSR matrix

template <typename IT>
__global__ void trace_partial(int64_t n, const IT *__restrict__ indptr, const int32_t *__restrict__ indices,
                              const double *__restrict__ data, int cplx, double *__restrict__ partial)
{
    double sr = 0.0, si = 0.0;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        for (int64_t k = indptr[r]; k < indptr[r + 1]; k++)
            if (indices[k] == r) {
                if (cplx) { sr += data[2 * k]; si += data[2 * k + 1]; }
                else sr += data[k];
            }
    }
    block_sum2(sr, si);
    if (threadIdx.x == 0) { partial[2 * blockIdx.x] = sr; partial[2 * blockIdx.x + 1] = si; }
}

// out[0..1] = trace (device).  data float64 (cplx=0) or complex128 (cplx=1).
extern "C" int qs_csr_trace(int64_t n, const void *indptr, int idx64, const int32_t *indices, const void *data,
                            int cplx, double *out, double *scratch, void *stream)
{
    if (n < 0 || !out || !scratch) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    int nb = red_blocks(n);
    if (idx64) trace_partial<int64_t><<<nb, RED_THREADS, 0, st>>>(n, (const int64_t *)indptr, indices, (const double *)data, cplx, scratch);
    else trace_partial<int32_t><<<nb, RED_THREADS, 0, st>>>(n, (const int32_t *)indptr, indices, (const double *)data, cplx, scratch);
    finish_sum2<<<1, RED_THREADS, 0, st>>>(nb, scratch, out, 0);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// column sums of |A + shift I| by atomics into colsum[n] (zeroed by caller)
template <typename IT>
__global__ void colsum_kernel(int64_t n, const IT *__restrict__ indptr, const int32_t *__restrict__ indices,
                              const double *__restrict__ data, int cplx, double shr, double shi,
                              double *__restrict__ colsum)
{
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        bool hasd = false;
        for (int64_t k = indptr[r]; k < indptr[r + 1]; k++) {
            int64_t c = indices[k];
            double vr = cplx ? data[2 * k] : data[k];
            double vi = cplx ? data[2 * k + 1] : 0.0;
            if (c == r) { vr += shr; vi += shi; hasd = true; }
            atomicAdd(&colsum[c], hypot(vr, vi));
        }
        if (!hasd) atomicAdd(&colsum[r], hypot(shr, shi));
    }
}

__global__ void max_partial(int64_t n, const double *__restrict__ x, double *__restrict__ partial)
{
    __shared__ double sm[32];
    double m = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = fmax(m, x[i]);
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t = fmax(t, sm[w]);
        partial[blockIdx.x] = t;
    }
}

// out[0] = max_c sum_r |A[r,c] + shift delta_rc|.  colsum: n doubles scratch.
extern "C" int qs_csr_1_norm(int64_t n, const void *indptr, int idx64, const int32_t *indices, const void *data,
                             int cplx, double sh_re, double sh_im, double *out, double *colsum, double *scratch,
                             void *stream)
{
    if (n < 0 || !out || !colsum || !scratch) return QS_ERR_ARG;
    cudaStream_t st = qs_stream(stream);
    QS_CHECK(cudaMemsetAsync(colsum, 0, sizeof(double) * (n > 0 ? n : 1), st));
    int nb = red_blocks(n);
    if (n > 0) {
        if (idx64) colsum_kernel<int64_t><<<nb, RED_THREADS, 0, st>>>(n, (const int64_t *)indptr, indices, (const double *)data, cplx, sh_re, sh_im, colsum);
        else colsum_kernel<int32_t><<<nb, RED_THREADS, 0, st>>>(n, (const int32_t *)indptr, indices, (const double *)data, cplx, sh_re, sh_im, colsum);
    }
    max_partial<<<nb, RED_THREADS, 0, st>>>(n, colsum, scratch);
    max_partial<<<1, RED_THREADS, 0, st>>>(nb, scratch, out);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// CSR SpMV / SpMM without FP64 instructions per nonzero.
//
// y = a A x (overwrite) or y += a A x, the contract of parallel-sparse-tools'
// _matvec (docs/modules/parallel_sparse_tools/matvec/matvec_core.html:146-201
// in the reference), in two arithmetic forms (csrc/lp_modes.cuh):
//
//   * paired single (qs_csr_matvec_pairs): float64 / complex128 x and y, the
//     matrix values as float pairs (qs_split_pairs).  x is first scaled by
//     the power of two at or below its largest component and split into
//     pairs (two streaming passes over x), the products and row sums run in
//     FP32 instructions with 48-bit significands, and the scale is undone
//     exactly when the row result is converted to double;
//   * single precision (qs_csr_matvec with float32 / complex64 x and values):
//     FP32 products and row sums, float32 / complex64 y.
//
// Row hand-out, lanes per row and entries in flight follow csrc/sparse.cu;
// after the butterfly reduction lanes 0 and 1 of a row group write the real
// and imaginary part of y.
#include "qs_common.cuh"
#include "pairf.cuh"
#include "lp_modes.cuh"

namespace {

template <class T> struct is_cx { static constexpr bool value = false; };
template <class S> struct is_cx<cx<S>> { static constexpr bool value = true; };

// real value times real x
template <class M>
__device__ __forceinline__ void rmul_acc(typename M::S &ar, typename M::S &, typename M::S d, typename M::S x)
{
    M::fma(ar, d, x);
}
// complex value times real x
template <class M>
__device__ __forceinline__ void rmul_acc(typename M::S &ar, typename M::S &ai, const cx<typename M::S> &d,
                                         typename M::S x)
{
    M::fma(ar, d.re, x);
    M::fma(ai, d.im, x);
}

// output stores: YT double / float (real) or cdbl / cflt (complex)
template <class M> __device__ __forceinline__ void st_out(double *y, int64_t e, int, typename M::S v, int k, int ow)
{
    double r = M::to_d(v, k);
    if (!ow) r += y[e];
    y[e] = r;
}
template <class M> __device__ __forceinline__ void st_out(cdbl *y, int64_t e, int comp, typename M::S v, int k, int ow)
{
    double *p = reinterpret_cast<double *>(y + e) + comp;
    double r = M::to_d(v, k);
    if (!ow) r += *p;
    *p = r;
}
template <class M> __device__ __forceinline__ void st_out(float *y, int64_t e, int, typename M::S v, int, int ow)
{
    float r = M::hi(v);
    if (!ow) r += y[e];
    y[e] = r;
}
template <class M> __device__ __forceinline__ void st_out(cflt *y, int64_t e, int comp, typename M::S v, int, int ow)
{
    float *p = reinterpret_cast<float *>(y + e) + comp;
    float r = M::hi(v);
    if (!ow) r += *p;
    *p = r;
}

// VM: 0 one value per nonzero; 1 coded: data holds a table of QS_CODE_TABLE
// values followed by one code byte per nonzero (pdtype QS_PF8 / QS_CPF8);
// 2 packed: indices holds col << 8 | code and data the table only (QS_PF8P /
// QS_CPF8P); 3 packed, one complex vector, the column words read four per
// 16-byte load (indices readable up to the next multiple of four words).
// The table is staged in shared memory.
template <class M, class DV, bool XC, class YT, class IT, int NB, int U, int VM>
__global__ void __launch_bounds__(256) spmv_lp_kernel(int64_t n, int lgG, const IT *__restrict__ indptr,
                                                      const int32_t *__restrict__ indices,
                                                      const DV *__restrict__ data, const void *__restrict__ xv,
                                                      YT *__restrict__ y, int64_t nvec, cdbl a, int overwrite,
                                                      const unsigned long long *__restrict__ xnorm)
{
    using S = typename M::S;
    using BE = typename M::BE;
    constexpr bool COUT = XC || is_cx<DV>::value;
    __shared__ S s_a[2];
    __shared__ int s_k;
    if (threadIdx.x == 0) s_a[0] = M::from_d(a.x);
    if (threadIdx.x == 1) s_a[1] = M::from_d(a.y);
    if (threadIdx.x == 2) s_k = xnorm ? scale_exp(__longlong_as_double((long long)*xnorm)) : 0;
    constexpr bool CODED = VM != 0;
    __shared__ DV s_tab[CODED ? QS_CODE_TABLE : 1];
    const uint8_t *codes = nullptr;
    if constexpr (CODED) {
        for (int i = threadIdx.x; i < QS_CODE_TABLE; i += blockDim.x) s_tab[i] = ldv(data + i);
        codes = reinterpret_cast<const uint8_t *>(data + QS_CODE_TABLE);
    }
    __syncthreads();
    const cx<S> av{s_a[0], s_a[1]};
    const int k2 = s_k;
    const unsigned long long keep = l2_keep_policy();
    const BE *xc = reinterpret_cast<const BE *>(xv);
    const S *xr = reinterpret_cast<const S *>(xv);

    const int G = 1 << lgG;
    const int GPW = 32 >> lgG;
    const int lane = threadIdx.x & (G - 1);
    const int comp = lane & 1;
    const int gsub = (threadIdx.x & 31) >> lgG;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t rb = warp * GPW; rb < n; rb += nwarps * GPW) {
        const int64_t r = rb + gsub;
        const bool valid = r < n;
        const bool writer = valid && (COUT ? lane < 2 : lane == 0);
        const IT k0 = valid ? indptr[r] : (IT)0, k1 = valid ? indptr[r + 1] : (IT)0;
        for (int64_t c0 = 0; c0 < nvec; c0 += NB) {
            S ar[NB], ai[NB];
#pragma unroll
            for (int b = 0; b < NB; b++) ar[b] = ai[b] = M::zero();
            if constexpr (VM == 3) {
                // one vector: the row's packed column words in 16-byte aligned
                // groups of four, group g of the row to lane g mod G
                for (IT c = (k0 & ~(IT)3) + 4 * lane; c < k1; c += (IT)(4 * G)) {
                    const uint4 w4 = __ldcs(reinterpret_cast<const uint4 *>(indices + c));
                    const uint32_t w[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
                    for (int h = 0; h < 4; h += 2) {
                        BE bv[2];
#pragma unroll
                        for (int i = 0; i < 2; i++)
                            bv[i] = (c + h + i >= k0 && c + h + i < k1) ? M::ldB(xc + (int32_t)(w[h + i] >> 8), keep)
                                                                        : BE{M::zero(), M::zero()};
#pragma unroll
                        for (int i = 0; i < 2; i++)
                            if (c + h + i >= k0 && c + h + i < k1) vmul_acc<M>(ar[0], ai[0], s_tab[w[h + i] & 255u], bv[i]);
                    }
                }
            } else {
            for (IT k = k0 + lane; k < k1; k += (IT)(G * U)) {
                int32_t col[U];
                DV d[U];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const IT kk = k + (IT)(u * G);
                    const bool in = kk < k1;
                    if constexpr (VM == 2) {
                        const uint32_t w = in ? (uint32_t)__ldcs(indices + kk) : 0u;
                        col[u] = (int32_t)(w >> 8);
                        d[u] = in ? s_tab[w & 255u] : vzero<DV>();
                    } else {
                        col[u] = in ? __ldcs(indices + kk) : 0;
                        if constexpr (VM == 1) d[u] = in ? s_tab[__ldcs(codes + kk)] : vzero<DV>();
                        else d[u] = in ? ldv(data + kk) : vzero<DV>();
                    }
                }
#pragma unroll
                for (int u = 0; u < U; u++) {
                    if (k + (IT)(u * G) < k1) {
#pragma unroll
                        for (int b = 0; b < NB; b++) {
                            if (NB == 1 || c0 + b < nvec) {
                                const int64_t xi = (int64_t)col[u] * nvec + c0 + b;
                                if constexpr (XC)
                                    vmul_acc<M>(ar[b], ai[b], d[u], NB == 1 ? M::ldB(xc + xi, keep) : M::ldB(xc + xi));
                                else rmul_acc<M>(ar[b], ai[b], d[u], M::ldS(xr + xi));
                            }
                        }
                    }
                }
            }
            }
#pragma unroll
            for (int b = 0; b < NB; b++) {
                for (int o = G >> 1; o > 0; o >>= 1) {
                    ar[b] = M::merge(ar[b], M::shfl_xor(ar[b], o));
                    if constexpr (COUT) ai[b] = M::merge(ai[b], M::shfl_xor(ai[b], o));
                }
            }
            if (writer) {
#pragma unroll
                for (int b = 0; b < NB; b++) {
                    if (c0 + b >= nvec) break;
                    const int64_t e = r * nvec + c0 + b;
                    const S accr = M::fin(ar[b]);
                    if constexpr (COUT) {
                        const S acci = M::fin(ai[b]);
                        const S v = comp ? M::add(M::mul(av.re, acci), M::mul(av.im, accr))
                                         : M::sub(M::mul(av.re, accr), M::mul(av.im, acci));
                        st_out<M>(y, e, comp, v, k2, overwrite);
                    } else {
                        st_out<M>(y, e, 0, M::mul(av.re, accr), k2, overwrite);
                    }
                }
            }
        }
    }
}

// largest |component| of a double array into *norm (bits of a double >= 0)
__global__ void xnorm_kernel(int64_t count, const double *__restrict__ x, unsigned long long *norm)
{
    double m = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        m = fmax(m, fabs(__ldcs(x + i)));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMax(norm, (unsigned long long)__double_as_longlong(m));
}

// xs[i] = pair(x[i] 2^-k), k from *norm
__global__ void xsplit_kernel(int64_t count, const double *__restrict__ x, float2 *__restrict__ xs,
                              const unsigned long long *__restrict__ norm)
{
    const double sc = pow2(-scale_exp(__longlong_as_double((long long)*norm)));
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        const pf v = pf_from_double(__ldcs(x + i) * sc);
        xs[i] = make_float2(v.h, v.l);
    }
}

struct SpmvArgs {
    int64_t n;
    const void *indptr;
    int idx64;
    const int32_t *indices;
    const void *data;
    const void *x;
    void *y;
    int64_t nvec;
    cdbl a;
    int overwrite;
    const unsigned long long *xnorm;
    int G, U;
    cudaStream_t st;
};

static int grid_rows(int64_t n, int G)
{
    int64_t gpb = 256 / G;
    int64_t b = (n + gpb - 1) / gpb;
    int64_t cap = (int64_t)qs_num_sms() * 16;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

template <class M, class DV, bool XC, class YT, class IT, int NB, int U, int VM>
int spmv_go(const SpmvArgs &a)
{
    int lg = 0;
    while ((1 << lg) < a.G) lg++;
    // persistent grid (grid-stride kernel): one wave of resident blocks
    static int resident = 0;
    auto k = spmv_lp_kernel<M, DV, XC, YT, IT, NB, U, VM>;
    const int blocks = qs_persistent_grid(k, 256, grid_rows(a.n, a.G), resident);
    k<<<blocks, 256, 0, a.st>>>(a.n, lg, (const IT *)a.indptr, a.indices, (const DV *)a.data, a.x, (YT *)a.y,
                                a.nvec, a.a, a.overwrite, a.xnorm);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

template <class M, class DV, bool XC, class YT, class IT, int VM>
int spmv_nb(const SpmvArgs &a)
{
    if constexpr (VM == 3) {
        if (a.nvec != 1 || !XC) return QS_ERR_ARG;
        return spmv_go<M, DV, XC, YT, IT, 1, 1, 3>(a);
    } else {
    if (a.nvec == 1) {
        if constexpr (sizeof(IT) == 4) {
            if (a.U >= 4) return spmv_go<M, DV, XC, YT, IT, 1, 4, VM>(a);
            if (a.U >= 2) return spmv_go<M, DV, XC, YT, IT, 1, 2, VM>(a);
        }
        return spmv_go<M, DV, XC, YT, IT, 1, 1, VM>(a);
    }
    if (a.nvec == 2) return spmv_go<M, DV, XC, YT, IT, 2, 1, VM>(a);
    if (a.nvec <= 4) return spmv_go<M, DV, XC, YT, IT, 4, 1, VM>(a);
    return spmv_go<M, DV, XC, YT, IT, 8, 1, VM>(a);
    }
}

// coded and packed values: int32 column indices only
template <class M, class DV, bool XC, class YT, int VM = 0>
int spmv_idx(const SpmvArgs &a)
{
    if constexpr (VM != 0) {
        if (a.idx64) return QS_ERR_ARG;
        return spmv_nb<M, DV, XC, YT, int32_t, VM>(a);
    } else {
        if (a.idx64) return spmv_nb<M, DV, XC, YT, int64_t, 0>(a);
        return spmv_nb<M, DV, XC, YT, int32_t, 0>(a);
    }
}

}  // namespace

// float32 / complex64 operands (called by qs_csr_matvec): 0 when handled,
// QS_ERR_UNSUPPORTED for type pairs left to the double kernels.
int spmv_lp_single(int64_t n, const void *indptr, int idx64, const int32_t *indices, const void *data, int dtype,
                   const void *x, int xtype, void *y, int64_t nvec, cdbl a, int overwrite, int G, int U,
                   cudaStream_t st)
{
    SpmvArgs s{n, indptr, idx64, indices, data, x, y, nvec, a, overwrite, nullptr, G, U, st};
    if (xtype == QS_F32 && dtype == QS_F32) return spmv_idx<ModeF32, float, false, float>(s);
    if (xtype == QS_C64 && dtype == QS_F32) return spmv_idx<ModeF32, float, true, cflt>(s);
    if (xtype == QS_C64 && dtype == QS_C64) return spmv_idx<ModeF32, cx<float>, true, cflt>(s);
    return QS_ERR_UNSUPPORTED;
}

// y = a A x (overwrite) or y += a A x with float64 / complex128 x and y and
// the matrix values as float pairs (pdtype QS_PF from float64 values,
// QS_CPF from complex128 values; a complex matrix needs complex x), or as
// one code byte per nonzero into a table of such pairs (QS_PF8 / QS_CPF8:
// QS_CODE_TABLE pairs, then nnz uint8 codes; int32 indices), or with the
// code packed into the low 8 bits of each column word (QS_PF8P / QS_CPF8P:
// indices holds col << 8 | code, col < 2^23; pdata the table only).
// xs: scratch of n*nvec*(8 or 16) bytes for the split x; norm: 8 bytes of
// device scratch.  group as for qs_csr_matvec.
extern "C" int qs_csr_matvec_pairs(int64_t n, int64_t nnz, const void *indptr, int idx64, const int32_t *indices,
                                   const void *pdata, int pdtype, const void *x, int xtype, void *y, int64_t nvec,
                                   double a_re, double a_im, int overwrite, int group, void *xs, void *norm,
                                   void *stream)
{
    if (n < 0 || nvec < 1 || (n > 0 && (!indptr || !x || !y || !xs || !norm))) return QS_ERR_ARG;
    if (n == 0) return QS_OK;
    const bool xc = xtype == QS_C128;
    if (!xc && xtype != QS_F64) return QS_ERR_ARG;
    const bool cvals = pdtype == QS_CPF || pdtype == QS_CPF8 || pdtype == QS_CPF8P;
    if (!xc && (a_im != 0.0 || cvals)) return QS_ERR_ARG;
    if (pdtype != QS_PF && pdtype != QS_CPF && pdtype != QS_PF8 && pdtype != QS_CPF8 && pdtype != QS_PF8P &&
        pdtype != QS_CPF8P)
        return QS_ERR_ARG;
    if (pdtype != QS_PF && pdtype != QS_CPF && idx64) return QS_ERR_ARG;
    int G = group > 0 ? (group & 0xff) : 2;
    int U = group > 0 ? ((group >> 8) & 0xff) : 1;
    if (U < 1) U = 1;
    if (G != 2 && G != 4 && G != 8 && G != 16 && G != 32) return QS_ERR_ARG;
    if (U != 1 && U != 2 && U != 4) return QS_ERR_ARG;
    (void)nnz;
    cudaStream_t st = qs_stream(stream);
    unsigned long long *nrm = reinterpret_cast<unsigned long long *>(norm);
    const int64_t count = n * nvec * (xc ? 2 : 1);
    QS_CHECK(cudaMemsetAsync(nrm, 0, sizeof(unsigned long long), st));
    int64_t b = (count + 255) / 256, cap = (int64_t)qs_num_sms() * 8;
    const int blocks = (int)(b > cap ? cap : b);
    xnorm_kernel<<<blocks, 256, 0, st>>>(count, (const double *)x, nrm);
    xsplit_kernel<<<blocks, 256, 0, st>>>(count, (const double *)x, (float2 *)xs, nrm);
    QS_CHECK(cudaGetLastError());
    SpmvArgs s{n, indptr, idx64, indices, pdata, xs, y, nvec, cdbl{a_re, a_im}, overwrite, nrm, G, U, st};
    if (pdtype == QS_PF8) return xc ? spmv_idx<ModePF, pf, true, cdbl, 1>(s) : spmv_idx<ModePF, pf, false, double, 1>(s);
    if (pdtype == QS_CPF8) return spmv_idx<ModePF, cpf, true, cdbl, 1>(s);
    const bool v4 = ((group >> 20) & 7) == 6 && group > 0;
    if (v4 && !(xc && nvec == 1 && (pdtype == QS_PF8P || pdtype == QS_CPF8P))) return QS_ERR_ARG;
    if (pdtype == QS_PF8P) {
        if (v4) return spmv_idx<ModePF, pf, true, cdbl, 3>(s);
        return xc ? spmv_idx<ModePF, pf, true, cdbl, 2>(s) : spmv_idx<ModePF, pf, false, double, 2>(s);
    }
    if (pdtype == QS_CPF8P) return v4 ? spmv_idx<ModePF, cpf, true, cdbl, 3>(s) : spmv_idx<ModePF, cpf, true, cdbl, 2>(s);
    if (!xc) return spmv_idx<ModePF, pf, false, double>(s);
    if (pdtype == QS_PF) return spmv_idx<ModePF, pf, true, cdbl>(s);
    return spmv_idx<ModePF, cpf, true, cdbl>(s);
}

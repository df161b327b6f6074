// Single-vector fused Taylor terms: a 32-row epilogue kernel and a
// persistent row-handout kernel.
//
// The same term as csrc/expm_lp.cu (new B = cf (A - mu) B, F += new B, both
// infinity norms and the stopping test of scipy's _expm_multiply_simple_core,
// which the reference's parallel-sparse-tools loop follows:
// expm_multiply_parallel_core.html:347-372), with the same arithmetic, so a
// term gives bit-identical B and F; what changes is how the work maps onto a
// warp.
//
// Measured on GB300 with the L=32 J1-J2 sector (4.7M rows, 34 nonzeros per
// row): with G lanes per row and the row epilogue (the complex float-pair
// products with the coefficients, the F update and the norms) executed right
// after each row's gathers, the epilogue is issued once per G-lane group, i.e.
// for only 32/G rows per warp instruction, and costs a quarter of the term at
// G = 4.  Here a warp owns units of 32 consecutive rows.  The gather loop
// still runs with G lanes per row (G passes of 32/G rows), but after each
// pass the row sums are shuffled to the lane whose index is the row's place
// in the unit; the epilogue then runs once for all 32 rows, one row per lane,
// both components per lane, with coalesced 16-byte loads and stores of B and
// F.  The grid is persistent (as many blocks as fit on the SMs), the unit's
// row pointers are one coalesced load per lane, and with the packed value
// form (QS_PF8P / QS_CPF8P) each nonzero's code byte travels in the low 8
// bits of its column word, so the gather loop issues one 4-byte load per
// nonzero besides the gather itself.
//
// Stopping test: the squared moduli of each new term element and each F
// element are formed in FP64 from the exact double values of the float pairs
// (as in csrc/expm_lp.cu).
#include "qs_common.cuh"
#include <type_traits>
#include "expm_ctl.cuh"
#include "pairf.cuh"
#include "lp_modes.cuh"

namespace {

constexpr unsigned FULL = 0xffffffffu;

template <class M>
__device__ __forceinline__ typename M::S shfl_idx(typename M::S v, int src);
template <>
__device__ __forceinline__ pf shfl_idx<ModePF>(pf v, int src)
{
    return pf{__shfl_sync(FULL, v.h, src), __shfl_sync(FULL, v.l, src)};
}
template <>
__device__ __forceinline__ float shfl_idx<ModeF32>(float v, int src)
{
    return __shfl_sync(FULL, v, src);
}

// VMODE: 0 one value per nonzero (data), 1 coded values (table, then one code
// byte per nonzero), 2 coded values with the code packed into the column word
// (indices holds col << 8 | code; data holds the table only), 3 the packed
// form read four words per 16-byte load (row hand-out kernel only).
template <class M, class DV, int VMODE, int G, int U>
__device__ __forceinline__ void r32_body(int64_t n, const int32_t *__restrict__ indptr,
                                         const int32_t *__restrict__ indices, const DV *__restrict__ data,
                                         const typename M::BE *__restrict__ Bin, typename M::BE *__restrict__ Bout,
                                         cdbl *__restrict__ F, cdbl mu0, const cdbl *__restrict__ coeff, int j,
                                         double tol, ExpmCtl *ctl)
{
    using S = typename M::S;
    using BE = typename M::BE;
    constexpr bool CODED = VMODE != 0;
    constexpr int GPW = 32 / G;            // rows per pass; G passes make the 32-row unit
    __shared__ S s_c[4];                   // cf.re, cf.im, (cf mu).re, (cf mu).im
    __shared__ int s_bexp;
    __shared__ DV s_tab[CODED ? QS_CODE_TABLE : 1];
    if (*((volatile int *)&ctl->done)) return;
    if (threadIdx.x == 0) s_bexp = *((volatile int *)&ctl->bexp);
    if (threadIdx.x == 1) {
        const cx<S> c{M::from_d(coeff[j].x), M::from_d(coeff[j].y)};
        const cx<S> m{M::from_d(mu0.x), M::from_d(mu0.y)};
        s_c[2] = M::sub(M::mul(c.re, m.re), M::mul(c.im, m.im));
        s_c[3] = M::add(M::mul(c.re, m.im), M::mul(c.im, m.re));
    }
    if (threadIdx.x == 32) s_c[0] = M::from_d(coeff[j].x);
    if (threadIdx.x == 33) s_c[1] = M::from_d(coeff[j].y);
    const uint8_t *codes = nullptr;
    if constexpr (CODED) {
        for (int i = threadIdx.x; i < QS_CODE_TABLE; i += blockDim.x) s_tab[i] = ldv(data + i);
        codes = reinterpret_cast<const uint8_t *>(data + QS_CODE_TABLE);
    }
    __syncthreads();
    const unsigned long long keep = l2_keep_policy();
    const int bexp = s_bexp;
    const double s_inv = pow2(-bexp);
    const S cf_re = s_c[0], cf_im = s_c[1], cm_re = s_c[2], cm_im = s_c[3];
    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);
    const int gsub = lane / G;
    const int64_t nunits = (n + 31) / 32;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double mb = 0.0, mf = 0.0;
    for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < nunits; u += nw) {
        const int64_t r = u * 32 + lane;                 // this lane's row in the epilogue
        const bool valid = r < n;
        const int32_t rp = __ldg(indptr + (valid ? r : n));
        const int64_t rlast = u * 32 + 32;
        const int32_t rend = __ldg(indptr + (rlast < n ? rlast : n));
        BE bo{M::zero(), M::zero()};
        double2 fv = make_double2(0.0, 0.0);
        if (valid) {
            bo = M::ldB(Bin + r);
            fv = __ldcs(reinterpret_cast<const double2 *>(F + r));
        }
        S sr = M::zero(), si = M::zero();
#pragma unroll 1
        for (int p = 0; p < G; p++) {
            const int rl = p * GPW + gsub;               // this group's row in the unit
            const int32_t k0 = __shfl_sync(FULL, rp, rl);
            const int32_t kn = __shfl_sync(FULL, rp, rl + 1 < 32 ? rl + 1 : 31);
            const int32_t k1 = rl + 1 < 32 ? kn : rend;
            S ar = M::zero(), ai = M::zero();
            for (int32_t k = k0 + gl; k < k1; k += G * U) {
                int32_t col[U];
                DV d[U];
#pragma unroll
                for (int uu = 0; uu < U; uu++) {
                    const int32_t kk = k + uu * G;
                    const bool in = kk < k1;
                    if constexpr (VMODE == 2) {
                        const uint32_t w = in ? (uint32_t)__ldcs(indices + kk) : 0u;
                        col[uu] = (int32_t)(w >> 8);
                        d[uu] = in ? s_tab[w & 255u] : vzero<DV>();
                    } else {
                        col[uu] = in ? __ldcs(indices + kk) : 0;
                        if constexpr (VMODE == 1) d[uu] = in ? s_tab[__ldcs(codes + kk)] : vzero<DV>();
                        else d[uu] = in ? ldv(data + kk) : vzero<DV>();
                    }
                }
#pragma unroll
                for (int uu = 0; uu < U; uu++)
                    if (k + uu * G < k1) vmul_acc<M>(ar, ai, d[uu], M::ldB(Bin + col[uu], keep));
            }
#pragma unroll
            for (int o = G >> 1; o > 0; o >>= 1) {
                ar = M::merge(ar, M::shfl_xor(ar, o));
                ai = M::merge(ai, M::shfl_xor(ai, o));
            }
            // the sum of row rl goes to lane rl
            const int src = ((lane - p * GPW) & (GPW - 1)) * G;
            const S vr = shfl_idx<M>(ar, src), vi = shfl_idx<M>(ai, src);
            if (lane / GPW == p) {
                sr = vr;
                si = vi;
            }
        }
        if (valid) {
            // new term = cf (A B) - (cf mu) B, both components (the arithmetic of csrc/expm_lp.cu)
            const S acc_re = M::fin(sr), acc_im = M::fin(si);
            const S mre = M::sub(M::add(M::mul(cf_re, acc_re), M::mul(M::neg(cf_im), acc_im)),
                                 M::add(M::mul(cm_re, bo.re), M::mul(M::neg(cm_im), bo.im)));
            const S mim = M::sub(M::add(M::mul(cf_re, acc_im), M::mul(cf_im, acc_re)),
                                 M::add(M::mul(cm_re, bo.im), M::mul(cm_im, bo.re)));
            M::st(Bout + r, BE{mre, mim});
            fv.x = M::add_to(fv.x, mre, bexp);
            fv.y = M::add_to(fv.y, mim, bexp);
            __stcs(reinterpret_cast<double2 *>(F + r), fv);
            const double dre = M::to_d(mre, 0), dim = M::to_d(mim, 0);
            const double fre = fv.x * s_inv, fim = fv.y * s_inv;
            mb = fmax(mb, __dadd_rn(__dmul_rn(dre, dre), __dmul_rn(dim, dim)));
            mf = fmax(mf, __dadd_rn(__dmul_rn(fre, fre), __dmul_rn(fim, fim)));
        }
    }
    fold_max2(mb, mf, &ctl->c2, &ctl->fn);
    if (last_block(ctl) && threadIdx.x == 0) {
        volatile ExpmCtl *vc = ctl;
        double c2 = sqrt(__longlong_as_double((long long)vc->c2));
        double fn = sqrt(__longlong_as_double((long long)vc->fn));
        const double sc = pow2(s_bexp);
        c2 *= sc;
        fn *= sc;
        vc->terms = vc->terms + 1;
        if (vc->c1 + c2 <= tol * fn) vc->done = 1;
        else vc->c1 = c2;
        vc->c2 = 0ull;
        vc->fn = 0ull;
        __threadfence();
        vc->arrive = 0u;
    }
}

// Row hand-out (G lanes per row, 32/G rows per warp at a time, the row
// epilogue right after each row's gathers) as in csrc/expm_lp.cu, specialised
// for one vector and one matrix, with a persistent grid and the packed value
// form.  Measured on the L=32 J1-J2 sector this shape at G = 2 is the
// fastest single-vector term: with two lanes per row both lanes of a group
// write (one component each), so no epilogue lane idles.
template <class M, class DV, int VMODE, int G, int U>
__device__ __forceinline__ void rows_body(int64_t n, const int32_t *__restrict__ indptr,
                                          const int32_t *__restrict__ indices, const DV *__restrict__ data,
                                          const typename M::BE *__restrict__ Bin, typename M::BE *__restrict__ Bout,
                                          cdbl *__restrict__ F, cdbl mu0, const cdbl *__restrict__ coeff, int j,
                                          double tol, ExpmCtl *ctl)
{
    using S = typename M::S;
    using BE = typename M::BE;
    constexpr bool CODED = VMODE != 0;
    constexpr int GPW = 32 / G;
    __shared__ S s_c[4];
    __shared__ int s_bexp;
    __shared__ DV s_tab[CODED ? QS_CODE_TABLE : 1];
    if (*((volatile int *)&ctl->done)) return;
    if (threadIdx.x == 0) s_bexp = *((volatile int *)&ctl->bexp);
    if (threadIdx.x == 1) {
        const cx<S> c{M::from_d(coeff[j].x), M::from_d(coeff[j].y)};
        const cx<S> m{M::from_d(mu0.x), M::from_d(mu0.y)};
        s_c[2] = M::sub(M::mul(c.re, m.re), M::mul(c.im, m.im));
        s_c[3] = M::add(M::mul(c.re, m.im), M::mul(c.im, m.re));
    }
    if (threadIdx.x == 32) s_c[0] = M::from_d(coeff[j].x);
    if (threadIdx.x == 33) s_c[1] = M::from_d(coeff[j].y);
    const uint8_t *codes = nullptr;
    if constexpr (CODED) {
        for (int i = threadIdx.x; i < QS_CODE_TABLE; i += blockDim.x) s_tab[i] = ldv(data + i);
        codes = reinterpret_cast<const uint8_t *>(data + QS_CODE_TABLE);
    }
    __syncthreads();
    const unsigned long long keep = l2_keep_policy();
    const int bexp = s_bexp;
    const double s_inv = pow2(-bexp);
    const int lane = threadIdx.x & (G - 1);
    const int comp = lane & 1;
    const int gsub = (threadIdx.x & 31) / G;
    const S cf_re = s_c[0], cm_re = s_c[2];
    const S cf_x = comp ? s_c[1] : M::neg(s_c[1]);
    const S cm_x = comp ? s_c[3] : M::neg(s_c[3]);
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double mb = 0.0, mf = 0.0;
    for (int64_t rb = warp * GPW; rb < n; rb += nwarps * GPW) {
        const int64_t r = rb + gsub;
        const bool valid = r < n;
        const bool writer = valid && lane < 2;
        const int32_t k0 = valid ? __ldg(indptr + r) : 0, k1 = valid ? __ldg(indptr + r + 1) : 0;
        BE bo{M::zero(), M::zero()};
        double fv = 0.0;
        if (writer) {
            bo = M::ldB(Bin + r);
            fv = __ldcs(reinterpret_cast<const double *>(F + r) + comp);
        }
        S ar = M::zero(), ai = M::zero();
        if constexpr (VMODE == 3) {
            // the row's column words in 16-byte aligned groups of four, group
            // g of the row to lane g mod G; words outside [k0, k1) are skipped
            for (int32_t c = (k0 & ~3) + 4 * lane; c < k1; c += 4 * G) {
                const uint4 w4 = __ldcs(reinterpret_cast<const uint4 *>(indices + c));
                const uint32_t w[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
                for (int h = 0; h < 4; h += 2) {     // two gathers in flight, as the U = 2 form
                    BE bv[2];
#pragma unroll
                    for (int i = 0; i < 2; i++)
                        bv[i] = (c + h + i >= k0 && c + h + i < k1) ? M::ldB(Bin + (int32_t)(w[h + i] >> 8), keep)
                                                                    : BE{M::zero(), M::zero()};
#pragma unroll
                    for (int i = 0; i < 2; i++)
                        if (c + h + i >= k0 && c + h + i < k1) vmul_acc<M>(ar, ai, s_tab[w[h + i] & 255u], bv[i]);
                }
            }
        } else {
            for (int32_t k = k0 + lane; k < k1; k += G * U) {
                int32_t col[U];
                DV d[U];
#pragma unroll
                for (int uu = 0; uu < U; uu++) {
                    const int32_t kk = k + uu * G;
                    const bool in = kk < k1;
                    if constexpr (VMODE == 2) {
                        const uint32_t w = in ? (uint32_t)__ldcs(indices + kk) : 0u;
                        col[uu] = (int32_t)(w >> 8);
                        d[uu] = in ? s_tab[w & 255u] : vzero<DV>();
                    } else {
                        col[uu] = in ? __ldcs(indices + kk) : 0;
                        if constexpr (VMODE == 1) d[uu] = in ? s_tab[__ldcs(codes + kk)] : vzero<DV>();
                        else d[uu] = in ? ldv(data + kk) : vzero<DV>();
                    }
                }
#pragma unroll
                for (int uu = 0; uu < U; uu++)
                    if (k + uu * G < k1) vmul_acc<M>(ar, ai, d[uu], M::ldB(Bin + col[uu], keep));
            }
        }
#pragma unroll
        for (int o = G >> 1; o > 0; o >>= 1) {
            ar = M::merge(ar, M::shfl_xor(ar, o));
            ai = M::merge(ai, M::shfl_xor(ai, o));
        }
        // new term = cf (A B) - (cf mu) B, this lane's component (as csrc/expm_lp.cu)
        const S acc_c = M::fin(comp ? ai : ar), acc_o = M::fin(comp ? ar : ai);
        const S bo_c = comp ? bo.im : bo.re, bo_o = comp ? bo.re : bo.im;
        const S mine = M::sub(M::add(M::mul(cf_re, acc_c), M::mul(cf_x, acc_o)),
                              M::add(M::mul(cm_re, bo_c), M::mul(cm_x, bo_o)));
        double md = 0.0, fs = 0.0;
        if (writer) {
            M::st_comp(Bout + r, comp, mine);
            fv = M::add_to(fv, mine, bexp);
            __stcs(reinterpret_cast<double *>(F + r) + comp, fv);
            md = M::to_d(mine, 0);
            fs = fv * s_inv;
        }
        double nb2 = __dmul_rn(md, md), f2 = __dmul_rn(fs, fs);
        nb2 = __dadd_rn(nb2, __shfl_xor_sync(FULL, nb2, 1));
        f2 = __dadd_rn(f2, __shfl_xor_sync(FULL, f2, 1));
        if (writer) {
            mb = fmax(mb, nb2);
            mf = fmax(mf, f2);
        }
    }
    fold_max2(mb, mf, &ctl->c2, &ctl->fn);
    if (last_block(ctl) && threadIdx.x == 0) {
        volatile ExpmCtl *vc = ctl;
        double c2 = sqrt(__longlong_as_double((long long)vc->c2));
        double fn = sqrt(__longlong_as_double((long long)vc->fn));
        const double sc = pow2(s_bexp);
        c2 *= sc;
        fn *= sc;
        vc->terms = vc->terms + 1;
        if (vc->c1 + c2 <= tol * fn) vc->done = 1;
        else vc->c1 = c2;
        vc->c2 = 0ull;
        vc->fn = 0ull;
        __threadfence();
        vc->arrive = 0u;
    }
}

#define R32_PARAMS                                                                                             \
    int64_t n, const int32_t *__restrict__ indptr, const int32_t *__restrict__ indices, const DV *__restrict__ data, \
        const typename M::BE *__restrict__ Bin, typename M::BE *__restrict__ Bout, cdbl *__restrict__ F, cdbl mu0,  \
        const cdbl *__restrict__ coeff, int j, double tol, ExpmCtl *ctl
#define R32_ARGS n, indptr, indices, data, Bin, Bout, F, mu0, coeff, j, tol, ctl

template <class M, class DV, int VMODE, int G, int U>
__global__ void __launch_bounds__(256, 4) taylor_r32_kernel(R32_PARAMS)
{
    r32_body<M, DV, VMODE, G, U>(R32_ARGS);
}
template <class M, class DV, int VMODE, int G, int U>
__global__ void __launch_bounds__(256, 6) taylor_r32_kernel_occ6(R32_PARAMS)
{
    r32_body<M, DV, VMODE, G, U>(R32_ARGS);
}

// persistent grid: every resident block, but no more blocks than 8-warp
// groups of 32-row units
template <class M, class DV, int VMODE, int G, int U>
__global__ void __launch_bounds__(256, 4) taylor_rows_kernel(R32_PARAMS)
{
    rows_body<M, DV, VMODE, G, U>(R32_ARGS);
}
template <class M, class DV, int VMODE, int G, int U>
__global__ void __launch_bounds__(256, 6) taylor_rows_kernel_occ6(R32_PARAMS)
{
    rows_body<M, DV, VMODE, G, U>(R32_ARGS);
}
template <class M, class DV, int VMODE, int G, int U>
__global__ void __launch_bounds__(256, 5) taylor_rows_kernel_occ5(R32_PARAMS)
{
    rows_body<M, DV, VMODE, G, U>(R32_ARGS);
}

template <class K>
int r32_blocks(K kern, const LpTerm &a, int &per_sm)
{
    if (per_sm < 0) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, 256, 0) != cudaSuccess) return -1;
        per_sm = b < 1 ? 1 : b;
    }
    const int64_t units = (a.n + 31) / 32;
    const int64_t need = (units + 7) / 8;
    const int64_t cap = (int64_t)qs_num_sms() * per_sm;
    return (int)(need < cap ? (need < 1 ? 1 : need) : cap);
}

template <class M, class DV, int VMODE, int G>
int rows_go(const LpTerm &a)
{
    constexpr int U = 2;
    using BE = typename M::BE;
    static int per_sm[3] = {-1, -1, -1};
    const int oc = a.occ == 1 || a.occ == 2 ? a.occ : 0;
    auto k = oc == 1 ? taylor_rows_kernel_occ6<M, DV, VMODE, G, U>
                     : (oc == 2 ? taylor_rows_kernel_occ5<M, DV, VMODE, G, U> : taylor_rows_kernel<M, DV, VMODE, G, U>);
    int &ps = per_sm[oc];
    if (ps < 0) {
        int b = 0;
        QS_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, 256, 0));
        ps = b < 1 ? 1 : b;
    }
    const int64_t need = (a.n + (256 / G) - 1) / (256 / G);
    const int64_t cap = (int64_t)qs_num_sms() * ps;
    const int blocks = (int)(need < cap ? (need < 1 ? 1 : need) : cap);
    k<<<blocks, 256, 0, a.st>>>(a.n, (const int32_t *)a.indptr, a.indices, (const DV *)a.data, (const BE *)a.Bin,
                                (BE *)a.Bout, a.F, a.mu0, a.coeff, a.j, a.tol, (ExpmCtl *)a.ctl);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

template <class M, class DV, int VMODE, int G>
int r32_go(const LpTerm &a)
{
    constexpr int U = 2;
    using BE = typename M::BE;
    if (a.occ == 1) {
        static int per_sm = -1;
        auto k = taylor_r32_kernel_occ6<M, DV, VMODE, G, U>;
        const int blocks = r32_blocks(k, a, per_sm);
        if (blocks < 1) return QS_ERR_CUDA;
        k<<<blocks, 256, 0, a.st>>>(a.n, (const int32_t *)a.indptr, a.indices, (const DV *)a.data,
                                    (const BE *)a.Bin, (BE *)a.Bout, a.F, a.mu0, a.coeff, a.j, a.tol,
                                    (ExpmCtl *)a.ctl);
    } else {
        static int per_sm = -1;
        auto k = taylor_r32_kernel<M, DV, VMODE, G, U>;
        const int blocks = r32_blocks(k, a, per_sm);
        if (blocks < 1) return QS_ERR_CUDA;
        k<<<blocks, 256, 0, a.st>>>(a.n, (const int32_t *)a.indptr, a.indices, (const DV *)a.data,
                                    (const BE *)a.Bin, (BE *)a.Bout, a.F, a.mu0, a.coeff, a.j, a.tol,
                                    (ExpmCtl *)a.ctl);
    }
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

template <class M, class DV, int VMODE>
int r32_g(const LpTerm &a)
{
    switch (a.staged) {
    case 1: return r32_go<M, DV, VMODE, 4>(a);
    case 2: return r32_go<M, DV, VMODE, 2>(a);
    case 3: return r32_go<M, DV, VMODE, 8>(a);
    case 4: return rows_go<M, DV, VMODE, 2>(a);
    case 5: return rows_go<M, DV, VMODE, 4>(a);
    case 6:
    case 7:
        if constexpr (VMODE == 2) return a.staged == 6 ? rows_go<M, DV, 3, 2>(a) : rows_go<M, DV, 3, 4>(a);
        else return QS_ERR_ARG;
    default: return QS_ERR_ARG;
    }
}

}  // namespace

// The single-vector terms of this file: a.staged = 1..3 the 32-row kernel
// with 4, 2 or 8 lanes per row in the gather loop, 4..5 the persistent
// row-handout kernel with 2 or 4 lanes per row, 6..7 the same with the
// packed column words read in aligned groups of four (packed operands only;
// the word buffer must be readable up to the next multiple of four words);
// a.occ = 1: registers capped for 6 blocks per SM, 2 (row hand-out only): 5,
// else 4.  One vector, int32 indptr and indices.
int st_taylor_term(const LpTerm &a)
{
    if (a.nvec != 1 || a.idx64 || a.staged < 1 || a.staged > 7) return QS_ERR_ARG;
    if (a.btype == QS_CPF) {
        switch (a.dtype) {
        case QS_PF8: return r32_g<ModePF, pf, 1>(a);
        case QS_CPF8: return r32_g<ModePF, cpf, 1>(a);
        case QS_PF8P: return r32_g<ModePF, pf, 2>(a);
        case QS_CPF8P: return r32_g<ModePF, cpf, 2>(a);
        case QS_PF: return r32_g<ModePF, pf, 0>(a);
        case QS_CPF: return r32_g<ModePF, cpf, 0>(a);
        default: return QS_ERR_ARG;
        }
    }
    if (a.btype == QS_C64) {
        switch (a.dtype) {
        case QS_F32: return r32_g<ModeF32, float, 0>(a);
        case QS_C64: return r32_g<ModeF32, cx<float>, 0>(a);
        default: return QS_ERR_ARG;
        }
    }
    return QS_ERR_ARG;
}

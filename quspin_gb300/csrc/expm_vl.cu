// Many-vector Taylor term with the vectors across the lanes.
//
// The same term as csrc/expm_lp.cu (new B = cf (A - mu) B, F += new B, the
// row sums of moduli of the new term and of F for the stopping test of
// scipy's _expm_multiply_simple_core, which the reference's
// parallel-sparse-tools loop follows: expm_multiply_parallel_core.html
// :347-372), for k > 1 vectors of one matrix or of a stack of sectors.
//
// The row hand-out kernel of csrc/expm_lp.cu gives each lane a share of a
// row's nonzeros and all of the row's vectors: for one nonzero a lane loads
// the vectors' entries of B (k consecutive 16-byte elements) with k warp
// instructions, each of which touches 32 different cache lines, one per lane.
// Measured with ncu on the L=22 Ising sectors (8 vectors), the L1TEX data
// pipe is then the busy unit (73% of its wavefronts, DRAM at 13%).  Here a
// group of 8 lanes owns a row and lane v owns vector c0 + v: one warp load
// gathers the whole 128-byte rows of B for four nonzeros (one per group), so
// a nonzero costs one wavefront instead of eight; each lane keeps one
// accumulator pair instead of eight, and a row's sums need no cross-lane
// merge.  The products, the epilogue and the F update use the arithmetic of
// csrc/expm_lp.cu; one lane sums a row's nonzeros in order, and the row sums
// of moduli add the vectors in a butterfly, so results agree with that kernel
// to float-pair rounding.
#include "qs_common.cuh"
#include <type_traits>
#include "expm_ctl.cuh"
#include "pairf.cuh"
#include "lp_modes.cuh"

namespace {

constexpr int VL = 8;    // lanes per row group = vectors per sweep of a row

template <class M, class DV, class IT, int U, bool MULTI, bool CODED>
__device__ __forceinline__ void vl_body(int64_t n, const IT *__restrict__ indptr, const int32_t *__restrict__ indices,
                                        const DV *__restrict__ data, const typename M::BE *__restrict__ Bin,
                                        typename M::BE *__restrict__ Bout, cdbl *__restrict__ F, int64_t nvec,
                                        cdbl mu0, const cdbl *__restrict__ mus, const int64_t *__restrict__ sec_off,
                                        const cdbl *__restrict__ coeff, int j, double tol, void *ctlp)
{
    using S = typename M::S;
    using BE = typename M::BE;
    constexpr int NS = MULTI ? QS_MAX_SECTORS : 1;
    __shared__ S s_cm[2 * NS];       // cf * mu per sector (the shift folded into the coefficient)
    __shared__ S s_cf[2];
    __shared__ int s_bexp[NS];
    __shared__ int s_done[NS];
    __shared__ int64_t s_off[NS + 1];
    __shared__ unsigned long long s_mb[NS], s_mf[NS];
    int nsec = 1;
    if constexpr (!MULTI) {
        ExpmCtl *ctl = reinterpret_cast<ExpmCtl *>(ctlp);
        if (*((volatile int *)&ctl->done)) return;
        if (threadIdx.x == 0) {
            s_bexp[0] = *((volatile int *)&ctl->bexp);
            s_done[0] = 0;
        }
        if (threadIdx.x == 1) {
            const cx<S> c{M::from_d(coeff[j].x), M::from_d(coeff[j].y)};
            const cx<S> m{M::from_d(mu0.x), M::from_d(mu0.y)};
            s_cm[0] = M::sub(M::mul(c.re, m.re), M::mul(c.im, m.im));
            s_cm[1] = M::add(M::mul(c.re, m.im), M::mul(c.im, m.re));
        }
    } else {
        MultiCtl *ctl = reinterpret_cast<MultiCtl *>(ctlp);
        nsec = ctl->nsec;
        for (int b = threadIdx.x; b <= nsec; b += blockDim.x) s_off[b] = sec_off[b];
        for (int b = threadIdx.x; b < nsec; b += blockDim.x) {
            s_done[b] = *((volatile int *)&ctl->done[b]);
            s_bexp[b] = ctl->bexp[b];
            const cdbl md = mus[b];
            const cx<S> c{M::from_d(coeff[j].x), M::from_d(coeff[j].y)};
            const cx<S> m{M::from_d(md.x), M::from_d(md.y)};
            s_cm[2 * b] = M::sub(M::mul(c.re, m.re), M::mul(c.im, m.im));
            s_cm[2 * b + 1] = M::add(M::mul(c.re, m.im), M::mul(c.im, m.re));
            s_mb[b] = 0ull;
            s_mf[b] = 0ull;
        }
    }
    if (threadIdx.x == 32) s_cf[0] = M::from_d(coeff[j].x);
    if (threadIdx.x == 33) s_cf[1] = M::from_d(coeff[j].y);
    __shared__ DV s_tab[CODED ? QS_CODE_TABLE : 1];
    const uint8_t *codes = nullptr;
    if constexpr (CODED) {
        for (int i = threadIdx.x; i < QS_CODE_TABLE; i += blockDim.x) s_tab[i] = ldv(data + i);
        codes = reinterpret_cast<const uint8_t *>(data + QS_CODE_TABLE);
    }
    __syncthreads();

    const int v = threadIdx.x & (VL - 1);
    const int grp = (threadIdx.x & 31) / VL;
    constexpr int RPW = 32 / VL;             // rows per warp and sweep
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const S cf_re = s_cf[0], cf_im = s_cf[1];
    double mb = 0.0, mf = 0.0;
    for (int64_t rb = warp * RPW; rb < n; rb += nwarps * RPW) {
        const int64_t r = rb + grp;
        int sec = 0;
        if constexpr (MULTI) sec = r < n ? sector_of(s_off, nsec, r) : 0;
        const bool valid = r < n && !s_done[sec];
        const IT k0 = valid ? indptr[r] : (IT)0, k1 = valid ? indptr[r + 1] : (IT)0;
        const int bexp = s_bexp[sec];
        const S cm_re = s_cm[2 * sec], cm_im = s_cm[2 * sec + 1];
        pf rbp{0.f, 0.f}, rfp{0.f, 0.f};
        for (int64_t c0 = 0; c0 < nvec; c0 += VL) {
            const int64_t c = c0 + v;
            const bool act = valid && c < nvec;
            S ar = M::zero(), ai = M::zero();
            for (IT k = k0; k < k1; k += (IT)U) {
                int32_t col[U];
                DV d[U];
                BE bv[U];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const bool in = k + (IT)u < k1;
                    col[u] = in ? __ldcs(indices + k + u) : 0;
                    if constexpr (CODED) d[u] = in ? s_tab[__ldcs(codes + k + u)] : vzero<DV>();
                    else d[u] = in ? ldv(data + k + u) : vzero<DV>();
                }
#pragma unroll
                for (int u = 0; u < U; u++)
                    bv[u] = (act && k + (IT)u < k1) ? M::ldB(Bin + (int64_t)col[u] * nvec + c) : BE{M::zero(), M::zero()};
#pragma unroll
                for (int u = 0; u < U; u++)
                    if (k + (IT)u < k1) vmul_acc<M>(ar, ai, d[u], bv[u]);
            }
            if (act) {
                const int64_t e = r * nvec + c;
                const BE bo = M::ldB(Bin + e);
                const S acc_re = M::fin(ar), acc_im = M::fin(ai);
                // new term = cf (A B) - (cf mu) B (the arithmetic of csrc/expm_lp.cu, both components)
                const S mre = M::sub(M::add(M::mul(cf_re, acc_re), M::mul(M::neg(cf_im), acc_im)),
                                     M::add(M::mul(cm_re, bo.re), M::mul(M::neg(cm_im), bo.im)));
                const S mim = M::sub(M::add(M::mul(cf_re, acc_im), M::mul(cf_im, acc_re)),
                                     M::add(M::mul(cm_re, bo.im), M::mul(cm_im, bo.re)));
                M::st(Bout + e, BE{mre, mim});
                double2 fv = __ldcs(reinterpret_cast<const double2 *>(F + e));
                fv.x = M::add_to(fv.x, mre, bexp);
                fv.y = M::add_to(fv.y, mim, bexp);
                __stcs(reinterpret_cast<double2 *>(F + e), fv);
                // moduli scaled by 2^-bexp in float-pair arithmetic
                const pf br = to_pair(mre), bi = to_pair(mim);
                const pf fr = pair_of_double_scaled(fv.x, bexp), fi = pair_of_double_scaled(fv.y, bexp);
                rbp = pf_add(rbp, pf_sqrt(pf_add(pf_mul(br, br), pf_mul(bi, bi))));
                rfp = pf_add(rfp, pf_sqrt(pf_add(pf_mul(fr, fr), pf_mul(fi, fi))));
            }
        }
        // the row's sums of moduli over its vectors: the group's eight lanes
#pragma unroll
        for (int o = 1; o < VL; o <<= 1) {
            rbp = pf_add(rbp, shfl_xor_pair(rbp, o));
            rfp = pf_add(rfp, shfl_xor_pair(rfp, o));
        }
        if (valid && v == 0) {
            const double rbn = pf_to_double_scaled(rbp, 0), rfn = pf_to_double_scaled(rfp, 0);
            if constexpr (MULTI) {
                atomicMax(&s_mb[sec], (unsigned long long)__double_as_longlong(rbn));
                atomicMax(&s_mf[sec], (unsigned long long)__double_as_longlong(rfn));
            } else {
                mb = fmax(mb, rbn);
                mf = fmax(mf, rfn);
            }
        }
    }

    // the stopping test, as in csrc/expm_lp.cu
    if constexpr (!MULTI) {
        ExpmCtl *ctl = reinterpret_cast<ExpmCtl *>(ctlp);
        fold_max2(mb, mf, &ctl->c2, &ctl->fn);
        if (last_block(ctl) && threadIdx.x == 0) {
            volatile ExpmCtl *vc = ctl;
            double c2 = __longlong_as_double((long long)vc->c2);
            double fn = __longlong_as_double((long long)vc->fn);
            const double sc = pow2(s_bexp[0]);
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
    } else {
        MultiCtl *ctl = reinterpret_cast<MultiCtl *>(ctlp);
        __syncthreads();
        for (int b = threadIdx.x; b < nsec; b += blockDim.x) {
            if (s_mb[b]) atomicMax(&ctl->c2[b], s_mb[b]);
            if (s_mf[b]) atomicMax(&ctl->fn[b], s_mf[b]);
        }
        if (last_block_multi(ctl) && threadIdx.x == 0) {
            volatile MultiCtl *vc = ctl;
            long long active = 0;
            for (int b = 0; b < nsec; b++) {
                if (vc->done[b]) continue;
                active++;
                double c2 = __longlong_as_double((long long)vc->c2[b]);
                double fn = __longlong_as_double((long long)vc->fn[b]);
                const double sc = pow2(vc->bexp[b]);
                c2 *= sc;
                fn *= sc;
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
}

#define VL_PARAMS                                                                                             \
    int64_t n, const IT *__restrict__ indptr, const int32_t *__restrict__ indices, const DV *__restrict__ data, \
        const typename M::BE *__restrict__ Bin, typename M::BE *__restrict__ Bout, cdbl *__restrict__ F,         \
        int64_t nvec, cdbl mu0, const cdbl *__restrict__ mus, const int64_t *__restrict__ sec_off,              \
        const cdbl *__restrict__ coeff, int j, double tol, void *ctlp
#define VL_ARGS n, indptr, indices, data, Bin, Bout, F, nvec, mu0, mus, sec_off, coeff, j, tol, ctlp

template <class M, class DV, class IT, int U, bool MULTI, bool CODED>
__global__ void __launch_bounds__(256, 4) taylor_vl_kernel(VL_PARAMS)
{
    vl_body<M, DV, IT, U, MULTI, CODED>(VL_ARGS);
}
template <class M, class DV, class IT, int U, bool MULTI, bool CODED>
__global__ void __launch_bounds__(256, 5) taylor_vl_kernel_occ5(VL_PARAMS)
{
    vl_body<M, DV, IT, U, MULTI, CODED>(VL_ARGS);
}

template <class M, class DV, class IT, int U, bool MULTI, bool CODED, bool OCC5>
int vl_go(const LpTerm &a)
{
    using BE = typename M::BE;
    static int resident = 0;
    auto k = OCC5 ? taylor_vl_kernel_occ5<M, DV, IT, U, MULTI, CODED> : taylor_vl_kernel<M, DV, IT, U, MULTI, CODED>;
    const int64_t need = (a.n + 31) / 32;          // 32 rows per block and sweep
    const int blocks = qs_persistent_grid(k, 256, need, resident);
    k<<<blocks, 256, 0, a.st>>>(a.n, (const IT *)a.indptr, a.indices, (const DV *)a.data, (const BE *)a.Bin,
                                (BE *)a.Bout, a.F, a.nvec, a.mu0, a.mus, a.sec_off, a.coeff, a.j, a.tol, a.ctl);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// a.staged: 1 four nonzeros in flight per lane, 4 blocks per SM; 2 two in
// flight, 4 blocks; 3 two in flight, registers capped for 5 blocks per SM
template <class M, class DV, class IT, bool MULTI, bool CODED>
int vl_shape(const LpTerm &a)
{
    switch (a.staged) {
    case 1: return vl_go<M, DV, IT, 4, MULTI, CODED, false>(a);
    case 2: return vl_go<M, DV, IT, 2, MULTI, CODED, false>(a);
    case 3: return vl_go<M, DV, IT, 2, MULTI, CODED, true>(a);
    default: return QS_ERR_ARG;
    }
}

template <class M, class DV, bool MULTI, bool CODED = false>
int vl_idx(const LpTerm &a)
{
    if constexpr (CODED) {
        if (a.idx64) return QS_ERR_ARG;
        return vl_shape<M, DV, int32_t, MULTI, true>(a);
    } else {
        if (a.idx64) return vl_shape<M, DV, int64_t, MULTI, false>(a);
        return vl_shape<M, DV, int32_t, MULTI, false>(a);
    }
}

}  // namespace

// The float forms' term for nvec > 1 vectors with the vectors across the
// lanes (a.staged = 1..3: see vl_shape); one matrix or a stack of sectors.
int vl_taylor_term(const LpTerm &a, bool multi)
{
    if (a.nvec < 2 || a.staged < 1 || a.staged > 3) return QS_ERR_ARG;
    if (multi && a.idx64) return QS_ERR_ARG;
    if (a.btype == QS_CPF) {
        if (a.dtype == QS_PF) return multi ? vl_idx<ModePF, pf, true>(a) : vl_idx<ModePF, pf, false>(a);
        if (a.dtype == QS_CPF) return multi ? vl_idx<ModePF, cpf, true>(a) : vl_idx<ModePF, cpf, false>(a);
        if (a.dtype == QS_PF8) return multi ? vl_idx<ModePF, pf, true, true>(a) : vl_idx<ModePF, pf, false, true>(a);
        if (a.dtype == QS_CPF8)
            return multi ? vl_idx<ModePF, cpf, true, true>(a) : vl_idx<ModePF, cpf, false, true>(a);
    } else if (a.btype == QS_C64) {
        if (a.dtype == QS_F32) return multi ? vl_idx<ModeF32, float, true>(a) : vl_idx<ModeF32, float, false>(a);
        if (a.dtype == QS_C64)
            return multi ? vl_idx<ModeF32, cx<float>, true>(a) : vl_idx<ModeF32, cx<float>, false>(a);
    }
    return QS_ERR_ARG;
}

// Fused Taylor term without FP64 instructions per nonzero.
//
// Same recurrence and stopping test as csrc/expm.cu (scipy's
// _expm_multiply_simple_core with the shift folded in, which the reference's
// parallel-sparse-tools==0.2.5 loop follows: expm_multiply_parallel_core.html
// :347-372), for two storage forms of the Taylor term B:
//
//   * QS_CPF  - paired single precision (csrc/pairf.cuh): B and the matrix
//               values are hi + lo float pairs, products and row sums run in
//               FP32 instructions with 48-bit significands; the default
//               "double" form of the Python layer.  The values come either
//               as one pair per nonzero (QS_PF / QS_CPF) or, for matrices
//               with at most 256 distinct values, as one code byte per
//               nonzero into a table of pairs (QS_PF8 / QS_CPF8): 1 byte of
//               value stream per nonzero instead of 8 or 16, same pairs,
//               same arithmetic, bit-identical results;
//   * QS_C64  - complex64 B and float32 / complex64 values with FP32 row sums:
//               the mixed form.
//
// In both, the Taylor partial sum F, the trace shift, the coefficients and
// the stopping test stay in IEEE double.  B is stored scaled by 2^-bexp,
// where 2^bexp is the power of two at or below ||F||_inf at the start of the
// substep, so the float exponent range covers any input scale; the scale is
// undone exactly on the exponent when a term is added to F.
//
// Per row the G lanes split the nonzeros; after the butterfly reduction every
// lane holds the row sum, lanes 0 and 1 write the real and imaginary part of
// the new term and of F (two FP64 adds each for the paired form), so the
// FP64 pipe sees a handful of fully used instructions per row instead of
// two per nonzero.  The stopping test: with one column, the squared modulus
// of each new term element and each F element is formed in FP64 from the
// exact double value of the float pair; with several columns the row sums of
// moduli are formed in float-pair arithmetic (squares to 2^-48, square roots
// to about 2^-44 relative: pf_sqrt), since a square root per element in FP64
// would load GB300's narrow FP64 pipe with a dozen instructions per element.
#include "qs_common.cuh"
#include <type_traits>
#include "expm_ctl.cuh"
#include "pairf.cuh"
#include "lp_modes.cuh"

namespace {

// One Taylor term; MULTI: block-diagonal stack of sectors (MultiCtl), else one
// matrix (ExpmCtl).  lgG: log2 of the lanes per row.  CODED: data holds a
// table of QS_CODE_TABLE values followed by one code byte per nonzero
// (dtype QS_PF8 / QS_CPF8); the table is staged in shared memory.
template <class M, class DV, class IT, int NB, int U, bool MULTI, bool CODED>
__device__ __forceinline__ void taylor_lp_body(int64_t n, int lgG, const IT *__restrict__ indptr,
                                                        const int32_t *__restrict__ indices,
                                                        const DV *__restrict__ data,
                                                        const typename M::BE *__restrict__ Bin,
                                                        typename M::BE *__restrict__ Bout, cdbl *__restrict__ F,
                                                        int64_t nvec, cdbl mu0, const cdbl *__restrict__ mus,
                                                        const int64_t *__restrict__ sec_off,
                                                        const cdbl *__restrict__ coeff, int j, double tol, void *ctlp,
                                                        double2 *__restrict__ rownorm)
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
    const unsigned long long keep = l2_keep_policy();

    const int G = 1 << lgG;
    const int GPW = 32 >> lgG;
    const int lane = threadIdx.x & (G - 1);
    const int comp = lane & 1;
    const int gsub = (threadIdx.x & 31) >> lgG;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    // lane comp computes component comp of the new term:
    //   re: cf.re acc.re - cf.im acc.im - (cm.re bo.re - cm.im bo.im)
    //   im: cf.re acc.im + cf.im acc.re - (cm.re bo.im + cm.im bo.re)
    const S cf_re = s_cf[0];
    const S cf_x = comp ? s_cf[1] : M::neg(s_cf[1]);
    double mb = 0.0, mf = 0.0;
    // Chunk-outer order (rownorm given, several NB-wide vector chunks): the
    // whole grid sweeps the rows once per chunk, so the gathered slice of B
    // is NB columns wide and can stay in L2 across the sweep; the row sums
    // of the stopping test are carried between sweeps in rownorm (the same
    // thread owns the same rows in every sweep).
    const int64_t nchunk = (nvec + NB - 1) / NB;
    const bool chunk_outer = rownorm != nullptr && nchunk > 1;
    const int64_t sweeps = chunk_outer ? nchunk : 1;
    const int64_t r_hi = n;
    for (int64_t sw = 0; sw < sweeps; sw++) {
    const int64_t c_begin = chunk_outer ? sw * NB : 0;
    const int64_t c_end = chunk_outer ? (c_begin + NB < nvec ? c_begin + NB : nvec) : nvec;
    // Rows are handed out per warp (GPW consecutive rows per warp and
    // iteration), so every lane reaches the full-mask shuffles.
    for (int64_t rb = warp * GPW; rb < r_hi; rb += nwarps * GPW) {
        const int64_t r = rb + gsub;
        int sec = 0;
        if constexpr (MULTI) sec = r < r_hi ? sector_of(s_off, nsec, r) : 0;
        const bool valid = r < r_hi && !s_done[sec];
        const bool writer = valid && lane < 2;
        const IT k0 = valid ? indptr[r] : (IT)0, k1 = valid ? indptr[r + 1] : (IT)0;
        const int bexp = s_bexp[sec];
        const double s_inv = pow2(-bexp);
        const S cm_re = s_cm[2 * sec];
        const S cm_x = comp ? s_cm[2 * sec + 1] : M::neg(s_cm[2 * sec + 1]);
        double rbn = 0.0, rfn = 0.0;
        pf rbp{0.f, 0.f}, rfp{0.f, 0.f};     // many columns: row sums of moduli as pairs
        BE bo_pre{M::zero(), M::zero()};
        double f_pre = 0.0;
        if (NB == 1 && writer) {
            bo_pre = M::ldB(Bin + r);
            f_pre = __ldcs(reinterpret_cast<const double *>(F + r) + comp);
        }
        for (int64_t c0 = c_begin; c0 < c_end; c0 += NB) {
            S ar[NB], ai[NB];
#pragma unroll
            for (int b = 0; b < NB; b++) ar[b] = ai[b] = M::zero();
            for (IT k = k0 + lane; k < k1; k += (IT)(G * U)) {
                int32_t col[U];
                DV d[U];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const IT kk = k + (IT)(u * G);
                    const bool in = kk < k1;
                    col[u] = in ? __ldcs(indices + kk) : 0;
                    if constexpr (CODED) d[u] = in ? s_tab[__ldcs(codes + kk)] : vzero<DV>();
                    else d[u] = in ? ldv(data + kk) : vzero<DV>();
                }
#pragma unroll
                for (int u = 0; u < U; u++) {
                    if (k + (IT)(u * G) < k1) {
#pragma unroll
                        for (int b = 0; b < NB; b++)
                            if (NB == 1 || c0 + b < nvec)
                                vmul_acc<M>(ar[b], ai[b], d[u],
                                            NB == 1 ? M::ldB(Bin + col[u], keep)
                                                    : M::ldB(Bin + (int64_t)col[u] * nvec + c0 + b));
                    }
                }
            }
#pragma unroll
            for (int b = 0; b < NB; b++) {
                for (int o = G >> 1; o > 0; o >>= 1) {
                    ar[b] = M::merge(ar[b], M::shfl_xor(ar[b], o));
                    ai[b] = M::merge(ai[b], M::shfl_xor(ai[b], o));
                }
            }
#pragma unroll
            for (int b = 0; b < NB; b++) {
                if (c0 + b >= nvec) break;
                const int64_t e = r * nvec + c0 + b;
                const BE bo = NB == 1 ? bo_pre : (writer ? M::ldB(Bin + e) : BE{M::zero(), M::zero()});
                // new term = cf (A B) - (cf mu) B, this lane's component only
                const S acc_c = M::fin(comp ? ai[b] : ar[b]), acc_o = M::fin(comp ? ar[b] : ai[b]);
                const S bo_c = comp ? bo.im : bo.re, bo_o = comp ? bo.re : bo.im;
                const S mine = M::sub(M::add(M::mul(cf_re, acc_c), M::mul(cf_x, acc_o)),
                                      M::add(M::mul(cm_re, bo_c), M::mul(cm_x, bo_o)));
                // moduli scaled by 2^-bexp: one column, squared moduli in FP64 (the square
                // root is taken once, at the end); several columns, row sums of moduli
                // formed in float-pair arithmetic (pf_sqrt)
                double md = 0.0, fs = 0.0;
                if (writer) {
                    M::st_comp(Bout + e, comp, mine);
                    double *fp = reinterpret_cast<double *>(F + e) + comp;
                    double fv = NB == 1 ? f_pre : __ldcs(fp);
                    fv = M::add_to(fv, mine, bexp);
                    __stcs(fp, fv);
                    if (NB == 1) {
                        md = M::to_d(mine, 0);
                        fs = fv * s_inv;
                    } else {
                        fs = fv;             // scaled by 2^-bexp in the pair split below
                    }
                }
                if constexpr (NB == 1) {
                    double nb2 = __dmul_rn(md, md), f2 = __dmul_rn(fs, fs);
                    nb2 = __dadd_rn(nb2, __shfl_xor_sync(0xffffffffu, nb2, 1));
                    f2 = __dadd_rn(f2, __shfl_xor_sync(0xffffffffu, f2, 1));
                    rbn = nb2;
                    rfn = f2;
                } else {
                    const pf bm = writer ? to_pair(mine) : pf{0.f, 0.f};
                    const pf fm = writer ? pair_of_double_scaled(fs, bexp) : pf{0.f, 0.f};
                    pf b2 = pf_mul(bm, bm), f2 = pf_mul(fm, fm);
                    b2 = pf_add(b2, shfl_xor_pair(b2, 1));
                    f2 = pf_add(f2, shfl_xor_pair(f2, 1));
                    rbp = pf_add(rbp, pf_sqrt(b2));
                    rfp = pf_add(rfp, pf_sqrt(f2));
                }
            }
        }
        if constexpr (NB > 1) {
            rbn = pf_to_double_scaled(rbp, 0);
            rfn = pf_to_double_scaled(rfp, 0);
        }
        if (chunk_outer && writer && lane == 0) {
            double2 acc = sw == 0 ? make_double2(0.0, 0.0) : rownorm[r];
            acc.x += rbn;
            acc.y += rfn;
            if (sw + 1 < sweeps) rownorm[r] = acc;
            rbn = acc.x;
            rfn = acc.y;
        }
        if (writer && sw + 1 == sweeps) {
            if constexpr (MULTI) {
                if (lane == 0) {
                    atomicMax(&s_mb[sec], (unsigned long long)__double_as_longlong(rbn));
                    atomicMax(&s_mf[sec], (unsigned long long)__double_as_longlong(rfn));
                }
            } else {
                mb = fmax(mb, rbn);
                mf = fmax(mf, rfn);
            }
        }
    }
    }

    if constexpr (!MULTI) {
        ExpmCtl *ctl = reinterpret_cast<ExpmCtl *>(ctlp);
        fold_max2(mb, mf, &ctl->c2, &ctl->fn);
        if (last_block(ctl) && threadIdx.x == 0) {
            volatile ExpmCtl *vc = ctl;
            double c2 = __longlong_as_double((long long)vc->c2);
            double fn = __longlong_as_double((long long)vc->fn);
            if (nvec == 1) { c2 = sqrt(c2); fn = sqrt(fn); }
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
                if (nvec == 1) { c2 = sqrt(c2); fn = sqrt(fn); }
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

#define TAYLOR_LP_PARAMS                                                                                      \
    int64_t n, int lgG, const IT *__restrict__ indptr, const int32_t *__restrict__ indices,                   \
        const DV *__restrict__ data, const typename M::BE *__restrict__ Bin, typename M::BE *__restrict__ Bout, \
        cdbl *__restrict__ F, int64_t nvec, cdbl mu0, const cdbl *__restrict__ mus,                           \
        const int64_t *__restrict__ sec_off, const cdbl *__restrict__ coeff, int j, double tol, void *ctlp, \
        double2 *__restrict__ rownorm
#define TAYLOR_LP_ARGS n, lgG, indptr, indices, data, Bin, Bout, F, nvec, mu0, mus, sec_off, coeff, j, tol, ctlp, rownorm

template <class M, class DV, class IT, int NB, int U, bool MULTI, bool CODED>
__global__ void __launch_bounds__(256) taylor_lp_kernel(TAYLOR_LP_PARAMS)
{
    taylor_lp_body<M, DV, IT, NB, U, MULTI, CODED>(TAYLOR_LP_ARGS);
}

// The eight-column shapes hold 32 pair accumulators per lane; capping them at
// three resident blocks per SM keeps 24 warps for the gathers.
template <class M, class DV, class IT, int NB, int U, bool MULTI, bool CODED>
__global__ void __launch_bounds__(256, 3) taylor_lp_kernel_wide(TAYLOR_LP_PARAMS)
{
    taylor_lp_body<M, DV, IT, NB, U, MULTI, CODED>(TAYLOR_LP_ARGS);
}

// Single-vector float-pair shapes with the registers capped for 6 or 8
// resident blocks per SM (more warps to cover the gather latency; the
// tuner decides whether the cap pays on the matrix at hand).
template <class M, class DV, class IT, int NB, int U, bool MULTI, bool CODED>
__global__ void __launch_bounds__(256, 6) taylor_lp_kernel_occ6(TAYLOR_LP_PARAMS)
{
    taylor_lp_body<M, DV, IT, NB, U, MULTI, CODED>(TAYLOR_LP_ARGS);
}
template <class M, class DV, class IT, int NB, int U, bool MULTI, bool CODED>
__global__ void __launch_bounds__(256, 8) taylor_lp_kernel_occ8(TAYLOR_LP_PARAMS)
{
    taylor_lp_body<M, DV, IT, NB, U, MULTI, CODED>(TAYLOR_LP_ARGS);
}

// F = eta F (per sector for MULTI) and the row-norm maximum; the last block
// sets c1 = ||F||_inf, the storage exponent bexp and clears the per-substep
// state (counting, at a substep end, a stopping test that never fired).
template <bool MULTI>
__global__ void __launch_bounds__(256) taylor_lp_norm_kernel(int64_t n, int64_t nvec, cdbl *__restrict__ F,
                                                             const cdbl *__restrict__ eta, int use_eta,
                                                             const int64_t *__restrict__ sec_off, void *ctlp,
                                                             int substep_end)
{
    constexpr int NS = MULTI ? QS_MAX_SECTORS : 1;
    __shared__ int64_t s_off[NS + 1];
    __shared__ unsigned long long s_m[NS];
    int nsec = 1;
    if constexpr (MULTI) {
        nsec = reinterpret_cast<MultiCtl *>(ctlp)->nsec;
        for (int b = threadIdx.x; b <= nsec; b += blockDim.x) s_off[b] = sec_off[b];
        for (int b = threadIdx.x; b < nsec; b += blockDim.x) s_m[b] = 0ull;
        __syncthreads();
    }
    double m = 0.0;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        int b = 0;
        if constexpr (MULTI) b = sector_of(s_off, nsec, r);
        const cdbl et = use_eta ? eta[b] : cdbl{1.0, 0.0};
        const bool scale = !(et.x == 1.0 && et.y == 0.0);
        double rs = 0.0;
        for (int64_t c = 0; c < nvec; c++) {
            const int64_t e = r * nvec + c;
            cdbl f = F[e];
            if (scale) {
                f = cdbl{et.x * f.x - et.y * f.y, et.x * f.y + et.y * f.x};
                F[e] = f;
            }
            rs += hypot(f.x, f.y);
        }
        if constexpr (MULTI) atomicMax(&s_m[b], (unsigned long long)__double_as_longlong(rs));
        else m = fmax(m, rs);
    }
    if constexpr (!MULTI) {
        ExpmCtl *ctl = reinterpret_cast<ExpmCtl *>(ctlp);
        fold_max2(m, 0.0, &ctl->c2, nullptr);
        if (last_block(ctl) && threadIdx.x == 0) {
            volatile ExpmCtl *vc = ctl;
            const double c1 = __longlong_as_double((long long)vc->c2);
            vc->c1 = c1;
            vc->bexp = scale_exp(c1);
            vc->c2 = 0ull;
            vc->fn = 0ull;
            if (substep_end && !vc->done) vc->nonconv = vc->nonconv + 1;
            vc->done = 0;
            __threadfence();
            vc->arrive = 0u;
        }
    } else {
        MultiCtl *ctl = reinterpret_cast<MultiCtl *>(ctlp);
        __syncthreads();
        for (int b = threadIdx.x; b < nsec; b += blockDim.x)
            if (s_m[b]) atomicMax(&ctl->c2[b], s_m[b]);
        if (last_block_multi(ctl) && threadIdx.x == 0) {
            volatile MultiCtl *vc = ctl;
            for (int b = 0; b < nsec; b++) {
                const double c1 = __longlong_as_double((long long)vc->c2[b]);
                vc->c1[b] = c1;
                vc->bexp[b] = scale_exp(c1);
                vc->c2[b] = 0ull;
                vc->fn[b] = 0ull;
                vc->done[b] = 0;
            }
            __threadfence();
            vc->arrive = 0u;
        }
    }
}

// B0 = F 2^-bexp in the storage form of M
template <class M, bool MULTI>
__global__ void __launch_bounds__(256) taylor_lp_load_kernel(int64_t n, int64_t nvec, const cdbl *__restrict__ F,
                                                             typename M::BE *__restrict__ B0,
                                                             const int64_t *__restrict__ sec_off, const void *ctlp)
{
    constexpr int NS = MULTI ? QS_MAX_SECTORS : 1;
    __shared__ int64_t s_off[NS + 1];
    __shared__ double s_sc[NS];
    int nsec = 1;
    if constexpr (MULTI) {
        const MultiCtl *ctl = reinterpret_cast<const MultiCtl *>(ctlp);
        nsec = ctl->nsec;
        for (int b = threadIdx.x; b <= nsec; b += blockDim.x) s_off[b] = sec_off[b];
        for (int b = threadIdx.x; b < nsec; b += blockDim.x) s_sc[b] = pow2(-ctl->bexp[b]);
    } else {
        if (threadIdx.x == 0) s_sc[0] = pow2(-reinterpret_cast<const ExpmCtl *>(ctlp)->bexp);
    }
    __syncthreads();
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        int b = 0;
        if constexpr (MULTI) b = sector_of(s_off, nsec, r);
        const double sc = s_sc[b];
        for (int64_t c = 0; c < nvec; c++) {
            const int64_t e = r * nvec + c;
            const cdbl f = F[e];
            M::st(B0 + e, typename M::BE{M::from_d(f.x * sc), M::from_d(f.y * sc)});
        }
    }
}

__global__ void split_pairs_kernel(int64_t count, const double *__restrict__ src, float2 *__restrict__ dst)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        const pf v = pf_from_double(src[i]);
        dst[i] = make_float2(v.h, v.l);
    }
}

template <class M, class DV, class IT, int NB, int U, bool MULTI, bool CODED>
int lp_go(const LpTerm &a)
{
    int lg = 0;
    while ((1 << lg) < a.G) lg++;
    // persistent grid: the kernels stride over row groups, so one wave of
    // resident blocks does all rows without per-block set-up repeated
    const int64_t need = taylor_grid(a.n, a.G);
    static int resident[4] = {0, 0, 0, 0};
    double2 *rn = a.chunk_outer ? (double2 *)a.rownorm : nullptr;
    if constexpr (NB == 1 && U <= 2 && sizeof(IT) == 4 && std::is_same<M, ModePF>::value) {
        if (a.occ == 1 || a.occ == 2) {
            auto k = a.occ == 1 ? taylor_lp_kernel_occ6<M, DV, IT, NB, U, MULTI, CODED>
                                : taylor_lp_kernel_occ8<M, DV, IT, NB, U, MULTI, CODED>;
            const int blocks = qs_persistent_grid(k, 256, need, resident[a.occ]);
            k<<<blocks, 256, 0, a.st>>>(a.n, lg, (const IT *)a.indptr, a.indices, (const DV *)a.data,
                                        (const typename M::BE *)a.Bin, (typename M::BE *)a.Bout, a.F, a.nvec, a.mu0,
                                        a.mus, a.sec_off, a.coeff, a.j, a.tol, a.ctl, rn);
            QS_CHECK(cudaGetLastError());
            return QS_OK;
        }
    }
    if constexpr (NB >= 8) {
        auto k = taylor_lp_kernel_wide<M, DV, IT, NB, U, MULTI, CODED>;
        const int blocks = qs_persistent_grid(k, 256, need, resident[3]);
        k<<<blocks, 256, 0, a.st>>>(a.n, lg, (const IT *)a.indptr, a.indices, (const DV *)a.data,
                                    (const typename M::BE *)a.Bin, (typename M::BE *)a.Bout, a.F, a.nvec, a.mu0,
                                    a.mus, a.sec_off, a.coeff, a.j, a.tol, a.ctl, rn);
    } else {
        auto k = taylor_lp_kernel<M, DV, IT, NB, U, MULTI, CODED>;
        const int blocks = qs_persistent_grid(k, 256, need, resident[0]);
        k<<<blocks, 256, 0, a.st>>>(a.n, lg, (const IT *)a.indptr, a.indices, (const DV *)a.data,
                                    (const typename M::BE *)a.Bin, (typename M::BE *)a.Bout, a.F, a.nvec, a.mu0,
                                    a.mus, a.sec_off, a.coeff, a.j, a.tol, a.ctl, rn);
    }
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

template <class M, class DV, class IT, bool MULTI, bool CODED>
int lp_nb(const LpTerm &a)
{
    if (a.nvec == 1) {
        if constexpr (sizeof(IT) == 4) {
            if (a.U >= 4 && !MULTI) return lp_go<M, DV, IT, 1, 4, MULTI, CODED>(a);
            if (a.U >= 2) return lp_go<M, DV, IT, 1, 2, MULTI, CODED>(a);
        }
        return lp_go<M, DV, IT, 1, 1, MULTI, CODED>(a);
    }
    if (a.nvec == 2) return lp_go<M, DV, IT, 2, 1, MULTI, CODED>(a);
    if (a.nvec <= 4 || (a.chunk_outer && a.narrow)) return lp_go<M, DV, IT, 4, 1, MULTI, CODED>(a);
    return lp_go<M, DV, IT, 8, 1, MULTI, CODED>(a);
}

// coded values: int32 column indices only
template <class M, class DV, bool MULTI, bool CODED = false>
int lp_idx(const LpTerm &a)
{
    if constexpr (CODED) {
        if (a.idx64) return QS_ERR_ARG;
        return lp_nb<M, DV, int32_t, MULTI, true>(a);
    } else {
        if constexpr (!MULTI) {
            if (a.idx64) return lp_nb<M, DV, int64_t, false, false>(a);
        }
        return lp_nb<M, DV, int32_t, MULTI, false>(a);
    }
}

}  // namespace

int lp_taylor_term(const LpTerm &a, bool multi)
{
    if (a.G != 2 && a.G != 4 && a.G != 8 && a.G != 16 && a.G != 32) return QS_ERR_ARG;
    if (multi && a.idx64) return QS_ERR_ARG;
    if (a.btype == QS_CPF) {
        if (a.dtype == QS_PF) return multi ? lp_idx<ModePF, pf, true>(a) : lp_idx<ModePF, pf, false>(a);
        if (a.dtype == QS_CPF) return multi ? lp_idx<ModePF, cpf, true>(a) : lp_idx<ModePF, cpf, false>(a);
        if (a.dtype == QS_PF8)
            return multi ? lp_idx<ModePF, pf, true, true>(a) : lp_idx<ModePF, pf, false, true>(a);
        if (a.dtype == QS_CPF8)
            return multi ? lp_idx<ModePF, cpf, true, true>(a) : lp_idx<ModePF, cpf, false, true>(a);
    } else if (a.btype == QS_C64) {
        if (a.dtype == QS_F32) return multi ? lp_idx<ModeF32, float, true>(a) : lp_idx<ModeF32, float, false>(a);
        if (a.dtype == QS_C64)
            return multi ? lp_idx<ModeF32, cx<float>, true>(a) : lp_idx<ModeF32, cx<float>, false>(a);
    }
    return QS_ERR_ARG;
}

int lp_taylor_rescale(int64_t n, int64_t nvec, cdbl *F, void *B0, int btype, const cdbl *eta, int use_eta,
                      const int64_t *sec_off, void *ctl, int substep_end, bool multi, cudaStream_t st)
{
    if (!lp_btype(btype)) return QS_ERR_ARG;
    int64_t b = (n + 255) / 256, cap = (int64_t)qs_num_sms() * 8;
    const int blocks = (int)(b > cap ? cap : b);
    if (multi) taylor_lp_norm_kernel<true><<<blocks, 256, 0, st>>>(n, nvec, F, eta, use_eta, sec_off, ctl, substep_end);
    else taylor_lp_norm_kernel<false><<<blocks, 256, 0, st>>>(n, nvec, F, eta, use_eta, sec_off, ctl, substep_end);
    QS_CHECK(cudaGetLastError());
    if (btype == QS_CPF) {
        if (multi) taylor_lp_load_kernel<ModePF, true><<<blocks, 256, 0, st>>>(n, nvec, F, (cpf *)B0, sec_off, ctl);
        else taylor_lp_load_kernel<ModePF, false><<<blocks, 256, 0, st>>>(n, nvec, F, (cpf *)B0, sec_off, ctl);
    } else {
        if (multi)
            taylor_lp_load_kernel<ModeF32, true><<<blocks, 256, 0, st>>>(n, nvec, F, (cx<float> *)B0, sec_off, ctl);
        else
            taylor_lp_load_kernel<ModeF32, false><<<blocks, 256, 0, st>>>(n, nvec, F, (cx<float> *)B0, sec_off, ctl);
    }
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// dst[i] = (hi, lo) with hi = float(src[i]), lo = float(src[i] - hi): the
// paired form of a double array (a complex128 array splits into the
// {re.hi, re.lo, im.hi, im.lo} layout of QS_CPF).
extern "C" int qs_split_pairs(int64_t count, const double *src, void *dst, void *stream)
{
    if (count < 0 || (count > 0 && (!src || !dst))) return QS_ERR_ARG;
    if (count == 0) return QS_OK;
    int64_t b = (count + 255) / 256, cap = (int64_t)qs_num_sms() * 8;
    split_pairs_kernel<<<(int)(b > cap ? cap : b), 256, 0, qs_stream(stream)>>>(count, src, (float2 *)dst);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

namespace {
__global__ void split_pairs_trunc_kernel(int64_t count, const double *__restrict__ src, int k, float2 *__restrict__ dst)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        const pf v = pair_of_double_scaled(src[i], k);
        dst[i] = make_float2(v.h, v.l);
    }
}
}  // namespace

// dst[i] = the pair of src[i] 2^-k that the many-vector stopping tests form
// for their moduli: hi = src[i] 2^-k truncated to 24 significant bits, lo =
// the rest truncated likewise (zero below the normal float range).
extern "C" int qs_split_pairs_trunc(int64_t count, const double *src, int k, void *dst, void *stream)
{
    if (count < 0 || (count > 0 && (!src || !dst))) return QS_ERR_ARG;
    if (count == 0) return QS_OK;
    int64_t b = (count + 255) / 256, cap = (int64_t)qs_num_sms() * 8;
    split_pairs_trunc_kernel<<<(int)(b > cap ? cap : b), 256, 0, qs_stream(stream)>>>(count, src, k, (float2 *)dst);
    QS_CHECK(cudaGetLastError());
    return QS_OK;
}

// Arithmetic policies of the float-instruction sparse kernels
// (csrc/expm_lp.cu, csrc/spmv_lp.cu): ModePF keeps values as float pairs
// (csrc/pairf.cuh), ModeF32 as plain floats.  Each gives the scalar type S,
// the complex element BE of the gathered vector, the product-accumulate and
// the butterfly merge of partial row sums, small complex arithmetic for the
// row epilogue and the conversions to IEEE double.
#pragma once
#include "qs_common.cuh"
#include "pairf.cuh"

namespace {

// L2 eviction priority for the gathered vector (createpolicy, PTX ISA 7.4+):
// single-vector gathers carry an evict_last policy so that the vector's
// lines outlive the streamed indices, values and partial sums (loaded and
// stored evict-first through __ldcs / __stcs) while a product or Taylor term
// runs.  Multi-vector blocks are far larger than L2 and keep the default.
__device__ __forceinline__ unsigned long long l2_keep_policy()
{
    unsigned long long pol;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ float4 ld_keep4(const float4 *p, unsigned long long pol)
{
    float4 v;
    asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ float2 ld_keep2(const float2 *p, unsigned long long pol)
{
    float2 v;
    asm("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(p), "l"(pol));
    return v;
}

struct ModePF {
    using S = pf;
    using BE = cpf;
    __device__ static S zero() { return pf{0.f, 0.f}; }
    __device__ static BE ldB(const BE *p)
    {
        const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
        return BE{pf{v.x, v.y}, pf{v.z, v.w}};
    }
    __device__ static BE ldB(const BE *p, unsigned long long pol)
    {
        const float4 v = ld_keep4(reinterpret_cast<const float4 *>(p), pol);
        return BE{pf{v.x, v.y}, pf{v.z, v.w}};
    }
    __device__ static void fma(S &acc, S a, S b) { pf_fma(acc, a.h, a.l, b.h, b.l); }
    __device__ static S merge(S a, S b) { return pf_merge(a, b); }
    __device__ static S fin(S a) { return pf_norm(a); }
    __device__ static S add(S a, S b) { return pf_add(a, b); }
    __device__ static S sub(S a, S b) { return pf_sub(a, b); }
    __device__ static S mul(S a, S b) { return pf_mul(a, b); }
    __device__ static S neg(S a) { return pf_neg(a); }
    __device__ static float hi(S a) { return a.h; }
    __device__ static S from_d(double x) { return pf_from_double(x); }
    __device__ static S shfl_xor(S a, int o)
    {
        return pf{__shfl_xor_sync(0xffffffffu, a.h, o), __shfl_xor_sync(0xffffffffu, a.l, o)};
    }
    __device__ static S ldS(const S *p)
    {
        const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
        return pf{v.x, v.y};
    }
    __device__ static double add_to(double f, S v, int k) { return (f + f2d_scaled(v.h, k)) + f2d_scaled(v.l, k); }
    __device__ static double to_d(S v, int k) { return f2d_scaled(v.h, k) + f2d_scaled(v.l, k); }
    __device__ static void st_comp(BE *p, int comp, S v)
    {
        __stcs(reinterpret_cast<float2 *>(p) + comp, make_float2(v.h, v.l));
    }
    __device__ static void st(BE *p, BE v)
    {
        __stcs(reinterpret_cast<float4 *>(p), make_float4(v.re.h, v.re.l, v.im.h, v.im.l));
    }
};

struct ModeF32 {
    using S = float;
    using BE = cx<float>;
    __device__ static S zero() { return 0.f; }
    __device__ static BE ldB(const BE *p)
    {
        const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
        return BE{v.x, v.y};
    }
    __device__ static BE ldB(const BE *p, unsigned long long pol)
    {
        const float2 v = ld_keep2(reinterpret_cast<const float2 *>(p), pol);
        return BE{v.x, v.y};
    }
    // explicit rounding everywhere (no contraction), so that every kernel
    // that uses this mode gives the same bits
    __device__ static void fma(S &acc, S a, S b) { acc = __fmaf_rn(a, b, acc); }
    __device__ static S merge(S a, S b) { return __fadd_rn(a, b); }
    __device__ static S fin(S a) { return a; }
    __device__ static S add(S a, S b) { return __fadd_rn(a, b); }
    __device__ static S sub(S a, S b) { return __fsub_rn(a, b); }
    __device__ static S mul(S a, S b) { return __fmul_rn(a, b); }
    __device__ static S neg(S a) { return -a; }
    __device__ static float hi(S a) { return a; }
    __device__ static S from_d(double x) { return (float)x; }
    __device__ static S shfl_xor(S a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
    __device__ static S ldS(const S *p) { return __ldg(p); }
    __device__ static double add_to(double f, S v, int k) { return f + f2d_scaled(v, k); }
    __device__ static double to_d(S v, int k) { return f2d_scaled(v, k); }
    __device__ static void st_comp(BE *p, int comp, S v) { __stcs(reinterpret_cast<float *>(p) + comp, v); }
    __device__ static void st(BE *p, BE v) { __stcs(reinterpret_cast<float2 *>(p), make_float2(v.re, v.im)); }
};

// streamed loads of the matrix values
__device__ __forceinline__ pf ldv(const pf *p)
{
    const float2 v = __ldcs(reinterpret_cast<const float2 *>(p));
    return pf{v.x, v.y};
}
__device__ __forceinline__ cpf ldv(const cpf *p)
{
    const float4 v = __ldcs(reinterpret_cast<const float4 *>(p));
    return cpf{pf{v.x, v.y}, pf{v.z, v.w}};
}
__device__ __forceinline__ float ldv(const float *p) { return __ldcs(p); }
__device__ __forceinline__ cx<float> ldv(const cx<float> *p)
{
    const float2 v = __ldcs(reinterpret_cast<const float2 *>(p));
    return cx<float>{v.x, v.y};
}
template <class DV> __device__ __forceinline__ DV vzero() { return DV{}; }

// acc += d x for a real value d and a complex x
template <class M>
__device__ __forceinline__ void vmul_acc(typename M::S &ar, typename M::S &ai, typename M::S d,
                                         const typename M::BE &x)
{
    M::fma(ar, d, x.re);
    M::fma(ai, d, x.im);
}
// acc += d x for a complex value d
template <class M>
__device__ __forceinline__ void vmul_acc(typename M::S &ar, typename M::S &ai, const cx<typename M::S> &d,
                                         const typename M::BE &x)
{
    M::fma(ar, d.re, x.re);
    M::fma(ar, M::neg(d.im), x.im);
    M::fma(ai, d.re, x.im);
    M::fma(ai, d.im, x.re);
}

// exponent of the largest power of two <= x (0 for 0, subnormal or non-finite x)
__device__ __forceinline__ int scale_exp(double x)
{
    const int E = (int)(((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ffull);
    if (E == 0 || E == 0x7ff) return 0;
    int k = E - 1023;
    return k < -1000 ? -1000 : (k > 1000 ? 1000 : k);
}

__device__ __forceinline__ double pow2(int k)   // 2^k for |k| <= 1000
{
    return __hiloint2double((1023 + k) << 20, 0);
}

// Moduli for the stopping test of the many-vector terms, in float-pair
// arithmetic on the FP32 pipe (GB300's FP64 pipe is a small fraction of its
// FP32 rate, and a square root in FP64 costs a dozen FP64 instructions per
// vector element).  pf_mul squares a pair with an error of order 2^-48
// relative; pf_sqrt takes the correctly rounded FP32 root of the high part
// and one correction with the exact FMA remainder, so the root of a pair is
// accurate to about 2^-44 relative.
__device__ __forceinline__ pf to_pair(pf v) { return v; }
__device__ __forceinline__ pf to_pair(float v) { return pf{v, 0.f}; }

__device__ __forceinline__ pf shfl_xor_pair(pf a, int o)
{
    return pf{__shfl_xor_sync(0xffffffffu, a.h, o), __shfl_xor_sync(0xffffffffu, a.l, o)};
}

// x 2^-k (exact, O(1)) as an unevaluated pair of floats, without FP64
// instructions: the high part is x's top 24 significant bits (d2f_scaled);
// the rest, x minus that, is exactly the low 29 bits of x's stored
// significand, made a float here by a leading-zero count and truncated to 24
// significant bits as d2f_scaled truncates (the same pair as truncating x
// 2^-k, subtracting the high part in FP64 and truncating the difference).
// Low parts below the normal float range are zero.
__device__ __forceinline__ pf pair_of_double_scaled(double x, int k)
{
    const float h = d2f_scaled(x, k);
    const uint32_t hi = (uint32_t)__double2hiint(x);
    const uint32_t m = (uint32_t)__double2loint(x) & 0x1fffffffu;
    if (m == 0u || (__float_as_uint(h) & 0x7fffffffu) == 0u || (__float_as_uint(h) & 0x7f800000u) == 0x7f800000u)
        return pf{h, 0.f};
    const int E = (int)((hi >> 20) & 0x7ffu);
    const int p = 31 - __clz(m);                     // leading bit of m, 0..28
    const int ef = E - 948 + p - k;                  // float exponent field of m 2^(E-1075-k)
    if (ef <= 0) return pf{h, 0.f};
    const uint32_t frac = (p >= 23 ? (m >> (p - 23)) : (m << (23 - p))) & 0x7fffffu;
    return pf{h, __uint_as_float((hi & 0x80000000u) | ((uint32_t)ef << 23) | frac)};
}

__device__ __forceinline__ pf pf_sqrt(pf x)
{
    if (!(x.h > 0.f)) return pf{0.f, 0.f};
    const float s = __fsqrt_rn(x.h);
    const float r = __fadd_rn(__fmaf_rn(-s, s, x.h), x.l);     // x - s^2 (the FMA remainder is exact)
    const float c = __fmul_rn(__fmul_rn(0.5f, r), __frcp_rn(s));
    return pf_norm(pf{s, c});
}


}  // namespace

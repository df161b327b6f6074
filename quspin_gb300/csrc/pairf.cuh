// Paired single-precision arithmetic for the sparse products.
//
// GB300 issues FP64 instructions at a small fraction of its FP32 rate: a
// sparse product with one or two FP64 fused multiply-adds per nonzero keeps
// the FP64 pipe busy long before the memory system is.  The hot loops
// therefore keep a real number as an unevaluated sum hi + lo of two floats
// (48 significant bits) and use only FP32 instructions per nonzero:
//
//   * error-free product: p = a*b, e = fma(a, b, -p) gives a*b = p + e exactly
//     (T. J. Dekker, "A floating-point technique for extending the available
//     precision", Numer. Math. 18 (1971) 224-242, with the fused multiply-add
//     in place of Dekker's splitting);
//   * error-free sum: Knuth's six-operation two-sum (D. E. Knuth, The Art of
//     Computer Programming vol. 2, 4.2.2, Theorem B) and the three-operation
//     fast two-sum for |a| >= |b| (Dekker 1971);
//   * dot-product accumulation in the style of T. Ogita, S. M. Rump and
//     S. Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26 (2005)
//     1955-1988 (Dot2): the high parts are chained through two-sum, every
//     rounding error is collected in one float and added once at the end.
//
// Only the per-row epilogue (the Taylor partial sum F, which stays in IEEE
// double) uses FP64 adds.  Conversions between float and double are done on
// the bit patterns with integer instructions, with an exact power-of-two
// scale folded into the exponent; subnormal floats are flushed to zero there
// (their contribution is below 2^-126 of the scaled vector).
#pragma once
#include <stdint.h>

struct pf { float h, l; };            // value = h + l
template <class S> struct cx { S re, im; };
using cpf = cx<pf>;                   // complex pair: {re.h, re.l, im.h, im.l}, 16 bytes

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

// accumulator of a dot product: h chained through two-sum, l collects errors
__device__ __forceinline__ void pf_fma(pf &acc, float ah, float al, float bh, float bl)
{
    const float p = __fmul_rn(ah, bh);
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    float s, t;
    two_sum(acc.h, p, s, t);
    acc.h = s;
    acc.l = __fadd_rn(acc.l, __fadd_rn(t, e));
}

// sum of two accumulators (unnormalised)
__device__ __forceinline__ pf pf_merge(pf a, pf b)
{
    float s, t;
    two_sum(a.h, b.h, s, t);
    return pf{s, __fadd_rn(__fadd_rn(a.l, b.l), t)};
}

__device__ __forceinline__ pf pf_norm(pf a)
{
    float s, t;
    fast_two_sum(a.h, a.l, s, t);
    return pf{s, t};
}

__device__ __forceinline__ pf pf_neg(pf a) { return pf{-a.h, -a.l}; }

__device__ __forceinline__ pf pf_add(pf a, pf b)
{
    float s, t;
    two_sum(a.h, b.h, s, t);
    t = __fadd_rn(t, __fadd_rn(a.l, b.l));
    fast_two_sum(s, t, s, t);
    return pf{s, t};
}

__device__ __forceinline__ pf pf_sub(pf a, pf b) { return pf_add(a, pf_neg(b)); }

__device__ __forceinline__ pf pf_mul(pf a, pf b)
{
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    float s, t;
    fast_two_sum(p, e, s, t);
    return pf{s, t};
}

// split of a double into hi + lo floats (FP64 instructions: used once per
// block for constants and once per element when a vector is loaded)
__device__ __forceinline__ pf pf_from_double(double x)
{
    const float h = (float)x;
    const float l = (float)(x - (double)h);
    return pf{h, l};
}

// float -> double times 2^k on the bit pattern (exact for normal results;
// results below the normal double range are truncated to subnormals, above
// it go to infinity; subnormal floats count as zero)
__device__ __forceinline__ double f2d_scaled(float f, int k)
{
    const uint32_t u = __float_as_uint(f);
    const uint32_t sgn = u & 0x80000000u;
    const int e = (int)((u >> 23) & 0xffu);
    uint32_t hi, lo;
    if (e == 0) {
        hi = sgn;
        lo = 0u;
    } else if (e == 0xff) {
        hi = sgn | 0x7ff00000u | ((u & 0x7fffffu) >> 3);
        lo = u << 29;
    } else {
        const int ed = e + 896 + k;
        if (ed <= 0) {
            const int sh = 1 - ed;   // significand with its leading one, shifted into the subnormal field
            const unsigned long long frac =
                sh < 64 ? ((unsigned long long)(0x800000u | (u & 0x7fffffu)) << 29) >> sh : 0ull;
            hi = sgn | (uint32_t)(frac >> 32);
            lo = (uint32_t)frac;
        } else if (ed >= 0x7ff) {
            hi = sgn | 0x7ff00000u;
            lo = 0u;
        } else {
            hi = sgn | ((uint32_t)ed << 20) | ((u & 0x7fffffu) >> 3);
            lo = u << 29;
        }
    }
    return __hiloint2double((int)hi, (int)lo);
}

// double times 2^-k -> float by truncation on the bit pattern (for norms)
__device__ __forceinline__ float d2f_scaled(double d, int k)
{
    const uint32_t hi = (uint32_t)__double2hiint(d);
    const uint32_t lo = (uint32_t)__double2loint(d);
    const uint32_t sgn = hi & 0x80000000u;
    const int E = (int)((hi >> 20) & 0x7ffu);
    if (E == 0) return __uint_as_float(sgn);
    if (E == 0x7ff) return __uint_as_float(sgn | 0x7f800000u | ((hi & 0xfffffu) << 3));
    const int ef = E - 896 - k;
    if (ef <= 0) return __uint_as_float(sgn);
    if (ef >= 0xff) return __uint_as_float(sgn | 0x7f800000u);
    return __uint_as_float(sgn | ((uint32_t)ef << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
}

// a pair times 2^k as one double: two exact conversions and one FP64 add
__device__ __forceinline__ double pf_to_double_scaled(pf a, int k)
{
    return f2d_scaled(a.h, k) + f2d_scaled(a.l, k);
}

// df64.cuh -- double-float arithmetic for the plain path's pair gates.
//
// GB300 executes FP64 at ~1.6 fused multiply-adds per clock per SM and
// converts between double and float at the same rate, against ~117 FP32
// FMAs (measured).  A general 2 x 2 complex gate needs 8 FP64 multiply-adds
// per amplitude, so in FP64 it runs at a quarter of HBM bandwidth.  This
// header restates the update in double-float (DF) form on the FP32 and
// integer pipes:
//   * a double x becomes hi + lo, two floats, by integer field operations
//     and one integer-to-float conversion (no FP64 instruction): hi is x
//     rounded to 24 significant bits, lo the signed remainder rounded to 24,
//     so |x - (hi + lo)| <= 2^-48 |x|;
//   * products are exact through the FMA (Dekker's TwoProduct in its FMA
//     form: p = a b, e = fma(a, b, -p)) and sums through Knuth's TwoSum;
//     the dot product of four DF terms follows the compensated scheme of
//     Ogita, Rump and Oishi (Dot2, SIAM J. Sci. Comput. 26, 2005), with the
//     cross terms a_hi b_lo + a_lo b_hi added to the error sum;
//   * the DF result goes back to a double by field operations: the high
//     float's fields placed in the double, the low float scaled to the
//     double's unit and converted to an integer (rounded to nearest), added
//     to the bit pattern.
// Range: doubles with 2^-126 <= |x| < 2^128 keep 2^-48 relative precision
// down to |x| ~ 2^-74 (then the low part leaves the float range); smaller
// magnitudes become 0, an absolute error below 2^-126.
// The result of a gate is within a few 2^-48 of the FP64 result, relative to
// the largest term.
//
// The functions compile for the device and, for the CPU unit test of the
// field manipulations (tests/test_df64.py), for the host.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define QG_DF_HD __host__ __device__ __forceinline__
#else
#define QG_DF_HD inline
#endif

namespace qg {
namespace df {

QG_DF_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}
QG_DF_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}
QG_DF_HD void d2words(double d, uint32_t& hi, uint32_t& lo) {
#if defined(__CUDA_ARCH__)
    hi = (uint32_t)__double2hiint(d);
    lo = (uint32_t)__double2loint(d);
#else
    uint64_t u;
    memcpy(&u, &d, 8);
    hi = (uint32_t)(u >> 32);
    lo = (uint32_t)u;
#endif
}
QG_DF_HD double words2d(uint32_t hi, uint32_t lo) {
#if defined(__CUDA_ARCH__)
    return __hiloint2double((int)hi, (int)lo);
#else
    const uint64_t u = ((uint64_t)hi << 32) | lo;
    double d;
    memcpy(&d, &u, 8);
    return d;
#endif
}
QG_DF_HD float fmaF(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return __builtin_fmaf(a, b, c);
#endif
}

// Products and sums that must stay rounded as written: the compiler would
// otherwise contract p + a * b into one FMA, which breaks the error-free
// transformations below
QG_DF_HD float mulR(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
QG_DF_HD float addR(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
QG_DF_HD float subR(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}

struct F2 {
    float h, l;
};

QG_DF_HD float i2f(int32_t v) {
#if defined(__CUDA_ARCH__)
    return __int2float_rn(v);
#else
    return (float)v;
#endif
}

// double -> hi + lo (integer field operations and one integer-to-float
// conversion; no FP64 instruction): hi is x rounded to 24 significant bits,
// lo the signed remainder (at most 29 bits) rounded to 24
QG_DF_HD F2 fromDouble(double x) {
    uint32_t hi, lo;
    d2words(x, hi, lo);
    const uint32_t ex = hi & 0x7FF00000u;                // biased exponent << 20
    const uint32_t sign = hi & 0x80000000u;
    // round the 52-bit fraction at bit 29 (a carry may reach the exponent)
    const uint32_t lo2 = lo + (1u << 28);
    const uint32_t hi2 = hi + (lo2 < lo ? 1u : 0u);
    // (hi2, lo2) << 3: the exponent's low 9 bits at 23..31 and the top 23
    // fraction bits below; rebiasing by 896 = 1023 - 127 is the same modulo
    // 2^9 for every exponent of the float range
    const uint32_t fs = (hi2 << 3) | (lo2 >> 29);
    const uint32_t hb = ((fs - (896u << 23)) & 0x7FFFFFFFu) | sign;
    // the remainder x - hi in units of 2^(E - 52): the low 29 fraction bits
    // as a signed 29-bit number (negative when hi was rounded up)
    const int32_t r = (int32_t)(lo << 3) >> 3;
    // 2^(E - 52) as a float: (e - 948) << 23 from the original exponent
    // (modulo 2^32, as above)
    const uint32_t scale = (ex << 3) - (948u << 23);
    const float l = mulR(i2f(r), u2f(scale));
    F2 f;
    f.h = ex >= (897u << 20) ? u2f(hb) : u2f(sign);     // |x| < 2^-126: 0
    f.l = ex >= (949u << 20) ? u2f(f2u(l) ^ sign) : 0.f;   // remainder below the float range: 0
    return f;
}

QG_DF_HD int32_t f2iRn(float f) {
#if defined(__CUDA_ARCH__)
    return __float2int_rn(f);
#else
    return (int32_t)__builtin_lrintf(f);
#endif
}

// hi + lo (|lo| below one ulp of hi, as fromDouble and dot4 give) ->
// double, rounded to nearest: the high float's fields placed in the double,
// then lo, scaled to units of the double's last place 2^(Eh - 52) by an
// exact power-of-two product and converted to an integer, added to the
// magnitude's bit pattern (|lo| < 2^29 units)
QG_DF_HD double toDouble(F2 v) {
    const uint32_t fh = f2u(v.h);
    const uint32_t ah = fh & 0x7FFFFFFFu, sh = fh & 0x80000000u;
    const uint32_t hi = ((ah >> 3) + (896u << 20)) | sh;
    const uint32_t lo = fh << 29;
    // lo against the magnitude: its sign flipped when hi is negative
    const float lm = u2f(f2u(v.l) ^ sh);
    // subtracting from a power of two crosses into the binade below, whose
    // unit is half as large: scale by 2^(53 - Eh) instead of 2^(52 - Eh)
    const bool down = (ah & 0x7FFFFFu) == 0u && lm < 0.f;
    const uint32_t scaleBits = ((down ? 307u : 306u) << 23) - (ah & 0x7F800000u);
    const int32_t d = f2iRn(mulR(lm, u2f(scaleBits)));
    const uint64_t w = (((uint64_t)hi << 32) | lo) + (uint64_t)(int64_t)d;
    // hi below 2^-75 (its unit would leave the float range) or zero: hi alone
    if (ah < (52u << 23)) return ah < 0x00800000u ? words2d(sh, 0u) : words2d(hi, lo);
    return words2d((uint32_t)(w >> 32), (uint32_t)w);
}

// Knuth's TwoSum: s + err = a + b exactly
QG_DF_HD void twoSum(float a, float b, float& s, float& err) {
    s = addR(a, b);
    const float bb = subR(s, a);
    err = addR(subR(a, subR(s, bb)), subR(b, bb));
}

// sum_k c_k x_k over four DF terms, as a DF result (Dot2 with the cross
// terms): the high products are summed by TwoSum, their rounding errors,
// the products' FMA errors and the cross terms go to the error sum
QG_DF_HD F2 dot4(const F2 c[4], const F2 x[4]) {
    float p = mulR(c[0].h, x[0].h);
    float s = fmaF(c[0].h, x[0].h, -p);
    s = fmaF(c[0].h, x[0].l, s);
    s = fmaF(c[0].l, x[0].h, s);
#pragma unroll
    for (int k = 1; k < 4; ++k) {
        const float h = mulR(c[k].h, x[k].h);
        const float r = fmaF(c[k].h, x[k].h, -h);
        float q;
        twoSum(p, h, p, q);
        s = fmaF(c[k].h, x[k].l, s);
        s = fmaF(c[k].l, x[k].h, s);
        s = addR(s, addR(q, r));
    }
    F2 out;
    twoSum(p, s, out.h, out.l);                         // |s| may exceed |p| when the terms cancel
    return out;
}

// a double as a DF constant (host side: exact split by rounding)
inline F2 splitConst(double c) {
    F2 r;
    r.h = (float)c;
    r.l = (float)(c - (double)r.h);
    return r;
}

}  // namespace df
}  // namespace qg

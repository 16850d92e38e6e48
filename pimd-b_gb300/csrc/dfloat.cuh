// Double-float ("double-word") arithmetic on the FP32 pipe.
//
// GB300 issues FP32 operations at 64 times its FP64 rate.  A value held as
// an unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2) carries 48
// significant bits, and the error-free transformations below keep sums and
// products of such values within a few units of 2^-48 relative, using FP32
// operations only.  The algorithms are the published ones:
//   two_sum        Knuth, TAOCP vol. 2 (6 operations, exact);
//   fast_two_sum   Dekker 1971, for |a| >= |b| (3 operations, exact);
//   two_prod       with a fused multiply-add (2 operations, exact);
//   add, add_sloppy, mul, mul_f: Joldes, Muller and Popescu, "Tight and
//   rigorous error bounds for basic building blocks of double-word
//   arithmetic", ACM TOMS 44(2), 2017 (AccurateDWPlusDW, relative error
//   below 3u^2; SloppyDWPlusDW, absolute error below a few u^2 (|x| + |y|);
//   DWTimesDW with FMA, below 5u^2; DWTimesFP, below 2u^2; u = 2^-24).
// Every operation is rounded to nearest with explicit intrinsics on the
// device, so the compiler's contraction of a*b+c never changes an
// error-free step.  The functions also compile for the host (used by the
// unit test of this arithmetic), where float operations round to nearest
// and fmaf is the correctly rounded fused multiply-add.
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD inline
#endif

namespace pimdb {
namespace dfl {

struct df {
    float hi, lo;
};

#if defined(__CUDA_ARCH__)
DF_HD float add_rn(float a, float b) { return __fadd_rn(a, b); }
DF_HD float sub_rn(float a, float b) { return __fsub_rn(a, b); }
DF_HD float mul_rn(float a, float b) { return __fmul_rn(a, b); }
DF_HD float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
DF_HD float bits_to_float(int b) { return __int_as_float(b); }
DF_HD int float_to_bits(float f) { return __float_as_int(f); }
DF_HD float rsqrt_approx(float x) { return rsqrtf(x); }
DF_HD float log_approx(float x) { return logf(x); }
#else
DF_HD float add_rn(float a, float b) { return a + b; }
DF_HD float sub_rn(float a, float b) { return a - b; }
DF_HD float mul_rn(float a, float b) { return a * b; }
DF_HD float fma_rn(float a, float b, float c) { return fmaf(a, b, c); }
DF_HD float bits_to_float(int b) {
    float f;
    __builtin_memcpy(&f, &b, 4);
    return f;
}
DF_HD int float_to_bits(float f) {
    int b;
    __builtin_memcpy(&b, &f, 4);
    return b;
}
DF_HD float rsqrt_approx(float x) { return 1.0f / sqrtf(x); }
DF_HD float log_approx(float x) { return logf(x); }
#endif

DF_HD df two_sum(float a, float b) {
    const float s = add_rn(a, b);
    const float bb = sub_rn(s, a);
    const float e = add_rn(sub_rn(a, sub_rn(s, bb)), sub_rn(b, bb));
    return {s, e};
}
DF_HD df fast_two_sum(float a, float b) {
    const float s = add_rn(a, b);
    return {s, sub_rn(b, sub_rn(s, a))};
}
DF_HD df two_prod(float a, float b) {
    const float p = mul_rn(a, b);
    return {p, fma_rn(a, b, -p)};
}
DF_HD df neg(df a) { return {-a.hi, -a.lo}; }

// AccurateDWPlusDW: relative error below 3u^2 whatever the signs.
DF_HD df add(df x, df y) {
    const df s = two_sum(x.hi, y.hi);
    const df t = two_sum(x.lo, y.lo);
    const float c = add_rn(s.lo, t.hi);
    const df v = fast_two_sum(s.hi, c);
    const float w = add_rn(t.lo, v.lo);
    return fast_two_sum(v.hi, w);
}
// SloppyDWPlusDW: absolute error of a few u^2 (|x| + |y|); the relative
// error is unbounded when x and y cancel, so it serves running sums whose
// error counts against the summands, not against the result.
DF_HD df add_sloppy(df x, df y) {
    const df s = two_sum(x.hi, y.hi);
    const float v = add_rn(x.lo, y.lo);
    const float w = add_rn(s.lo, v);
    return fast_two_sum(s.hi, w);
}
// DWPlusFP: x + y with y a float (relative error below 2u^2).
DF_HD df add_f(df x, float y) {
    const df s = two_sum(x.hi, y);
    const float v = add_rn(x.lo, s.lo);
    return fast_two_sum(s.hi, v);
}
// DWTimesDW with FMA: relative error below 5u^2.
DF_HD df mul(df x, df y) {
    const df c = two_prod(x.hi, y.hi);
    const float tl0 = mul_rn(x.lo, y.lo);
    const float tl1 = fma_rn(x.hi, y.lo, tl0);
    const float cl2 = fma_rn(x.lo, y.hi, tl1);
    const float cl3 = add_rn(c.lo, cl2);
    return fast_two_sum(c.hi, cl3);
}
// DWTimesFP with FMA: relative error below 2u^2.
DF_HD df mul_f(df x, float y) {
    const df c = two_prod(x.hi, y);
    const float cl3 = fma_rn(x.lo, y, c.lo);
    return fast_two_sum(c.hi, cl3);
}
// x^2 (a mul with the cross term doubled).
DF_HD df sqr(df x) {
    const df c = two_prod(x.hi, x.hi);
    const float cl = fma_rn(add_rn(x.hi, x.hi), x.lo, c.lo);
    return fast_two_sum(c.hi, cl);
}

// 1/sqrt(x) for x > 0 whose float image is a normal number: from a seed y0
// of rsqrt(hi) (relative error e0; the hardware's is a few 2^-24), one
// Newton step with the
// second-order term, y = y0 + y0 (e/2 + 3e^2/8), e = 1 - x y0^2 formed
// in double-float (x y0^2 = 1 - e cancels, so e is exact to about u^2).
// Relative error of order e0^3 + u^2.
DF_HD df rsqrt_from(df x, float y0) {
    const df xy = mul_f(x, y0);
    const df xyy = mul_f(xy, y0);
    const float e = sub_rn(sub_rn(1.0f, xyy.hi), xyy.lo);  // 1 - xyy.hi is exact (Sterbenz)
    const float corr = mul_rn(y0, mul_rn(e, fma_rn(e, 0.375f, 0.5f)));
    return fast_two_sum(y0, corr);
}
DF_HD df rsqrt(df x) { return rsqrt_from(x, rsqrt_approx(x.hi)); }

// Double-float image of a double (hi = nearest float, lo = nearest float of
// the remainder): 48 of the 53 bits.
DF_HD df from_double(double v) {
    const float h = (float)v;
    return {h, (float)(v - (double)h)};
}
DF_HD double to_double(df a) { return (double)a.hi + (double)a.lo; }

// exp(x) for a double-float x with x.hi in [-87, 87]: Tang's table-driven
// reduction (P. T. P. Tang, ACM TOMS 15(2), 1989) with 256 table entries,
// x = (256 m + j) ln2/256 + t, |t| <= ln2/512, exp(x) = 2^m 2^(j/256) exp(t),
// exp(t) - 1 = t + t^2/2 + t^3/6 + t^4/24 (remainder below 4e-17).
// ln2/256 = L1 + L2 + L3 with L1 of 12 significant bits: for |x| < 88
// (|n| < 2^15) the exact x.hi - n L1 needs at most 24 bits, so the fused
// multiply-add that forms it does not round; n L2 is split exactly by
// two_prod.  `tbl` holds 2^(j/256) as double-floats (hi[256], lo[256]).
// Relative error a few u^2 plus the propagation of x's own error for
// x >= -69 (results above 2^-100); below that the low word turns subnormal
// and the relative error grows to 1e-11 at x = -80 and 1e-8 at x = -87.
// Results whose exponent falls below the normal float range return 0.
struct ExpTable {
    float hi[256], lo[256];
};
constexpr float kLn2_256_1 = 0x1.62ep-9f;      // 12 significant bits (2839 * 2^-20)
constexpr float kLn2_256_2 = 0x1.0bfbe8p-23f;  // the next 24 bits
constexpr float kLn2_256_3 = 0x1.cf79acp-48f;  // the remainder (sum within 5e-23 of ln2/256)
constexpr float kInvLn2_256 = 369.32992553710938f;  // 256 / ln2 rounded to float

constexpr float kRoundShift = 12582912.0f;  // 1.5 * 2^23: adding it rounds |v| < 2^22 to an integer

DF_HD df exp(df x, const ExpTable& tbl) {
    // outside [-88, 88] the result is below the normal range (0) or
    // overflows; NaN passes through
    if (x.hi < -88.0f) return {0.0f, 0.0f};
    if (!(x.hi <= 88.0f)) return {x.hi * 3.0e38f, 0.0f};  // +inf, or NaN
    // n = round(x.hi 256/ln2) by the shifter: the sum's low mantissa bits
    // hold n, and no rounding or float-to-integer instruction is issued
    // (those run on the FP64/conversion pipe on this GPU)
    const float tsh = fma_rn(x.hi, kInvLn2_256, kRoundShift);
    const int n = float_to_bits(tsh) - float_to_bits(kRoundShift);
    const float nf = sub_rn(tsh, kRoundShift);
    // t = x - n ln2/256, in double-float
    const float r1 = fma_rn(-nf, kLn2_256_1, x.hi);      // exact: n L1 has <= 24 bits, r1 ~ x.hi - n L1 (Sterbenz)
    const df p2 = two_prod(nf, kLn2_256_2);              // n L2 exactly
    const df t0 = two_sum(r1, -p2.hi);
    // x.lo (up to ulp(x.hi)/2, far above t's low word) joins exactly
    const df t1 = two_sum(t0.hi, x.lo);
    const float tl = add_rn(add_rn(t1.lo, t0.lo), fma_rn(-nf, kLn2_256_3, -p2.lo));
    const df t = fast_two_sum(t1.hi, tl);
    // exp(t) - 1 = t + t^2/2 + (t^3/6 + t^4/24)
    const df q = sqr(t);
    const float small = mul_rn(q.hi, fma_rn(q.hi, 1.0f / 24.0f, mul_rn(t.hi, 1.0f / 6.0f)));
    df pm = add_sloppy(t, {mul_rn(q.hi, 0.5f), mul_rn(q.lo, 0.5f)});
    pm = add_f(pm, small);
    // 1 + pm, then the table entry
    const df one_p = add_f(fast_two_sum(1.0f, pm.hi), pm.lo);
    const int j = n & 255;
    const df y = mul(one_p, df{tbl.hi[j], tbl.lo[j]});
    const int m = n >> 8;  // floor division by 256
    if (m < -126) return {0.0f, 0.0f};
    const float sc = bits_to_float((m + 127) << 23);  // 2^m, a normal float for m in [-126, 127]
    return {mul_rn(y.hi, sc), mul_rn(y.lo, sc)};
}

// log(y) for a double-float y with y.hi in [1e-30, 1e30]: x0 = logf(y.hi)
// on the FP32 pipe (a few float ulps), r = y exp(-x0) - 1 (|r| < 2^-16),
// log y = x0 + r - r^2/2 + r^3/3 (the next term is below 2^-64).  About
// 2^-46 absolute plus 2^-46 relative.
DF_HD df log(df y, const ExpTable& tbl) {
    const float x0 = log_approx(y.hi);
    const df r = add_f(mul(y, exp(df{-x0, 0.0f}, tbl)), -1.0f);
    const df lp = add_f(r, mul_rn(mul_rn(r.hi, r.hi), fma_rn(r.hi, 1.0f / 3.0f, -0.5f)));
    return add(df{x0, 0.0f}, lp);
}

}  // namespace dfl
}  // namespace pimdb

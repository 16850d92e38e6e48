// Pair and external potential gradients on the device, shared by the
// one-system force kernels (forces.cu) and the batched-replica kernel
// (batch.cu).  Reference: the potentials' gradV
// (src/potentials/{harmonic,aziz,dipole,double_well,cosine}.cpp).
#pragma once

#include "common.cuh"

namespace pimdb {

// Aziz HFDHE2 (reference aziz.cpp:6-13, aziz.h:25-34).
struct Aziz {
    static constexpr double rm = 5.60738, A = 0.5448504e6, eps = 3.42016E-5, alpha = 13.353384, D = 1.241314,
                            C6 = 1.3732412, C8 = 0.4253785, C10 = 0.1781;
};

// exp(x) by Tang's table-driven method (P. T. P. Tang, "Table-driven
// implementation of the exponential function in IEEE floating-point
// arithmetic", ACM TOMS 15(2), 1989): x = (32 m + j) ln2/32 + r with
// |r| <= ln2/64, exp(x) = 2^m 2^(j/32) exp(r), exp(r) - 1 by its Taylor
// polynomial to degree 6 (remainder below 4e-18).  n = 32 m + j comes from
// the round-to-nearest of x 32/ln2 (the 1.5 * 2^52 shift); ln2/32 is split
// into L1 (low 17 bits clear, so n L1 is exact for |n| < 2^17) and L2.
// `tbl` holds 2^(j/32), j = 0..31, rounded to double (kExp2Table; shared
// memory, so lanes with different j do not serialise).  Valid for
// x < 709; results below 2^-1010 (x < -700) are returned as 0.  Measured on
// GB300: within one ulp of CUDA's exp on [-745, 5] and 1.34x its
// throughput (11 FP64 operations).
static __constant__ double kExp2Table[32] = {
    0x1.0000000000000p+0, 0x1.059b0d3158574p+0, 0x1.0b5586cf9890fp+0, 0x1.11301d0125b51p+0,
    0x1.172b83c7d517bp+0, 0x1.1d4873168b9aap+0, 0x1.2387a6e756238p+0, 0x1.29e9df51fdee1p+0,
    0x1.306fe0a31b715p+0, 0x1.371a7373aa9cbp+0, 0x1.3dea64c123422p+0, 0x1.44e086061892dp+0,
    0x1.4bfdad5362a27p+0, 0x1.5342b569d4f82p+0, 0x1.5ab07dd485429p+0, 0x1.6247eb03a5585p+0,
    0x1.6a09e667f3bcdp+0, 0x1.71f75e8ec5f74p+0, 0x1.7a11473eb0187p+0, 0x1.82589994cce13p+0,
    0x1.8ace5422aa0dbp+0, 0x1.93737b0cdc5e5p+0, 0x1.9c49182a3f090p+0, 0x1.a5503b23e255dp+0,
    0x1.ae89f995ad3adp+0, 0x1.b7f76f2fb5e47p+0, 0x1.c199bdd85529cp+0, 0x1.cb720dcef9069p+0,
    0x1.d5818dcfba487p+0, 0x1.dfc97337b9b5fp+0, 0x1.ea4afa2a490dap+0, 0x1.f50765b6e4540p+0};

__device__ __forceinline__ double exp_tang(double x, const double* tbl) {
    const double shifter = 6755399441055744.0;  // 1.5 * 2^52
    const double t = fma(x, 46.16624130844683, shifter);  // 32 / ln2
    const int n = __double2loint(t);
    const double nd = t - shifter;
    double r = fma(nd, -0.021660849392446835, x);  // L1
    r = fma(nd, -5.145609244655338e-14, r);        // L2
    double q = fma(r, 1.0 / 720.0, 1.0 / 120.0);
    q = fma(q, r, 1.0 / 24.0);
    q = fma(q, r, 1.0 / 6.0);
    q = fma(q, r, 0.5);
    const double p = fma(r * r, q, r);
    const double tj = tbl[n & 31];
    const double y = fma(tj, p, tj);
    const int hi = __double2hiint(y) + ((n >> 5) << 20);
    return n < -32318 ? 0.0 : __hiloint2double(hi, __double2loint(y));
}

// grad V(r) = s(r) * r for the radial pair potentials.  `r2` is |r|^2.
template <typename R>
__device__ __forceinline__ R pair_scale(int kind, R r2, R param);

// FP64 gradient scale; with `tbl` the exponentials use exp_tang.
template <bool kTang>
__device__ __forceinline__ double pair_scale_d(int kind, double r2, double param, const double* tbl) {
    auto ex = [&](double v) { return kTang ? exp_tang(v, tbl) : exp(v); };
    if (kind == POT_HARMONIC) return param;  // harmonic.cpp:21-23, k = m w^2
    // one reciprocal square root serves |r|, 1/r_scaled and the final 1/|r|
    const double rinv = rsqrt(r2);
    if (kind == POT_DIPOLE) {  // dipole.cpp:24-45: -3 D / |r|^5
        const double ri2 = rinv * rinv;
        return -3.0 * param * (ri2 * ri2 * rinv);
    }
    // POT_AZIZ, aziz.cpp:56-106 (same terms, factored)
    const double norm = r2 * rinv;
    const double rs = norm * (1.0 / Aziz::rm);
    const double T1 = -Aziz::A * Aziz::alpha * ex(-Aziz::alpha * rs);
    double g;
    if (rs > 1.0E-7 && rs < 0.01) {
        g = T1 * (Aziz::eps / Aziz::rm);
    } else {
        const double ix = Aziz::rm * rinv;  // 1 / r_scaled
        const double ix2 = ix * ix;
        const double ix6 = ix2 * ix2 * ix2;
        double tail = 0.0;
        if (rs < Aziz::D) {
            // T2 + T3 = F(rs) [ix^7 (6 C6 + 8 C8 ix^2 + 10 C10 ix^4)
            //                  - 2 D ix^2 (D ix - 1) ix^6 (C6 + C8 ix^2 + C10 ix^4)]
            const double t = Aziz::D * ix - 1.0;
            const double e = ex(-t * t);
            const double pa = fma(fma(10.0 * Aziz::C10, ix2, 8.0 * Aziz::C8), ix2, 6.0 * Aziz::C6);
            const double pb = fma(fma(Aziz::C10, ix2, Aziz::C8), ix2, Aziz::C6);
            tail = e * ix6 * (ix * pa - 2.0 * Aziz::D * ix2 * t * pb);
        } else {
            const double pa = fma(fma(10.0 * Aziz::C10, ix2, 8.0 * Aziz::C8), ix2, 6.0 * Aziz::C6);
            tail = ix6 * ix * pa;  // F = 1, dF = 0
        }
        g = (Aziz::eps / Aziz::rm) * (T1 + tail);
    }
    return g * rinv;
}

template <>
__device__ __forceinline__ double pair_scale<double>(int kind, double r2, double param) {
    return pair_scale_d<false>(kind, r2, param, nullptr);
}

// ln(A alpha eps / r_m) of the Aziz parameters above (aziz.cpp:6-13).
constexpr double kAzizLnK = 3.7927146577859623;

// Aziz gradient scale outside the damping radius (r_s >= D, where F = 1 and
// dF = 0): (eps/r_m) [-A alpha exp(-alpha r_s) + ix^7 (6 C6 + 8 C8 ix^2 +
// 10 C10 ix^4)] / |r|, with the prefactors folded into the exponent and the
// polynomial.  Branch-free; the caller checks r_s >= D (aziz_is_far) and
// uses pair_scale_d otherwise.
__device__ __forceinline__ double aziz_far_scale(double r2, const double* tbl) {
    constexpr double k = Aziz::eps / Aziz::rm;
    const double rinv = rsqrt(r2);
    const double norm = r2 * rinv;
    const double e = exp_tang(fma(-(Aziz::alpha / Aziz::rm), norm, kAzizLnK), tbl);
    const double ix = Aziz::rm * rinv;
    const double ix2 = ix * ix;
    const double ix7 = ix2 * ix2 * ix2 * ix;
    const double pa = fma(fma(10.0 * Aziz::C10 * k, ix2, 8.0 * Aziz::C8 * k), ix2, 6.0 * Aziz::C6 * k);
    return fma(ix7, pa, -e) * rinv;
}
// r_s = |r| / r_m >= D, on r2 = |r|^2
__device__ __forceinline__ bool aziz_is_far(double r2) {
    return r2 >= (Aziz::D * Aziz::rm) * (Aziz::D * Aziz::rm);
}

template <>
__device__ __forceinline__ float pair_scale<float>(int kind, float r2, float param) {
    if (kind == POT_HARMONIC) return param;
    const float rinv = rsqrtf(r2);
    if (kind == POT_DIPOLE) {
        const float ri2 = rinv * rinv;
        return -3.0f * param * ri2 * ri2 * rinv;
    }
    const float norm = r2 * rinv;
    const float rs = norm * (float)(1.0 / Aziz::rm);
    const float T1 = (float)(-Aziz::A * Aziz::alpha) * expf(-(float)Aziz::alpha * rs);
    float g;
    if (rs > 1.0E-7f && rs < 0.01f) {
        g = T1 * (float)(Aziz::eps / Aziz::rm);
    } else {
        const float ix = (float)Aziz::rm * rinv;
        const float ix2 = ix * ix;
        const float ix6 = ix2 * ix2 * ix2;
        const float ix7 = ix6 * ix, ix8 = ix6 * ix2, ix9 = ix8 * ix, ix10 = ix8 * ix2, ix11 = ix10 * ix;
        float F = 1.0f, dF = 0.0f;
        if (rs < (float)Aziz::D) {
            const float t = (float)Aziz::D * ix - 1.0f;
            const float e = expf(-t * t);
            F = e;
            dF = 2.0f * (float)Aziz::D * ix2 * t * e;
        }
        const float T2 = ((float)(6.0 * Aziz::C6) * ix7 + (float)(8.0 * Aziz::C8) * ix9 +
                          (float)(10.0 * Aziz::C10) * ix11) * F;
        const float T3 = -((float)Aziz::C6 * ix6 + (float)Aziz::C8 * ix8 + (float)Aziz::C10 * ix10) * dF;
        g = (float)(Aziz::eps / Aziz::rm) * (T1 + T2 + T3);
    }
    return g * rinv;
}

// -grad V_ext for one particle (double_well.cpp:22-40, cosine.cpp:23-35,
// harmonic.cpp:21-23).
template <int D>
__device__ __forceinline__ void ext_force(const Sys& s, const double* xi, double* out) {
    if (s.ext_kind == POT_HARMONIC) {
#pragma unroll
        for (int a = 0; a < D; ++a) out[a] = -(xi[a] * s.ext_a);
    } else if (s.ext_kind == POT_DOUBLE_WELL) {
        double r2 = 0.0;
#pragma unroll
        for (int a = 0; a < D; ++a) r2 += xi[a] * xi[a];
        const double pre = s.ext_a * (r2 - s.ext_b);
#pragma unroll
        for (int a = 0; a < D; ++a) out[a] = -(pre * xi[a]);
    } else if (s.ext_kind == POT_COSINE) {
#pragma unroll
        for (int a = 0; a < D; ++a) out[a] = -(s.ext_a * sin(s.ext_b * xi[a] + s.ext_c));
    } else {
#pragma unroll
        for (int a = 0; a < D; ++a) out[a] = 0.0;
    }
}

// Pair potential V(r) of one separation (`r2` = |r|^2), the reference's
// V() for one distance vector: harmonic.cpp:7-19 (1/2 k r^2), dipole.cpp:5-20
// (D / r^3), aziz.cpp:18-54 with F of aziz.h:25-27.
__device__ inline double pair_value(int kind, double r2, double param) {
    if (kind == POT_HARMONIC) return 0.5 * param * r2;
    const double r = sqrt(r2);
    if (kind == POT_DIPOLE) return param / (r * r * r);
    if (kind != POT_AZIZ) return 0.0;
    const double rs = r / Aziz::rm;
    const double urep = Aziz::A * exp(-Aziz::alpha * rs);
    if (rs > 1.0E-7 && rs < 0.01) return Aziz::eps * urep;
    const double ix2 = 1.0 / (rs * rs);
    const double ix6 = ix2 * ix2 * ix2;
    const double ix8 = ix6 * ix2;
    const double ix10 = ix8 * ix2;
    const double t = Aziz::D / rs - 1.0;
    const double F = rs < Aziz::D ? exp(-t * t) : 1.0;
    const double uatt = -(Aziz::C6 * ix6 + Aziz::C8 * ix8 + Aziz::C10 * ix10) * F;
    return Aziz::eps * (urep + uatt);
}

// External potential of one particle: harmonic.cpp:7-19 (1/2 k |x|^2),
// double_well.cpp:6-20 (m s sum_a (x_a^2 - loc^2)^2), cosine.cpp:9-21
// (A sum_a cos(k x_a + phase)).  Sys holds ext_a = m w^2 | 4 m s | -A k,
// ext_b = - | loc^2 | k, ext_c = - | m s | phase.
template <int D>
__device__ __forceinline__ double ext_value(const Sys& s, const double* xi) {
    double v = 0.0;
    if (s.ext_kind == POT_HARMONIC) {
#pragma unroll
        for (int a = 0; a < D; ++a) v += xi[a] * xi[a];
        return 0.5 * s.ext_a * v;
    }
    if (s.ext_kind == POT_DOUBLE_WELL) {
#pragma unroll
        for (int a = 0; a < D; ++a) v += (xi[a] * xi[a] - s.ext_b) * (xi[a] * xi[a] - s.ext_b);
        return s.ext_c * v;
    }
    if (s.ext_kind == POT_COSINE) {
#pragma unroll
        for (int a = 0; a < D; ++a) v += cos(s.ext_b * xi[a] + s.ext_c);
        return (-s.ext_a / s.ext_b) * v;
    }
    return 0.0;
}

}  // namespace pimdb

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

// grad V(r) = s(r) * r for the radial pair potentials.  `r2` is |r|^2.
template <typename R>
__device__ __forceinline__ R pair_scale(int kind, R r2, R param);

template <>
__device__ __forceinline__ double pair_scale<double>(int kind, double r2, double param) {
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
    const double T1 = -Aziz::A * Aziz::alpha * exp(-Aziz::alpha * rs);
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
            const double e = exp(-t * t);
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

// Pair and external potential gradients on the device, shared by the
// one-system force kernels (forces.cu) and the batched-replica kernel
// (batch.cu).  Reference: the potentials' gradV
// (src/potentials/{harmonic,aziz,dipole,double_well,cosine}.cpp).
#pragma once

#include "aziz_df.cuh"
#include "common.cuh"

namespace pimdb {

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
    // the result would be returned as 0 below: skip the polynomial (most of
    // a large system's exchange weights land here)
    if (n < -32318) return 0.0;
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
    return __hiloint2double(hi, __double2loint(y));
}

// The same method with a 256-entry table (kExp2Table256: 2^(j/256), j =
// 0..255, correctly rounded): |r| <= ln2/512, so the Taylor polynomial of
// exp(r) - 1 stops at degree 4 (remainder below 4e-17 relative) and the
// evaluation costs 9 FP64 operations instead of 11.  ln2/256 = L1 + L2 with
// L1 of 30 significant bits (n L1 exact for |n| < 2^23).  Valid for x < 709;
// results below 2^-1010 are returned as 0.
static __constant__ double kExp2Table256[256] = {
    0x1.0000000000000p+0, 0x1.00b1afa5abcbfp+0, 0x1.0163da9fb3335p+0, 0x1.02168143b0281p+0,
    0x1.02c9a3e778061p+0, 0x1.037d42e11bbccp+0, 0x1.04315e86e7f85p+0, 0x1.04e5f72f654b1p+0,
    0x1.059b0d3158574p+0, 0x1.0650a0e3c1f89p+0, 0x1.0706b29ddf6dep+0, 0x1.07bd42b72a836p+0,
    0x1.0874518759bc8p+0, 0x1.092bdf66607e0p+0, 0x1.09e3ecac6f383p+0, 0x1.0a9c79b1f3919p+0,
    0x1.0b5586cf9890fp+0, 0x1.0c0f145e46c85p+0, 0x1.0cc922b7247f7p+0, 0x1.0d83b23395decp+0,
    0x1.0e3ec32d3d1a2p+0, 0x1.0efa55fdfa9c5p+0, 0x1.0fb66affed31bp+0, 0x1.1073028d7233ep+0,
    0x1.11301d0125b51p+0, 0x1.11edbab5e2ab6p+0, 0x1.12abdc06c31ccp+0, 0x1.136a814f204abp+0,
    0x1.1429aaea92de0p+0, 0x1.14e95934f312ep+0, 0x1.15a98c8a58e51p+0, 0x1.166a45471c3c2p+0,
    0x1.172b83c7d517bp+0, 0x1.17ed48695bbc0p+0, 0x1.18af9388c8deap+0, 0x1.1972658375d2fp+0,
    0x1.1a35beb6fcb75p+0, 0x1.1af99f8138a1cp+0, 0x1.1bbe084045cd4p+0, 0x1.1c82f95281c6bp+0,
    0x1.1d4873168b9aap+0, 0x1.1e0e75eb44027p+0, 0x1.1ed5022fcd91dp+0, 0x1.1f9c18438ce4dp+0,
    0x1.2063b88628cd6p+0, 0x1.212be3578a819p+0, 0x1.21f49917ddc96p+0, 0x1.22bdda27912d1p+0,
    0x1.2387a6e756238p+0, 0x1.2451ffb82140ap+0, 0x1.251ce4fb2a63fp+0, 0x1.25e85711ece75p+0,
    0x1.26b4565e27cddp+0, 0x1.2780e341ddf29p+0, 0x1.284dfe1f56381p+0, 0x1.291ba7591bb70p+0,
    0x1.29e9df51fdee1p+0, 0x1.2ab8a66d10f13p+0, 0x1.2b87fd0dad990p+0, 0x1.2c57e39771b2fp+0,
    0x1.2d285a6e4030bp+0, 0x1.2df961f641589p+0, 0x1.2ecafa93e2f56p+0, 0x1.2f9d24abd886bp+0,
    0x1.306fe0a31b715p+0, 0x1.31432edeeb2fdp+0, 0x1.32170fc4cd831p+0, 0x1.32eb83ba8ea32p+0,
    0x1.33c08b26416ffp+0, 0x1.3496266e3fa2dp+0, 0x1.356c55f929ff1p+0, 0x1.36431a2de883bp+0,
    0x1.371a7373aa9cbp+0, 0x1.37f26231e754ap+0, 0x1.38cae6d05d866p+0, 0x1.39a401b7140efp+0,
    0x1.3a7db34e59ff7p+0, 0x1.3b57fbfec6cf4p+0, 0x1.3c32dc313a8e5p+0, 0x1.3d0e544ede173p+0,
    0x1.3dea64c123422p+0, 0x1.3ec70df1c5175p+0, 0x1.3fa4504ac801cp+0, 0x1.40822c367a024p+0,
    0x1.4160a21f72e2ap+0, 0x1.423fb2709468ap+0, 0x1.431f5d950a897p+0, 0x1.43ffa3f84b9d4p+0,
    0x1.44e086061892dp+0, 0x1.45c2042a7d232p+0, 0x1.46a41ed1d0057p+0, 0x1.4786d668b3237p+0,
    0x1.486a2b5c13cd0p+0, 0x1.494e1e192aed2p+0, 0x1.4a32af0d7d3dep+0, 0x1.4b17dea6db7d7p+0,
    0x1.4bfdad5362a27p+0, 0x1.4ce41b817c114p+0, 0x1.4dcb299fddd0dp+0, 0x1.4eb2d81d8abffp+0,
    0x1.4f9b2769d2ca7p+0, 0x1.508417f4531eep+0, 0x1.516daa2cf6642p+0, 0x1.5257de83f4eefp+0,
    0x1.5342b569d4f82p+0, 0x1.542e2f4f6ad27p+0, 0x1.551a4ca5d920fp+0, 0x1.56070dde910d2p+0,
    0x1.56f4736b527dap+0, 0x1.57e27dbe2c4cfp+0, 0x1.58d12d497c7fdp+0, 0x1.59c0827ff07ccp+0,
    0x1.5ab07dd485429p+0, 0x1.5ba11fba87a03p+0, 0x1.5c9268a5946b7p+0, 0x1.5d84590998b93p+0,
    0x1.5e76f15ad2148p+0, 0x1.5f6a320dceb71p+0, 0x1.605e1b976dc09p+0, 0x1.6152ae6cdf6f4p+0,
    0x1.6247eb03a5585p+0, 0x1.633dd1d1929fdp+0, 0x1.6434634ccc320p+0, 0x1.652b9febc8fb7p+0,
    0x1.6623882552225p+0, 0x1.671c1c70833f6p+0, 0x1.68155d44ca973p+0, 0x1.690f4b19e9538p+0,
    0x1.6a09e667f3bcdp+0, 0x1.6b052fa75173ep+0, 0x1.6c012750bdabfp+0, 0x1.6cfdcddd47645p+0,
    0x1.6dfb23c651a2fp+0, 0x1.6ef9298593ae5p+0, 0x1.6ff7df9519484p+0, 0x1.70f7466f42e87p+0,
    0x1.71f75e8ec5f74p+0, 0x1.72f8286ead08ap+0, 0x1.73f9a48a58174p+0, 0x1.74fbd35d7cbfdp+0,
    0x1.75feb564267c9p+0, 0x1.77024b1ab6e09p+0, 0x1.780694fde5d3fp+0, 0x1.790b938ac1cf6p+0,
    0x1.7a11473eb0187p+0, 0x1.7b17b0976cfdbp+0, 0x1.7c1ed0130c132p+0, 0x1.7d26a62ff86f0p+0,
    0x1.7e2f336cf4e62p+0, 0x1.7f3878491c491p+0, 0x1.80427543e1a12p+0, 0x1.814d2add106d9p+0,
    0x1.82589994cce13p+0, 0x1.8364c1eb941f7p+0, 0x1.8471a4623c7adp+0, 0x1.857f4179f5b21p+0,
    0x1.868d99b4492edp+0, 0x1.879cad931a436p+0, 0x1.88ac7d98a6699p+0, 0x1.89bd0a478580fp+0,
    0x1.8ace5422aa0dbp+0, 0x1.8be05bad61778p+0, 0x1.8cf3216b5448cp+0, 0x1.8e06a5e0866d9p+0,
    0x1.8f1ae99157736p+0, 0x1.902fed0282c8ap+0, 0x1.9145b0b91ffc6p+0, 0x1.925c353aa2fe2p+0,
    0x1.93737b0cdc5e5p+0, 0x1.948b82b5f98e5p+0, 0x1.95a44cbc8520fp+0, 0x1.96bdd9a7670b3p+0,
    0x1.97d829fde4e50p+0, 0x1.98f33e47a22a2p+0, 0x1.9a0f170ca07bap+0, 0x1.9b2bb4d53fe0dp+0,
    0x1.9c49182a3f090p+0, 0x1.9d674194bb8d5p+0, 0x1.9e86319e32323p+0, 0x1.9fa5e8d07f29ep+0,
    0x1.a0c667b5de565p+0, 0x1.a1e7aed8eb8bbp+0, 0x1.a309bec4a2d33p+0, 0x1.a42c980460ad8p+0,
    0x1.a5503b23e255dp+0, 0x1.a674a8af46052p+0, 0x1.a799e1330b358p+0, 0x1.a8bfe53c12e59p+0,
    0x1.a9e6b5579fdbfp+0, 0x1.ab0e521356ebap+0, 0x1.ac36bbfd3f37ap+0, 0x1.ad5ff3a3c2774p+0,
    0x1.ae89f995ad3adp+0, 0x1.afb4ce622f2ffp+0, 0x1.b0e07298db666p+0, 0x1.b20ce6c9a8952p+0,
    0x1.b33a2b84f15fbp+0, 0x1.b468415b749b1p+0, 0x1.b59728de5593ap+0, 0x1.b6c6e29f1c52ap+0,
    0x1.b7f76f2fb5e47p+0, 0x1.b928cf22749e4p+0, 0x1.ba5b030a1064ap+0, 0x1.bb8e0b79a6f1fp+0,
    0x1.bcc1e904bc1d2p+0, 0x1.bdf69c3f3a207p+0, 0x1.bf2c25bd71e09p+0, 0x1.c06286141b33dp+0,
    0x1.c199bdd85529cp+0, 0x1.c2d1cd9fa652cp+0, 0x1.c40ab5fffd07ap+0, 0x1.c544778fafb22p+0,
    0x1.c67f12e57d14bp+0, 0x1.c7ba88988c933p+0, 0x1.c8f6d9406e7b5p+0, 0x1.ca3405751c4dbp+0,
    0x1.cb720dcef9069p+0, 0x1.ccb0f2e6d1675p+0, 0x1.cdf0b555dc3fap+0, 0x1.cf3155b5bab74p+0,
    0x1.d072d4a07897cp+0, 0x1.d1b532b08c968p+0, 0x1.d2f87080d89f2p+0, 0x1.d43c8eacaa1d6p+0,
    0x1.d5818dcfba487p+0, 0x1.d6c76e862e6d3p+0, 0x1.d80e316c98398p+0, 0x1.d955d71ff6075p+0,
    0x1.da9e603db3285p+0, 0x1.dbe7cd63a8315p+0, 0x1.dd321f301b460p+0, 0x1.de7d5641c0658p+0,
    0x1.dfc97337b9b5fp+0, 0x1.e11676b197d17p+0, 0x1.e264614f5a129p+0, 0x1.e3b333b16ee12p+0,
    0x1.e502ee78b3ff6p+0, 0x1.e653924676d76p+0, 0x1.e7a51fbc74c83p+0, 0x1.e8f7977cdb740p+0,
    0x1.ea4afa2a490dap+0, 0x1.eb9f4867cca6ep+0, 0x1.ecf482d8e67f1p+0, 0x1.ee4aaa2188510p+0,
    0x1.efa1bee615a27p+0, 0x1.f0f9c1cb6412ap+0, 0x1.f252b376bba97p+0, 0x1.f3ac948dd7274p+0,
    0x1.f50765b6e4540p+0, 0x1.f6632798844f8p+0, 0x1.f7bfdad9cbe14p+0, 0x1.f91d802243c89p+0,
    0x1.fa7c1819e90d8p+0, 0x1.fbdba3692d514p+0, 0x1.fd3c22b8f71f1p+0, 0x1.fe9d96b2a23d9p+0};

__device__ __forceinline__ double exp_tang256(double x, const double* tbl) {
    const double shifter = 6755399441055744.0;  // 1.5 * 2^52
    const double t = fma(x, 369.3299304675746, shifter);  // 256 / ln2
    const int n = __double2loint(t);
    const double nd = t - shifter;
    double r = fma(nd, -0x1.62e42ffp-9, x);     // L1
    r = fma(nd, 1.6409824502660487e-13, r);   // -L2
    double q = fma(r, 1.0 / 24.0, 1.0 / 6.0);
    q = fma(q, r, 0.5);
    const double p = fma(r * r, q, r);
    const double tj = tbl[n & 255];
    const double y = fma(tj, p, tj);
    const int hi = __double2hiint(y) + ((n >> 8) << 20);
    return n < -258560 ? 0.0 : __hiloint2double(hi, __double2loint(y));
}

// A double as a normalised double-float, by bit patterns (no FP64 or
// conversion-pipe instruction).
__device__ __forceinline__ dfl::df split_df(double x) {
    float h, l;
    split_f32(x, h, l);
    return dfl::fast_two_sum(h, l);
}
// A double rounded to float (to within 2^-24 ulp of round-to-nearest).
__device__ __forceinline__ float round_f32(double x) {
    float h, l;
    split_f32(x, h, l);
    return h + l;
}
// The double of a double-float: the one FP64 instruction of the conversion.
__device__ __forceinline__ double df_to_f64(dfl::df v) { return f32_to_f64(v.hi) + f32_to_f64(v.lo); }
// Whether a double is +-0 (integer compare, not a DSETP).
__device__ __forceinline__ bool f64_is_zero(double x) { return (__double_as_longlong(x) << 1) == 0; }

// A block fills `t` with 2^(j/256) as double-floats (bit patterns of the
// FP64 table; no FP64 instruction).  The caller synchronises.
__device__ __forceinline__ void fill_exp_table_df(dfl::ExpTable& t) {
    for (int j = threadIdx.x; j < 256; j += blockDim.x) {
        float h, l;
        split_f32(kExp2Table256[j], h, l);
        const dfl::df n = dfl::fast_two_sum(h, l);
        t.hi[j] = n.hi;
        t.lo[j] = n.lo;
    }
}

// exp(a) of a double through the double-float exponential (about 2^-46
// relative, plus a's own rounding to 48 bits times |a|); outside [-87, 87]
// CUDA's FP64 exp.  One FP64 instruction (the final add) in range.
__device__ __forceinline__ double exp_df(double a, const dfl::ExpTable& et) {
    float h, l;
    split_f32(a, h, l);
    if (!(fabsf(h) <= 87.0f)) return exp(a);
    const dfl::df v = dfl::exp(dfl::fast_two_sum(h, l), et);
    return f32_to_f64(v.hi) + f32_to_f64(v.lo);
}

// log(y) of a double y > 0 through the double-float logarithm (dfl::log);
// outside [1e-30, 1e30] CUDA's FP64 log.  One FP64 instruction in range.
__device__ __forceinline__ double log_df(double y, const dfl::ExpTable& et) {
    float h, l;
    split_f32(y, h, l);
    if (!(h > 1e-30f && h < 1e30f)) return log(y);
    const dfl::df v = dfl::log(dfl::fast_two_sum(h, l), et);
    return f32_to_f64(v.hi) + f32_to_f64(v.lo);
}

// 1/sqrt(r2) for a positive normal double whose float image is normal:
// Newton-Raphson with the second-order term, y = y0 (1 + e/2 + 3 e^2/8),
// e = 1 - r2 y0^2, from the FP32 approximation y0 = rsqrtf(r2).  r2 reaches
// the FP32 unit and y0 comes back through the bit patterns (truncation of
// the mantissa, no FP64 conversion instruction); |e| < 1e-6 leaves an error
// of order e^3 below one ulp.  5 FP64 operations.
__device__ __forceinline__ double rsqrt_newton(double r2) {
    const int hi = __double2hiint(r2);
    const unsigned lo = (unsigned)__double2loint(r2);
    const float xf = __int_as_float(((hi - ((1023 - 127) << 20)) << 3) | (int)(lo >> 29));
    const int yb = __float_as_int(rsqrtf(xf));
    const double y0 = __hiloint2double((yb >> 3) + ((1023 - 127) << 20), yb << 29);
    const double e = fma(-(r2 * y0), y0, 1.0);
    return fma(y0, e * fma(e, 0.375, 0.5), y0);
}

// grad V(r) = s(r) * r for the radial pair potentials.  `r2` is |r|^2.
template <typename R>
__device__ __forceinline__ R pair_scale(int kind, R r2, R param);

// FP64 gradient scale; with `tbl` (kExp2Table256) the exponentials use exp_tang256.
template <bool kTang>
__device__ __forceinline__ double pair_scale_d(int kind, double r2, double param, const double* tbl) {
    auto ex = [&](double v) { return kTang ? exp_tang256(v, tbl) : exp(v); };
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

// Aziz gradient scale outside the damping radius (r_s >= D, where F = 1 and
// dF = 0): (eps/r_m) [-A alpha exp(-alpha r_s) + ix^7 (6 C6 + 8 C8 ix^2 +
// 10 C10 ix^4)] / |r| with ix = r_m/|r|, written as
// r^-8 (c6 + c8 r^-2 + c10 r^-4) - exp(ln(A alpha eps/r_m) - alpha |r|/r_m) / |r|
// (c_n = n C_n r_m^n eps).  Branch-free; the caller checks r_s >= D
// (aziz_is_far) and uses pair_scale_d otherwise.  `tbl` is kExp2Table256.
__device__ __forceinline__ double aziz_far_scale(double r2, const double* tbl) {
    constexpr double rm2 = Aziz::rm * Aziz::rm, rm6 = rm2 * rm2 * rm2, rm8 = rm6 * rm2, rm10 = rm8 * rm2;
    constexpr double c6 = 6.0 * Aziz::C6 * Aziz::eps * rm6, c8 = 8.0 * Aziz::C8 * Aziz::eps * rm8,
                     c10 = 10.0 * Aziz::C10 * Aziz::eps * rm10;
    const double rinv = rsqrt_newton(r2);
    const double e = exp_tang256(fma(-(Aziz::alpha / Aziz::rm), r2 * rinv, kAzizLnK), tbl);
    const double ri2 = rinv * rinv;
    const double ri4 = ri2 * ri2;
    const double pa = fma(fma(c10, ri2, c8), ri2, c6);
    return fma(ri4 * ri4, pa, -e * rinv);
}
// r_s = |r| / r_m >= D, on r2 = |r|^2 (a compare of the bit patterns: r2 >= 0)
__device__ __forceinline__ bool aziz_is_far(double r2) {
    constexpr double far2 = (Aziz::D * Aziz::rm) * (Aziz::D * Aziz::rm);
    return __double_as_longlong(r2) >= __double_as_longlong(far2);
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

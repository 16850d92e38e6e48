// The Aziz HFDHE2 pair gradient outside its damping radius, evaluated in
// double-float on the FP32 pipe (dfloat.cuh).  Parameters of the reference
// (src/potentials/aziz.cpp:6-13); compiles for the host too, where the unit
// test of this arithmetic checks it against an extended-precision form.
#pragma once

#include "dfloat.cuh"

namespace pimdb {

// Aziz HFDHE2 (reference aziz.cpp:6-13, aziz.h:25-34), bohr and hartree.
struct Aziz {
    static constexpr double rm = 5.60738, A = 0.5448504e6, eps = 3.42016E-5, alpha = 13.353384, D = 1.241314,
                            C6 = 1.3732412, C8 = 0.4253785, C10 = 0.1781;
};

// ln(A alpha eps / r_m) of the Aziz parameters above (aziz.cpp:6-13).
constexpr double kAzizLnK = 3.7927146577859623;

// Gradient scale s(r) = (dV/dr) / r for r_s = r / r_m >= D (F = 1, dF = 0):
//   s = r^-8 (c6 + c8 r^-2 + c10 r^-4) - exp(ln(A alpha eps / r_m) - alpha r / r_m) / r,
// c_n = n C_n r_m^n eps, the same factoring as the FP64 far-field scale.
// r2 = |r|^2 as a double-float.  Relative error a few 2^-48 (the attractive
// and repulsive terms do not cancel beyond the damping radius).
DF_HD dfl::df aziz_far_scale_df(dfl::df r2, const dfl::ExpTable& tbl) {
    using namespace dfl;
    constexpr double rm2 = Aziz::rm * Aziz::rm, rm6 = rm2 * rm2 * rm2, rm8 = rm6 * rm2, rm10 = rm8 * rm2;
    constexpr double c6 = 6.0 * Aziz::C6 * Aziz::eps * rm6, c8 = 8.0 * Aziz::C8 * Aziz::eps * rm8,
                     c10 = 10.0 * Aziz::C10 * Aziz::eps * rm10, ka = Aziz::alpha / Aziz::rm;
    constexpr float c6h = (float)c6, c6l = (float)(c6 - (double)c6h);
    constexpr float c8h = (float)c8, c8l = (float)(c8 - (double)c8h);
    constexpr float c10h = (float)c10, c10l = (float)(c10 - (double)c10h);
    constexpr float kah = (float)ka, kal = (float)(ka - (double)kah);
    constexpr float lkh = (float)kAzizLnK, lkl = (float)(kAzizLnK - (double)lkh);
    const df rinv = rsqrt(r2);
    const df r = mul(r2, rinv);
    const df arg = add(df{lkh, lkl}, neg(mul(df{kah, kal}, r)));
    const df e = dfl::exp(arg, tbl);
    const df ri2 = sqr(rinv);
    const df ri4 = sqr(ri2);
    const df pa = add_sloppy(mul(add_sloppy(mul(df{c10h, c10l}, ri2), df{c8h, c8l}), ri2), df{c6h, c6l});
    return add(mul(sqr(ri4), pa), neg(mul(e, rinv)));
}

// Gradient scale inside the damping radius, r_s = r / r_m in [0.01, D): the
// reference's general form (aziz.cpp:56-106, F and dF of aziz.h:25-34) with
// F = exp(-t^2), t = D ix - 1, ix = 1/r_s, dF = 2 D ix^2 t F:
//   s = (eps/r_m) [-A alpha exp(-alpha r_s)
//        + F ix^6 (ix (6 C6 + 8 C8 ix^2 + 10 C10 ix^4) - 2 D ix^2 t (C6 + C8 ix^2 + C10 ix^4))] / r.
// The repulsive and attractive terms cancel near r_m; the absolute error
// stays a few 2^-48 of their size.  r_s < 0.01 (the reference's
// short-range branch) is left to the FP64 path.
constexpr double kAzizNearMinR2 = (0.01 * Aziz::rm) * (0.01 * Aziz::rm);

// r_s >= D on a double-float r2 (the reference compares r_s = r / r_m with
// D; at the boundary F = 1 and dF = 0 on both sides, so a decision that
// differs from the FP64 one within the double-float rounding of r2 changes
// the result by far less than that rounding).
DF_HD bool aziz_is_far_df(dfl::df r2) {
    constexpr double far2 = (Aziz::D * Aziz::rm) * (Aziz::D * Aziz::rm);
    constexpr float fh = (float)far2, fl = (float)(far2 - (double)fh);
    return r2.hi > fh || (r2.hi == fh && r2.lo >= fl);
}

#if defined(__CUDA_ARCH__)
// out of line on the device: a pass over the few entries inside the damping
// radius per tile calls it, and the pair kernel's hot loop stays smaller
__device__ __noinline__
#else
inline
#endif
dfl::df aziz_near_scale_df(dfl::df r2, const dfl::ExpTable& tbl) {
    using namespace dfl;
    constexpr double irm = 1.0 / Aziz::rm, aal = Aziz::A * Aziz::alpha, erm = Aziz::eps / Aziz::rm,
                     c6a = 6.0 * Aziz::C6, c8a = 8.0 * Aziz::C8, c10a = 10.0 * Aziz::C10, d2 = 2.0 * Aziz::D;
#define PIMDB_DF_CONST(name, v) constexpr float name##h = (float)(v), name##l = (float)((v) - (double)name##h)
    PIMDB_DF_CONST(irm, irm);
    PIMDB_DF_CONST(rm, Aziz::rm);
    PIMDB_DF_CONST(al, Aziz::alpha);
    PIMDB_DF_CONST(aal, aal);
    PIMDB_DF_CONST(dd, Aziz::D);
    PIMDB_DF_CONST(d2, d2);
    PIMDB_DF_CONST(erm, erm);
    PIMDB_DF_CONST(c6, Aziz::C6);
    PIMDB_DF_CONST(c8, Aziz::C8);
    PIMDB_DF_CONST(c10, Aziz::C10);
    PIMDB_DF_CONST(c6a, c6a);
    PIMDB_DF_CONST(c8a, c8a);
    PIMDB_DF_CONST(c10a, c10a);
#undef PIMDB_DF_CONST
    const df rinv = rsqrt(r2);
    const df rs = mul(mul(r2, rinv), df{irmh, irml});
    const df t1 = mul(dfl::exp(neg(mul(rs, df{alh, all})), tbl), df{-aalh, -aall});
    const df ix = mul(rinv, df{rmh, rml});
    const df ix2 = sqr(ix);
    const df ix6 = mul(sqr(ix2), ix2);
    const df t = add_f(mul(ix, df{ddh, ddl}), -1.0f);
    const df f = dfl::exp(neg(sqr(t)), tbl);
    const df pa = add_sloppy(mul(add_sloppy(mul(df{c10ah, c10al}, ix2), df{c8ah, c8al}), ix2), df{c6ah, c6al});
    const df pb = add_sloppy(mul(add_sloppy(mul(df{c10h, c10l}, ix2), df{c8h, c8l}), ix2), df{c6h, c6l});
    const df inner = add(mul(ix, pa), neg(mul(mul(ix2, t), mul(pb, df{d2h, d2l}))));
    const df g = mul(add(t1, mul(mul(f, ix6), inner)), df{ermh, erml});
    return mul(g, rinv);
}

}  // namespace pimdb

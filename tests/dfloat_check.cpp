// Host check of the double-float arithmetic the pair kernels use
// (pimd-b_gb300/csrc/dfloat.cuh, aziz_df.cuh) against long double.  Prints
// the largest relative error of each function over its test range; the
// Python test reads the numbers.  Inputs are seeded and deterministic.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <random>

#include "../pimd-b_gb300/csrc/aziz_df.cuh"

using namespace pimdb;
using dfl::df;
typedef long double ld;

static ld val(df a) { return (ld)a.hi + (ld)a.lo; }
static df mk(ld v) {
    const float h = (float)v;
    return {h, (float)(v - (ld)h)};
}
static ld rel(ld got, ld want) { return fabsl(got - want) / fabsl(want); }

int main() {
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    dfl::ExpTable tbl;
    for (int j = 0; j < 256; ++j) {
        const df e = mk(exp2l((ld)j / 256.0L));
        tbl.hi[j] = e.hi;
        tbl.lo[j] = e.lo;
    }
    ld e_add = 0, e_mul = 0, e_sqr = 0, e_exp = 0, e_rsqrt = 0, e_rsqrt_seed = 0, e_aziz = 0, e_sloppy_abs = 0;
    for (int k = 0; k < 400000; ++k) {
        const ld a = (U(rng) - 0.5) * powl(2.0L, (int)(U(rng) * 40) - 20);
        const ld b = (U(rng) - 0.5) * powl(2.0L, (int)(U(rng) * 40) - 20);
        const df da = mk(a), db = mk(b);
        const ld A = val(da), B = val(db);
        if (A + B != 0) e_add = std::max(e_add, rel(val(dfl::add(da, db)), A + B));
        e_sloppy_abs = std::max(e_sloppy_abs, fabsl(val(dfl::add_sloppy(da, db)) - (A + B)) / (fabsl(A) + fabsl(B)));
        e_mul = std::max(e_mul, rel(val(dfl::mul(da, db)), A * B));
        e_sqr = std::max(e_sqr, rel(val(dfl::sqr(da)), A * A));
    }
    // exp over [-69, 80] (below -69 the low word of the result is subnormal)
    for (int k = 0; k < 400000; ++k) {
        const ld x = -69.0L + 149.0L * U(rng);
        const df dx = mk(x);
        const ld X = val(dx);
        const df y = dfl::exp(dx, tbl);
        e_exp = std::max(e_exp, rel(val(y), expl(X)));
    }
    // rsqrt over [1e-3, 1e5], with the library seed and with seeds off by up to 8 float ulps
    for (int k = 0; k < 400000; ++k) {
        const ld x = powl(10.0L, -3.0L + 8.0L * U(rng));
        const df dx = mk(x);
        const ld X = val(dx);
        e_rsqrt = std::max(e_rsqrt, rel(val(dfl::rsqrt(dx)), 1.0L / sqrtl(X)));
        const float y0 = (float)(1.0L / sqrtl(X)) * (1.0f + (float)((U(rng) - 0.5) * 16.0 * 0x1p-24));
        e_rsqrt_seed = std::max(e_rsqrt_seed, rel(val(dfl::rsqrt_from(dx, y0)), 1.0L / sqrtl(X)));
    }
    // the Aziz far-field gradient scale, r in [D r_m, 30 bohr]
    const ld rm = Aziz::rm, eps = Aziz::eps, al = Aziz::alpha;
    for (int k = 0; k < 400000; ++k) {
        const ld r = (ld)Aziz::D * rm + (30.0L - (ld)Aziz::D * rm) * U(rng);
        const df r2 = mk(r * r);
        const ld R = sqrtl(val(r2));
        const ld ix = rm / R;
        const ld want = (eps / rm) *
                        (-(ld)Aziz::A * al * expl(-al * R / rm) +
                         (6.0L * Aziz::C6 * powl(ix, 7) + 8.0L * Aziz::C8 * powl(ix, 9) + 10.0L * Aziz::C10 * powl(ix, 11))) /
                        R;
        e_aziz = std::max(e_aziz, rel(val(aziz_far_scale_df(r2, tbl)), want));
    }
    // inside the damping radius, r_s in [0.01, D): error against the size of
    // the terms (the force crosses zero at r_m)
    ld e_near = 0;
    for (int k = 0; k < 400000; ++k) {
        const ld r = rm * (0.01L + ((ld)Aziz::D - 0.01L) * U(rng));
        const df r2 = mk(r * r);
        const ld R = sqrtl(val(r2));
        const ld x = R / rm, ix = 1.0L / x, D = Aziz::D;
        const ld F = expl(-(D * ix - 1.0L) * (D * ix - 1.0L));
        const ld dF = 2.0L * D * ix * ix * (D * ix - 1.0L) * F;
        const ld T1 = -(ld)Aziz::A * al * expl(-al * x);
        const ld T2 = (6.0L * Aziz::C6 * powl(ix, 7) + 8.0L * Aziz::C8 * powl(ix, 9) + 10.0L * Aziz::C10 * powl(ix, 11)) * F;
        const ld T3 = -(Aziz::C6 * powl(ix, 6) + Aziz::C8 * powl(ix, 8) + Aziz::C10 * powl(ix, 10)) * dF;
        const ld want = (eps / rm) * (T1 + T2 + T3) / R;
        const ld size = (eps / rm) * (fabsl(T1) + fabsl(T2) + fabsl(T3)) / R;
        e_near = std::max(e_near, fabsl(val(aziz_near_scale_df(r2, tbl)) - want) / size);
    }
    std::printf("aziz_near %.3Le\n", e_near);
    // log over [1e-20, 1e20] (log-uniform) and just around 1: error against
    // max(|log y|, 1)
    ld e_log = 0;
    for (int k = 0; k < 400000; ++k) {
        const ld y = (k & 1) ? powl(10.0L, -20.0L + 40.0L * U(rng)) : 1.0L + (U(rng) - 0.5) * 1e-3L;
        const df dy = mk(y);
        const ld Y = val(dy);
        e_log = std::max(e_log, fabsl(val(dfl::log(dy, tbl)) - logl(Y)) / std::max(fabsl(logl(Y)), 1.0L));
    }
    std::printf("log %.3Le\n", e_log);
    std::printf("add %.3Le\nadd_sloppy_abs %.3Le\nmul %.3Le\nsqr %.3Le\nexp %.3Le\nrsqrt %.3Le\nrsqrt_seed8ulp %.3Le\n"
                "aziz_far %.3Le\n",
                e_add, e_sloppy_abs, e_mul, e_sqr, e_exp, e_rsqrt, e_rsqrt_seed, e_aziz);
    return 0;
}

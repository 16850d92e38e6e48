// Shared device-side definitions for the PIMD-B++ hot path on GB300 (sm_103a).
//
// Device layout of one ring polymer ("system"): structure of arrays, bead
// major: a[bead][axis][particle], particle rows padded to `ld` (a multiple of
// 32 doubles = 256 bytes) so that every row starts on a 256-byte boundary.
// Padding entries hold zeros and are never part of a sum.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace pimdb {

enum PotKind : int {
    POT_FREE = 0,
    POT_HARMONIC = 1,
    POT_DOUBLE_WELL = 2,
    POT_COSINE = 3,
    POT_AZIZ = 4,
    POT_DIPOLE = 5,
};

// Error bits written by kernels into the per-system error word.
enum ErrBits : int {
    ERRB_NONFINITE_VB = 1,
    ERRB_BOUNDS = 2,
    ERRB_TIMEOUT = 4,
};

// Everything a kernel needs to know about one system, passed by value.
struct Sys {
    int N;          // particles
    int P;          // beads
    int ld;         // padded particle stride (multiple of 32)
    int bosonic;    // exchange on beads 0 and P-1
    int pbc;
    double L, invL; // box edge and its inverse
    double mass, dt;
    double dt_m;    // dt / mass (the drift multiplies: FP64 division costs ~8 FP64 operations)
    double kappa;   // spring constant m omega_p^2
    double beta_ex; // exchange beta = beta/P
    double inv_beta_ex;  // 1 / beta_ex
    double omega_p;
    double c1, c2;  // Langevin friction and noise coefficients
    double cutoff;  // effective pair cutoff: 0 none, < 0 all pairs
    int ext_kind;
    double ext_a, ext_b, ext_c; // harmonic: k | double well: 4 m s, loc^2, m s | cosine: -A k, k, phase
    int int_kind;
    double int_a;               // harmonic pair: k | dipole: strength
    int pair_cap;               // pair-tile gradient capacity per warp (0: the default)
    int reserve_sms;            // SMs (the highest ids) the pair tiles leave to the exchange's
                                // one-block passes running beside them (0: none)
    int eflat;                  // cycle energies from link prefix sums (given a work array)
    uint64_t seed;
    uint32_t replica;
    // device arrays
    double* x;      // [P][D][ld]
    double* p;
    double* f;      // total forces (Simulation::forces)
    double* fphys;  // physical forces (normal-mode propagator's ext_forces member)
    double* fx;     // exterior (exchange) spring forces of beads 0 and P-1: [2][D][ld]
    double* E;      // packed cycle energies: row v (0-based), column u <= v at v(v+1)/2 + u
    double* V;      // forward potentials V[0..N]
    double* Vb;     // backward potentials V_backwards[0..N]
    double* scal;   // exchange scalars: V_B, prim, P_distinct, P_longest
    double* red;    // reduction partials
    int* err;       // error word
    // exchange work arrays
    double* Vh;     // FP32-accurate estimate of V (stored as double), N+1
    double* Vbh;    // estimate of V_backwards, N+1
    double* yf;     // y_m = exp(-beta (V_m - Vh_m)), N+1
    double* yb;     // y_l = exp(-beta (Vb_l - Vbh_l)), N+1
    double* Wf;     // forward weights, packed like E
    double* Wb;     // backward weights, packed by backward node (see exchange.cu)
    double* Et;     // E re-packed by backward node
    double* rowR;   // per-row factors exp(-beta (Vh[l+1] + Vb[l+1] - V[N])), N
    double* rowC;   // cut probabilities exp(-beta (V[l+1] + Vb[l+1] - V[N])), N
    double* Vp;     // V and V_backwards of the previous evaluation, [2][N+1]
                    // (null: the next estimate is the last result, not extrapolated)
    int* xflags;    // [0] forward used the exact fallback, [1] backward, [2] completion counter
    // Langevin normals drawn by the reference's RanMars streams (one per
    // bead, seeded seed + bead) for the current and the previous MD step:
    // [t & 3][bead-or-mode][axis][ld] with t = 2 step + substep.  Null when
    // the noise is the counter-based Philox stream.
    const double* noise;
};

// MD step index of a launch: `off`, plus the value at `base` when the launch
// belongs to a replayed CUDA graph (base = the handle's device-side step
// counter, which the graph itself advances).
struct StepRef {
    const long long* base;
    long long off;
    __device__ __forceinline__ long long get() const { return off + (base ? *base : 0); }
};

template <int D>
__host__ __device__ inline size_t idx(const Sys& s, int b, int a, int i) {
    return ((size_t)b * D + a) * s.ld + i;
}

// applyMinimumImage (reference common.cpp:41-43): dx - L floor(dx/L + 1/2).
__device__ __forceinline__ double min_image(double dx, double L, double invL) {
    return dx - L * floor(dx * invL + 0.5);
}
__device__ __forceinline__ float min_image_f(float dx, float L, float invL) {
    return dx - L * floorf(dx * invL + 0.5f);
}

// ---------------------------------------------------------------- reductions
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide reductions; `sh` must hold blockDim.x/32 doubles.  Every thread
// receives the result.  Contains two __syncthreads().
__device__ __forceinline__ double block_sum(double v, double* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    for (int k = 0; k < nw; ++k) t += sh[k];
    __syncthreads();
    return t;
}
__device__ __forceinline__ double block_min(double v, double* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_min(v);
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = sh[0];
    for (int k = 1; k < nw; ++k) t = fmin(t, sh[k]);
    __syncthreads();
    return t;
}

// ------------------------------------------------------------------- noise
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) followed by Box-Muller.
// Normal number for (bead-or-mode b, axis a, particle i) at (step, substep):
// counter = {pair, replica, t_lo, t_hi} with pair = (b*D + a)*ceil(N/2) + i/2
// and t = 2*step + substep; even i takes the cosine branch, odd i the sine.
__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint64_t seed) {
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
        const uint32_t n0 = hi1 ^ c[1] ^ k0;
        const uint32_t n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
    }
}

// Box-Muller on the FP32 pipe (FP64 runs at 1/64 of the FP32 rate, so FP64
// transcendentals would cost as much as a pair interaction).  Its log, sin and
// cos are evaluated here from their series with correctly rounded IEEE
// operations only (explicit round-to-nearest intrinsics, nothing contracted),
// so a C restatement with fmaf draws bit-identical numbers.
//   u1 = (k + 1) 2^-24 from the top 24 bits k of word 0, exact (|z| <= 5.8);
//   log u1 = e ln2 + 2 atanh((m - 1)/(m + 1)), m in [sqrt(1/2), sqrt(2)),
//            the atanh series to s^9 (next term below 3e-9 relative);
//   theta = 2 pi u2, u2 from 26 bits of word 2: the top 2 bits select the
//            quadrant, the next 24 give phi in [0, pi/2), where the Taylor
//            series of sin to phi^13 and cos to phi^14 are within 7e-10.
__device__ __forceinline__ float bm_log(float u) {
    const unsigned bits = __float_as_uint(u);
    int e = (int)((bits >> 23) & 0xffu) - 127;
    float m = __uint_as_float((bits & 0x7fffffu) | 0x3f800000u);
    if (m > 1.41421354f) {
        m = __fmul_rn(m, 0.5f);
        e += 1;
    }
    const float sv = __fdiv_rn(__fsub_rn(m, 1.0f), __fadd_rn(m, 1.0f));
    const float s2 = __fmul_rn(sv, sv);
    float q = __fmaf_rn(0.111111112f, s2, 0.142857149f);
    q = __fmaf_rn(q, s2, 0.2f);
    q = __fmaf_rn(q, s2, 0.333333343f);
    q = __fmaf_rn(q, s2, 1.0f);
    const float lm = __fmul_rn(__fmul_rn(2.0f, sv), q);
    const float ef = (float)e;
    return __fmaf_rn(ef, 0.693145752f, __fmaf_rn(ef, 1.42860677e-06f, lm));
}

__device__ __forceinline__ void bm_sincos_2pi(unsigned w, float* sn, float* cs) {
    const unsigned quad = w >> 30;
    const float ph = __fmul_rn(__fmul_rn((float)((w >> 6) & 0xffffffu), 5.96046448e-08f), 1.57079637f);
    const float p2 = __fmul_rn(ph, ph);
    float sp = __fmaf_rn(1.60590444e-10f, p2, -2.50521079e-08f);
    sp = __fmaf_rn(sp, p2, 2.75573188e-06f);
    sp = __fmaf_rn(sp, p2, -1.98412701e-04f);
    sp = __fmaf_rn(sp, p2, 8.33333377e-03f);
    sp = __fmaf_rn(sp, p2, -0.166666672f);
    sp = __fmaf_rn(__fmul_rn(sp, p2), ph, ph);
    float cp = __fmaf_rn(-1.14707454e-11f, p2, 2.08767559e-09f);
    cp = __fmaf_rn(cp, p2, -2.75573188e-07f);
    cp = __fmaf_rn(cp, p2, 2.48015876e-05f);
    cp = __fmaf_rn(cp, p2, -1.38888892e-03f);
    cp = __fmaf_rn(cp, p2, 4.16666679e-02f);
    cp = __fmaf_rn(cp, p2, -0.5f);
    cp = __fmaf_rn(cp, p2, 1.0f);
    const float a = (quad & 1u) ? cp : sp, b = (quad & 1u) ? sp : cp;
    *sn = (quad & 2u) ? -a : a;
    *cs = ((quad + 1u) & 2u) ? -b : b;
}

__device__ __forceinline__ float2 philox_normal_pair_f32(uint64_t seed, uint32_t replica, uint64_t t, uint32_t pair) {
    uint32_t c[4] = {pair, replica, (uint32_t)t, (uint32_t)(t >> 32)};
    philox4x32_10(c, seed);
    const float u1 = __fmul_rn((float)((c[0] >> 8) + 1u), 5.96046448e-08f);  // exact
    const float r = __fsqrt_rn(__fmul_rn(-2.0f, bm_log(u1)));
    float sn, cs;
    bm_sincos_2pi(c[2], &sn, &cs);
    return make_float2(__fmul_rn(r, cs), __fmul_rn(r, sn));
}

// float -> double by bit patterns (exact), so that no FP64-pipe conversion
// is issued (on GB300 a conversion takes the FP64 pipe at half its add
// rate); zero, subnormal, infinite and NaN values take the conversion.
__device__ __forceinline__ double f32_to_f64(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned ef = (u >> 23) & 0xffu;
    if (ef == 0u || ef == 0xffu) return (double)f;
    return __hiloint2double((int)((u & 0x80000000u) | ((ef + 896u) << 20) | ((u & 0x7fffffu) >> 3)), (int)(u << 29));
}
// x = hi + lo by bit patterns: hi holds the sign, exponent and leading 24
// significand bits of x (truncated), lo the remaining 29 bits, truncated to
// a float's 24 (|lo| < 2^-23 |x|; hi + lo carries 47 or more bits of x).
// Outside 2^-60 <= |x| < 2^100 (and for zero) the conversions are used.
__device__ __forceinline__ void split_f32(double x, float& hi, float& lo) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ffu);
    if (e < 1023 - 60 || e >= 1023 + 100) {
        hi = (float)x;
        lo = (float)(x - (double)hi);
        return;
    }
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const unsigned long long m = b & 0xfffffffffffffULL;  // 52 fraction bits
    hi = __uint_as_float(sign | ((unsigned)(e - 1023 + 127) << 23) | (unsigned)(m >> 29));
    const unsigned m29 = (unsigned)(m & 0x1fffffffu);  // value m29 2^(e - 1075)
    if (m29 == 0u) {
        lo = 0.0f;
        return;
    }
    const int top = 31 - __clz((int)m29);  // leading bit of m29, 0..28
    const unsigned frac = top >= 23 ? (m29 >> (top - 23)) & 0x7fffffu : (m29 << (23 - top)) & 0x7fffffu;
    lo = __uint_as_float(sign | ((unsigned)(e - 1075 + top + 127) << 23) | frac);
}

__device__ __forceinline__ double2 philox_normal_pair(uint64_t seed, uint32_t replica, uint64_t t, uint32_t pair) {
    const float2 z = philox_normal_pair_f32(seed, replica, t, pair);
    return make_double2(f32_to_f64(z.x), f32_to_f64(z.y));
}

// The two Langevin normals of (bead-or-mode k, axis a, particles 2 i2 and
// 2 i2 + 1) at noise counter t = 2 step + substep (half = ceil(N / 2)): the
// Philox pair, or the RanMars streams' normals staged in s.noise.
template <int D>
__device__ __forceinline__ double2 langevin_pair(const Sys& s, uint64_t t, int k, int a, int i2, int half) {
    if (s.noise) {
        const double* z = s.noise + (((size_t)(t & 3) * s.P + k) * D + a) * s.ld + 2 * i2;
        return make_double2(z[0], z[1]);
    }
    return philox_normal_pair(s.seed, s.replica, t, (uint32_t)((size_t)(k * D + a) * half + i2));
}

}  // namespace pimdb

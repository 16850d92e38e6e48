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
    double kappa;   // spring constant m omega_p^2
    double beta_ex; // exchange beta = beta/P
    double omega_p;
    double c1, c2;  // Langevin friction and noise coefficients
    double cutoff;  // effective pair cutoff: 0 none, < 0 all pairs
    int ext_kind;
    double ext_a, ext_b, ext_c; // harmonic: k | double well: 4 m s, loc^2, m s | cosine: -A k, k, phase
    int int_kind;
    double int_a;               // harmonic pair: k | dipole: strength
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

__device__ __forceinline__ double2 philox_normal_pair(uint64_t seed, uint32_t replica, uint64_t t, uint32_t pair) {
    uint32_t c[4] = {pair, replica, (uint32_t)t, (uint32_t)(t >> 32)};
    philox4x32_10(c, seed);
    const uint64_t a = ((((uint64_t)c[1]) << 32) | c[0]) >> 11;
    const uint64_t b = ((((uint64_t)c[3]) << 32) | c[2]) >> 11;
    const double u1 = ((double)a + 0.5) * 0x1p-53;
    const double u2 = ((double)b + 0.5) * 0x1p-53;
    const double r = sqrt(-2.0 * log(u1));
    double sn, cs;
    sincos(6.283185307179586 * u2, &sn, &cs);
    return make_double2(r * cs, r * sn);
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

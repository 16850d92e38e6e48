// Integrator pieces of the OBABO step (src/simulation.cpp:236-260):
//   Langevin O-step, Cartesian coupling  langevin.cpp:15-27, thermostat_coupling.cpp:11-25
//   Langevin O-step, normal-mode coupling thermostat_coupling.cpp:29-47, normal_modes.cpp:99-139
//   centre-of-mass momentum removal      simulation.cpp:581-603
//   velocity-Verlet B and A              velocity_verlet.cpp:7-38
//   normal-mode propagator               normal_modes_propagator.cpp:19-103
// plus the layout conversions between the reference's per-bead dVec order
// [bead][particle][axis] and the device order [bead][axis][particle].
//
// The centre-of-mass correction needs a sum over every bead and particle.
// The kernel that last changed the momenta writes per-block partial sums
// (`red_out`); the next kernel reduces them in a fixed order at start-up
// (`red_in`), so the result is deterministic.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace pimdb {

template <int D>
__global__ void k_pack(Sys s, const double* __restrict__ src, double* __restrict__ dst) {
    const size_t n = (size_t)s.P * s.N * D;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int a = (int)(e % D);
        const size_t bi = e / D;
        const int i = (int)(bi % s.N);
        const int b = (int)(bi / s.N);
        dst[idx<D>(s, b, a, i)] = src[e];
    }
}

template <int D>
__global__ void k_unpack(Sys s, const double* __restrict__ src, double* __restrict__ dst) {
    const size_t n = (size_t)s.P * s.N * D;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int a = (int)(e % D);
        const size_t bi = e / D;
        const int i = (int)(bi % s.N);
        const int b = (int)(bi / s.N);
        dst[e] = src[idx<D>(s, b, a, i)];
    }
}

// State in, one launch: x and p in host order (either may be absent; device
// staging or page-locked host memory, read directly) and every force array
// zeroed (as after the reference's
// constructor, src/simulation.cpp:16-101).  The exchange keeps reusing its
// last potentials as the estimate: where new coordinates make that estimate
// fail, its retry phase draws a fresh one.
template <int D>
__global__ void k_state_in(Sys s, const double* __restrict__ sx, const double* __restrict__ sp) {
    const size_t n = (size_t)s.P * s.N * D;
    const size_t nsoa = (size_t)s.P * D * s.ld;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    for (size_t e = t0; e < n; e += stride) {
        const int a = (int)(e % D);
        const size_t bi = e / D;
        const size_t o = idx<D>(s, (int)(bi / s.N), a, (int)(bi % s.N));
        if (sx) s.x[o] = sx[e];
        if (sp) s.p[o] = sp[e];
    }
    for (size_t q = t0; q < nsoa; q += stride) {
        s.f[q] = 0.0;
        s.fphys[q] = 0.0;
        if (q < (size_t)2 * D * s.ld) s.fx[q] = 0.0;
    }
}

// State out, one launch: x, p and f (each output may be null) in host
// order.  The outputs are device staging or page-locked host memory, which
// the kernel writes directly.
template <int D>
__global__ void k_state_out(Sys s, double* __restrict__ ox, double* __restrict__ op, double* __restrict__ of) {
    const size_t n = (size_t)s.P * s.N * D;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int a = (int)(e % D);
        const size_t bi = e / D;
        const size_t o = idx<D>(s, (int)(bi / s.N), a, (int)(bi % s.N));
        if (ox) ox[e] = s.x[o];
        if (op) op[e] = s.p[o];
        if (of) of[e] = s.f[o];
    }
}

template <int D>
__device__ __forceinline__ void com_from_partials(const Sys& s, const double* red_in, int nred, double* cm,
                                                  double* shred) {
    double acc[3] = {0.0, 0.0, 0.0};
    for (int k = threadIdx.x; k < nred; k += blockDim.x) {
#pragma unroll
        for (int a = 0; a < D; ++a) acc[a] += red_in[3 * k + a];
    }
    const double inv = 1.0 / ((double)s.N * (double)s.P);
#pragma unroll
    for (int a = 0; a < D; ++a) cm[a] = block_sum(acc[a], shred) * inv;
}

template <int D>
__device__ __forceinline__ void com_write_partials(double* part, double* red_out, double* shred) {
#pragma unroll
    for (int a = 0; a < D; ++a) {
        const double t = block_sum(part[a], shred);
        if (threadIdx.x == 0) red_out[3 * blockIdx.x + a] = t;
    }
}

// Kick source for the normal-mode propagator (normal_modes_propagator.cpp:73-103):
// physical forces, plus on bosonic beads the exchange spring minus the
// distinguishable inner springs.
template <int D>
__device__ __forceinline__ double nm_kick_force(const Sys& s, int b, int a, int i) {
    const size_t o = idx<D>(s, b, a, i);
    double fk = s.fphys[o];
    if (s.bosonic && (b == 0 || b == s.P - 1)) {
        const int bp = (b - 1 + s.P) % s.P, bn = (b + 1) % s.P;
        const double inner = -s.kappa * (2 * s.x[o] - s.x[idx<D>(s, bp, a, i)] - s.x[idx<D>(s, bn, a, i)]);
        fk = fk + s.fx[((size_t)(b == 0 ? 0 : 1) * D + a) * s.ld + i] - inner;
    }
    return fk;
}

// One thread per (bead, axis, particle pair).
template <int D>
__global__ void k_cart_update(Sys s, int flags, const double* __restrict__ red_in, int nred_in,
                              double* __restrict__ red_out, StepRef sref, int substep, int kick_nm) {
    const long long step = sref.get();
    __shared__ double shred[32];
    const int half = (s.N + 1) / 2;
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t total = (size_t)s.P * D * half;
    double cm[3] = {0.0, 0.0, 0.0};
    if (flags & SF_COM_APPLY) com_from_partials<D>(s, red_in, nred_in, cm, shred);
    double part[3] = {0.0, 0.0, 0.0};
    if (t < total) {
        const int i2 = (int)(t % half);
        const int ba = (int)(t / half);
        const int a = ba % D;
        const int b = ba / D;
        double2 z = make_double2(0.0, 0.0);
        if (flags & SF_LANGEVIN)
            z = langevin_pair<D>(s, 2ull * (unsigned long long)step + substep, b, a, i2, half);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i = 2 * i2 + h;
            if (i >= s.N) break;
            const size_t o = idx<D>(s, b, a, i);
            double p = s.p[o];
            if (flags & SF_COM_APPLY) p -= cm[a];
            if (flags & SF_KICK) {
                const double fk = kick_nm ? nm_kick_force<D>(s, b, a, i) : s.f[o];
                p += 0.5 * s.dt * fk;
            }
            if (flags & SF_LANGEVIN) p = s.c1 * p + s.c2 * (h == 0 ? z.x : z.y);
            if (flags & SF_DRIFT) s.x[o] = fma(p, s.dt_m, s.x[o]);
            s.p[o] = p;
            part[a] += p;
        }
    }
    if (flags & SF_COM_PARTIAL) com_write_partials<D>(part, red_out, shred);
}

constexpr int kNmTile = 4;                           // particles per block
static_assert(sizeof(double) * 4 * (size_t)kNmMaxBeads * kNmTile + 4096 <= 227 * 1024,
              "k_nm_propagate's shared memory at the most beads");
constexpr int kNmPairs = kNmTile / 2;                // particle pairs per block
constexpr int kNmGroups = 64;                        // mode groups
constexpr int kNmThreads = kNmPairs * kNmGroups;

// Langevin O-step on the normal modes: p_nm = C p, p_nm <- c1 p_nm + c2 xi,
// p = C^T p_nm.  One block per (kNmTile-particle tile, axis); thread (pair pp,
// group g) handles particles 2pp, 2pp+1 of the tile for modes g, g+64, ...
// and then for beads g, g+64, ...
template <int D>
__global__ void __launch_bounds__(kNmThreads) k_nm_thermo(Sys s, const double* __restrict__ C,
                                                          const double* __restrict__ T, int flags,
                                                          const double* __restrict__ red_in, int nred_in,
                                                          double* __restrict__ red_out, StepRef sref,
                                                          int substep) {
    const long long step = sref.get();
    extern __shared__ double sm[];
    __shared__ double shred[32];
    const int P = s.P;
    double* sp = sm;                 // [P][kNmTile]
    double* sq = sm + P * kNmTile;   // [P][kNmTile]
    const int a = blockIdx.y;
    const int i0 = blockIdx.x * kNmTile;
    const int pp = threadIdx.x % kNmPairs, g = threadIdx.x / kNmPairs;
    double cm[3] = {0.0, 0.0, 0.0};
    if (flags & SF_COM_APPLY) com_from_partials<D>(s, red_in, nred_in, cm, shred);
    for (int e = threadIdx.x; e < P * kNmTile; e += blockDim.x) {
        const int b = e / kNmTile, il = e % kNmTile, i = i0 + il;
        sp[e] = i < s.N ? s.p[idx<D>(s, b, a, i)] - cm[a] : 0.0;
    }
    __syncthreads();
    const int half = (s.N + 1) / 2;
    const uint64_t t = 2ull * (unsigned long long)step + substep;
    for (int k = g; k < P; k += kNmGroups) {
        double q0 = 0.0, q1 = 0.0;
        const double* ck = C + (size_t)k * P;
        for (int b = 0; b < P; ++b) {
            const double c = ck[b];
            q0 += c * sp[b * kNmTile + 2 * pp];
            q1 += c * sp[b * kNmTile + 2 * pp + 1];
        }
        const int ie = i0 + 2 * pp;
        const double2 z = langevin_pair<D>(s, t, k, a, ie >> 1, half);
        sq[k * kNmTile + 2 * pp] = s.c1 * q0 + s.c2 * z.x;
        sq[k * kNmTile + 2 * pp + 1] = s.c1 * q1 + s.c2 * z.y;
    }
    __syncthreads();
    double part = 0.0;
    for (int j = g; j < P; j += kNmGroups) {
        double v0 = 0.0, v1 = 0.0;
        const double* tj = T + (size_t)j * P;
        for (int k = 0; k < P; ++k) {
            const double c = tj[k];
            v0 += c * sq[k * kNmTile + 2 * pp];
            v1 += c * sq[k * kNmTile + 2 * pp + 1];
        }
        const int ie = i0 + 2 * pp;
        if (ie < s.N) {
            s.p[idx<D>(s, j, a, ie)] = v0;
            part += v0;
        }
        if (ie + 1 < s.N) {
            s.p[idx<D>(s, j, a, ie + 1)] = v1;
            part += v1;
        }
    }
    if (flags & SF_COM_PARTIAL) {
        const int bid = blockIdx.y * gridDim.x + blockIdx.x;
        const double tsum = block_sum(part, shred);
        if (threadIdx.x == 0) {
#pragma unroll
            for (int ax = 0; ax < D; ++ax) red_out[3 * bid + ax] = ax == a ? tsum : 0.0;
        }
    }
}

// Normal-mode propagator step up to the force evaluation
// (normal_modes_propagator.cpp:19-63): half-kick with the stored physical
// forces, Cartesian -> normal modes, exact free ring-polymer rotation, back
// to Cartesian.  rot[4 k ..] = {cos(w_k dt), sin(w_k dt), m w_k,
// sin(w_k dt) / (m w_k)} (w_0 = 0 is the free-particle drift).
template <int D>
__global__ void __launch_bounds__(kNmThreads) k_nm_propagate(Sys s, const double* __restrict__ C,
                                                             const double* __restrict__ T,
                                                             const double* __restrict__ rot, int com_apply,
                                                             const double* __restrict__ red_in, int nred_in) {
    extern __shared__ double sm[];
    __shared__ double shred[32];
    const int P = s.P;
    double* sx = sm;
    double* sp = sm + P * kNmTile;
    double* sq = sm + 2 * P * kNmTile;
    double* spi = sm + 3 * P * kNmTile;
    const int a = blockIdx.y;
    const int i0 = blockIdx.x * kNmTile;
    const int pp = threadIdx.x % kNmPairs, g = threadIdx.x / kNmPairs;
    double cm[3] = {0.0, 0.0, 0.0};
    if (com_apply) com_from_partials<D>(s, red_in, nred_in, cm, shred);
    for (int e = threadIdx.x; e < P * kNmTile; e += blockDim.x) {
        const int b = e / kNmTile, il = e % kNmTile, i = i0 + il;
        double x = 0.0, p = 0.0;
        if (i < s.N) {
            const size_t o = idx<D>(s, b, a, i);
            x = s.x[o];
            p = s.p[o] - cm[a];
            p += 0.5 * s.dt * nm_kick_force<D>(s, b, a, i);
        }
        sx[e] = x;
        sp[e] = p;
    }
    __syncthreads();
    for (int k = g; k < P; k += kNmGroups) {
        double q0 = 0.0, q1 = 0.0, p0 = 0.0, p1 = 0.0;
        const double* ck = C + (size_t)k * P;
        for (int b = 0; b < P; ++b) {
            const double c = ck[b];
            q0 += c * sx[b * kNmTile + 2 * pp];
            q1 += c * sx[b * kNmTile + 2 * pp + 1];
            p0 += c * sp[b * kNmTile + 2 * pp];
            p1 += c * sp[b * kNmTile + 2 * pp + 1];
        }
        const double cs = rot[4 * k], sn = rot[4 * k + 1], mw = rot[4 * k + 2], snw = rot[4 * k + 3];
        double qa, qb, pa, pb;
        if (mw == 0.0) {
            qa = q0 + s.dt_m * p0;
            qb = q1 + s.dt_m * p1;
            pa = p0;
            pb = p1;
        } else {
            qa = cs * q0 + snw * p0;
            qb = cs * q1 + snw * p1;
            pa = -mw * sn * q0 + cs * p0;
            pb = -mw * sn * q1 + cs * p1;
        }
        sq[k * kNmTile + 2 * pp] = qa;
        sq[k * kNmTile + 2 * pp + 1] = qb;
        spi[k * kNmTile + 2 * pp] = pa;
        spi[k * kNmTile + 2 * pp + 1] = pb;
    }
    __syncthreads();
    for (int j = g; j < P; j += kNmGroups) {
        double x0 = 0.0, x1 = 0.0, v0 = 0.0, v1 = 0.0;
        const double* tj = T + (size_t)j * P;
        for (int k = 0; k < P; ++k) {
            const double c = tj[k];
            x0 += c * sq[k * kNmTile + 2 * pp];
            x1 += c * sq[k * kNmTile + 2 * pp + 1];
            v0 += c * spi[k * kNmTile + 2 * pp];
            v1 += c * spi[k * kNmTile + 2 * pp + 1];
        }
        const int ie = i0 + 2 * pp;
        if (ie < s.N) {
            const size_t o = idx<D>(s, j, a, ie);
            s.x[o] = x0;
            s.p[o] = v0;
        }
        if (ie + 1 < s.N) {
            const size_t o = idx<D>(s, j, a, ie + 1);
            s.x[o] = x1;
            s.p[o] = v1;
        }
    }
}

// ---------------------------------------------------------------------------
// Normal-mode transforms by FFT (P a power of two).  C's rows are the scaled
// real DFT: for X_k = sum_b x_b exp(-2 pi i k b / P),
//   q_0 = X_0 / sqrt(P), q_{P/2} = X_{P/2} / sqrt(P),
//   q_k = sqrt(2/P) Re X_k (0 < k < P/2), q_k = sqrt(2/P) Im X_k (k > P/2)
// (with Im X_{P-k} = -Im X_k for real input)
// (normal_modes.cpp:52-79).  Two particles share one complex FFT (real and
// imaginary parts); radix-2 Stockham stages in shared memory with twiddles
// tw[t] = exp(-2 pi i t / P), t < P/2.  The inverse builds the Hermitian
// spectra of C^T and runs the conjugate transform.
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// One Stockham radix-2 pass structure for `nf` transforms; stage 0 gets its
// operands from `load(f, b)`.  Returns the buffer holding out[f * P + k].
template <class Load>
__device__ double2* fft_stages(Load load, int nf, int P, int logP, const double2* __restrict__ tw, bool inv,
                               double2* w0, double2* w1) {
    const int half = P >> 1;
    const double2* src = nullptr;
    double2* dst = w0;
    for (int st = 0, Ns = 1; st < logP; ++st, Ns <<= 1) {
        for (int e = threadIdx.x; e < nf * half; e += blockDim.x) {
            const int f = e / half, j = e - f * half;
            double2 v0, v1;
            if (st == 0) {
                v0 = load(f, j);
                v1 = load(f, j + half);
            } else {
                v0 = src[f * P + j];
                v1 = src[f * P + j + half];
            }
            const int k = j & (Ns - 1);
            double2 t = tw[k * (half / Ns)];
            if (inv) t.y = -t.y;
            const double2 bb = cmul(v1, t);
            const int o = f * P + (j - k) * 2 + k;
            dst[o] = make_double2(v0.x + bb.x, v0.y + bb.y);
            dst[o + Ns] = make_double2(v0.x - bb.x, v0.y - bb.y);
        }
        __syncthreads();
        src = dst;
        dst = (dst == w0) ? w1 : w0;
    }
    return const_cast<double2*>(src);
}

// in[n] -> out[n] for n < narr: arrays of [P][kNmTile] doubles (bead or mode major).
struct NmArrays {
    const double* in[3];
    double* out[3];
};

__device__ void nm_forward_fft(const NmArrays& ar, int narr, int P, int logP, const double2* __restrict__ tw,
                               double2* w0, double2* w1) {
    const int nf = narr * (kNmTile / 2);
    auto load = [&](int f, int b) {
        const double* a = ar.in[f / (kNmTile / 2)] + 2 * (f % (kNmTile / 2));
        return make_double2(a[b * kNmTile], a[b * kNmTile + 1]);
    };
    const double2* R = fft_stages(load, nf, P, logP, tw, false, w0, w1);
    const int half = P >> 1;
    const double c = sqrt(2.0 / P), c0 = 1.0 / sqrt((double)P);
    for (int e = threadIdx.x; e < nf * (half + 1); e += blockDim.x) {
        const int f = e / (half + 1), k = e - f * (half + 1);
        const double2 Zk = R[f * P + k], Zm = R[f * P + ((P - k) & (P - 1))];
        const double xar = 0.5 * (Zk.x + Zm.x), xai = 0.5 * (Zk.y - Zm.y);
        const double xbr = 0.5 * (Zk.y + Zm.y), xbi = 0.5 * (Zm.x - Zk.x);
        double* o = ar.out[f / (kNmTile / 2)] + 2 * (f % (kNmTile / 2));
        if (k == 0 || k == half) {
            o[k * kNmTile] = c0 * xar;
            o[k * kNmTile + 1] = c0 * xbr;
        } else {
            o[k * kNmTile] = c * xar;
            o[k * kNmTile + 1] = c * xbr;
            // q_{P-k} = sqrt(2/P) Im X_{P-k} = -sqrt(2/P) Im X_k (real input)
            o[(P - k) * kNmTile] = -c * xai;
            o[(P - k) * kNmTile + 1] = -c * xbi;
        }
    }
    __syncthreads();
}

// Normal modes -> Cartesian for ar.in[0..narr); result[f * P + j] = x_a + i x_b
// for particles 2 (f % 4), 2 (f % 4) + 1 of array f / 4.
__device__ const double2* nm_inverse_fft(const NmArrays& ar, int narr, int P, int logP,
                                         const double2* __restrict__ tw, double2* w0, double2* w1) {
    const int nf = narr * (kNmTile / 2);
    const int half = P >> 1;
    const double c = 0.5 * sqrt(2.0 / P), c0 = 1.0 / sqrt((double)P);
    auto load = [&](int f, int k) {
        const double* a = ar.in[f / (kNmTile / 2)] + 2 * (f % (kNmTile / 2));
        double zar, zai, zbr, zbi;
        if (k == 0 || k == half) {
            zar = c0 * a[k * kNmTile];
            zbr = c0 * a[k * kNmTile + 1];
            zai = zbi = 0.0;
        } else if (k < half) {
            zar = c * a[k * kNmTile];
            zai = -c * a[(P - k) * kNmTile];
            zbr = c * a[k * kNmTile + 1];
            zbi = -c * a[(P - k) * kNmTile + 1];
        } else {
            zar = c * a[(P - k) * kNmTile];
            zai = c * a[k * kNmTile];
            zbr = c * a[(P - k) * kNmTile + 1];
            zbi = c * a[k * kNmTile + 1];
        }
        return make_double2(zar - zbi, zai + zbr);
    };
    return fft_stages(load, nf, P, logP, tw, true, w0, w1);
}

// ---------------------------------------------------------------------------
// Fused normal-mode step for the normal-mode propagator with the
// normal-mode Langevin thermostat.  Between two force evaluations the
// reference applies (normal_modes_propagator.cpp:19-103,
// thermostat_coupling.cpp:29-47, simulation.cpp:246-259):
//   tail of step s-1:  kick(F), O (normal modes), COM removal
//   head of step s:    O (normal modes), COM removal, kick(F), free ring rotation
// Every piece is linear in the normal-mode frame, so one kernel transforms
// p, the kick force F and x once, applies all of it in that frame and
// transforms x and p back: 5 bead transforms instead of 8.  The COM removal
// becomes a shift of the centroid mode (C's first row is 1/sqrt(P), every
// other row sums to zero), which needs the sum over all particles: blocks
// meet at a grid barrier (cooperative launch, so all blocks are resident; the
// barrier gives up after a bounded number of polls and raises ERRB_TIMEOUT).
// mode bit 0: tail of step-1, bit 1: head of step.

__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned nblocks, int* err) {
    __syncthreads();
    __shared__ int timed_out;
    if (threadIdx.x == 0) {
        timed_out = 0;
        volatile unsigned* gen = bar + 1;
        const unsigned my = *gen;
        __threadfence();
        if (atomicAdd(bar, 1u) == nblocks - 1) {
            bar[0] = 0;
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            unsigned it = 0;
            while (*gen == my) {
                if (++it > (1u << 24)) {
                    atomicOr(err, ERRB_TIMEOUT);
                    timed_out = 1;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return !timed_out;
}

template <int D>
__global__ void __launch_bounds__(kNmThreads) k_nm_fused(Sys s, const double* __restrict__ C,
                                                         const double* __restrict__ T,
                                                         const double* __restrict__ rot, double* cmpart,
                                                         unsigned* bar, int mode, StepRef sref, int fixcom,
                                                         const double2* __restrict__ tw, int logP) {
    const long long step = sref.get();
    extern __shared__ double sm[];
    __shared__ double shred[32];
    const int P = s.P;
    double* sp = sm;                    // p, later C p
    double* sf = sm + P * kNmTile;      // kick force, later C F
    double* sx = sm + 2 * P * kNmTile;  // x, later C x
    double* sq = sm + 3 * P * kNmTile;  // normal-mode p
    double* sg = sm + 4 * P * kNmTile;  // normal-mode F
    double* sy = sm + 5 * P * kNmTile;  // normal-mode x
    const int a = blockIdx.y;
    const int i0 = blockIdx.x * kNmTile;
    const int pp = threadIdx.x % kNmPairs, g = threadIdx.x / kNmPairs;
    const int nblocks = gridDim.x * gridDim.y;
    const int bid = blockIdx.y * gridDim.x + blockIdx.x;
    const bool head = mode & 2, tail = mode & 1;
    for (int e = threadIdx.x; e < P * kNmTile; e += blockDim.x) {
        const int b = e / kNmTile, il = e % kNmTile, i = i0 + il;
        double x = 0.0, p = 0.0, f = 0.0;
        if (i < s.N) {
            const size_t o = idx<D>(s, b, a, i);
            x = s.x[o];
            p = s.p[o];
            f = nm_kick_force<D>(s, b, a, i);
        }
        sx[e] = x;
        sp[e] = p;
        sf[e] = f;
    }
    __syncthreads();
    double2* w0 = reinterpret_cast<double2*>(sm + 6 * P * kNmTile);
    double2* w1 = w0 + 3 * (kNmTile / 2) * P;
    if (tw) {
        NmArrays ar = {{sp, sf, sx}, {sq, sg, sy}};
        nm_forward_fft(ar, head ? 3 : 2, P, logP, tw, w0, w1);
    } else {
    for (int k = g; k < P; k += kNmGroups) {
        double q0 = 0.0, q1 = 0.0, f0 = 0.0, f1 = 0.0, x0 = 0.0, x1 = 0.0;
        const double* ck = C + (size_t)k * P;
        for (int b = 0; b < P; ++b) {
            const double c = ck[b];
            const int o = b * kNmTile + 2 * pp;
            q0 += c * sp[o];
            q1 += c * sp[o + 1];
            f0 += c * sf[o];
            f1 += c * sf[o + 1];
            if (head) {
                x0 += c * sx[o];
                x1 += c * sx[o + 1];
            }
        }
        const int o = k * kNmTile + 2 * pp;
        sq[o] = q0;
        sq[o + 1] = q1;
        sg[o] = f0;
        sg[o + 1] = f1;
        sy[o] = x0;
        sy[o + 1] = x1;
    }
    __syncthreads();
    }
    const int half = (s.N + 1) / 2;
    const double hdt = 0.5 * s.dt;
    const double sqrtP = sqrt((double)P);
    const double cm_scale = sqrtP * sqrtP / ((double)s.N * (double)P);  // q0 -> sqrt(P) cm
    auto thermostat = [&](uint64_t t) {
        for (int k = g; k < P; k += kNmGroups) {
            const int o = k * kNmTile + 2 * pp;
            const int ie = i0 + 2 * pp;
            const double2 z = langevin_pair<D>(s, t, k, a, ie >> 1, half);
            sq[o] = s.c1 * sq[o] + s.c2 * z.x;
            sq[o + 1] = s.c1 * sq[o + 1] + s.c2 * z.y;
        }
        __syncthreads();
    };
    auto remove_com = [&](int buf) -> bool {
        // centroid sum of this tile (real particles only), grid barrier,
        // then every block subtracts sqrt(P) cm from its centroid mode.  The
        // two removals of one launch use separate halves of cmpart.
        double* cp = cmpart + (size_t)buf * nblocks;
        double part = 0.0;
        if (threadIdx.x < kNmTile && i0 + (int)threadIdx.x < s.N) part = sq[threadIdx.x];
        const double tsum = block_sum(part, shred);
        if (threadIdx.x == 0) cp[bid] = tsum;
        if (!grid_barrier(bar, nblocks, s.err)) return false;
        double acc = 0.0;
        for (int k = threadIdx.x; k < gridDim.x; k += blockDim.x) acc += ((volatile double*)cp)[a * gridDim.x + k];
        const double shift = block_sum(acc, shred) * cm_scale;  // sqrt(P) * cm
        if (threadIdx.x < kNmTile) sq[threadIdx.x] -= shift;
        __syncthreads();
        return true;
    };
    if (tail) {
        for (int e = threadIdx.x; e < P * kNmTile; e += blockDim.x) sq[e] += hdt * sg[e];
        __syncthreads();
        thermostat(2ull * (unsigned long long)(step - 1) + 1);
        // With the head in the same launch one removal, after the head's
        // O-step, stands for both: the removal is a linear projection and the
        // O-step affine, so COM(O2(COM(O1 p))) = COM(O2(O1 p)).
        if (fixcom && !head && !remove_com(0)) return;
    }
    if (head) {
        thermostat(2ull * (unsigned long long)step);
        if (fixcom && !remove_com(1)) return;
        for (int k = g; k < P; k += kNmGroups) {
            const double cs = rot[4 * k], sn = rot[4 * k + 1], mw = rot[4 * k + 2], snw = rot[4 * k + 3];
            for (int h2 = 0; h2 < 2; ++h2) {
                const int o = k * kNmTile + 2 * pp + h2;
                const double q = sy[o];
                const double pk = sq[o] + hdt * sg[o];
                if (mw == 0.0) {
                    sy[o] = q + s.dt_m * pk;
                    sq[o] = pk;
                } else {
                    sy[o] = cs * q + snw * pk;
                    sq[o] = -mw * sn * q + cs * pk;
                }
            }
        }
        __syncthreads();
    }
    if (tw) {
        NmArrays ar = {{sq, sy, nullptr}, {nullptr, nullptr, nullptr}};
        const double2* R = nm_inverse_fft(ar, head ? 2 : 1, P, logP, tw, w0, w1);
        for (int e = threadIdx.x; e < P * (kNmTile / 2); e += blockDim.x) {
            const int j = e / (kNmTile / 2), q = e % (kNmTile / 2);
            const int ie = i0 + 2 * q;
            const double2 pv = R[q * P + j];
            double2 xv = make_double2(0.0, 0.0);
            if (head) xv = R[((kNmTile / 2) + q) * P + j];
            if (ie < s.N) {
                const size_t o = idx<D>(s, j, a, ie);
                s.p[o] = pv.x;
                if (head) s.x[o] = xv.x;
            }
            if (ie + 1 < s.N) {
                const size_t o = idx<D>(s, j, a, ie + 1);
                s.p[o] = pv.y;
                if (head) s.x[o] = xv.y;
            }
        }
        return;
    }
    for (int j = g; j < P; j += kNmGroups) {
        double x0 = 0.0, x1 = 0.0, v0 = 0.0, v1 = 0.0;
        const double* tj = T + (size_t)j * P;
        for (int k = 0; k < P; ++k) {
            const double c = tj[k];
            const int o = k * kNmTile + 2 * pp;
            v0 += c * sq[o];
            v1 += c * sq[o + 1];
            if (head) {
                x0 += c * sy[o];
                x1 += c * sy[o + 1];
            }
        }
        const int ie = i0 + 2 * pp;
        if (ie < s.N) {
            const size_t o = idx<D>(s, j, a, ie);
            s.p[o] = v0;
            if (head) s.x[o] = x0;
        }
        if (ie + 1 < s.N) {
            const size_t o = idx<D>(s, j, a, ie + 1);
            s.p[o] = v1;
            if (head) s.x[o] = x1;
        }
    }
}

// ---------------------------------------------------------------------------
// The same fused step with the transforms in registers, for P = 32 E
// (E = 1, 2, 4).  One warp per (particle pair, axis): the pair's two real
// sequences are the real and imaginary parts of one complex sequence, and
// lane l holds beads l + 32 e.  Forward: with n = 32 e + l and k = k1 + E k2,
//   Z_k = sum_l W_32^(l k2) [W_P^(l k1) sum_e z_(32e+l) W_E^(e k1)]:
// an E-point DFT in the lane, the twiddles, then a 32-point radix-2
// decimation in frequency across lanes (shuffles, no block barriers); mode k
// ends in element k1 of lane bitrev5(k2).  Every normal-mode operation (kick,
// O-step, COM shift, free rotation) is per mode, in registers.  The inverse
// runs the same steps backwards (decimation in time across lanes from the
// bit-reversed order), which leaves bead n = 32 e + l in element e of lane l.
// Only the COM removal still meets at a grid barrier.

__device__ __forceinline__ double2 shfl_xor_d2(double2 v, int m) {
    return make_double2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}
__device__ __forceinline__ double2 shfl_d2(double2 v, int src) {
    return make_double2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}
// W_P^t = exp(-2 pi i t / P), 0 <= t < P, from tw[t] (t < P/2)
__device__ __forceinline__ double2 twid(const double2* tw, int t, int half) {
    const double2 w = tw[t & (half - 1)];
    return t < half ? w : make_double2(-w.x, -w.y);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }

template <int E>
__device__ __forceinline__ void warp_fft_fwd(double2 (&z)[E], const double2* tw, int P, int lane) {
    const int half = P >> 1;
    if constexpr (E == 2) {
        const double2 a = z[0], b = z[1];
        z[0] = cadd(a, b);
        z[1] = csub(a, b);
    } else if constexpr (E == 4) {
        const double2 a = cadd(z[0], z[2]), b = csub(z[0], z[2]), c = cadd(z[1], z[3]), d = csub(z[1], z[3]);
        z[0] = cadd(a, c);
        z[2] = csub(a, c);
        z[1] = make_double2(b.x + d.y, b.y - d.x);  // b - i d
        z[3] = make_double2(b.x - d.y, b.y + d.x);  // b + i d
    }
#pragma unroll
    for (int k1 = 1; k1 < E; ++k1) z[k1] = cmul(z[k1], twid(tw, lane * k1, half));
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
        const bool upper = (lane & d) != 0;
        const double2 w = upper ? twid(tw, (lane & (d - 1)) * (P / (2 * d)), half) : make_double2(1.0, 0.0);
#pragma unroll
        for (int k1 = 0; k1 < E; ++k1) {
            const double2 o = shfl_xor_d2(z[k1], d);
            const double2 own = upper ? make_double2(-z[k1].x, -z[k1].y) : z[k1];
            z[k1] = cmul(cadd(o, own), w);  // lower: own + other; upper: (other - own) w
        }
    }
}

template <int E>
__device__ __forceinline__ void warp_fft_inv(double2 (&z)[E], const double2* tw, int P, int lane) {
    const int half = P >> 1;
#pragma unroll
    for (int d = 1; d <= 16; d <<= 1) {
        const bool upper = (lane & d) != 0;
        const double2 w = cconj(twid(tw, (lane & (d - 1)) * (P / (2 * d)), half));
#pragma unroll
        for (int k1 = 0; k1 < E; ++k1) {
            const double2 o = shfl_xor_d2(z[k1], d);
            const double2 t = cmul(upper ? z[k1] : o, w);   // the upper element, turned
            const double2 lo = upper ? o : z[k1];
            z[k1] = upper ? csub(lo, t) : cadd(lo, t);
        }
    }
#pragma unroll
    for (int k1 = 1; k1 < E; ++k1) z[k1] = cmul(z[k1], cconj(twid(tw, lane * k1, half)));
    if constexpr (E == 2) {
        const double2 a = z[0], b = z[1];
        z[0] = cadd(a, b);
        z[1] = csub(a, b);
    } else if constexpr (E == 4) {
        const double2 a = cadd(z[0], z[2]), b = csub(z[0], z[2]), c = cadd(z[1], z[3]), d = csub(z[1], z[3]);
        z[0] = cadd(a, c);
        z[2] = csub(a, c);
        z[1] = make_double2(b.x - d.y, b.y + d.x);  // b + i d
        z[3] = make_double2(b.x + d.y, b.y - d.x);  // b - i d
    }
}

// The value that element k1 of lane `lane` holds for mode P - k.
template <int E>
__device__ __forceinline__ double2 mode_partner(const double2 (&v)[E], int k1, int lane) {
    if (k1 == 0) {
        const int k2 = (int)(__brev((unsigned)lane) >> 27);
        return shfl_d2(v[0], (int)(__brev((unsigned)((32 - k2) & 31)) >> 27));
    }
    return shfl_d2(v[E - k1], lane ^ 31);
}

// Spectrum Z of two real sequences -> their normal-mode coordinates (a, b):
//   q_k = c0 Re X_k (k = 0, P/2), c Re X_k (k < P/2), c Im X_k (k > P/2).
template <int E>
__device__ __forceinline__ void warp_to_modes(double2 (&z)[E], int P, int lane) {
    const double c = sqrt(2.0 / P), c0 = 1.0 / sqrt((double)P);
    const int half = P >> 1;
    double2 q[E];
#pragma unroll
    for (int k1 = 0; k1 < E; ++k1) {
        const double2 zp = mode_partner<E>(z, k1, lane);
        const int k = k1 + E * (int)(__brev((unsigned)lane) >> 27);
        const double xar = 0.5 * (z[k1].x + zp.x), xai = 0.5 * (z[k1].y - zp.y);
        const double xbr = 0.5 * (z[k1].y + zp.y), xbi = 0.5 * (zp.x - z[k1].x);
        if (k == 0 || k == half) q[k1] = make_double2(c0 * xar, c0 * xbr);
        else if (k < half) q[k1] = make_double2(c * xar, c * xbr);
        else q[k1] = make_double2(c * xai, c * xbi);
    }
#pragma unroll
    for (int k1 = 0; k1 < E; ++k1) z[k1] = q[k1];
}

// Normal-mode coordinates (a, b) -> the spectrum whose conjugate transform
// gives x_a + i x_b (the block kernel's nm_inverse_fft load).
template <int E>
__device__ __forceinline__ void warp_from_modes(double2 (&q)[E], int P, int lane) {
    const double c = 0.5 * sqrt(2.0 / P), c0 = 1.0 / sqrt((double)P);
    const int half = P >> 1;
    double2 z[E];
#pragma unroll
    for (int k1 = 0; k1 < E; ++k1) {
        const double2 qp = mode_partner<E>(q, k1, lane);
        const int k = k1 + E * (int)(__brev((unsigned)lane) >> 27);
        double zar, zai, zbr, zbi;
        if (k == 0 || k == half) {
            zar = c0 * q[k1].x;
            zbr = c0 * q[k1].y;
            zai = zbi = 0.0;
        } else if (k < half) {
            zar = c * q[k1].x;
            zai = -c * qp.x;
            zbr = c * q[k1].y;
            zbi = -c * qp.y;
        } else {
            zar = c * qp.x;
            zai = c * q[k1].x;
            zbr = c * qp.y;
            zbi = c * q[k1].y;
        }
        z[k1] = make_double2(zar - zbi, zai + zbr);
    }
#pragma unroll
    for (int k1 = 0; k1 < E; ++k1) q[k1] = z[k1];
}

template <int D, int E>
__global__ void __launch_bounds__(256) k_nm_warp(Sys s, const double* __restrict__ rot, double* cmpart, unsigned* bar,
                                                 int mode, StepRef sref, int fixcom, const double2* __restrict__ tw_g) {
    constexpr int P = 32 * E;
    __shared__ double2 tw[P / 2];
    for (int t = threadIdx.x; t < P / 2; t += blockDim.x) tw[t] = tw_g[t];
    __syncthreads();
    const long long step = sref.get();
    const int lane = threadIdx.x & 31;
    const int half = (s.N + 1) / 2;
    const int nwarps = D * half;
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const bool live = w < nwarps;  // idle warps still meet the block's barriers
    const int a = live ? w / half : 0, i2 = live ? w % half : 0;
    const int ia = 2 * i2, ib = 2 * i2 + 1;
    const bool va = live && ia < s.N, vb = live && ib < s.N;
    const bool head = mode & 2, tail = mode & 1;
    double2 zp[E], zf[E], zx[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int b = 32 * e + lane;
        zp[e] = zf[e] = zx[e] = make_double2(0.0, 0.0);
        if (va) {
            const size_t o = idx<D>(s, b, a, ia);
            zp[e].x = s.p[o];
            zx[e].x = s.x[o];
            zf[e].x = nm_kick_force<D>(s, b, a, ia);
        }
        if (vb) {
            const size_t o = idx<D>(s, b, a, ib);
            zp[e].y = s.p[o];
            zx[e].y = s.x[o];
            zf[e].y = nm_kick_force<D>(s, b, a, ib);
        }
    }
    warp_fft_fwd<E>(zp, tw, P, lane);
    warp_fft_fwd<E>(zf, tw, P, lane);
    if (head) warp_fft_fwd<E>(zx, tw, P, lane);
    warp_to_modes<E>(zp, P, lane);
    warp_to_modes<E>(zf, P, lane);
    if (head) warp_to_modes<E>(zx, P, lane);
    const double hdt = 0.5 * s.dt;
    const int k2 = (int)(__brev((unsigned)lane) >> 27);
    auto thermostat = [&](uint64_t t) {
#pragma unroll
        for (int k1 = 0; k1 < E; ++k1) {
            const double2 z = langevin_pair<D>(s, t, k1 + E * k2, a, i2, half);
            zp[k1].x = s.c1 * zp[k1].x + s.c2 * z.x;
            zp[k1].y = s.c1 * zp[k1].y + s.c2 * z.y;
        }
    };
    // centroid (mode 0: element 0 of lane 0) of every particle, one partial
    // per warp; after the grid barrier each warp adds its axis' partials in
    // order and shifts its own centroid mode by sqrt(P) cm
    const double cm_scale = 1.0 / (double)s.N;
    auto remove_com = [&](int buf) -> bool {
        double* cp = cmpart + (size_t)buf * nwarps;
        if (live && lane == 0) cp[w] = (va ? zp[0].x : 0.0) + (vb ? zp[0].y : 0.0);
        if (!grid_barrier(bar, gridDim.x, s.err)) return false;
        double acc = 0.0;
        if (live)
            for (int k = lane; k < half; k += 32) acc += ((volatile double*)cp)[a * half + k];
        const double shift = warp_sum(acc) * cm_scale;
        if (lane == 0) {
            zp[0].x -= shift;
            zp[0].y -= shift;
        }
        return true;
    };
    if (tail) {
#pragma unroll
        for (int k1 = 0; k1 < E; ++k1) {
            zp[k1].x += hdt * zf[k1].x;
            zp[k1].y += hdt * zf[k1].y;
        }
        thermostat(2ull * (unsigned long long)(step - 1) + 1);
        // with the head in this launch one removal after its O-step stands
        // for both (the removal commutes through the affine O-step)
        if (fixcom && !head && !remove_com(0)) return;
    }
    if (head) {
        thermostat(2ull * (unsigned long long)step);
        if (fixcom && !remove_com(1)) return;
#pragma unroll
        for (int k1 = 0; k1 < E; ++k1) {
            const int k = k1 + E * k2;
            const double cs = rot[4 * k], sn = rot[4 * k + 1], mw = rot[4 * k + 2], snw = rot[4 * k + 3];
            // kick, then the free ring rotation of (q, p) in mode k
            auto turn = [&](double& q, double& pm, double g) {
                const double q0 = q, pk = pm + hdt * g;
                if (mw == 0.0) {
                    q = q0 + s.dt_m * pk;
                    pm = pk;
                } else {
                    q = cs * q0 + snw * pk;
                    pm = -mw * sn * q0 + cs * pk;
                }
            };
            turn(zx[k1].x, zp[k1].x, zf[k1].x);
            turn(zx[k1].y, zp[k1].y, zf[k1].y);
        }
    }
    warp_from_modes<E>(zp, P, lane);
    warp_fft_inv<E>(zp, tw, P, lane);
    if (head) {
        warp_from_modes<E>(zx, P, lane);
        warp_fft_inv<E>(zx, tw, P, lane);
    }
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int b = 32 * e + lane;
        if (va) {
            const size_t o = idx<D>(s, b, a, ia);
            s.p[o] = zp[e].x;
            if (head) s.x[o] = zx[e].x;
        }
        if (vb) {
            const size_t o = idx<D>(s, b, a, ib);
            s.p[o] = zp[e].y;
            if (head) s.x[o] = zx[e].y;
        }
    }
}

// Three warps per (particle pair, axis): warp 0 transforms p, warp 1 the
// kick force, warp 2 x, each in registers as above, so the transforms run
// side by side; the modes of F and x meet warp 0's in shared memory for the
// per-mode operations, and warps 0 and 2 transform p and x back.  Used when
// every block can be resident (the COM removal's grid barrier).
template <int D, int E>
__global__ void __launch_bounds__(96) k_nm_warp3(Sys s, const double* __restrict__ rot, double* cmpart, unsigned* bar,
                                                 int mode, StepRef sref, int fixcom, const double2* __restrict__ tw_g,
                                                 double2* __restrict__ mp, double2* __restrict__ mx, int use_modes) {
    constexpr int P = 32 * E;
    __shared__ double2 tw[P / 2];
    __shared__ double2 sF[E][32], sX[E][32];
    for (int t = threadIdx.x; t < P / 2; t += blockDim.x) tw[t] = tw_g[t];
    __syncthreads();
    const long long step = sref.get();
    const int lane = threadIdx.x & 31, role = threadIdx.x >> 5;  // 0: p, 1: F, 2: x
    const int half = (s.N + 1) / 2;
    const int u = blockIdx.x;  // (axis, particle pair)
    const int a = u / half, i2 = u % half;
    const int ia = 2 * i2, ib = 2 * i2 + 1;
    const bool va = ia < s.N, vb = ib < s.N;
    const bool head = mode & 2, tail = mode & 1;
    const int k2 = (int)(__brev((unsigned)lane) >> 27);
    double2 z[E];
    // The normal modes of p and x as the previous head left them (in this
    // warp's register order), when nothing has changed x or p since: no
    // forward transform for those two.
    const size_t mbase = (size_t)blockIdx.x * E * 32 + lane;
    const bool cached = use_modes && mp && (role == 0 || (role == 2 && head));
    if (cached) {
        const double2* src = role == 0 ? mp : mx;
#pragma unroll
        for (int k1 = 0; k1 < E; ++k1) z[k1] = src[mbase + (size_t)k1 * 32];
        if (role == 2) {
#pragma unroll
            for (int k1 = 0; k1 < E; ++k1) sX[k1][lane] = z[k1];
        }
    } else if (role == 0 || role == 1 || head) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int b = 32 * e + lane;
            z[e] = make_double2(0.0, 0.0);
            if (va) {
                const size_t o = idx<D>(s, b, a, ia);
                z[e].x = role == 0 ? s.p[o] : role == 2 ? s.x[o] : nm_kick_force<D>(s, b, a, ia);
            }
            if (vb) {
                const size_t o = idx<D>(s, b, a, ib);
                z[e].y = role == 0 ? s.p[o] : role == 2 ? s.x[o] : nm_kick_force<D>(s, b, a, ib);
            }
        }
        warp_fft_fwd<E>(z, tw, P, lane);
        warp_to_modes<E>(z, P, lane);
        if (role == 1) {
#pragma unroll
            for (int k1 = 0; k1 < E; ++k1) sF[k1][lane] = z[k1];
        } else if (role == 2) {
#pragma unroll
            for (int k1 = 0; k1 < E; ++k1) sX[k1][lane] = z[k1];
        }
    }
    __syncthreads();
    const double hdt = 0.5 * s.dt;
    auto thermostat = [&](uint64_t t) {
#pragma unroll
        for (int k1 = 0; k1 < E; ++k1) {
            const double2 zn = langevin_pair<D>(s, t, k1 + E * k2, a, i2, half);
            z[k1].x = s.c1 * z[k1].x + s.c2 * zn.x;
            z[k1].y = s.c1 * z[k1].y + s.c2 * zn.y;
        }
    };
    const int nunits = gridDim.x;
    const double cm_scale = 1.0 / (double)s.N;
    // every thread of the block takes part (the barrier's block syncs); the
    // centroid mode is element 0 of warp 0's lane 0
    auto remove_com = [&](int buf) -> bool {
        double* cp = cmpart + (size_t)buf * nunits;
        if (threadIdx.x == 0) cp[u] = (va ? z[0].x : 0.0) + (vb ? z[0].y : 0.0);
        if (!grid_barrier(bar, gridDim.x, s.err)) return false;
        if (role == 0) {
            double acc = 0.0;
            for (int k = lane; k < half; k += 32) acc += ((volatile double*)cp)[a * half + k];
            const double shift = warp_sum(acc) * cm_scale;
            if (lane == 0) {
                z[0].x -= shift;
                z[0].y -= shift;
            }
        }
        return true;
    };
    if (tail) {
        if (role == 0) {
#pragma unroll
            for (int k1 = 0; k1 < E; ++k1) {
                const double2 g = sF[k1][lane];
                z[k1].x += hdt * g.x;
                z[k1].y += hdt * g.y;
            }
            thermostat(2ull * (unsigned long long)(step - 1) + 1);
        }
        if (fixcom && !head && !remove_com(0)) return;
    }
    if (head) {
        if (role == 0) thermostat(2ull * (unsigned long long)step);
        if (fixcom && !remove_com(1)) return;
        if (role == 0) {
#pragma unroll
            for (int k1 = 0; k1 < E; ++k1) {
                const int k = k1 + E * k2;
                const double cs = rot[4 * k], sn = rot[4 * k + 1], mw = rot[4 * k + 2], snw = rot[4 * k + 3];
                const double2 g = sF[k1][lane];
                double2 q = sX[k1][lane];
                auto turn = [&](double& qv, double& pm, double gv) {
                    const double q0 = qv, pk = pm + hdt * gv;
                    if (mw == 0.0) {
                        qv = q0 + s.dt_m * pk;
                        pm = pk;
                    } else {
                        qv = cs * q0 + snw * pk;
                        pm = -mw * sn * q0 + cs * pk;
                    }
                };
                turn(q.x, z[k1].x, g.x);
                turn(q.y, z[k1].y, g.y);
                sX[k1][lane] = q;
            }
        }
        __syncthreads();
        if (role == 2) {
#pragma unroll
            for (int k1 = 0; k1 < E; ++k1) z[k1] = sX[k1][lane];
        }
        // the modes of this head, for the next launch
        if (mp && (role == 0 || role == 2)) {
            double2* dst = role == 0 ? mp : mx;
#pragma unroll
            for (int k1 = 0; k1 < E; ++k1) dst[mbase + (size_t)k1 * 32] = z[k1];
        }
    }
    if (role == 0 || (role == 2 && head)) {
        warp_from_modes<E>(z, P, lane);
        warp_fft_inv<E>(z, tw, P, lane);
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int b = 32 * e + lane;
            double* dst = role == 0 ? s.p : s.x;
            if (va) dst[idx<D>(s, b, a, ia)] = z[e].x;
            if (vb) dst[idx<D>(s, b, a, ib)] = z[e].y;
        }
    }
}

template <int D, int E>
static bool nm_warp3_fits(const Sys& s) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_nm_warp3<D, E>, 96, 0) != cudaSuccess) return false;
    return (long long)D * ((s.N + 1) / 2) <= (long long)per * sms;
}

// The normal-mode propagator's step (normal_modes_propagator.cpp:19-71:
// [COM], half-kick, free ring rotation) with the transforms in registers,
// for P = 32, 64, 128: two warps per (particle pair, axis), warp 0 on p and
// warp 1 on x; they swap modes in shared memory for the rotation.  No grid
// barrier: the pending COM correction comes reduced (`cmv`, or null).
template <int D, int E>
__global__ void __launch_bounds__(64) k_nm_prop_warp(Sys s, const double* __restrict__ rot,
                                                     const double* __restrict__ cmv,
                                                     const double2* __restrict__ tw_g) {
    constexpr int P = 32 * E;
    __shared__ double2 tw[P / 2];
    __shared__ double2 sm2[2][E][32];  // [0] p modes, [1] x modes
    for (int t = threadIdx.x; t < P / 2; t += blockDim.x) tw[t] = tw_g[t];
    __syncthreads();
    const int lane = threadIdx.x & 31, role = threadIdx.x >> 5;  // 0: p, 1: x
    const int half = (s.N + 1) / 2;
    const int u = blockIdx.x;
    const int a = u / half, i2 = u % half;
    const int ia = 2 * i2, ib = 2 * i2 + 1;
    const bool va = ia < s.N, vb = ib < s.N;
    const double cm = cmv ? cmv[a] : 0.0, hdt = 0.5 * s.dt;
    double2 z[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int b = 32 * e + lane;
        z[e] = make_double2(0.0, 0.0);
        if (va) {
            const size_t o = idx<D>(s, b, a, ia);
            z[e].x = role == 0 ? (s.p[o] - cm) + hdt * nm_kick_force<D>(s, b, a, ia) : s.x[o];
        }
        if (vb) {
            const size_t o = idx<D>(s, b, a, ib);
            z[e].y = role == 0 ? (s.p[o] - cm) + hdt * nm_kick_force<D>(s, b, a, ib) : s.x[o];
        }
    }
    warp_fft_fwd<E>(z, tw, P, lane);
    warp_to_modes<E>(z, P, lane);
#pragma unroll
    for (int k1 = 0; k1 < E; ++k1) sm2[role][k1][lane] = z[k1];
    __syncthreads();
    const int k2 = (int)(__brev((unsigned)lane) >> 27);
#pragma unroll
    for (int k1 = 0; k1 < E; ++k1) {
        const int k = k1 + E * k2;
        const double cs = rot[4 * k], sn = rot[4 * k + 1], mw = rot[4 * k + 2], snw = rot[4 * k + 3];
        const double2 pm = sm2[0][k1][lane], q = sm2[1][k1][lane];
        auto turn = [&](double q0, double p0) -> double {
            if (mw == 0.0) return role == 0 ? p0 : q0 + s.dt_m * p0;
            return role == 0 ? -mw * sn * q0 + cs * p0 : cs * q0 + snw * p0;
        };
        z[k1] = make_double2(turn(q.x, pm.x), turn(q.y, pm.y));
    }
    warp_from_modes<E>(z, P, lane);
    warp_fft_inv<E>(z, tw, P, lane);
    double* dst = role == 0 ? s.p : s.x;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int b = 32 * e + lane;
        if (va) dst[idx<D>(s, b, a, ia)] = z[e].x;
        if (vb) dst[idx<D>(s, b, a, ib)] = z[e].y;
    }
}

// The pending COM correction reduced once: cm[a] from the partial sums.
template <int D>
__global__ void k_com_mean(Sys s, const double* __restrict__ red_in, int nred, double* __restrict__ cm) {
    __shared__ double shred[32];
    double c[3] = {0.0, 0.0, 0.0};
    com_from_partials<D>(s, red_in, nred, c, shred);
    if (threadIdx.x == 0)
        for (int a = 0; a < D; ++a) cm[a] = c[a];
}

// Warps per block of the warp kernel: the fewest (spreading the pairs over
// the most SMs) with which every block is resident at once; 0 if none fits.
template <int D, int E>
static int nm_warp_block(const Sys& s) {
    if (nm_warp3_fits<D, E>(s)) return 3;  // three warps per pair and axis
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long nwarps = (long long)D * ((s.N + 1) / 2);
    for (int wpb = 1; wpb <= 8; wpb <<= 1) {  // one warp per pair and axis
        int per = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_nm_warp<D, E>, 32 * wpb, 0) != cudaSuccess) return 0;
        if ((nwarps + wpb - 1) / wpb <= (long long)per * sms) return wpb;
    }
    return 0;
}

template <int D>
static int nm_warp_block_d(const Sys& s) {
    if (s.P == 32) return nm_warp_block<D, 1>(s);
    if (s.P == 64) return nm_warp_block<D, 2>(s);
    if (s.P == 128) return nm_warp_block<D, 4>(s);
    return 0;
}

static int nm_warp_block_any(const Sys& s, int D) {
    if (D == 1) return nm_warp_block_d<1>(s);
    if (D == 2) return nm_warp_block_d<2>(s);
    return nm_warp_block_d<3>(s);
}

template <int D, int E>
static cudaError_t nm_warp_t(const Sys& s, const double* rot, double* cmpart, unsigned* bar, int mode, StepRef step,
                             int fixcom, const double2* tw, int wpb, cudaStream_t st, const NmModes* modes) {
    const long long nwarps = (long long)D * ((s.N + 1) / 2);
    if (wpb == 3) {
        Sys sc = s;
        double2* mp = modes ? modes->p : nullptr;
        double2* mx = modes ? modes->x : nullptr;
        int use = modes ? modes->use : 0;
        if (modes) modes->written = (mode & 2) != 0;
        void* args[] = {&sc, &rot, &cmpart, &bar, &mode, &step, &fixcom, &tw, &mp, &mx, &use};
        return cudaLaunchCooperativeKernel((void*)k_nm_warp3<D, E>, dim3((unsigned)nwarps), dim3(96), args, 0, st);
    }
    dim3 grid((unsigned)((nwarps + wpb - 1) / wpb));
    Sys sc = s;
    void* args[] = {&sc, &rot, &cmpart, &bar, &mode, &step, &fixcom, &tw};
    return cudaLaunchCooperativeKernel((void*)k_nm_warp<D, E>, grid, dim3(32 * wpb), args, 0, st);
}

template <int D>
static cudaError_t nm_warp_d(const Sys& s, const double* rot, double* cmpart, unsigned* bar, int mode, StepRef step,
                             int fixcom, const double2* tw, int wpb, cudaStream_t st, const NmModes* modes) {
    if (s.P == 32) return nm_warp_t<D, 1>(s, rot, cmpart, bar, mode, step, fixcom, tw, wpb, st, modes);
    if (s.P == 64) return nm_warp_t<D, 2>(s, rot, cmpart, bar, mode, step, fixcom, tw, wpb, st, modes);
    return nm_warp_t<D, 4>(s, rot, cmpart, bar, mode, step, fixcom, tw, wpb, st, modes);
}

// [6][P][kNmTile] arrays plus two FFT work buffers of 3 kNmPairs complex transforms
size_t nm_fused_smem(const Sys& s) {
    return sizeof(double) * (6 * (size_t)s.P * kNmTile + 2 * 2 * 3 * (kNmTile / 2) * (size_t)s.P);
}

template <int D>
static bool nm_fused_fits_t(const Sys& s) {
    const size_t smem = nm_fused_smem(s);
    if (smem > 200 * 1024) return false;
    // the kernel also has static shared memory, so opt in whenever the dynamic
    // part alone reaches the 48 KiB default
    if (cudaFuncSetAttribute(k_nm_fused<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return false;
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_nm_fused<D>, kNmThreads, smem) != cudaSuccess) return false;
    const long long need = (long long)((s.N + kNmTile - 1) / kNmTile) * D;
    return need <= (long long)per * sms;
}

bool nm_block_fits(const Sys& s, int D) {
    if (D == 1) return nm_fused_fits_t<1>(s);
    if (D == 2) return nm_fused_fits_t<2>(s);
    return nm_fused_fits_t<3>(s);
}

bool nm_fused_fits(const Sys& s, int D) { return nm_warp_block_any(s, D) > 0 || nm_block_fits(s, D); }

// one block per (axis, particle pair), E x 32 complex values each (P = 32 E)
size_t nm_mode_doubles(const Sys& s, int D) { return 2 * (size_t)D * ((s.N + 1) / 2) * (size_t)s.P; }

size_t nm_fused_partials(const Sys& s, int D) {
    return 2 * std::max((size_t)nm_blocks(s, D), (size_t)D * ((s.N + 1) / 2));
}

template <int D>
static cudaError_t nm_fused_t(const Sys& s, const double* C, const double* T, const double* rot, double* cmpart,
                              unsigned* bar, int mode, StepRef step, int fixcom, const double2* tw, int logP,
                              cudaStream_t st) {
    dim3 grid((s.N + kNmTile - 1) / kNmTile, D);
    Sys sc = s;
    void* args[] = {&sc, &C, &T, &rot, &cmpart, &bar, &mode, &step, &fixcom, &tw, &logP};
    return cudaLaunchCooperativeKernel((void*)k_nm_fused<D>, grid, dim3(kNmThreads), args, nm_fused_smem(s), st);
}

cudaError_t launch_nm_fused(const Sys& s, int D, const double* C, const double* T, const double* rot, double* cmpart,
                            unsigned* bar, int mode, StepRef step, int fixcom, const double2* tw, int logP,
                            cudaStream_t st, const NmModes* modes) {
    // the warp kernel when P = 32, 64 or 128 and the FFTs are selected (or
    // the block kernel cannot be resident); the block kernel otherwise
    if (modes) modes->written = false;
    static int wpb_cache[4] = {-1, -1, -1, -1};
    static long long wpb_key[4] = {-1, -1, -1, -1};
    const long long key = ((long long)s.N << 20) | s.P;
    if (wpb_key[D] != key) {
        wpb_cache[D] = nm_warp_block_any(s, D);
        wpb_key[D] = key;
    }
    const int wpb = wpb_cache[D];
    if (wpb > 0 && tw) {
        if (D == 1) return nm_warp_d<1>(s, rot, cmpart, bar, mode, step, fixcom, tw, wpb, st, modes);
        if (D == 2) return nm_warp_d<2>(s, rot, cmpart, bar, mode, step, fixcom, tw, wpb, st, modes);
        return nm_warp_d<3>(s, rot, cmpart, bar, mode, step, fixcom, tw, wpb, st, modes);
    }
    if (D == 1) return nm_fused_t<1>(s, C, T, rot, cmpart, bar, mode, step, fixcom, tw, logP, st);
    if (D == 2) return nm_fused_t<2>(s, C, T, rot, cmpart, bar, mode, step, fixcom, tw, logP, st);
    return nm_fused_t<3>(s, C, T, rot, cmpart, bar, mode, step, fixcom, tw, logP, st);
}

// ---------------------------------------------------------------------------
// Nose-Hoover chains (src/thermostats/nose_hoover.cpp): one chain per bead
// over all its degrees of freedom (variant 0), per bead and particle (1), or
// per degree of freedom (2); with the normal-mode coupling the "beads" are
// the normal modes of momenta transformed by k_bead_transform.  Every chain
// integrates singleChainStep (:98-144, Tuckerman et al. 2006) in the
// reference's operation order and rescales its momenta.

// singleChainStep on one chain; returns the momentum scale
__device__ __forceinline__ double nh_chain_step(const NHPar& q, double current_energy, double* eta, double* eta_dot,
                                                double* eta_dd) {
    const int M = q.nchains;
    double exp_factor = 0.0;
    eta_dd[0] = (current_energy - q.required) / q.Q1;
    eta_dot[M - 1] += eta_dd[M - 1] * q.dt4;
    for (int i = M - 2; i >= 0; i--) {
        exp_factor = exp(-q.dt8 * eta_dot[i + 1]);
        eta_dot[i] *= exp_factor;
        eta_dot[i] += eta_dd[i] * q.dt4;
        eta_dot[i] *= exp_factor;
    }
    const double scale = exp(-q.dt2 * eta_dot[0]);
    for (int i = 0; i < M; i++) eta[i] += q.dt2 * eta_dot[i];
    eta_dd[0] = (current_energy * scale * scale - q.required) / q.Q1;
    eta_dot[0] *= exp_factor;
    eta_dot[0] += eta_dd[0] * q.dt4;
    eta_dot[0] *= exp_factor;
    double Q_former = q.Q1;
    for (int i = 1; i < M - 1; i++) {
        exp_factor = exp(-q.dt8 * eta_dot[i + 1]);
        eta_dot[i] *= exp_factor;
        eta_dd[i] = (Q_former * eta_dot[i - 1] * eta_dot[i - 1] - 1 / q.thermo_beta) / q.Qi;
        eta_dot[i] += eta_dd[i] * q.dt4;
        eta_dot[i] *= exp_factor;
        Q_former = q.Qi;
    }
    eta_dd[M - 1] = (q.Qi * eta_dot[M - 2] * eta_dot[M - 2] - 1 / q.thermo_beta) / q.Qi;
    eta_dot[M - 1] += eta_dd[M - 1] * q.dt4;
    return scale;
}

template <int D>
__global__ void k_nose_hoover(Sys s, NHPar q, double* __restrict__ pa) {
    const int M = q.nchains;
    if (q.variant == 0) {  // one chain per bead: block b
        __shared__ double red[32];
        __shared__ double sscale;
        const int b = blockIdx.x;
        double e = 0.0;
        for (int t = threadIdx.x; t < D * s.N; t += blockDim.x) {
            const int a = t / s.N, i = t - a * s.N;
            const double pv = pa[idx<D>(s, b, a, i)];
            e += pv * pv;
        }
        e = block_sum(e, red);
        if (threadIdx.x == 0) {
            const size_t c = (size_t)b * M;
            sscale = nh_chain_step(q, e / s.mass, q.eta + c, q.eta_dot + c, q.eta_dd + c);
        }
        __syncthreads();
        const double scale = sscale;
        for (int t = threadIdx.x; t < D * s.N; t += blockDim.x) {
            const int a = t / s.N, i = t - a * s.N;
            const size_t o = idx<D>(s, b, a, i);
            pa[o] = pa[o] * scale;
        }
        return;
    }
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (q.variant == 1) {  // one chain per bead and particle
        if (t >= (size_t)s.P * s.N) return;
        const int b = (int)(t / s.N), i = (int)(t % s.N);
        double e = 0.0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            const double pv = pa[idx<D>(s, b, a, i)];
            e += pv * pv;
        }
        const size_t c = t * M;
        const double scale = nh_chain_step(q, e / s.mass, q.eta + c, q.eta_dot + c, q.eta_dd + c);
#pragma unroll
        for (int a = 0; a < D; ++a) {
            const size_t o = idx<D>(s, b, a, i);
            pa[o] = pa[o] * scale;
        }
        return;
    }
    // one chain per degree of freedom, chain ((b N + i) D + a)
    if (t >= (size_t)s.P * s.N * D) return;
    const int a = (int)(t % D);
    const size_t bi = t / D;
    const int b = (int)(bi / s.N), i = (int)(bi % s.N);
    const size_t o = idx<D>(s, b, a, i);
    const double pv = pa[o];
    const size_t c = t * M;
    const double scale = nh_chain_step(q, pv * pv / s.mass, q.eta + c, q.eta_dot + c, q.eta_dd + c);
    pa[o] = pv * scale;
}

// out[k][a][i] = sum_j M[k][j] in[j][a][i] (bead <-> normal-mode rows, j
// ascending as in normal_modes.cpp:86-139)
template <int D>
__global__ void k_bead_transform(Sys s, const double* __restrict__ Mx, const double* __restrict__ in,
                                 double* __restrict__ out) {
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= (size_t)s.P * D * s.N) return;
    const int i = (int)(t % s.N);
    const size_t ka = t / s.N;
    const int a = (int)(ka % D), k = (int)(ka / D);
    double acc = 0.0;
    for (int j = 0; j < s.P; ++j) acc += Mx[(size_t)k * s.P + j] * in[idx<D>(s, j, a, i)];
    out[idx<D>(s, k, a, i)] = acc;
}

template <int D>
static void nose_hoover_t(const Sys& s, const NHPar& q, const double* C, const double* T, double* pnm,
                          cudaStream_t st) {
    const size_t ne = (size_t)s.P * D * s.N;
    const unsigned gt = (unsigned)((ne + 255) / 256);
    double* target = s.p;
    if (C) {
        k_bead_transform<D><<<gt, 256, 0, st>>>(s, C, s.p, pnm);
        target = pnm;
    }
    if (q.variant == 0) k_nose_hoover<D><<<s.P, 256, 0, st>>>(s, q, target);
    else if (q.variant == 1) k_nose_hoover<D><<<(unsigned)(((size_t)s.P * s.N + 255) / 256), 256, 0, st>>>(s, q, target);
    else k_nose_hoover<D><<<gt, 256, 0, st>>>(s, q, target);
    if (C) k_bead_transform<D><<<gt, 256, 0, st>>>(s, T, pnm, s.p);
}

int launch_nose_hoover(const Sys& s, int D, const NHPar& q, const double* C, const double* T, double* pnm,
                       cudaStream_t st) {
    if (D == 1) nose_hoover_t<1>(s, q, C, T, pnm, st);
    else if (D == 2) nose_hoover_t<2>(s, q, C, T, pnm, st);
    else nose_hoover_t<3>(s, q, C, T, pnm, st);
    return C ? 3 : 1;
}

// ------------------------------------------------------------------ launchers
static int pack_grid(size_t n) {
    size_t g = (n + 255) / 256;
    return (int)(g > 4096 ? 4096 : (g ? g : 1));
}

void launch_pack(const Sys& s, int D, const double* src, double* dst, cudaStream_t st) {
    const int g = pack_grid((size_t)s.P * s.N * D);
    if (D == 1) k_pack<1><<<g, 256, 0, st>>>(s, src, dst);
    else if (D == 2) k_pack<2><<<g, 256, 0, st>>>(s, src, dst);
    else k_pack<3><<<g, 256, 0, st>>>(s, src, dst);
}

void launch_unpack(const Sys& s, int D, const double* src, double* dst, cudaStream_t st) {
    const int g = pack_grid((size_t)s.P * s.N * D);
    if (D == 1) k_unpack<1><<<g, 256, 0, st>>>(s, src, dst);
    else if (D == 2) k_unpack<2><<<g, 256, 0, st>>>(s, src, dst);
    else k_unpack<3><<<g, 256, 0, st>>>(s, src, dst);
}

void launch_state_in(const Sys& s, int D, const double* sx, const double* sp, cudaStream_t st) {
    const size_t n = std::max((size_t)s.P * s.N * D, (size_t)s.P * D * s.ld);
    const int g = pack_grid(n);
    if (D == 1) k_state_in<1><<<g, 256, 0, st>>>(s, sx, sp);
    else if (D == 2) k_state_in<2><<<g, 256, 0, st>>>(s, sx, sp);
    else k_state_in<3><<<g, 256, 0, st>>>(s, sx, sp);
}

void launch_state_out(const Sys& s, int D, double* ox, double* op, double* of, cudaStream_t st) {
    const int g = pack_grid((size_t)s.P * s.N * D);
    if (D == 1) k_state_out<1><<<g, 256, 0, st>>>(s, ox, op, of);
    else if (D == 2) k_state_out<2><<<g, 256, 0, st>>>(s, ox, op, of);
    else k_state_out<3><<<g, 256, 0, st>>>(s, ox, op, of);
}

int cart_update_blocks(const Sys& s, int D) {
    const size_t total = (size_t)s.P * D * ((s.N + 1) / 2);
    return (int)((total + 255) / 256);
}

int nm_blocks(const Sys& s, int D) { return ((s.N + kNmTile - 1) / kNmTile) * D; }

void launch_cart_update(const Sys& s, int D, int flags, const double* red_in, int nred_in, double* red_out,
                        StepRef step, int substep, int kick_nm, cudaStream_t st) {
    const int g = cart_update_blocks(s, D);
    if (D == 1) k_cart_update<1><<<g, 256, 0, st>>>(s, flags, red_in, nred_in, red_out, step, substep, kick_nm);
    else if (D == 2) k_cart_update<2><<<g, 256, 0, st>>>(s, flags, red_in, nred_in, red_out, step, substep, kick_nm);
    else k_cart_update<3><<<g, 256, 0, st>>>(s, flags, red_in, nred_in, red_out, step, substep, kick_nm);
}

template <int D>
static void nm_thermo_launch(const Sys& s, const double* C, const double* T, int flags, const double* red_in,
                             int nred_in, double* red_out, StepRef step, int substep, cudaStream_t st) {
    const size_t smem = sizeof(double) * 2 * (size_t)s.P * kNmTile;
    cudaFuncSetAttribute(k_nm_thermo<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid((s.N + kNmTile - 1) / kNmTile, D);
    k_nm_thermo<D><<<grid, kNmThreads, smem, st>>>(s, C, T, flags, red_in, nred_in, red_out, step, substep);
}

void launch_nm_thermo(const Sys& s, int D, const double* C, const double* T, int flags, const double* red_in,
                      int nred_in, double* red_out, StepRef step, int substep, cudaStream_t st) {
    if (D == 1) nm_thermo_launch<1>(s, C, T, flags, red_in, nred_in, red_out, step, substep, st);
    else if (D == 2) nm_thermo_launch<2>(s, C, T, flags, red_in, nred_in, red_out, step, substep, st);
    else nm_thermo_launch<3>(s, C, T, flags, red_in, nred_in, red_out, step, substep, st);
}

template <int D>
static void nm_prop_launch(const Sys& s, const double* C, const double* T, const double* rot, int com_apply,
                           const double* red_in, int nred_in, cudaStream_t st) {
    const size_t smem = sizeof(double) * 4 * (size_t)s.P * kNmTile;
    cudaFuncSetAttribute(k_nm_propagate<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid((s.N + kNmTile - 1) / kNmTile, D);
    k_nm_propagate<D><<<grid, kNmThreads, smem, st>>>(s, C, T, rot, com_apply, red_in, nred_in);
}

template <int D, int E>
static void nm_prop_warp_t(const Sys& s, const double* rot, int com_apply, const double* red_in, int nred_in,
                           const double2* tw, double* cm, cudaStream_t st) {
    if (com_apply) k_com_mean<D><<<1, 256, 0, st>>>(s, red_in, nred_in, cm);
    const unsigned units = (unsigned)(D * ((s.N + 1) / 2));
    k_nm_prop_warp<D, E><<<units, 64, 0, st>>>(s, rot, com_apply ? cm : nullptr, tw);
}

template <int D>
static bool nm_prop_warp_d(const Sys& s, const double* rot, int com_apply, const double* red_in, int nred_in,
                           const double2* tw, double* cm, cudaStream_t st) {
    if (s.P == 32) nm_prop_warp_t<D, 1>(s, rot, com_apply, red_in, nred_in, tw, cm, st);
    else if (s.P == 64) nm_prop_warp_t<D, 2>(s, rot, com_apply, red_in, nred_in, tw, cm, st);
    else if (s.P == 128) nm_prop_warp_t<D, 4>(s, rot, com_apply, red_in, nred_in, tw, cm, st);
    else return false;
    return true;
}

int launch_nm_propagate(const Sys& s, int D, const double* C, const double* T, const double* rot, int com_apply,
                        const double* red_in, int nred_in, const double2* tw, double* cm, cudaStream_t st) {
    if (tw && cm) {
        bool done = false;
        if (D == 1) done = nm_prop_warp_d<1>(s, rot, com_apply, red_in, nred_in, tw, cm, st);
        else if (D == 2) done = nm_prop_warp_d<2>(s, rot, com_apply, red_in, nred_in, tw, cm, st);
        else done = nm_prop_warp_d<3>(s, rot, com_apply, red_in, nred_in, tw, cm, st);
        if (done) return com_apply ? 2 : 1;
    }
    if (D == 1) nm_prop_launch<1>(s, C, T, rot, com_apply, red_in, nred_in, st);
    else if (D == 2) nm_prop_launch<2>(s, C, T, rot, com_apply, red_in, nred_in, st);
    else nm_prop_launch<3>(s, C, T, rot, com_apply, red_in, nred_in, st);
    return 1;
}

}  // namespace pimdb

// ---------------------------------------------------------------------------
// RanMars parity noise: the reference's Langevin noise (langevin.cpp:15-27
// draws sim.mars_gen->gaussian() per particle and axis; one RanMars stream
// per bead rank, seeded seed + rank, simulation.cpp:54-59).  RANMAR is a
// lagged-Fibonacci generator (Marsaglia, Zaman & Tsang; F. James, Comp. Phys.
// Comm. 60, 329 (1990), as in libs/random_mars.cpp) with Marsaglia's polar
// Gaussian; each stream is sequential, so one thread per stream draws the
// step's 2 N D normals into s.noise.  Not a fast path: it exists to replay
// the reference's Langevin trajectories.
namespace pimdb {

void ranmars_seed(int seed, RanMarsState& r) {
    // libs/random_mars.cpp:11-47 (seed checked by the caller)
    r = RanMarsState{};
    int ij = (seed - 1) / 30082;
    int kl = (seed - 1) - 30082 * ij;
    int i = (ij / 177) % 177 + 2, j = ij % 177 + 2, k = (kl / 169) % 178 + 1, l = kl % 169;
    for (int n = 1; n <= 97; ++n) {
        double acc = 0.0, bit = 0.5;
        for (int b = 0; b < 24; ++b) {
            const int m = ((i * j) % 179) * k % 179;
            i = j;
            j = k;
            k = m;
            l = (53 * l + 1) % 169;
            if ((l * m) % 64 >= 32) acc = acc + bit;
            bit = 0.5 * bit;
        }
        r.u[n] = acc;
    }
    r.c = 362436.0 / 16777216.0;
    r.cd = 7654321.0 / 16777216.0;
    r.cm = 16777213.0 / 16777216.0;
    r.i97 = 97;
    r.j97 = 33;
    // the constructor draws one uniform (random_mars.cpp:46)
    double uni = r.u[r.i97] - r.u[r.j97];
    if (uni < 0.0) uni += 1.0;
    r.u[r.i97] = uni;
    if (--r.i97 == 0) r.i97 = 97;
    if (--r.j97 == 0) r.j97 = 97;
    r.c -= r.cd;
    if (r.c < 0.0) r.c += r.cm;
}

namespace {

// RanMars::uniform (random_mars.cpp:59-78) on a stream held in shared memory.
__device__ double ranmars_uniform(RanMarsState& r) {
    double uni = __dsub_rn(r.u[r.i97], r.u[r.j97]);
    if (uni < 0.0) uni = __dadd_rn(uni, 1.0);
    r.u[r.i97] = uni;
    if (--r.i97 == 0) r.i97 = 97;
    if (--r.j97 == 0) r.j97 = 97;
    r.c = __dsub_rn(r.c, r.cd);
    if (r.c < 0.0) r.c = __dadd_rn(r.c, r.cm);
    uni = __dsub_rn(uni, r.c);
    if (uni < 0.0) uni = __dadd_rn(uni, 1.0);
    return uni;
}

// RanMars::gaussian (random_mars.cpp:84-103): the polar method, the second
// variate of each accepted pair kept for the next call.  Products and sums
// are rounded separately (no contraction), so the acceptance test sees the
// same rsq as the reference's.
__device__ double ranmars_gaussian(RanMarsState& r) {
    if (r.save) {
        r.save = 0;
        return r.second;
    }
    double v1, v2, rsq;
    int tries = 0;
    do {
        v1 = __dsub_rn(__dmul_rn(2.0, ranmars_uniform(r)), 1.0);
        v2 = __dsub_rn(__dmul_rn(2.0, ranmars_uniform(r)), 1.0);
        rsq = __dadd_rn(__dmul_rn(v1, v1), __dmul_rn(v2, v2));
    } while ((rsq >= 1.0 || rsq == 0.0) && ++tries < (1 << 20));
    const double fac = sqrt(__ddiv_rn(__dmul_rn(-2.0, log(rsq)), rsq));
    r.second = __dmul_rn(v1, fac);
    r.save = 1;
    return __dmul_rn(v2, fac);
}

// One block per stream (bead): lane 0 draws both O-steps' normals of the
// current MD step into the step-parity half of `noise`, in the reference's
// order (particle-major, then axis).
template <int D>
__global__ void k_ranmars_draw(Sys s, RanMarsState* __restrict__ states, double* __restrict__ noise, StepRef sref) {
    __shared__ RanMarsState r;
    const int b = blockIdx.x;
    const int words = (int)(sizeof(RanMarsState) / sizeof(double));
    double* sh = reinterpret_cast<double*>(&r);
    const double* g = reinterpret_cast<const double*>(states + b);
    for (int w = threadIdx.x; w < words; w += blockDim.x) sh[w] = g[w];
    __syncthreads();
    if (threadIdx.x == 0) {
        const long long step = sref.get();
        for (int o = 0; o < 2; ++o) {
            double* out = noise + ((size_t)((step & 1) * 2 + o) * s.P + b) * D * s.ld;
            for (int i = 0; i < s.N; ++i)
#pragma unroll
                for (int a = 0; a < D; ++a) out[(size_t)a * s.ld + i] = ranmars_gaussian(r);
        }
    }
    __syncthreads();
    double* gw = reinterpret_cast<double*>(states + b);
    for (int w = threadIdx.x; w < words; w += blockDim.x) gw[w] = sh[w];
}

}  // namespace

void launch_ranmars_draw(const Sys& s, int D, RanMarsState* states, double* noise, StepRef step, cudaStream_t st) {
    if (D == 1) k_ranmars_draw<1><<<s.P, 32, 0, st>>>(s, states, noise, step);
    else if (D == 2) k_ranmars_draw<2><<<s.P, 32, 0, st>>>(s, states, noise, step);
    else k_ranmars_draw<3><<<s.P, 32, 0, st>>>(s, states, noise, step);
}

}  // namespace pimdb

// Batched replicas: many independent ring polymers, each with its own N, P,
// temperature, potentials and noise key, advanced together by one launch
// per MD step.
//
// The reference runs one system per MPI job (src/pimdb.cpp:31-68,
// src/simulation.cpp:236-260); an ensemble of small systems is many jobs.
// Here a persistent grid takes whole replicas from a work counter, largest
// first, and one CTA runs the complete step of one replica:
//   head    O-step (substep 0), COM removal, B half-kick, A drift
//   forces  external + pair forces per bead (one warp per bead, positions
//           staged in shared memory), interior springs, and on bosonic
//           replicas the Feldman-Hirshberg exchange on beads 1 and P
//           (the block-level pieces shared with the one-system kernels)
//   tail    B half-kick, O-step (substep 1), COM removal
// in the order of src/simulation.cpp:246-259 with the cartesian propagator
// (src/propagators/velocity_verlet.cpp:7-38) or the normal-mode one
// (src/propagators/normal_modes_propagator.cpp:19-71) and the Langevin
// thermostat (src/thermostats/langevin.cpp:10-27) in either frame.  Nothing
// waits on another CTA: the only cross-CTA state is the work counter, reset
// by the CTA that finishes last, which also advances the device-side step
// counter, so a sequence of step launches can be captured once in a CUDA
// graph and replayed.
//
// Precision: `R` is the pair-force arithmetic.  R = double is the FP64 path
// (same noise, formulas and exchange as the one-system path; harmonic and
// dipole pairs in double-float, bead_pairs_df).  R = float computes pair
// separations from hi/lo float pairs and pair gradients in FP32, sums each
// 32-particle tile in FP32 and accumulates tiles in FP64, forms the
// exchange weights in double-float and the exterior spring forces in FP32
// with compensated sums; the potentials, the triangular solve, the cycle
// energies and the integrator stay FP64.  Both draw the Langevin normals
// with FP32 Box-Muller from the same Philox bits.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "config.h"
#include "exchange_dev.cuh"
#include "forces_dev.cuh"
#include "kernels.h"

namespace pimdb {

enum BatchFlags : int { BF_LANGEVIN = 1, BF_FIXCOM = 2, BF_NM = 4, BF_NMTHERMO = 8 };
enum BatchMode : int { BM_HEAD = 1, BM_FORCES = 2, BM_TAIL = 4, BM_ADVANCE = 8, BM_ESTIMATORS = 16 };

// Normal-mode tables of one replica (BF_NM or BF_NMTHERMO), transposed so
// that a warp's lanes (one mode or one bead each) read P consecutive
// doubles: Ct[b P + k] = C[k][b], Tt[k P + j] = T[j][k]; rot[4 k ..] as the
// one-system path's.
struct NmTabs {
    const double* Ct;
    const double* Tt;
    const double* rot;
};

struct BatchRep {
    Sys s;
    int flags;  // BatchFlags
    int pad;
    NmTabs nm;
};

constexpr int kBatchMaxThreads = 512;
// Beads of a replica with normal modes: each warp holds 8 P doubles of one
// particle pair's lines in shared memory.
constexpr int kBatchMaxNmBeads = 256;

template <typename R>
__device__ __forceinline__ void normal_pair(const Sys& s, long long step, int substep, uint32_t pair, double& z0,
                                            double& z1) {
    const uint64_t t = 2ull * (unsigned long long)step + substep;
    // the one-system path's normals (drawn on the FP32 pipe in either precision)
    const float2 z = philox_normal_pair_f32(s.seed, s.replica, t, pair);
    z0 = f32_to_f64(z.x);
    z1 = f32_to_f64(z.y);
}

// Sums v[0..D) over the block; every thread receives the totals.  `sh`
// holds 3 * 32 doubles.
template <int D>
__device__ __forceinline__ void block_sum_axes(double* v, double* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int a = 0; a < D; ++a) {
        const double t = warp_sum(v[a]);
        if (lane == 0) sh[a * 32 + w] = t;
    }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < D; ++a) {
        double t = 0.0;
        for (int k = 0; k < nw; ++k) t += sh[a * 32 + k];
        v[a] = t;
    }
    __syncthreads();
}

// The normal-mode propagator's kick force of elements (b, a, i0) and
// (b, a, i0 + 1), as the one-system path forms it (nm_kick_force): the
// physical force, and on the bosonic end beads the exchange's spring force
// fx less the distinguishable ring spring the free propagation carries.
// All stored forces are zero until the first force evaluation after a state
// is set, as in the reference.
template <int D>
__device__ __forceinline__ double2 nm_kick_pair(const Sys& s, int b, int a, int i0) {
    const size_t o = idx<D>(s, b, a, i0);
    double2 fk = *reinterpret_cast<const double2*>(s.fphys + o);
    if (s.bosonic && (b == 0 || b == s.P - 1)) {
        const int bp = (b - 1 + s.P) % s.P, bn = (b + 1) % s.P;
        const double2 x = *reinterpret_cast<const double2*>(s.x + o);
        const double2 xp = *reinterpret_cast<const double2*>(s.x + idx<D>(s, bp, a, i0));
        const double2 xn = *reinterpret_cast<const double2*>(s.x + idx<D>(s, bn, a, i0));
        const double2 fx = *reinterpret_cast<const double2*>(s.fx + ((size_t)(b == 0 ? 0 : 1) * D + a) * s.ld + i0);
        const double in0 = -s.kappa * (2 * x.x - xp.x - xn.x), in1 = -s.kappa * (2 * x.y - xp.y - xn.y);
        fk.x = fk.x + fx.x - in0;
        fk.y = fk.y + fx.y - in1;
    }
    return fk;
}

// One pass over the momenta of a replica, element pairs (i, i+1) per thread
// so that one Philox call serves both normals (pair index as in the
// one-system kernels: (b D + a) ceil(N/2) + i/2).
//   com_in:  subtract cm (a COM correction computed before this pass)
//   kick:    p += dt/2 f (nmkick: the normal-mode propagator's kick force,
//            nm_kick_pair)
//   o:       p = c1 p + c2 xi (substep)
//   drift:   x += dt p / m
// Returns the per-axis sums of the new p in `sum` (this thread's share).
// The pair (2 i2, 2 i2 + 1) is one aligned 16-byte word of each array (the
// leading dimension is a multiple of 32 and every array starts on 256
// bytes; for odd N the second element of the last pair is padding, loaded
// and stored back unchanged).  Each thread loads kPassUnroll pairs of every
// array it touches before it computes any of them: the passes stream state
// that left L2 a step ago, and one pair's loads in flight per thread leave
// them latency-bound.  The elements are taken in the same per-thread order
// as one pair at a time (the same sums, bit for bit).
constexpr int kPassUnroll = 4;
template <int D, typename R>
__device__ __forceinline__ void momenta_pass(const Sys& s, long long step, int substep, const double* cm, bool com_in,
                                             bool kick, bool o, bool drift, double* sum, bool nmkick = false) {
    const int N = s.N, H = (N + 1) / 2;
    const int total = s.P * H, stride = blockDim.x;
    // loop constants kept in registers (opaque: not recomputed per element)
    double hdt = 0.5 * s.dt, c1 = s.c1, c2 = s.c2, dt_m = s.dt_m;
    asm volatile("" : "+d"(hdt), "+d"(c1), "+d"(c2), "+d"(dt_m));
#pragma unroll 1
    for (int a = 0; a < D; ++a) {
        double sa = 0.0;
        const double cma = com_in ? cm[a] : 0.0;
        for (int q0 = threadIdx.x; q0 < total; q0 += kPassUnroll * stride) {
            double2 pv[kPassUnroll], fv[kPassUnroll], xv[kPassUnroll];
#pragma unroll
            for (int k = 0; k < kPassUnroll; ++k) {
                const int q = min(q0 + k * stride, total - 1);  // past the end: a repeat, not stored
                const int b = q / H, i2 = q - b * H;
                const size_t e = idx<D>(s, b, a, 2 * i2);
                pv[k] = *reinterpret_cast<const double2*>(s.p + e);
                if (kick && !nmkick) fv[k] = *reinterpret_cast<const double2*>(s.f + e);
                if (drift) xv[k] = *reinterpret_cast<const double2*>(s.x + e);
                if (kick && nmkick) fv[k] = nm_kick_pair<D>(s, b, a, 2 * i2);
            }
#pragma unroll
            for (int k = 0; k < kPassUnroll; ++k) {
                const int q = q0 + k * stride;
                if (q < total) {
                    const int b = q / H, i2 = q - b * H;
                    const size_t e = idx<D>(s, b, a, 2 * i2);
                    const bool two = 2 * i2 + 1 < N;
                    double z0 = 0.0, z1 = 0.0;
                    if (o) normal_pair<R>(s, step, substep, (uint32_t)((b * D + a) * H + i2), z0, z1);
                    double p0 = pv[k].x, p1 = pv[k].y;
                    if (com_in) {
                        p0 -= cma;
                        p1 -= cma;
                    }
                    if (kick) {
                        p0 += hdt * fv[k].x;
                        p1 += hdt * fv[k].y;
                    }
                    if (o) {
                        p0 = c1 * p0 + c2 * z0;
                        p1 = c1 * p1 + c2 * z1;
                    }
                    if (!two) p1 = pv[k].y;  // padding: unchanged
                    if (drift)
                        *reinterpret_cast<double2*>(s.x + e) =
                            make_double2(fma(p0, dt_m, xv[k].x), two ? fma(p1, dt_m, xv[k].y) : xv[k].y);
                    *reinterpret_cast<double2*>(s.p + e) = make_double2(p0, p1);
                    sa += p0;
                    if (two) sa += p1;
                }
            }
        }
        sum[a] = sa;
    }
}

// Bytes of one particle's staged position: FP64, x y | z (one 16-byte and
// one 8-byte shared load per pair in 3D); mixed, hx hy hz lx | ly lz.
template <int D>
__host__ __device__ constexpr int stage_bytes() { return D == 3 ? 32 : 8 * D; }

// R = float: the hi/lo layout, hi + lo a normalised double-float of x
// (the mixed path's FP32 separations, the FP64 path's double-float pairs).
template <int D, typename R>
__device__ __forceinline__ void stage_put(unsigned char* st, int j, const double* x) {
    unsigned char* q = st + (size_t)j * stage_bytes<D>();
    if constexpr (sizeof(R) == 8) {
        if constexpr (D == 3) {
            *reinterpret_cast<double2*>(q) = make_double2(x[0], x[1]);
            *reinterpret_cast<double*>(q + 16) = x[2];
        } else if constexpr (D == 2) {
            *reinterpret_cast<double2*>(q) = make_double2(x[0], x[1]);
        } else {
            *reinterpret_cast<double*>(q) = x[0];
        }
    } else {
        float h[D], l[D];
#pragma unroll
        for (int a = 0; a < D; ++a) {
            const dfl::df v = split_df(x[a]);  // no FP64-pipe instruction
            h[a] = v.hi;
            l[a] = v.lo;
        }
        if constexpr (D == 3) {
            *reinterpret_cast<float4*>(q) = make_float4(h[0], h[1], h[2], l[0]);
            *reinterpret_cast<float2*>(q + 16) = make_float2(l[1], l[2]);
        } else if constexpr (D == 2) {
            *reinterpret_cast<float4*>(q) = make_float4(h[0], h[1], l[0], l[1]);
        } else {
            *reinterpret_cast<float2*>(q) = make_float2(h[0], l[0]);
        }
    }
}

template <int D, typename R>
__device__ __forceinline__ void stage_get(const unsigned char* st, int j, R* h, R* l) {
    const unsigned char* q = st + (size_t)j * stage_bytes<D>();
    if constexpr (sizeof(R) == 8) {
        if constexpr (D == 3) {
            const double2 v = *reinterpret_cast<const double2*>(q);
            h[0] = v.x;
            h[1] = v.y;
            h[2] = *reinterpret_cast<const double*>(q + 16);
        } else if constexpr (D == 2) {
            const double2 v = *reinterpret_cast<const double2*>(q);
            h[0] = v.x;
            h[1] = v.y;
        } else {
            h[0] = *reinterpret_cast<const double*>(q);
        }
#pragma unroll
        for (int a = 0; a < D; ++a) l[a] = 0.0;
    } else {
        if constexpr (D == 3) {
            const float4 v = *reinterpret_cast<const float4*>(q);
            const float2 w = *reinterpret_cast<const float2*>(q + 16);
            h[0] = v.x;
            h[1] = v.y;
            h[2] = v.z;
            l[0] = v.w;
            l[1] = w.x;
            l[2] = w.y;
        } else if constexpr (D == 2) {
            const float4 v = *reinterpret_cast<const float4*>(q);
            h[0] = v.x;
            h[1] = v.y;
            l[0] = v.z;
            l[1] = v.w;
        } else {
            const float2 v = *reinterpret_cast<const float2*>(q);
            h[0] = v.x;
            l[0] = v.y;
        }
    }
}

// The pair gradient sum of particle i of bead b (FP64 path, harmonic or
// dipole pair potential) in double-float on the FP32 pipe: separations as
// double-float differences of the staged hi/lo positions (about 2^-47
// relative), the gradient scale (k, or -3 D |r|^-5 from the double-float
// 1/sqrt) and the sum over j in double-float (AccurateDWPlusDW).  A pair
// within 1e-6 L of the half-box edge (the image must be the FP64 one) or
// within 1e-5 of the cutoff (the in/out decision must be the FP64 one) is
// evaluated in FP64 from the FP64 positions, as the FP64 loop does.  The
// all-pairs harmonic force needs no distance: r^2 is not formed.
template <int D>
__device__ __noinline__ void bead_pairs_df(const Sys& s, int b, int i, const double* xi, const unsigned char* stage,
                                           double* g) {
    using dfl::df;
    const int N = s.N;
    const bool harm = s.int_kind == POT_HARMONIC;
    const double cut = s.cutoff;
    const bool need_r2 = !(harm && cut < 0.0);
    const float cut2f = cut < 0.0 ? INFINITY : round_f32(cut * cut);
    const float shell = 1e-5f * cut2f;
    const float Lf = round_f32(s.L), halfL = 0.5f * Lf, amb = 1e-6f * Lf;
    const df Ldf = split_df(s.L);
    const df K = split_df(harm ? s.int_a : -3.0 * s.int_a);  // harmonic k; dipole -3 D
    float hi[D], lo[D];
    stage_get<D, float>(stage, i, hi, lo);
    df acc[D];
    double accx[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
        acc[a] = df{0.0f, 0.0f};
        accx[a] = 0.0;
    }
    for (int j = 0; j < N; ++j) {
        float hj[D], lj[D];
        stage_get<D, float>(stage, j, hj, lj);
        df d[D];
        bool exact = false;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            d[a] = dfl::add(df{hi[a], lo[a]}, df{-hj[a], -lj[a]});
            if (s.pbc) {
                exact |= fabsf(fabsf(d[a].hi) - halfL) <= amb;
                if (fabsf(d[a].hi) > halfL) d[a] = dfl::add(d[a], d[a].hi > 0.0f ? dfl::neg(Ldf) : Ldf);
            }
        }
        bool use = j != i;
        df sc = K;
        if (need_r2) {
            df r2 = dfl::sqr(d[0]);
#pragma unroll
            for (int a = 1; a < D; ++a) r2 = dfl::add_sloppy(r2, dfl::sqr(d[a]));  // non-negative terms
            if (fabsf(r2.hi - cut2f) <= shell) exact = true;
            use = use && r2.hi < cut2f;
            if (!harm) {  // dipole: -3 D |r|^-5
                const df ri = dfl::rsqrt(r2);
                const df ri2 = dfl::sqr(ri);
                sc = dfl::mul(K, dfl::mul(dfl::sqr(ri2), ri));
            }
        }
        if (exact && j != i) {
            // FP64, as the FP64 pair loop
            double r[D], q2 = 0.0;
#pragma unroll
            for (int a = 0; a < D; ++a) {
                double dd = xi[a] - s.x[idx<D>(s, b, a, j)];
                if (s.pbc) dd = min_image(dd, s.L, s.invL);
                r[a] = dd;
                q2 += dd * dd;
            }
            if (!(q2 >= (cut < 0.0 ? INFINITY : cut * cut))) {
                const double scd = pair_scale<double>(s.int_kind, q2, s.int_a);
#pragma unroll
                for (int a = 0; a < D; ++a) accx[a] -= scd * r[a];
            }
        } else if (use) {
#pragma unroll
            for (int a = 0; a < D; ++a) acc[a] = dfl::add(acc[a], dfl::neg(dfl::mul(sc, d[a])));
        }
    }
#pragma unroll
    for (int a = 0; a < D; ++a) g[a] = df_to_f64(acc[a]) + accx[a];
}

// Physical forces of bead b plus its interior springs, by one warp.  The
// bead's positions are staged in `stage` (N slots of stage_bytes<D>()).
// Bosonic end beads keep the physical part only: the exchange adds their
// springs.  Global loads are issued in groups (kStageUnroll particles per
// lane when staging; a particle's own and both neighbour positions at once)
// so that a warp waits once per group rather than once per load.
constexpr int kStageUnroll = 4;
template <int D, typename R>
__device__ void bead_forces_warp(const Sys& s, int b, int lane, unsigned char* stage) {
    const int N = s.N;
    const bool pairs = s.int_kind != POT_FREE && s.cutoff != 0.0;
    // FP64 with the harmonic or dipole pair potential: pairs in double-float
    // (bead_pairs_df), from the hi/lo layout
    const bool dfp = sizeof(R) == 8 && (s.int_kind == POT_HARMONIC || s.int_kind == POT_DIPOLE);
    if (pairs) {
        for (int j0 = lane; j0 < N; j0 += 32 * kStageUnroll) {
            double xs[kStageUnroll][D];
#pragma unroll
            for (int k = 0; k < kStageUnroll; ++k) {
                const int j = min(j0 + 32 * k, N - 1);  // past the end: a repeat, not stored
#pragma unroll
                for (int a = 0; a < D; ++a) xs[k][a] = s.x[idx<D>(s, b, a, j)];
            }
#pragma unroll
            for (int k = 0; k < kStageUnroll; ++k)
                if (j0 + 32 * k < N) {
                    if (dfp) stage_put<D, float>(stage, j0 + 32 * k, xs[k]);
                    else stage_put<D, R>(stage, j0 + 32 * k, xs[k]);
                }
        }
        __syncwarp();
    }
    const double cut = s.cutoff;
    // The loop constants are made opaque (an empty asm that takes them as
    // in/out operands): under register pressure the compiler otherwise
    // recomputes them from the shared Sys inside the pair loop, a DMUL and a
    // conversion per pair on the FP64 pipe.  All pairs: an infinite cutoff.
    R cut2 = cut < 0.0 ? (R)INFINITY : (R)(cut * cut);
    R param = (R)s.int_a;
    if constexpr (sizeof(R) == 4) asm volatile("" : "+f"(cut2), "+f"(param));
    else asm volatile("" : "+d"(cut2), "+d"(param));
    const bool bosonic_bead = s.bosonic && (b == 0 || b == s.P - 1);
    const int bp = (b - 1 + s.P) % s.P, bn = (b + 1) % s.P;
    for (int i = lane; i < N; i += 32) {
        double xi[D], xp[D], xn[D];
#pragma unroll
        for (int a = 0; a < D; ++a) {
            xi[a] = s.x[idx<D>(s, b, a, i)];
            if (!bosonic_bead) {
                xp[a] = s.x[idx<D>(s, bp, a, i)];
                xn[a] = s.x[idx<D>(s, bn, a, i)];
            }
        }
        // the interior springs' separations (simulation.cpp:405-419), added
        // after the physical forces as before
        double sp[D];
#pragma unroll
        for (int a = 0; a < D; ++a) {
            sp[a] = 0.0;
            if (!bosonic_bead) {
                double dp = xp[a] - xi[a];
                double dn = xn[a] - xi[a];
                if (s.pbc) {
                    dp = min_image(dp, s.L, s.invL);
                    dn = min_image(dn, s.L, s.invL);
                }
                sp[a] = dp + dn;
            }
        }
        double acc[D];
        ext_force<D>(s, xi, acc);
        if (pairs && dfp) {
            double g[D];
            bead_pairs_df<D>(s, b, i, xi, stage, g);
#pragma unroll
            for (int a = 0; a < D; ++a) acc[a] += g[a];
        } else if (pairs) {
            R hi[D], lo[D];
            stage_get<D, R>(stage, i, hi, lo);
            // FP32: the 32-pair partial sums are added up error-free in two
            // floats (Knuth's two-sum), so the FP64 pipe is not touched
            // until the particle's total
            R ch[D], cl[D];
#pragma unroll
            for (int a = 0; a < D; ++a) ch[a] = cl[a] = (R)0;
            for (int j0 = 0; j0 < N; j0 += 32) {
                const int jn = min(32, N - j0);
                R t[D];
#pragma unroll
                for (int a = 0; a < D; ++a) t[a] = (R)0;
#pragma unroll 4
                for (int jj = 0; jj < jn; ++jj) {
                    const int j = j0 + jj;
                    R hj[D], lj[D];
                    stage_get<D, R>(stage, j, hj, lj);
                    R r[D];
                    R r2 = (R)0;
#pragma unroll
                    for (int a = 0; a < D; ++a) {
                        R d;
                        if constexpr (sizeof(R) == 8) {
                            d = hi[a] - hj[a];
                            if (s.pbc) d = min_image(d, s.L, s.invL);
                        } else {
                            d = (hi[a] - hj[a]) + (lo[a] - lj[a]);
                            if (s.pbc) d = min_image_f(d, (float)s.L, (float)s.invL);
                        }
                        r[a] = d;
                        r2 += d * d;
                    }
                    // a select, not a branch: the self term (r = 0) may be
                    // infinite for the dipole and must not enter
                    const bool use = j != i && !(r2 >= cut2);  // a NaN separation still enters
                    const R sc = pair_scale<R>(s.int_kind, r2, param);
#pragma unroll
                    for (int a = 0; a < D; ++a) t[a] -= use ? sc * r[a] : (R)0;
                }
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    if constexpr (sizeof(R) == 8) {
                        acc[a] += t[a];
                    } else {
                        const R sum = ch[a] + t[a];
                        const R bb = sum - ch[a];
                        cl[a] += (ch[a] - (sum - bb)) + (t[a] - bb);
                        ch[a] = sum;
                    }
                }
            }
            if constexpr (sizeof(R) == 4) {
#pragma unroll
                for (int a = 0; a < D; ++a) acc[a] += f32_to_f64(ch[a]) + f32_to_f64(cl[a]);
            }
        }
#pragma unroll
        for (int a = 0; a < D; ++a) {
            const size_t o = idx<D>(s, b, a, i);
            s.f[o] = bosonic_bead ? acc[a] : s.kappa * sp[a] + acc[a];  // simulation.cpp:363-373
            if (s.fphys) s.fphys[o] = acc[a];  // the normal-mode propagator's kick force
        }
    }
    __syncwarp();
}

// ------------------------------------------------ mixed-precision exchange
// This GPU's FP64 pipe finishes about one warp-wide FP64 instruction per 16
// SM cycles, against 4 FP32 ones per cycle, so the mixed path moves the two
// largest FP64 parts of the exchange to the FP32 pipe: the weights in
// double-float (about 2^-44 relative) and the exterior spring forces in FP32
// with compensated sums (about 2e-7 relative per term).  The potentials, the
// triangular solve and the energies stay FP64, as on the FP64 path.

// Shared floats batch_exchange_forces_f32 stages.
__host__ __device__ constexpr size_t xforces_f32_floats(int D, int N) { return 4 * (size_t)D * N + 3 * (size_t)N; }

// The exterior spring forces of exch_force_row (accumulated into f) in FP32:
// probabilities Wf y R and 1 - C rounded to float, separations from hi/lo
// floats, each lane's terms and the warp's lanes summed with two-sum error
// terms.  Lanes 0..D-1 add the interior neighbour spring and write axis
// a = lane: one FP64 add per row joins the result to f.
template <int D>
__device__ void batch_exchange_forces_f32(const Sys& s, float* sm) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int N = s.N, P = s.P;
    float* xh = sm;  // (side D + a) N + i; side 0 bead 1, 1 bead P
    float* xl = xh + 2 * D * N;
    float* yv = xl + 2 * D * N;  // y_l
    float* rr = yv + N;          // R_l
    float* cc = rr + N;          // 1 - C_l
    for (int e = threadIdx.x; e < 2 * D * N; e += blockDim.x) {
        const int side = e / (D * N), a = (e / N) % D, i = e % N;
        split_f32(s.x[idx<D>(s, side ? P - 1 : 0, a, i)], xh[e], xl[e]);
    }
    for (int l = threadIdx.x; l < N; l += blockDim.x) {
        yv[l] = round_f32(s.yf[l]);
        rr[l] = round_f32(s.rowR[l]);
        cc[l] = round_f32(1.0 - s.rowC[l]);
    }
    __syncthreads();
    const float Lf = round_f32(s.L), invLf = round_f32(s.invL), kf = round_f32(s.kappa);
    for (int w = warp; w < 2 * N; w += nw) {
        const bool lastb = w < N;  // bead P, particle l (row l); else bead 1 (column l)
        const int l = lastb ? w : w - N, side = lastb ? 1 : 0, other = 1 - side;
        float ph[D], pl[D], sh[D], sl[D];
#pragma unroll
        for (int a = 0; a < D; ++a) {
            ph[a] = xh[(side * D + a) * N + l];
            pl[a] = xl[(side * D + a) * N + l];
            sh[a] = sl[a] = 0.0f;
        }
        auto add_term = [&](float pr, int n) {
#pragma unroll
            for (int a = 0; a < D; ++a) {
                float d = (xh[(other * D + a) * N + n] - ph[a]) + (xl[(other * D + a) * N + n] - pl[a]);
                if (s.pbc) d = min_image_f(d, Lf, invLf);
                const float t = pr * d;
                const float sum = sh[a] + t, bb = sum - sh[a];
                sl[a] += (sh[a] - (sum - bb)) + (t - bb);
                sh[a] = sum;
            }
        };
        if (lastb) {  // n <= l + 1: close-cycle entries, then the direct link
            const size_t r = tri(l);
            const float Rl = rr[l];
            const int nmax = min(l + 1, N - 1);
            for (int n = lane; n <= nmax; n += 32) {
                if (n <= l) {
                    const double wd = s.Wf[r + n];
                    if (f64_is_zero(wd)) continue;  // a cycle too costly to contribute adds exactly 0
                    add_term(round_f32(wd) * yv[n] * Rl, n);
                } else {
                    add_term(cc[l], n);
                }
            }
        } else {  // q >= l - 1: the direct link, then close-cycle entries
            const float yl = yv[l];
            for (int q = max(0, l - 1) + lane; q < N; q += 32) {
                if (q >= l) {
                    const double wd = s.Wf[tri(q) + l];
                    if (f64_is_zero(wd)) continue;
                    add_term(round_f32(wd) * yl * rr[q], q);
                } else {
                    add_term(cc[q], q);
                }
            }
        }
#pragma unroll
        for (int a = 0; a < D; ++a) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float oh = __shfl_xor_sync(0xffffffffu, sh[a], o), ol = __shfl_xor_sync(0xffffffffu, sl[a], o);
                const float sum = sh[a] + oh, bb = sum - sh[a];
                sl[a] = (sl[a] + ol) + ((sh[a] - (sum - bb)) + (oh - bb));
                sh[a] = sum;
            }
        }
        if (lane < D) {
            const int a = lane;
            float hs = sh[0], ls = sl[0], hb = ph[0], lb = pl[0];
#pragma unroll
            for (int k = 1; k < D; ++k)
                if (a == k) {
                    hs = sh[k];
                    ls = sl[k];
                    hb = ph[k];
                    lb = pl[k];
                }
            const int bead = lastb ? P - 1 : 0, nb = lastb ? (P - 2 + P) % P : 1 % P;
            float nh, nl;
            split_f32(s.x[idx<D>(s, nb, a, l)], nh, nl);
            float d = (nh - hb) + (nl - lb);
            if (s.pbc) d = min_image_f(d, Lf, invLf);
            const float fs = kf * ((hs + d) + ls);
            const size_t o = idx<D>(s, bead, a, l);
            const double fsd = f32_to_f64(fs);
            s.fx[((size_t)side * D + a) * s.ld + l] = fsd;
            s.f[o] = fsd + s.f[o];
        }
    }
}

// The Feldman-Hirshberg exchange of one replica by the whole block; adds the
// exterior springs to f on beads 1 and P (which hold the physical forces).
// R = float: weights and exterior forces on the FP32 pipe (above).
template <int D, typename R>
__device__ void batch_exchange(const Sys& s, unsigned char* work, const double* tbl, const dfl::ExpTable* etbl) {
    constexpr bool kMixed = sizeof(R) == 4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int N = s.N;
    // the interior links |x1_{u+1} - xP_u|^2 once per u (shared memory),
    // instead of once per cycle-energy entry
    double* link = reinterpret_cast<double*>(work);
    for (int u = threadIdx.x; u < N - 1; u += blockDim.x) link[u] = sepsq<D>(s, s.P - 1, u, 0, u + 1);
    __syncthreads();
    for (int v = warp; v < N; v += nw) energy_row<D>(s, v, lane, link);
    __syncthreads();
    int fresh = ((volatile int*)s.xflags)[3];
    __syncthreads();
    for (int attempt = 0; attempt < 2; ++attempt) {
        if (fresh) {
            estimate_direction(s, 0, reinterpret_cast<float*>(work));
            __syncthreads();
            estimate_direction(s, 1, reinterpret_cast<float*>(work));
            __syncthreads();
        }
        if (kMixed) {
            weights_df_block(s, *etbl, reinterpret_cast<float*>(work));
        } else {
            for (int p = warp; p < N; p += nw) {
                const double inv = recip_row(p);
                for (int u = lane; u <= p; u += 32) exch_weight(s, p, u, inv, tbl);
            }
        }
        __syncthreads();
        // a reused estimate that fails is replaced by a fresh one (second
        // attempt) rather than by the exact recursion
        solve_direction(s, 0, 0, reinterpret_cast<double*>(work), fresh, nullptr, 1, etbl);
        __syncthreads();
        solve_direction(s, 1, 0, reinterpret_cast<double*>(work), fresh, nullptr, 1, etbl);
        __syncthreads();
        const int retry = ((volatile int*)s.xflags)[6];
        __syncthreads();
        if (!retry) break;
        if (threadIdx.x == 0) s.xflags[6] = 0;
        fresh = 1;
        __syncthreads();
    }
    solve_finish(s, 0, etbl);
    // the exact fallback's probabilities come from their exponentials: FP64 rows
    if (kMixed && !((volatile int*)s.xflags)[0]) {
        __syncthreads();
        batch_exchange_forces_f32<D>(s, reinterpret_cast<float*>(work));
        return;
    }
    // beads 1 and P staged in the (now free) shared scratch for the forces
    double* xs = reinterpret_cast<double*>(work);
    for (int e = threadIdx.x; e < 2 * D * N; e += blockDim.x) {
        const int side = e / (D * N), a = (e / N) % D, i = e % N;
        xs[e] = s.x[idx<D>(s, side ? s.P - 1 : 0, a, i)];
    }
    __syncthreads();
    for (int w = warp; w < 2 * N; w += nw) exch_force_row<D>(s, w, lane, 1, xs);
}

// ------------------------------------------------------------ normal modes
// The normal-mode propagator (normal_modes_propagator.cpp:19-71) and the
// Langevin O-step in the normal-mode frame, with the one-system path's
// P x P transforms (k_nm_propagate, k_nm_thermo): every mode and every bead
// is a sum over beads (modes) in ascending order.  One warp per (axis,
// particle pair), both particles in shared memory (`wsm`: 8 P doubles per
// warp); lanes take modes (beads) k, k + 32, ...

// [COM], half-kick with the normal-mode kick force, Cartesian -> modes, the
// exact free ring-polymer rotation, modes -> Cartesian; x and p written.
template <int D>
__device__ __noinline__ void nm_propagate_block(const Sys& s, const NmTabs& nm, const double* cm, bool com_in, double* wsm) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int P = s.P, N = s.N, H = (N + 1) / 2;
    double* w = wsm + (size_t)warp * 8 * P;  // x0 x1 p0 p1 | q0 q1 u0 u1
    const double hdt = 0.5 * s.dt;
    for (int line = warp; line < D * H; line += nw) {
        const int a = line / H, i0 = 2 * (line - a * H);
        const bool two = i0 + 1 < N;
        const double ca = com_in ? cm[a] : 0.0;
        for (int b = lane; b < P; b += 32) {
            const size_t o = idx<D>(s, b, a, i0);
            const double2 fk = nm_kick_pair<D>(s, b, a, i0);
            const double2 x = *reinterpret_cast<const double2*>(s.x + o);
            const double2 pv = *reinterpret_cast<const double2*>(s.p + o);
            double p0 = pv.x - ca, p1 = pv.y - ca;
            p0 += hdt * fk.x;
            p1 += hdt * fk.y;
            // the second particle of an odd N's last pair is padding: zeros,
            // as outside the one-system kernels' range
            w[b] = x.x;
            w[P + b] = two ? x.y : 0.0;
            w[2 * P + b] = p0;
            w[3 * P + b] = two ? p1 : 0.0;
        }
        __syncwarp();
        for (int k = lane; k < P; k += 32) {
            double q0 = 0.0, q1 = 0.0, p0 = 0.0, p1 = 0.0;
            for (int b = 0; b < P; ++b) {
                const double c = nm.Ct[(size_t)b * P + k];
                q0 += c * w[b];
                q1 += c * w[P + b];
                p0 += c * w[2 * P + b];
                p1 += c * w[3 * P + b];
            }
            const double cs = nm.rot[4 * k], sn = nm.rot[4 * k + 1], mw = nm.rot[4 * k + 2], snw = nm.rot[4 * k + 3];
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
            w[4 * P + k] = qa;
            w[5 * P + k] = qb;
            w[6 * P + k] = pa;
            w[7 * P + k] = pb;
        }
        __syncwarp();
        for (int j = lane; j < P; j += 32) {
            double x0 = 0.0, x1 = 0.0, v0 = 0.0, v1 = 0.0;
            for (int k = 0; k < P; ++k) {
                const double c = nm.Tt[(size_t)k * P + j];
                x0 += c * w[4 * P + k];
                x1 += c * w[5 * P + k];
                v0 += c * w[6 * P + k];
                v1 += c * w[7 * P + k];
            }
            const size_t o = idx<D>(s, j, a, i0);
            s.x[o] = x0;
            s.p[o] = v0;
            if (two) {
                s.x[o + 1] = x1;
                s.p[o + 1] = v1;
            }
        }
        __syncwarp();
    }
}

// [COM], then the Langevin O-step on the normal modes of p (the normals of
// mode k drawn as the Cartesian ones of bead k: pair index (k D + a)
// ceil(N/2) + i/2); p written, and its per-axis sums (this thread's share)
// in `sum`.
template <int D, typename R>
__device__ __noinline__ void nm_thermo_block(const Sys& s, const NmTabs& nm, long long step, int substep, const double* cm,
                                bool com_in, double* sum, double* wsm) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int P = s.P, N = s.N, H = (N + 1) / 2;
    double* w = wsm + (size_t)warp * 8 * P;  // p0 p1 | u0 u1
    for (int a = 0; a < D; ++a) sum[a] = 0.0;
    for (int line = warp; line < D * H; line += nw) {
        const int a = line / H, i2 = line - a * H, i0 = 2 * i2;
        const bool two = i0 + 1 < N;
        const double ca = com_in ? cm[a] : 0.0;
        for (int b = lane; b < P; b += 32) {
            w[b] = s.p[idx<D>(s, b, a, i0)] - ca;
            w[P + b] = two ? s.p[idx<D>(s, b, a, i0 + 1)] - ca : 0.0;
        }
        __syncwarp();
        for (int k = lane; k < P; k += 32) {
            double q0 = 0.0, q1 = 0.0;
            for (int b = 0; b < P; ++b) {
                const double c = nm.Ct[(size_t)b * P + k];
                q0 += c * w[b];
                q1 += c * w[P + b];
            }
            double z0, z1;
            normal_pair<R>(s, step, substep, (uint32_t)((k * D + a) * H + i2), z0, z1);
            w[2 * P + k] = s.c1 * q0 + s.c2 * z0;
            w[3 * P + k] = s.c1 * q1 + s.c2 * z1;
        }
        __syncwarp();
        double part = 0.0;
        for (int j = lane; j < P; j += 32) {
            double v0 = 0.0, v1 = 0.0;
            for (int k = 0; k < P; ++k) {
                const double c = nm.Tt[(size_t)k * P + j];
                v0 += c * w[2 * P + k];
                v1 += c * w[3 * P + k];
            }
            const size_t o = idx<D>(s, j, a, i0);
            s.p[o] = v0;
            part += v0;
            if (two) {
                s.p[o + 1] = v1;
                part += v1;
            }
        }
#pragma unroll
        for (int c = 0; c < D; ++c)
            if (c == a) sum[c] += part;
        __syncwarp();
    }
}

template <int D, typename R>
__device__ void batch_replica(const Sys& s, int flags, const NmTabs& nm, long long step, int mode, double* red,
                              unsigned char* work, const double* tbl, const dfl::ExpTable* etbl) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const bool langevin = flags & BF_LANGEVIN, fixcom = flags & BF_FIXCOM;
    const bool nmprop = flags & BF_NM, nmthermo = langevin && (flags & BF_NMTHERMO);
    const bool cart_langevin = langevin && !nmthermo;
    double* wsm = reinterpret_cast<double*>(work);  // normal-mode lines (free outside the force phase)
    const double inv_np = 1.0 / ((double)s.N * s.P);
    double cm[D], sum[D];
#pragma unroll
    for (int a = 0; a < D; ++a) cm[a] = 0.0;
    if (mode & BM_HEAD) {
        // O-step (substep 0) and the sums for the COM removal
        if (nmthermo || cart_langevin || fixcom) {
            if (nmthermo) nm_thermo_block<D, R>(s, nm, step, 0, cm, false, sum, wsm);
            else momenta_pass<D, R>(s, step, 0, cm, false, false, cart_langevin, false, sum);
            if (fixcom) {
                block_sum_axes<D>(sum, red);
#pragma unroll
                for (int a = 0; a < D; ++a) cm[a] = sum[a] * inv_np;
            } else {
                __syncthreads();
            }
        }
        // [COM], B, A (velocity_verlet.cpp:9-12) or the normal-mode
        // propagation up to the forces (normal_modes_propagator.cpp:19-63)
        if (nmprop) nm_propagate_block<D>(s, nm, cm, fixcom, wsm);
        else momenta_pass<D, R>(s, step, 0, cm, fixcom, true, false, true, sum);
        __syncthreads();
    }
    if (mode & BM_FORCES) {
        unsigned char* stage = work + (size_t)warp * stage_bytes<D>() * s.N;
        for (int b = warp; b < s.P; b += nw) bead_forces_warp<D, R>(s, b, lane, stage);
        __syncthreads();
        if (s.bosonic) {
            batch_exchange<D, R>(s, work, tbl, etbl);
            __syncthreads();
        }
    }
    if (mode & BM_TAIL) {
        // B (the normal-mode kick force under the normal-mode propagator),
        // O-step (substep 1), COM removal
        if (nmthermo) {
            if (nmprop) momenta_pass<D, R>(s, step, 1, cm, false, true, false, false, sum, true);
            else momenta_pass<D, R>(s, step, 1, cm, false, true, false, false, sum, false);
            __syncthreads();
            nm_thermo_block<D, R>(s, nm, step, 1, cm, false, sum, wsm);
        } else if (nmprop) {
            momenta_pass<D, R>(s, step, 1, cm, false, true, cart_langevin, false, sum, true);
        } else {
            momenta_pass<D, R>(s, step, 1, cm, false, true, cart_langevin, false, sum, false);
        }
        if (fixcom) {
            block_sum_axes<D>(sum, red);
#pragma unroll
            for (int a = 0; a < D; ++a) cm[a] = sum[a] * inv_np;
            momenta_pass<D, R>(s, step, 1, cm, true, false, false, false, sum);
        }
        __syncthreads();
    }
    if (mode & BM_ESTIMATORS) {
        if (s.bosonic) estimators_block(s, s.P, reinterpret_cast<double*>(work));
        __syncthreads();
    }
}

// One launch: every replica through `mode`.  ctl[0] is the work counter,
// ctl[1] counts finished CTAs; the last CTA resets both and, with
// BM_ADVANCE, advances the step counter.
template <int D, typename R>
__global__ void __launch_bounds__(kBatchMaxThreads)
    k_batch(const BatchRep* __restrict__ reps, const int* __restrict__ order, int nrep, int* ctl,
            long long* step_ctr, int mode) {
    extern __shared__ __align__(16) unsigned char bsm[];
    double* red = reinterpret_cast<double*>(bsm);
    unsigned char* work = bsm + 3 * 32 * sizeof(double);
    __shared__ Sys ss;
    __shared__ NmTabs snm;
    __shared__ int item, sflags;
    __shared__ double tbl[32];  // exp_tang's table
    __shared__ dfl::ExpTable etbl;  // 2^(j/256) as double-floats (bit patterns)
    if (threadIdx.x < 32) tbl[threadIdx.x] = kExp2Table[threadIdx.x];
    fill_exp_table_df(etbl);
    const long long step = *(volatile long long*)step_ctr;
    for (;;) {
        if (threadIdx.x == 0) item = atomicAdd(&ctl[0], 1);
        __syncthreads();
        const int k = item;
        if (k < nrep && threadIdx.x == 0) {
            ss = reps[order[k]].s;
            sflags = reps[order[k]].flags;
            snm = reps[order[k]].nm;
        }
        __syncthreads();
        if (k >= nrep) break;
        batch_replica<D, R>(ss, sflags, snm, step, mode, red, work, tbl, &etbl);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&ctl[1], 1) == (int)gridDim.x - 1) {
            ctl[0] = 0;
            ctl[1] = 0;
            if (mode & BM_ADVANCE) *step_ctr = step + 1;
            __threadfence();
        }
    }
}

// Host-layout <-> device-layout copies for every replica (blockIdx.y =
// replica): which = 0 x, 1 p, 2 f.
template <int D>
__global__ void k_batch_pack(const BatchRep* __restrict__ reps, const size_t* __restrict__ hoff,
                             const double* __restrict__ src, int which) {
    const Sys& s = reps[blockIdx.y].s;
    double* dst = which == 0 ? s.x : (which == 1 ? s.p : s.f);
    const size_t n = (size_t)s.P * s.N * D;
    const double* in = src + hoff[blockIdx.y];
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int a = (int)(e % D);
        const size_t bi = e / D;
        const int i = (int)(bi % s.N), b = (int)(bi / s.N);
        dst[idx<D>(s, b, a, i)] = in[e];
    }
}

template <int D>
__global__ void k_batch_unpack(const BatchRep* __restrict__ reps, const size_t* __restrict__ hoff,
                               double* __restrict__ out_all, int which) {
    const Sys& s = reps[blockIdx.y].s;
    const double* src = which == 0 ? s.x : (which == 1 ? s.p : s.f);
    const size_t n = (size_t)s.P * s.N * D;
    double* out = out_all + hoff[blockIdx.y];
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int a = (int)(e % D);
        const size_t bi = e / D;
        const int i = (int)(bi % s.N), b = (int)(bi / s.N);
        out[e] = src[idx<D>(s, b, a, i)];
    }
}

// After new coordinates: forces to zero (the reference's constructor never
// evaluates them), a fresh FP32 exchange estimate, cleared error word.
__global__ void k_batch_reset(const BatchRep* __restrict__ reps, int D) {
    const Sys& s = reps[blockIdx.x].s;
    const size_t n = (size_t)s.P * D * s.ld;
    for (size_t e = threadIdx.x; e < n; e += blockDim.x) s.f[e] = 0.0;
    if (s.fphys)
        for (size_t e = threadIdx.x; e < n; e += blockDim.x) s.fphys[e] = 0.0;
    for (size_t e = threadIdx.x; e < (size_t)2 * D * s.ld; e += blockDim.x) s.fx[e] = 0.0;
    if (threadIdx.x < 8) s.xflags[threadIdx.x] = threadIdx.x == 3 ? 1 : 0;
    if (threadIdx.x == 0) *s.err = 0;
}

}  // namespace pimdb

using namespace pimdb;

// --------------------------------------------------------------------- host
struct pimdb_batch {
    int nrep = 0, D = 3, mixed = 0;
    std::vector<pimdb_config> cfgs;
    std::vector<BatchRep> reps;
    std::vector<size_t> hoff;  // replica offsets in the host layout (doubles)
    size_t htotal = 0;
    std::vector<int> order;
    BatchRep* d_reps = nullptr;
    int* d_order = nullptr;
    size_t* d_hoff = nullptr;
    int* d_ctl = nullptr;
    long long* d_step = nullptr;
    int* d_err = nullptr;       // one word per replica
    int* d_iflags = nullptr;    // 8 exchange flags per replica
    double* d_scal = nullptr;   // [nrep][4]
    double* pool = nullptr;
    size_t pool_doubles = 0;
    double* d_stage = nullptr;  // host-layout staging (htotal doubles)
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int threads = 256, ctas_per_sm = 2, grid = 1, maxN = 1, sms = 1, maxPnm = 0;
    size_t smem = 0;
    bool use_graph = true;
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0, graph_threads = 0, graph_grid = 0;
    long long step = 0;
    long long launches = 0;
    std::string err;
};

static thread_local std::string g_batch_error;

static int bfail(pimdb_batch* b, int code, const std::string& msg) {
    if (b) b->err = msg;
    g_batch_error = msg;
    return code;
}

#define BATCH_CUDA(b, expr)                                                               \
    do {                                                                                  \
        cudaError_t e_ = (expr);                                                          \
        if (e_ != cudaSuccess) return bfail(b, PIMDB_ERR_CUDA, cudaGetErrorString(e_));   \
    } while (0)

static size_t batch_smem(int D, int maxN, int threads, int maxPnm) {
    const size_t nw = threads / 32;
    const size_t stage = nw * (size_t)maxN * (D == 3 ? stage_bytes<3>() : D == 2 ? stage_bytes<2>() : stage_bytes<1>());
    const size_t est = sizeof(float) * 3 * (size_t)(maxN + 1);
    const size_t solve = sizeof(double) * (2 * (size_t)(maxN + 1) + 32);
    const size_t xforces = sizeof(double) * 2 * (size_t)D * maxN;  // beads 1 and P for the exchange forces
    const size_t xforces32 = sizeof(float) * std::max(xforces_f32_floats(D, maxN), 4 * (size_t)(maxN + 1));
    const size_t estim = sizeof(double) * ((size_t)maxN + 1 + 32);
    const size_t nmlines = sizeof(double) * nw * 8 * (size_t)maxPnm;  // normal-mode lines, 8 P per warp
    return 3 * 32 * sizeof(double) +
           std::max(std::max(std::max(stage, est), std::max(solve, estim)),
                    std::max(std::max(xforces, xforces32), nmlines));
}

template <typename F>
static void with_kernel(int D, int mixed, F&& f) {
    if (mixed) {
        if (D == 1) f(k_batch<1, float>);
        else if (D == 2) f(k_batch<2, float>);
        else f(k_batch<3, float>);
    } else {
        if (D == 1) f(k_batch<1, double>);
        else if (D == 2) f(k_batch<2, double>);
        else f(k_batch<3, double>);
    }
}

static int configure_launch(pimdb_batch* b, int threads, int ctas_per_sm) {
    if (threads < 32 || threads > kBatchMaxThreads || threads % 32) return bfail(b, PIMDB_ERR_ARG, "threads must be a multiple of 32 in [32, 512]");
    if (ctas_per_sm < 1) return bfail(b, PIMDB_ERR_ARG, "ctas_per_sm must be >= 1");
    const size_t smem = batch_smem(b->D, b->maxN, threads, b->maxPnm);
    // every warp stages the largest replica's positions: with many warps a
    // large replica needs more shared memory than a block can have
    int dev = 0, optin = 0;
    size_t stat = 0;
    if (cudaGetDevice(&dev) == cudaSuccess)
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    with_kernel(b->D, b->mixed, [&](auto k) {
        cudaFuncAttributes fa{};
        if (cudaFuncGetAttributes(&fa, k) == cudaSuccess) stat = fa.sharedSizeBytes;
    });
    cudaGetLastError();
    if (optin > 0 && smem + stat > (size_t)optin)
        return bfail(b, PIMDB_ERR_CONFIG, "the batched kernel needs " + std::to_string(smem + stat) +
                                              " bytes of shared memory for " + std::to_string(b->maxN) +
                                              " particles at " + std::to_string(threads) + " threads per block");
    int resident = 0;
    cudaError_t e = cudaSuccess;
    with_kernel(b->D, b->mixed, [&](auto k) {
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k, threads, smem);
    });
    if (e != cudaSuccess) {
        cudaGetLastError();
        return bfail(b, PIMDB_ERR_CUDA, cudaGetErrorString(e));
    }
    if (resident < 1) return bfail(b, PIMDB_ERR_CONFIG, "batched kernel does not fit on an SM with this block size");
    b->threads = threads;
    b->ctas_per_sm = std::min(ctas_per_sm, resident);
    b->smem = smem;
    b->grid = std::max(1, std::min(b->nrep, b->sms * b->ctas_per_sm));
    return PIMDB_OK;
}

static void launch_batch(pimdb_batch* b, int mode) {
    with_kernel(b->D, b->mixed, [&](auto k) {
        k<<<b->grid, b->threads, b->smem, b->stream>>>(b->d_reps, b->d_order, b->nrep, b->d_ctl, b->d_step, mode);
    });
    ++b->launches;
}

static void free_batch(pimdb_batch* b) {
    if (!b) return;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    cudaFree(b->d_reps);
    cudaFree(b->d_order);
    cudaFree(b->d_hoff);
    cudaFree(b->d_ctl);
    cudaFree(b->d_step);
    cudaFree(b->d_err);
    cudaFree(b->d_iflags);
    cudaFree(b->d_scal);
    cudaFree(b->pool);
    cudaFree(b->d_stage);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

extern "C" int pimdb_batch_create(const pimdb_config* cfgs, int nreplicas, void* cuda_stream, pimdb_batch** out) {
    if (!cfgs || !out || nreplicas < 1) return bfail(nullptr, PIMDB_ERR_ARG, "NULL argument or no replicas");
    *out = nullptr;
    const int D = cfgs[0].ndim, precision = cfgs[0].precision;
    for (int r = 0; r < nreplicas; ++r) {
        const pimdb_config& c = cfgs[r];
        const std::string why = validate_config(c);
        if (!why.empty()) return bfail(nullptr, PIMDB_ERR_CONFIG, "replica " + std::to_string(r) + ": " + why);
        if (c.ndim != D) return bfail(nullptr, PIMDB_ERR_CONFIG, "every replica of a batch must have the same ndim");
        if (c.precision != precision)
            return bfail(nullptr, PIMDB_ERR_CONFIG, "every replica of a batch must have the same precision");
        if (c.thermostat >= PIMDB_THERMO_NOSE_HOOVER)
            return bfail(nullptr, PIMDB_ERR_CONFIG,
                         "replica " + std::to_string(r) +
                             ": the batched engine runs the Langevin thermostat (cartesian or normal-mode) or none");
        if ((c.propagator == PIMDB_PROP_NORMAL_MODES || c.nmthermostat) && c.nbeads > kBatchMaxNmBeads)
            return bfail(nullptr, PIMDB_ERR_CONFIG,
                         "replica " + std::to_string(r) + ": the batched engine's normal modes take at most " +
                             std::to_string(kBatchMaxNmBeads) + " beads");
        if (c.natoms > 2048) return bfail(nullptr, PIMDB_ERR_CONFIG, "the batched engine supports at most 2048 particles per replica");
        if (c.rng != PIMDB_RNG_PHILOX)
            return bfail(nullptr, PIMDB_ERR_CONFIG,
                         "replica " + std::to_string(r) + ": the batched engine draws counter-based (Philox) noise");
        if (c.exchange != PIMDB_EXCHANGE_FELDMAN_HIRSHBERG && c.bosonic && c.nbeads > 1)
            return bfail(nullptr, PIMDB_ERR_CONFIG,
                         "replica " + std::to_string(r) + ": the batched engine runs the Feldman-Hirshberg exchange");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return bfail(nullptr, PIMDB_ERR_NO_DEVICE, "no CUDA device visible");
    }
    pimdb_batch* b = new (std::nothrow) pimdb_batch();
    if (!b) return bfail(nullptr, PIMDB_ERR_ARG, "out of host memory");
    b->nrep = nreplicas;
    b->D = D;
    b->mixed = precision == PIMDB_MIXED;
    b->cfgs.assign(cfgs, cfgs + nreplicas);
    b->reps.resize(nreplicas);
    b->hoff.resize(nreplicas);
    // pool layout: every array rounded up to 32 doubles (256 bytes)
    auto up = [](size_t n) { return (n + 31) / 32 * 32; };
    std::vector<std::vector<size_t>> offs(nreplicas);
    size_t off = 0, hoff = 0;
    for (int r = 0; r < nreplicas; ++r) {
        Sys s{};
        sys_params_from_config(cfgs[r], s);
        b->maxN = std::max(b->maxN, s.N);
        const size_t nstate = (size_t)s.P * D * s.ld;
        const size_t ntri = s.bosonic ? (size_t)s.N * (s.N + 1) / 2 : 1;
        const bool nm = cfgs[r].propagator == PIMDB_PROP_NORMAL_MODES || cfgs[r].nmthermostat;
        const size_t sizes[] = {nstate, nstate, nstate, (size_t)2 * D * s.ld, ntri, ntri, ntri, ntri,
                                (size_t)s.N + 1, (size_t)s.N + 1, (size_t)s.N + 1, (size_t)s.N + 1,
                                (size_t)s.N + 1, (size_t)s.N + 1, (size_t)s.N, (size_t)s.N,
                                // normal-mode tables Ct, Tt, rot and the physical forces
                                // (empty without normal modes)
                                nm ? (size_t)s.P * s.P : 0, nm ? (size_t)s.P * s.P : 0, nm ? (size_t)4 * s.P : 0,
                                nm ? nstate : 0};
        for (size_t n : sizes) {
            offs[r].push_back(off);
            off += up(n);
        }
        if (nm) b->maxPnm = std::max(b->maxPnm, s.P);
        b->reps[r].s = s;
        b->reps[r].flags = (cfgs[r].thermostat == PIMDB_THERMO_LANGEVIN ? BF_LANGEVIN : 0) |
                           (cfgs[r].fixcom ? BF_FIXCOM : 0) |
                           (cfgs[r].propagator == PIMDB_PROP_NORMAL_MODES ? BF_NM : 0) |
                           (cfgs[r].nmthermostat ? BF_NMTHERMO : 0);
        b->hoff[r] = hoff;
        hoff += (size_t)s.P * s.N * D;
    }
    b->pool_doubles = off;
    b->htotal = hoff;
    cudaError_t e = cudaSuccess;
    if (cuda_stream) {
        b->stream = (cudaStream_t)cuda_stream;
    } else {
        e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
        b->own_stream = (e == cudaSuccess);
    }
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->pool, std::max<size_t>(off, 1) * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(b->pool, 0, std::max<size_t>(off, 1) * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_err, sizeof(int) * nreplicas);
    if (e == cudaSuccess) e = cudaMemset(b->d_err, 0, sizeof(int) * nreplicas);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_iflags, sizeof(int) * 8 * nreplicas);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_scal, sizeof(double) * 4 * nreplicas);
    if (e == cudaSuccess) e = cudaMemset(b->d_scal, 0, sizeof(double) * 4 * nreplicas);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_ctl, sizeof(int) * 2);
    if (e == cudaSuccess) e = cudaMemset(b->d_ctl, 0, sizeof(int) * 2);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_step, sizeof(long long));
    if (e == cudaSuccess) e = cudaMemset(b->d_step, 0, sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_stage, std::max<size_t>(hoff, 1) * sizeof(double));
    if (e != cudaSuccess) {
        free_batch(b);
        return bfail(nullptr, PIMDB_ERR_CUDA, cudaGetErrorString(e));
    }
    std::vector<int> iflags(8 * (size_t)nreplicas, 0);
    for (int r = 0; r < nreplicas; ++r) {
        Sys& s = b->reps[r].s;
        const size_t* o = offs[r].data();
        double* P = b->pool;
        s.x = P + o[0];
        s.p = P + o[1];
        s.f = P + o[2];
        s.fphys = (b->reps[r].flags & BF_NM) ? P + o[19] : nullptr;  // the normal-mode kick force
        s.fx = P + o[3];
        s.E = P + o[4];
        s.Et = P + o[5];
        s.Wf = P + o[6];
        s.Wb = P + o[7];
        s.V = P + o[8];
        s.Vb = P + o[9];
        s.Vh = P + o[10];
        s.Vbh = P + o[11];
        s.yf = P + o[12];
        s.yb = P + o[13];
        s.rowR = P + o[14];
        s.rowC = P + o[15];
        s.scal = b->d_scal + 4 * (size_t)r;
        s.red = nullptr;
        s.err = b->d_err + r;
        s.xflags = b->d_iflags + 8 * (size_t)r;
        iflags[8 * (size_t)r + 3] = 1;
        b->reps[r].nm = NmTabs{nullptr, nullptr, nullptr};
        if (b->reps[r].flags & (BF_NM | BF_NMTHERMO)) {
            // the one-system path's tables, transposed for the warps' reads
            std::vector<double> C, T, rot;
            nm_tables(s.P, s.omega_p, s.mass, s.dt, C, T, rot);
            std::vector<double> Ct(C.size()), Tt(T.size());
            for (int k = 0; k < s.P; ++k)
                for (int j = 0; j < s.P; ++j) {
                    Ct[(size_t)j * s.P + k] = C[(size_t)k * s.P + j];
                    Tt[(size_t)k * s.P + j] = T[(size_t)j * s.P + k];
                }
            b->reps[r].nm = NmTabs{P + o[16], P + o[17], P + o[18]};
            if (e == cudaSuccess) e = cudaMemcpy(P + o[16], Ct.data(), Ct.size() * sizeof(double), cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = cudaMemcpy(P + o[17], Tt.data(), Tt.size() * sizeof(double), cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = cudaMemcpy(P + o[18], rot.data(), rot.size() * sizeof(double), cudaMemcpyHostToDevice);
        }
    }
    // largest replicas first: pair work P N^2, exchange N^2 FP64 exponentials
    b->order.resize(nreplicas);
    std::iota(b->order.begin(), b->order.end(), 0);
    auto cost = [&](int r) {
        const Sys& s = b->reps[r].s;
        const double n = s.N, p = s.P;
        const int fl = b->reps[r].flags;
        const double nm = ((fl & BF_NM) ? 4.0 : 0.0) + ((fl & BF_NMTHERMO) && (fl & BF_LANGEVIN) ? 4.0 : 0.0);
        return p * n * (n + 32.0) + (s.bosonic ? 64.0 * n * n : 0.0) + nm * 64.0 * n * p * p;
    };
    std::stable_sort(b->order.begin(), b->order.end(), [&](int a, int c) { return cost(a) > cost(c); });
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_reps, sizeof(BatchRep) * nreplicas);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_reps, b->reps.data(), sizeof(BatchRep) * nreplicas, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_order, sizeof(int) * nreplicas);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_order, b->order.data(), sizeof(int) * nreplicas, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_hoff, sizeof(size_t) * nreplicas);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_hoff, b->hoff.data(), sizeof(size_t) * nreplicas, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_iflags, iflags.data(), sizeof(int) * iflags.size(), cudaMemcpyHostToDevice);
    int dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) {
        free_batch(b);
        return bfail(nullptr, PIMDB_ERR_CUDA, cudaGetErrorString(e));
    }
    // 256 threads unless the largest replica's staging needs smaller blocks
    int st = PIMDB_ERR_CONFIG;
    for (int t = 256; t >= 32 && st == PIMDB_ERR_CONFIG; t /= 2) st = configure_launch(b, t, 2);
    if (st != PIMDB_OK) {
        const std::string msg = b->err;
        free_batch(b);
        return bfail(nullptr, st, msg);
    }
    *out = b;
    return PIMDB_OK;
}

extern "C" int pimdb_batch_destroy(pimdb_batch* b) {
    if (!b) return bfail(nullptr, PIMDB_ERR_ARG, "NULL batch");
    cudaStreamSynchronize(b->stream);
    free_batch(b);
    return PIMDB_OK;
}

extern "C" int pimdb_batch_size(const pimdb_batch* b, int* nreplicas, long long* host_doubles) {
    if (!b) return bfail(nullptr, PIMDB_ERR_ARG, "NULL batch");
    if (nreplicas) *nreplicas = b->nrep;
    if (host_doubles) *host_doubles = (long long)b->htotal;
    return PIMDB_OK;
}

static int check_errors(pimdb_batch* b) {
    std::vector<int> errs(b->nrep);
    BATCH_CUDA(b, cudaMemcpyAsync(errs.data(), b->d_err, sizeof(int) * b->nrep, cudaMemcpyDeviceToHost, b->stream));
    BATCH_CUDA(b, cudaStreamSynchronize(b->stream));
    for (int r = 0; r < b->nrep; ++r)
        if (errs[r] & ERRB_NONFINITE_VB)
            return bfail(b, PIMDB_ERR_NONFINITE_VB,
                         "replica " + std::to_string(r) + ": Invalid sig_denom in bosonic exchange potential");
    return PIMDB_OK;
}

// All replicas from host arrays concatenated in replica order, each
// [bead][particle][axis]; x or p may be NULL to keep the current values.
extern "C" int pimdb_batch_set_states(pimdb_batch* b, const double* x, const double* p) {
    if (!b) return bfail(nullptr, PIMDB_ERR_ARG, "NULL batch");
    const double* src[2] = {x, p};
    for (int k = 0; k < 2; ++k) {
        if (!src[k]) continue;
        BATCH_CUDA(b, cudaMemcpyAsync(b->d_stage, src[k], b->htotal * sizeof(double), cudaMemcpyHostToDevice, b->stream));
        dim3 grid(8, b->nrep);
        if (b->D == 1) k_batch_pack<1><<<grid, 256, 0, b->stream>>>(b->d_reps, b->d_hoff, b->d_stage, k);
        else if (b->D == 2) k_batch_pack<2><<<grid, 256, 0, b->stream>>>(b->d_reps, b->d_hoff, b->d_stage, k);
        else k_batch_pack<3><<<grid, 256, 0, b->stream>>>(b->d_reps, b->d_hoff, b->d_stage, k);
        ++b->launches;
    }
    k_batch_reset<<<b->nrep, 256, 0, b->stream>>>(b->d_reps, b->D);
    ++b->launches;
    BATCH_CUDA(b, cudaGetLastError());
    BATCH_CUDA(b, cudaStreamSynchronize(b->stream));
    return PIMDB_OK;
}

extern "C" int pimdb_batch_get_states(pimdb_batch* b, double* x, double* p, double* f) {
    if (!b) return bfail(nullptr, PIMDB_ERR_ARG, "NULL batch");
    double* dst[3] = {x, p, f};
    for (int k = 0; k < 3; ++k) {
        if (!dst[k]) continue;
        dim3 grid(8, b->nrep);
        if (b->D == 1) k_batch_unpack<1><<<grid, 256, 0, b->stream>>>(b->d_reps, b->d_hoff, b->d_stage, k);
        else if (b->D == 2) k_batch_unpack<2><<<grid, 256, 0, b->stream>>>(b->d_reps, b->d_hoff, b->d_stage, k);
        else k_batch_unpack<3><<<grid, 256, 0, b->stream>>>(b->d_reps, b->d_hoff, b->d_stage, k);
        ++b->launches;
        BATCH_CUDA(b, cudaMemcpyAsync(dst[k], b->d_stage, b->htotal * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    }
    BATCH_CUDA(b, cudaGetLastError());
    BATCH_CUDA(b, cudaStreamSynchronize(b->stream));
    return PIMDB_OK;
}

extern "C" int pimdb_batch_set_step(pimdb_batch* b, long long step) {
    if (!b) return bfail(nullptr, PIMDB_ERR_ARG, "NULL batch");
    BATCH_CUDA(b, cudaMemcpyAsync(b->d_step, &step, sizeof(long long), cudaMemcpyHostToDevice, b->stream));
    BATCH_CUDA(b, cudaStreamSynchronize(b->stream));
    b->step = step;
    return PIMDB_OK;
}

extern "C" int pimdb_batch_get_step(pimdb_batch* b, long long* step) {
    if (!b || !step) return bfail(b, PIMDB_ERR_ARG, "NULL argument");
    BATCH_CUDA(b, cudaMemcpyAsync(step, b->d_step, sizeof(long long), cudaMemcpyDeviceToHost, b->stream));
    BATCH_CUDA(b, cudaStreamSynchronize(b->stream));
    return PIMDB_OK;
}

extern "C" int pimdb_batch_compute_forces(pimdb_batch* b) {
    if (!b) return bfail(nullptr, PIMDB_ERR_ARG, "NULL batch");
    launch_batch(b, BM_FORCES);
    BATCH_CUDA(b, cudaGetLastError());
    return check_errors(b);
}

static int enqueue_batch_steps(pimdb_batch* b, int nsteps) {
    const int mode = BM_HEAD | BM_FORCES | BM_TAIL | BM_ADVANCE;
    if (!b->use_graph || nsteps == 1) {
        for (int k = 0; k < nsteps; ++k) launch_batch(b, mode);
        BATCH_CUDA(b, cudaGetLastError());
        return PIMDB_OK;
    }
    if (!b->graph || b->graph_steps != nsteps || b->graph_threads != b->threads || b->graph_grid != b->grid) {
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        cudaGraph_t g = nullptr;
        BATCH_CUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        const long long before = b->launches;
        for (int k = 0; k < nsteps; ++k) launch_batch(b, mode);
        b->launches = before;
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->graph = nullptr;
            return bfail(b, PIMDB_ERR_CUDA, cudaGetErrorString(e));
        }
        b->graph_steps = nsteps;
        b->graph_threads = b->threads;
        b->graph_grid = b->grid;
    }
    BATCH_CUDA(b, cudaGraphLaunch(b->graph, b->stream));
    b->launches += nsteps;
    return PIMDB_OK;
}

extern "C" int pimdb_batch_step_async(pimdb_batch* b, int nsteps) {
    if (!b) return bfail(nullptr, PIMDB_ERR_ARG, "NULL batch");
    if (nsteps < 0) return bfail(b, PIMDB_ERR_ARG, "nsteps < 0");
    if (nsteps == 0) return PIMDB_OK;
    const int st = enqueue_batch_steps(b, nsteps);
    if (st == PIMDB_OK) b->step += nsteps;
    return st;
}

extern "C" int pimdb_batch_step(pimdb_batch* b, int nsteps) {
    const int st = pimdb_batch_step_async(b, nsteps);
    if (st != PIMDB_OK) return st;
    return check_errors(b);
}

extern "C" int pimdb_batch_synchronize(pimdb_batch* b) {
    if (!b) return bfail(nullptr, PIMDB_ERR_ARG, "NULL batch");
    return check_errors(b);
}

// V_B, primEstimator, P_distinct and P_longest of every replica at the
// current coordinates (forces are evaluated first); scalars [nrep][4]
// (zeros for distinguishable replicas).
extern "C" int pimdb_batch_exchange(pimdb_batch* b, double* scalars) {
    if (!b || !scalars) return bfail(b, PIMDB_ERR_ARG, "NULL argument");
    launch_batch(b, BM_FORCES | BM_ESTIMATORS);
    BATCH_CUDA(b, cudaGetLastError());
    const int st = check_errors(b);
    if (st != PIMDB_OK) return st;
    BATCH_CUDA(b, cudaMemcpyAsync(scalars, b->d_scal, sizeof(double) * 4 * b->nrep, cudaMemcpyDeviceToHost, b->stream));
    BATCH_CUDA(b, cudaStreamSynchronize(b->stream));
    return PIMDB_OK;
}

extern "C" int pimdb_batch_set_option(pimdb_batch* b, const char* name, int value) {
    if (!b || !name) return bfail(b, PIMDB_ERR_ARG, "NULL argument");
    if (!strcmp(name, "threads")) return configure_launch(b, value, b->ctas_per_sm);
    if (!strcmp(name, "ctas_per_sm")) return configure_launch(b, b->threads, value);
    if (!strcmp(name, "graph")) {
        b->use_graph = value != 0;
        return PIMDB_OK;
    }
    return bfail(b, PIMDB_ERR_ARG, std::string("unknown option ") + name);
}

extern "C" int pimdb_batch_get_launch(pimdb_batch* b, int* threads, int* ctas_per_sm, int* grid, long long* launches) {
    if (!b) return bfail(nullptr, PIMDB_ERR_ARG, "NULL batch");
    if (threads) *threads = b->threads;
    if (ctas_per_sm) *ctas_per_sm = b->ctas_per_sm;
    if (grid) *grid = b->grid;
    if (launches) *launches = b->launches;
    return PIMDB_OK;
}

// Block shape of the step kernel chosen by measurement: every candidate
// (threads per CTA x CTAs per SM that fit) runs `steps` steps from a copy of
// the current device state, timed with events; the fastest is kept and the
// state, the exchange estimates and the step counter are restored.
extern "C" int pimdb_batch_autotune(pimdb_batch* b, int steps, int* threads, int* ctas_per_sm) {
    if (!b) return bfail(nullptr, PIMDB_ERR_ARG, "NULL batch");
    if (steps < 1) steps = 2;
    double* snap = nullptr;
    int* fsnap = nullptr;
    long long step0 = 0;
    BATCH_CUDA(b, cudaStreamSynchronize(b->stream));
    BATCH_CUDA(b, cudaMalloc((void**)&snap, b->pool_doubles * sizeof(double)));
    cudaError_t e = cudaMalloc((void**)&fsnap, sizeof(int) * 8 * b->nrep);
    if (e == cudaSuccess) e = cudaMemcpyAsync(snap, b->pool, b->pool_doubles * sizeof(double), cudaMemcpyDeviceToDevice, b->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fsnap, b->d_iflags, sizeof(int) * 8 * b->nrep, cudaMemcpyDeviceToDevice, b->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&step0, b->d_step, sizeof(long long), cudaMemcpyDeviceToHost, b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    const int old_threads = b->threads, old_ctas = b->ctas_per_sm;
    const bool old_graph = b->use_graph;
    b->use_graph = false;
    int best_t = old_threads, best_c = old_ctas;
    float best_ms = 1e30f;
    const int cand_t[] = {128, 256, 512};
    const int cand_c[] = {1, 2, 3, 4};
    for (int ti = 0; ti < 3 && e == cudaSuccess; ++ti) {
        for (int ci = 0; ci < 4 && e == cudaSuccess; ++ci) {
            if (configure_launch(b, cand_t[ti], cand_c[ci]) != PIMDB_OK) continue;
            if (b->ctas_per_sm != cand_c[ci]) continue;  // does not fit
            enqueue_batch_steps(b, 1);  // warm-up
            e = cudaEventRecord(t0, b->stream);
            if (e == cudaSuccess) enqueue_batch_steps(b, steps);
            if (e == cudaSuccess) e = cudaEventRecord(t1, b->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(t1);
            float ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
            if (e == cudaSuccess && ms < best_ms) {
                best_ms = ms;
                best_t = cand_t[ti];
                best_c = cand_c[ci];
            }
            if (e == cudaSuccess) e = cudaMemcpyAsync(b->pool, snap, b->pool_doubles * sizeof(double), cudaMemcpyDeviceToDevice, b->stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_iflags, fsnap, sizeof(int) * 8 * b->nrep, cudaMemcpyDeviceToDevice, b->stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(b->d_step, &step0, sizeof(long long), cudaMemcpyHostToDevice, b->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
        }
    }
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    cudaFree(snap);
    cudaFree(fsnap);
    b->use_graph = old_graph;
    if (e != cudaSuccess) return bfail(b, PIMDB_ERR_CUDA, cudaGetErrorString(e));
    const int st = configure_launch(b, best_t, best_c);
    if (st != PIMDB_OK) return st;
    if (threads) *threads = b->threads;
    if (ctas_per_sm) *ctas_per_sm = b->ctas_per_sm;
    return check_errors(b);
}

extern "C" int pimdb_batch_last_error(const pimdb_batch* b, char* buf, int len) {
    const std::string& m = b ? b->err : g_batch_error;
    if (buf && len > 0) {
        std::snprintf(buf, (size_t)len, "%s", m.c_str());
    }
    return PIMDB_OK;
}

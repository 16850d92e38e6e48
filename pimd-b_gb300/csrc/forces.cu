// Per-bead forces: external potential, all-pairs interaction (shared-memory
// tiled, minimum image, cutoff) and the distinguishable ring springs.
//
// Reference: Simulation::updateForces / updateSpringForces /
// updatePhysicalForces (src/simulation.cpp:353-455) and the potentials'
// gradV (src/potentials/{harmonic,aziz,dipole,double_well,cosine}.cpp).
//
// One thread owns one particle of one bead and sums the pair gradient over
// every other particle of the same bead (j ascending), so no atomics are
// needed and the result is deterministic.  Precision: `R` is the arithmetic
// type of the pair gradient (double for the plain path, float for the mixed
// path, which reconstructs separations from hi/lo float pairs and adds each
// tile's float partial sum into a double accumulator).
#include "forces_dev.cuh"
#include "kernels.h"

namespace pimdb {

constexpr int kPairThreads = 128;

template <int D, typename R>
__global__ void __launch_bounds__(kPairThreads) k_bead_forces(Sys s, int write_phys) {
    __shared__ double xs[D][kPairThreads];
    const int b = blockIdx.y;
    const int i = blockIdx.x * kPairThreads + threadIdx.x;
    const bool active = i < s.N;
    double xi[D];
#pragma unroll
    for (int a = 0; a < D; ++a) xi[a] = active ? s.x[idx<D>(s, b, a, i)] : 0.0;

    double acc[D];
    ext_force<D>(s, xi, acc);

    const bool pairs = s.int_kind != POT_FREE && s.cutoff != 0.0;
    if (pairs) {
        const double cut = s.cutoff;
        const R cutR = (R)cut;
        const R paramR = (R)s.int_a;
        R hi[D], lo[D];
#pragma unroll
        for (int a = 0; a < D; ++a) {
            hi[a] = (R)xi[a];
            lo[a] = (R)(xi[a] - (double)hi[a]);
        }
        for (int j0 = 0; j0 < s.N; j0 += kPairThreads) {
            const int jl = j0 + threadIdx.x;
            __syncthreads();
#pragma unroll
            for (int a = 0; a < D; ++a) xs[a][threadIdx.x] = jl < s.N ? s.x[idx<D>(s, b, a, jl)] : 0.0;
            __syncthreads();
            if (!active) continue;
            const int jn = min(kPairThreads, s.N - j0);
            R t[D];
#pragma unroll
            for (int a = 0; a < D; ++a) t[a] = (R)0;
            for (int jj = 0; jj < jn; ++jj) {
                const int j = j0 + jj;
                if (j == i) continue;
                R r[D];
                R r2 = (R)0;
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    R d;
                    if constexpr (sizeof(R) == 8) {
                        d = xi[a] - xs[a][jj];
                        if (s.pbc) d = min_image(d, s.L, s.invL);
                    } else {
                        const double xj = xs[a][jj];
                        const float hj = (float)xj;
                        const float lj = (float)(xj - (double)hj);
                        d = (hi[a] - hj) + (lo[a] - lj);
                        if (s.pbc) d = min_image_f(d, (float)s.L, (float)s.invL);
                    }
                    r[a] = d;
                    r2 += d * d;
                }
                if (cut < 0.0 || (sizeof(R) == 8 ? sqrt((double)r2) < cut : r2 < cutR * cutR)) {
                    const R sc = pair_scale<R>(s.int_kind, r2, paramR);
#pragma unroll
                    for (int a = 0; a < D; ++a) t[a] -= sc * r[a];
                }
            }
#pragma unroll
            for (int a = 0; a < D; ++a) acc[a] += (double)t[a];
        }
    }
    if (!active) return;

    const bool bosonic_bead = s.bosonic && (b == 0 || b == s.P - 1);
    const int bp = (b - 1 + s.P) % s.P, bn = (b + 1) % s.P;
#pragma unroll
    for (int a = 0; a < D; ++a) {
        const size_t o = idx<D>(s, b, a, i);
        if (write_phys) s.fphys[o] = acc[a];
        if (bosonic_bead) {
            s.f[o] = acc[a];  // the exchange kernels add the exterior springs
        } else {
            double dp = s.x[idx<D>(s, bp, a, i)] - xi[a];
            double dn = s.x[idx<D>(s, bn, a, i)] - xi[a];
            if (s.pbc) {
                dp = min_image(dp, s.L, s.invL);
                dn = min_image(dn, s.L, s.invL);
            }
            s.f[o] = s.kappa * (dp + dn) + acc[a];  // simulation.cpp:405-419, :363-373
        }
    }
}

// ---------------------------------------------------------------------------
// Newton's-third-law pair forces.  The N x N pair matrix of one bead is cut
// into 32 x 32 tiles; one warp owns one tile (it, jt) with jt >= it.  Lane t
// holds particle i = 32 it + t and, rotating one lane per step, every j of
// tile jt together with j's force accumulator, so each unordered pair is
// evaluated once and no atomics are needed.  The warp writes its two partial
// sums into part[b][slot][axis][particle], slot = the other tile's index;
// every (particle, slot) is written exactly once, and k_bead_finish adds the
// slots in ascending order (deterministic).
constexpr int kTile = 32;

template <typename R, int D>
struct PairPos {
    R h[D], l[D];  // value = h + l (for R = double, l = 0)
};

template <typename R, int D>
__device__ __forceinline__ PairPos<R, D> split_pos(const double* x) {
    PairPos<R, D> q;
#pragma unroll
    for (int a = 0; a < D; ++a) {
        q.h[a] = (R)x[a];
        q.l[a] = (R)(x[a] - (double)q.h[a]);
    }
    return q;
}

template <int D, typename R>
__device__ __forceinline__ bool pair_force(const Sys& s, const PairPos<R, D>& pi, const PairPos<R, D>& pj,
                                           R* g) {
    const double cut = s.cutoff;
    if constexpr (sizeof(R) == 8) {
        // cheap FP32 screen: pairs clearly beyond the cutoff skip the FP64 work
        if (cut > 0.0) {
            float r2f = 0.0f;
#pragma unroll
            for (int a = 0; a < D; ++a) {
                float d = (float)pi.h[a] - (float)pj.h[a];
                if (s.pbc) d = min_image_f(d, (float)s.L, (float)s.invL);
                r2f += d * d;
            }
            if (r2f > (float)(cut * cut) * 1.0001f) return false;
        }
    }
    R r[D];
    R r2 = (R)0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
        R d;
        if constexpr (sizeof(R) == 8) {
            d = pi.h[a] - pj.h[a];
            if (s.pbc) d = min_image(d, s.L, s.invL);
        } else {
            d = (pi.h[a] - pj.h[a]) + (pi.l[a] - pj.l[a]);
            if (s.pbc) d = min_image_f(d, (float)s.L, (float)s.invL);
        }
        r[a] = d;
        r2 += d * d;
    }
    bool in;
    if (cut < 0.0) in = true;
    else if constexpr (sizeof(R) == 8) in = r2 < cut * cut;  // |r| < cutoff (simulation.cpp:444)
    else in = r2 < (float)(cut * cut);
    if (!in) return false;
    const R sc = pair_scale<R>(s.int_kind, r2, (R)s.int_a);
#pragma unroll
    for (int a = 0; a < D; ++a) g[a] = sc * r[a];  // grad V(r_i - r_j)
    return true;
}

template <typename R, int D>
__device__ __forceinline__ void rotate(PairPos<R, D>& q, R* acc, int& jidx, int lane) {
    const int src = (lane + 1) & 31;
#pragma unroll
    for (int a = 0; a < D; ++a) {
        q.h[a] = __shfl_sync(0xffffffffu, q.h[a], src);
        if constexpr (sizeof(R) == 4) q.l[a] = __shfl_sync(0xffffffffu, q.l[a], src);
        acc[a] = __shfl_sync(0xffffffffu, acc[a], src);
    }
    jidx = __shfl_sync(0xffffffffu, jidx, src);
}

template <int D, typename R>
__global__ void __launch_bounds__(128) k_pair_tiles(Sys s, double* __restrict__ part, int T, int npairs) {
    const int w = blockIdx.x * 4 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.y;
    if (w >= npairs) return;
    // tile pair (it, jt), jt >= it, row-major over the upper triangle
    int it = (int)((2.0 * T + 1.0 - sqrt((2.0 * T + 1.0) * (2.0 * T + 1.0) - 8.0 * w)) * 0.5);
    while (it > 0 && it * T - it * (it - 1) / 2 > w) --it;
    while ((it + 1) * T - (it + 1) * it / 2 <= w) ++it;
    const int jt = it + (w - (it * T - it * (it - 1) / 2));
    const bool diag = it == jt;

    const int i = it * kTile + lane;
    int jidx = jt * kTile + lane;
    double xi[D], xj[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
        xi[a] = i < s.N ? s.x[idx<D>(s, b, a, i)] : 0.0;
        xj[a] = jidx < s.N ? s.x[idx<D>(s, b, a, jidx)] : 0.0;
    }
    const PairPos<R, D> pi = split_pos<R, D>(xi);
    PairPos<R, D> pj = split_pos<R, D>(xj);
    R ai[D], aj[D];
#pragma unroll
    for (int a = 0; a < D; ++a) ai[a] = aj[a] = (R)0;
    int rot = 0;
    const int first = diag ? 1 : 0, lastS = diag ? 16 : 31;
    if (diag) {
        rotate<R, D>(pj, aj, jidx, lane);
        ++rot;
    }
    for (int st = first; st <= lastS; ++st) {
        const bool act = i < s.N && jidx < s.N && (!diag || st < 16 || lane < 16);
        if (act) {
            R g[D];
            if (pair_force<D, R>(s, pi, pj, g)) {
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    ai[a] -= g[a];
                    aj[a] += g[a];
                }
            }
        }
        rotate<R, D>(pj, aj, jidx, lane);
        ++rot;
    }
    while (rot & 31) {  // bring every j accumulator back to its home lane
        rotate<R, D>(pj, aj, jidx, lane);
        ++rot;
    }
    const size_t base_b = (size_t)b * T;
    if (diag) {
        if (i < s.N) {
#pragma unroll
            for (int a = 0; a < D; ++a)
                part[((base_b + it) * D + a) * s.ld + i] = (double)ai[a] + (double)aj[a];
        }
    } else {
        if (i < s.N) {
#pragma unroll
            for (int a = 0; a < D; ++a) part[((base_b + jt) * D + a) * s.ld + i] = (double)ai[a];
        }
        if (jidx < s.N) {
#pragma unroll
            for (int a = 0; a < D; ++a) part[((base_b + it) * D + a) * s.ld + jidx] = (double)aj[a];
        }
    }
}

// ---------------------------------------------------------------------------
// FP64 pair tiles with lane compaction (plain path with a finite cutoff).
// A warp-instruction on the FP64 pipe costs the same whether or not its lanes
// are active, so evaluating the Aziz gradient only in the lanes whose pair is
// inside the cutoff wastes the pipe on the others.  Each warp therefore
//   1. screens its tile's pairs with FP32 distances and records, per i lane,
//      the j's inside the cutoff (plus a small margin), and per j lane the
//      (i, position) of those entries;
//   2. lays the entries out i-major and evaluates them 32 at a time in FP64,
//      every lane busy, storing each gradient in shared memory;
//   3. sums the gradients per i and per j in list order (deterministic).
// Same result as k_pair_tiles; the exact FP64 cutoff test is applied in step 2.
constexpr int kCompactWarps = 2;

template <int D>
struct CompactSmem {
    double xi[kTile][D], xj[kTile][D];
    double g[kTile * kTile][D];
    unsigned char ilist[kTile][kTile];     // j's of lane i
    unsigned short jlist[kTile][kTile];    // (i << 8 | k) entries of lane j
    int icnt[kTile], jcnt[kTile], off[kTile];
    unsigned char fi[kTile * kTile], fj[kTile * kTile];
};

template <int D>
__global__ void __launch_bounds__(32 * kCompactWarps) k_pair_tiles_compact(Sys s, double* __restrict__ part, int T,
                                                                          int npairs) {
    extern __shared__ __align__(16) unsigned char csm_raw[];
    CompactSmem<D>& sm = reinterpret_cast<CompactSmem<D>*>(csm_raw)[threadIdx.x >> 5];
    const int w = blockIdx.x * kCompactWarps + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.y;
    if (w >= npairs) return;
    int it = (int)((2.0 * T + 1.0 - sqrt((2.0 * T + 1.0) * (2.0 * T + 1.0) - 8.0 * w)) * 0.5);
    while (it > 0 && it * T - it * (it - 1) / 2 > w) --it;
    while ((it + 1) * T - (it + 1) * it / 2 <= w) ++it;
    const int jt = it + (w - (it * T - it * (it - 1) / 2));
    const bool diag = it == jt;
    const int i = it * kTile + lane, j = jt * kTile + lane;
#pragma unroll
    for (int a = 0; a < D; ++a) {
        sm.xi[lane][a] = i < s.N ? s.x[idx<D>(s, b, a, i)] : 0.0;
        sm.xj[lane][a] = j < s.N ? s.x[idx<D>(s, b, a, j)] : 0.0;
    }
    sm.icnt[lane] = 0;
    sm.jcnt[lane] = 0;
    __syncwarp();
    // 1. FP32 screen, one rotation step at a time (lane i meets j = i + st)
    const double cut = s.cutoff;
    const float cut2f = (float)(cut * cut) * 1.0001f;
    const float Lf = (float)s.L, invLf = (float)s.invL;
    float xif[D];
#pragma unroll
    for (int a = 0; a < D; ++a) xif[a] = (float)sm.xi[lane][a];
    int icnt = 0;
    const int first = diag ? 1 : 0, lastS = diag ? 16 : 31;
    for (int st = first; st <= lastS; ++st) {
        const int jl = (lane + st) & 31;
        bool in = i < s.N && jt * kTile + jl < s.N && (!diag || st < 16 || lane < 16);
        if (in) {
            float r2 = 0.0f;
#pragma unroll
            for (int a = 0; a < D; ++a) {
                float d = xif[a] - (float)sm.xj[jl][a];
                if (s.pbc) d = min_image_f(d, Lf, invLf);
                r2 += d * d;
            }
            in = r2 <= cut2f;
        }
        if (in) {
            const int jc = sm.jcnt[jl];  // lanes of one step hit distinct j's
            sm.jlist[jl][jc] = (unsigned short)((lane << 8) | icnt);
            sm.jcnt[jl] = jc + 1;
            sm.ilist[lane][icnt++] = (unsigned char)jl;
        }
        __syncwarp();
    }
    sm.icnt[lane] = icnt;
    // 2. i-major layout: offsets by a warp scan of the counts
    int off = icnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, off, o);
        if (lane >= o) off += y;
    }
    const int total = __shfl_sync(0xffffffffu, off, 31);
    off -= icnt;
    sm.off[lane] = off;
    for (int k = 0; k < icnt; ++k) {
        sm.fi[off + k] = (unsigned char)lane;
        sm.fj[off + k] = sm.ilist[lane][k];
    }
    __syncwarp();
    for (int f = lane; f < total; f += 32) {
        const int il = sm.fi[f], jl = sm.fj[f];
        double r[D];
        double r2 = 0.0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            double d = sm.xi[il][a] - sm.xj[jl][a];
            if (s.pbc) d = min_image(d, s.L, s.invL);
            r[a] = d;
            r2 += d * d;
        }
        const double sc = r2 < cut * cut ? pair_scale<double>(s.int_kind, r2, s.int_a) : 0.0;
#pragma unroll
        for (int a = 0; a < D; ++a) sm.g[f][a] = sc * r[a];  // grad V(r_i - r_j)
    }
    __syncwarp();
    // 3. deterministic sums: i side over its own (contiguous) entries, j side
    //    over its list in recording order
    double ai[D], aj[D];
#pragma unroll
    for (int a = 0; a < D; ++a) ai[a] = aj[a] = 0.0;
    for (int k = 0; k < icnt; ++k)
#pragma unroll
        for (int a = 0; a < D; ++a) ai[a] -= sm.g[off + k][a];
    const int jc = sm.jcnt[lane];
    for (int k = 0; k < jc; ++k) {
        const int e = sm.jlist[lane][k];
        const int f = sm.off[e >> 8] + (e & 255);
#pragma unroll
        for (int a = 0; a < D; ++a) aj[a] += sm.g[f][a];
    }
    const size_t base_b = (size_t)b * T;
    if (diag) {
        if (i < s.N) {
#pragma unroll
            for (int a = 0; a < D; ++a) part[((base_b + it) * D + a) * s.ld + i] = ai[a] + aj[a];
        }
    } else {
        if (i < s.N) {
#pragma unroll
            for (int a = 0; a < D; ++a) part[((base_b + jt) * D + a) * s.ld + i] = ai[a];
        }
        if (j < s.N) {
#pragma unroll
            for (int a = 0; a < D; ++a) part[((base_b + it) * D + a) * s.ld + j] = aj[a];
        }
    }
}

// f = springs + (-grad V_ext + sum of the pair slots), one thread per
// (bead, axis, particle).  T = 0 when there are no pair forces.
template <int D>
__global__ void k_bead_finish(Sys s, const double* __restrict__ part, int T, int write_phys) {
    const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const int i = (int)(e % s.ld);
    const size_t ba = e / s.ld;
    if (ba >= (size_t)s.P * D || i >= s.N) return;
    const int a = (int)(ba % D), b = (int)(ba / D);
    double xi[D];
#pragma unroll
    for (int c = 0; c < D; ++c) xi[c] = s.x[idx<D>(s, b, c, i)];
    double fe[D];
    ext_force<D>(s, xi, fe);
    double acc = fe[a];
    for (int q = 0; q < T; ++q) acc += part[(((size_t)b * T + q) * D + a) * s.ld + i];
    const size_t o = idx<D>(s, b, a, i);
    if (write_phys) s.fphys[o] = acc;
    if (s.bosonic && (b == 0 || b == s.P - 1)) {
        s.f[o] = acc;
    } else {
        const int bp = (b - 1 + s.P) % s.P, bn = (b + 1) % s.P;
        double dp = s.x[idx<D>(s, bp, a, i)] - xi[a];
        double dn = s.x[idx<D>(s, bn, a, i)] - xi[a];
        if (s.pbc) {
            dp = min_image(dp, s.L, s.invL);
            dn = min_image(dn, s.L, s.invL);
        }
        s.f[o] = s.kappa * (dp + dn) + acc;
    }
}

size_t pair_partial_doubles(const Sys& s, int D) {
    const int T = (s.N + kTile - 1) / kTile;
    return (size_t)s.P * T * D * s.ld;
}

template <int D>
static void tiles_launch(const Sys& s, int mixed, int write_phys, double* part, cudaStream_t st) {
    const bool pairs = s.int_kind != POT_FREE && s.cutoff != 0.0;
    const int T = pairs ? (s.N + kTile - 1) / kTile : 0;
    if (pairs) {
        const int np = T * (T + 1) / 2;
        if (!mixed && s.cutoff > 0.0) {
            const size_t smem = sizeof(CompactSmem<D>) * kCompactWarps;
            static bool attr = false;
            if (!attr) {
                cudaFuncSetAttribute(k_pair_tiles_compact<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                attr = true;
            }
            dim3 grid((np + kCompactWarps - 1) / kCompactWarps, s.P);
            k_pair_tiles_compact<D><<<grid, 32 * kCompactWarps, smem, st>>>(s, part, T, np);
        } else {
            dim3 grid((np + 3) / 4, s.P);
            if (mixed) k_pair_tiles<D, float><<<grid, 128, 0, st>>>(s, part, T, np);
            else k_pair_tiles<D, double><<<grid, 128, 0, st>>>(s, part, T, np);
        }
    }
    const size_t n = (size_t)s.P * D * s.ld;
    k_bead_finish<D><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s, part, T, write_phys);
}

void launch_pair_tiles_and_finish(const Sys& s, int D, int mixed, int write_phys, double* part, cudaStream_t st) {
    if (D == 1) tiles_launch<1>(s, mixed, write_phys, part, st);
    else if (D == 2) tiles_launch<2>(s, mixed, write_phys, part, st);
    else tiles_launch<3>(s, mixed, write_phys, part, st);
}

template <int D>
void launch_bead_forces(const Sys& s, int mixed, int write_phys, cudaStream_t st) {
    dim3 grid((s.N + kPairThreads - 1) / kPairThreads, s.P);
    if (mixed)
        k_bead_forces<D, float><<<grid, kPairThreads, 0, st>>>(s, write_phys);
    else
        k_bead_forces<D, double><<<grid, kPairThreads, 0, st>>>(s, write_phys);
}

void launch_bead_forces(const Sys& s, int D, int mixed, int write_phys, cudaStream_t st) {
    if (D == 1) launch_bead_forces<1>(s, mixed, write_phys, st);
    else if (D == 2) launch_bead_forces<2>(s, mixed, write_phys, st);
    else launch_bead_forces<3>(s, mixed, write_phys, st);
}

// ---------------------------------------------------------------------------
// Potential energy, the function whose negative gradient the force kernels
// evaluate: external + pair energies of every bead (each pair once, same
// cutoff and minimum image as the forces) and the ring springs that do not
// take part in the exchange (all P links when distinguishable; links
// b -> b+1, b < P-1, when bosonic, whose exterior links live in V_B).
// Spring energy as classicalSpringEnergy (simulation.cpp:464-486).
constexpr int kEnergyThreads = 128;

template <int D>
__device__ __forceinline__ double link_energy(const Sys& s, int b, int bn, int i) {
    double e = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
        double d = s.x[idx<D>(s, bn, a, i)] - s.x[idx<D>(s, b, a, i)];
        if (s.pbc) d = min_image(d, s.L, s.invL);
        e += d * d;
    }
    return 0.5 * s.kappa * e;
}

template <int D>
__device__ __forceinline__ double pair_energy_ij(const Sys& s, const double* xi, const double* xj) {
    double r2 = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
        double d = xi[a] - xj[a];
        if (s.pbc) d = min_image(d, s.L, s.invL);
        r2 += d * d;
    }
    if (s.cutoff > 0.0 && !(sqrt(r2) < s.cutoff)) return 0.0;
    return pair_value(s.int_kind, r2, s.int_a);
}

// part[(b * gridDim.x + block) * 3 + {0 external, 1 pair, 2 spring}]
template <int D>
__global__ void __launch_bounds__(kEnergyThreads) k_energy_terms(Sys s, double* __restrict__ part) {
    __shared__ double xs[D][kEnergyThreads];
    __shared__ double red[3 * 32];
    const int b = blockIdx.y;
    const int i = blockIdx.x * kEnergyThreads + threadIdx.x;
    const bool active = i < s.N;
    double xi[D];
#pragma unroll
    for (int a = 0; a < D; ++a) xi[a] = active ? s.x[idx<D>(s, b, a, i)] : 0.0;
    double e[3] = {0.0, 0.0, 0.0};
    if (active) {
        e[0] = ext_value<D>(s, xi);
        if (s.P > 1 && (!s.bosonic || b < s.P - 1)) e[2] = link_energy<D>(s, b, (b + 1) % s.P, i);
    }
    const bool pairs = s.int_kind != POT_FREE && s.cutoff != 0.0;
    if (pairs) {
        for (int j0 = blockIdx.x * kEnergyThreads; j0 < s.N; j0 += kEnergyThreads) {
            __syncthreads();
            const int jl = j0 + threadIdx.x;
#pragma unroll
            for (int a = 0; a < D; ++a) xs[a][threadIdx.x] = jl < s.N ? s.x[idx<D>(s, b, a, jl)] : 0.0;
            __syncthreads();
            if (!active) continue;
            const int jn = min(kEnergyThreads, s.N - j0);
            for (int jj = 0; jj < jn; ++jj) {
                const int j = j0 + jj;
                if (j <= i) continue;
                double xj[D];
#pragma unroll
                for (int a = 0; a < D; ++a) xj[a] = xs[a][jj];
                e[1] += pair_energy_ij<D>(s, xi, xj);
            }
        }
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double t = warp_sum(e[k]);
        if (lane == 0) red[k * 32 + w] = t;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int q = 0; q < nw; ++q) t += red[threadIdx.x * 32 + q];
        part[((size_t)b * gridDim.x + blockIdx.x) * 3 + threadIdx.x] = t;
    }
}

// Energy of every term that involves particle i of bead b (one warp per
// item): its external energy, its pair energies with every other particle
// of the bead, and its non-exchange springs.  The derivative of this sum
// (plus V_B on bosonic beads 1 and P) with respect to x_bi is -f_bi.
template <int D>
__global__ void k_local_energy(Sys s, int n, const int* __restrict__ items, double* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (w >= n) return;
    const int b = items[2 * w], i = items[2 * w + 1];
    if (b < 0 || b >= s.P || i < 0 || i >= s.N) {
        if (lane == 0) {
            atomicOr(s.err, ERRB_BOUNDS);
            out[w] = 0.0;
        }
        return;
    }
    double xi[D];
#pragma unroll
    for (int a = 0; a < D; ++a) xi[a] = s.x[idx<D>(s, b, a, i)];
    double e = 0.0;
    if (s.int_kind != POT_FREE && s.cutoff != 0.0) {
        for (int j = lane; j < s.N; j += 32) {
            if (j == i) continue;
            double xj[D];
#pragma unroll
            for (int a = 0; a < D; ++a) xj[a] = s.x[idx<D>(s, b, a, j)];
            e += pair_energy_ij<D>(s, xi, xj);
        }
    }
    e = warp_sum(e);
    if (lane == 0) {
        e += ext_value<D>(s, xi);
        if (s.P > 1) {
            const int bp = (b - 1 + s.P) % s.P, bn = (b + 1) % s.P;
            if (!s.bosonic || b > 0) e += link_energy<D>(s, bp, b, i);
            if (!s.bosonic || b < s.P - 1) e += link_energy<D>(s, b, bn, i);
        }
        out[w] = e;
    }
}

int energy_blocks(const Sys& s) { return (s.N + kEnergyThreads - 1) / kEnergyThreads; }

void launch_energy_terms(const Sys& s, int D, double* part, cudaStream_t st) {
    dim3 grid(energy_blocks(s), s.P);
    if (D == 1) k_energy_terms<1><<<grid, kEnergyThreads, 0, st>>>(s, part);
    else if (D == 2) k_energy_terms<2><<<grid, kEnergyThreads, 0, st>>>(s, part);
    else k_energy_terms<3><<<grid, kEnergyThreads, 0, st>>>(s, part);
}

void launch_local_energy(const Sys& s, int D, int n, const int* items, double* out, cudaStream_t st) {
    const int warps = 4;
    const int grid = (n + warps - 1) / warps;
    if (grid == 0) return;
    if (D == 1) k_local_energy<1><<<grid, 32 * warps, 0, st>>>(s, n, items, out);
    else if (D == 2) k_local_energy<2><<<grid, 32 * warps, 0, st>>>(s, n, items, out);
    else k_local_energy<3><<<grid, 32 * warps, 0, st>>>(s, n, items, out);
}

}  // namespace pimdb

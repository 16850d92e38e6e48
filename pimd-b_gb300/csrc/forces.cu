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
#include <algorithm>
#include <cmath>
#include <mutex>

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
//   1. screens its tile's pairs with FP32 distances: lane i meets the j lanes
//      one rotation step at a time (j positions by shuffle) and sets bit j
//      of its mask for a pair inside the cutoff plus a small margin (and of
//      a second mask inside the Aziz damping radius D r_m); the steps are
//      independent, so they overlap;
//   2. lays the entries out i-major (ascending j within a lane: entry f of
//      lane i at off_i + its rank in the mask), evaluates all of them 32 (two
//      per lane) at a time in FP64 on the branch-free path of the potential
//      (the Aziz form beyond the damping radius), every lane busy, storing
//      each gradient in shared memory, then evaluates the few entries inside
//      the damping radius again on the general path (compacted by ballot so
//      that the branch occupies a single 32-entry pass);
//   3. sums the gradients per i over its contiguous entries and per j over
//      the column of the masks in ascending i (deterministic: the
//      evaluation order does not enter any sum).
// Under PBC the tile's positions are wrapped into the box once, so a
// separation lies in (-L, L).  On the far path each axis is one FP64
// subtraction from the image the FP32 screen chose (x_j - L, x_j or x_j + L,
// kept in shared memory); an entry whose FP32 test lies within 1e-6 L of the
// half-box edge, where the FP32 and FP64 choices could differ, joins the
// damping-radius list, whose exact path takes the minimum image as one
// conditional shift (a compare of the bit patterns and one FP64 add) instead
// of dx - L floor(dx/L + 1/2).  The exponentials use exp_tang256.  Same
// result as k_pair_tiles up to rounding; the exact FP64 cutoff test is
// applied in step 2.
constexpr int kCompactWarps = 2;
// gradient capacity per warp unless Sys::pair_cap says otherwise: 384
// entries let six blocks share an SM; a tile with more entries is summed in
// two chunks (measured on the benchmark system: 82 us at 384 against 86 at
// 544 and 85 at 640)
constexpr int kCompactDefaultCap = 384;
// entries of the damping-radius list evaluated per pass
constexpr int kCompactNear = 256;

// Per-warp shared memory: the fixed part below, then the gradients of up to
// `cap` entries (double[cap][D]).  A tile with more entries inside the
// cutoff than `cap` is evaluated and summed in chunks of `cap` entries.
template <int D>
struct CompactSmem {
    double xi[kTile][D], xj[kTile][D];   // wrapped into the box under PBC
    float xif[kTile][D], xjf[kTile][D];  // FP32 hi parts (nearest floats)
    float xil[kTile][D], xjl[kTile][D];  // double-float path: x - hi, the low words
    union {
        double xjs[2][kTile][D];         // FP64 path under PBC: xj - L, xj + L
        float lo[2][kTile][D];           // mixed path: x - hi of i, of j
        struct {
            float h[2][kTile][D], l[2][kTile][D];
        } img;                           // double-float path under PBC: xj - L, xj + L
    } u;
    unsigned mask[kTile];                // lane i: bit j for each entry (i, j)
    int off[kTile];                      // lane i's first entry
    unsigned short fe[kTile * kTile];    // entry f: near << 15 | i << 5 | j
    unsigned short nl[kCompactNear];     // damping-radius entries of one pass
};
constexpr int kCompactMaxCap = kTile * kTile;
// bytes of one warp's shared memory for a gradient capacity of `cap` entries
template <int D>
__host__ __device__ constexpr size_t compact_warp_bytes(int cap) {
    return (sizeof(CompactSmem<D>) + (size_t)cap * D * sizeof(double) + 15) / 16 * 16;
}

// d in (-L, L) -> its minimum image; `half_bits` = bit pattern of L/2.
__device__ __forceinline__ double min_image_wrapped(double d, double L, long long half_bits) {
    const long long bits = __double_as_longlong(d);
    const double sh = ((bits & 0x7fffffffffffffffLL) > half_bits) ? copysign(L, d) : 0.0;
    return d - sh;
}

// The FP64 gradient scale of the rare entries the tiles evaluate exactly
// (half-box edge, cutoff shell, the reference's short-range branch), out of
// line: the general Aziz form is long, and inlined into the tile loop it
// enlarges the code every warp runs through (instruction-cache misses).
__device__ __noinline__ double pair_scale_exact(int kind, double r2, double param, const double* tbl) {
    return pair_scale_d<true>(kind, r2, param, tbl);
}

// One tile task: bead b, tile pair w (it <= jt) of the bead's T(T+1)/2.
// kMixed: entries beyond the Aziz damping radius (and every entry of the
// other potentials) are evaluated in FP32 from hi/lo separations; entries
// inside it stay FP64, where the repulsive and attractive terms nearly
// cancel and FP32 would lose the difference.  Sums are FP64 either way.
//
// kDf (FP64 path with the Aziz potential): the entries are evaluated in
// double-float on the FP32 pipe (aziz_far_scale_df beyond the damping radius,
// aziz_near_scale_df inside it; about 2^-43 relative), their gradients kept
// as double-floats and every sum formed in double-float; only the entries
// within 1e-6 L of the half-box edge or within 1e-5 of the cutoff (where the
// image or the in/out decision must be the FP64 one) take the exact FP64
// path, as every marked entry does without kDf.
template <int D, bool kMixed, bool kDf>
__device__ __forceinline__ void compact_tile(const Sys& s, double* __restrict__ part, int T, int b, int w,
                                             CompactSmem<D>& sm, double (*g)[D], int cap, const double* tbl,
                                             const dfl::ExpTable* etbl, int lane) {
    using dfl::df;
    auto gd = reinterpret_cast<float2 (*)[D]>(g);  // kDf: gradient entries as (hi, lo)
    int it = 0, rem = w;  // row it holds the T - it tile pairs (it, it..T-1)
    while (rem >= T - it) {
        rem -= T - it;
        ++it;
    }
    const int jt = it + rem;
    const bool diag = it == jt;
    const int i = it * kTile + lane, j = jt * kTile + lane;
    float xif[D], xjf[D];
    const df Ldf{(float)s.L, (float)(s.L - f32_to_f64((float)s.L))};
#pragma unroll
    for (int a = 0; a < D; ++a) {
        double xv = i < s.N ? s.x[idx<D>(s, b, a, i)] : 0.0;
        double yv = j < s.N ? s.x[idx<D>(s, b, a, j)] : 0.0;
        if (s.pbc) {
            xv -= s.L * rint(xv * s.invL);
            yv -= s.L * rint(yv * s.invL);
        }
        sm.xi[lane][a] = xv;
        sm.xj[lane][a] = yv;
        xif[a] = (float)xv;
        xjf[a] = (float)yv;
        sm.xif[lane][a] = xif[a];
        sm.xjf[lane][a] = xjf[a];
        if (kMixed) {
            sm.u.lo[0][lane][a] = (float)(xv - (double)xif[a]);
            sm.u.lo[1][lane][a] = (float)(yv - (double)xjf[a]);
        } else if (kDf) {
            // x = hi + lo exactly in double, lo rounded to float: 48 bits
            sm.xil[lane][a] = (float)(xv - f32_to_f64(xif[a]));
            const float yl = (float)(yv - f32_to_f64(xjf[a]));
            sm.xjl[lane][a] = yl;
            if (s.pbc) {
                const df m = dfl::add(df{xjf[a], yl}, dfl::neg(Ldf));
                const df q = dfl::add(df{xjf[a], yl}, Ldf);
                sm.u.img.h[0][lane][a] = m.hi;
                sm.u.img.l[0][lane][a] = m.lo;
                sm.u.img.h[1][lane][a] = q.hi;
                sm.u.img.l[1][lane][a] = q.lo;
            }
        } else if (s.pbc) {
            sm.u.xjs[0][lane][a] = yv - s.L;
            sm.u.xjs[1][lane][a] = yv + s.L;
        }
    }
    // 1. FP32 screen
    const double cut = s.cutoff;
    const float cut2f = (float)(cut * cut) * 1.0001f;
    const bool aziz = s.int_kind == POT_AZIZ;
    const float near2f = aziz ? (float)(Aziz::D * Aziz::rm * Aziz::D * Aziz::rm) * 1.0001f : -1.0f;
    const float Lf = (float)s.L, halfLf = 0.5f * (float)s.L;
    const int nj = min(kTile, s.N - jt * kTile);  // valid j lanes
    const bool ivalid = i < s.N;
    unsigned mask = 0u, nmask = 0u, xmask = 0u;
    const int first = diag ? 1 : 0, lastS = diag ? 16 : 31;
    // |dx| within this of L/2 in FP32: the FP32 image choice might differ
    // from the FP64 one, so the entry takes the exact path (with the
    // damping-radius entries).  Bound on the FP32 error: 2.5 2^-24 L.
    const float amb = 1e-6f * Lf;
    // the double-float path applies no cutoff test: entries within 1e-5 of
    // the cutoff (far above the FP32 error of r2) take the exact FP64 path
    const float shell2f = (float)(cut * cut) * (1.0f - 1e-5f);
#pragma unroll 4
    for (int st = first; st <= lastS; ++st) {
        const int jl = (lane + st) & 31;
        float r2 = 0.0f;
        bool edge = false;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            float d = xif[a] - __shfl_sync(0xffffffffu, xjf[a], jl);
            if (s.pbc) {
                edge |= fabsf(fabsf(d) - halfLf) <= amb;
                if (fabsf(d) > halfLf) d -= copysignf(Lf, d);
            }
            r2 = fmaf(d, d, r2);
        }
        const bool in = ivalid && jl < nj && (!diag || st < 16 || lane < 16) && r2 <= cut2f;
        mask |= (unsigned)in << jl;
        const bool exact = aziz && (edge || (kDf && r2 >= shell2f));
        nmask |= (unsigned)(in && (r2 < near2f || exact)) << jl;
        xmask |= (unsigned)(in && exact) << jl;
    }
    // 2. i-major layout: offsets by a warp scan of the counts
    const int icnt = __popc(mask);
    int off = icnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, off, o);
        if (lane >= o) off += y;
    }
    const int total = __shfl_sync(0xffffffffu, off, 31);
    off -= icnt;
    sm.mask[lane] = mask;
    sm.off[lane] = off;
    {
        unsigned mm = mask;
        for (int f = off; mm; ++f) {
            const int jj = __ffs(mm) - 1;
            mm &= mm - 1u;
            // bit 15: redo on the near path; bit 14: on the exact FP64 path
            sm.fe[f] = (unsigned short)((((nmask >> jj) & 1u) << 15) | (((xmask >> jj) & 1u) << 14) | (lane << 5) |
                                        jj);
        }
    }
    // the column of lane j: the i's whose masks hold bit j
    unsigned col = 0u;
#pragma unroll
    for (int t = 0; t < 32; ++t) {
        const unsigned bt = __ballot_sync(0xffffffffu, (mask >> t) & 1u);
        if (lane == t) col = bt;
    }
    __syncwarp();
    const long long half_bits = __double_as_longlong(0.5 * s.L);
    const double cut2 = cut * cut;
    const long long cut2_bits = __double_as_longlong(cut2);
    auto separation = [&](int f, double* r) {
        const int e = sm.fe[f], il = (e >> 5) & 31, jl = e & 31;
        double r2 = 0.0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            double d = sm.xi[il][a] - sm.xj[jl][a];
            if (s.pbc) d = min_image_wrapped(d, s.L, half_bits);
            r[a] = d;
            r2 += d * d;
        }
        return r2;
    };
    // The far path's separation: the image is the one the FP32 screen chose
    // (xj - L, xj or xj + L, each rounded once), so one FP64 subtraction per
    // axis; entries where that choice is not certain were marked above.
    auto separation_far = [&](int f, double* r) {
        const int e = sm.fe[f], il = (e >> 5) & 31, jl = e & 31;
        double r2 = 0.0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            double xjv = sm.xj[jl][a];
            if (s.pbc) {
                const float df = sm.xif[il][a] - sm.xjf[jl][a];
                if (fabsf(df) > halfLf) xjv = sm.u.xjs[df > 0.0f ? 1 : 0][jl][a];
            }
            const double d = sm.xi[il][a] - xjv;
            r[a] = d;
            r2 += d * d;
        }
        return r2;
    };
    // The double-float far path's separation: the image the FP32 screen
    // chose (xj - L, xj or xj + L as double-floats), one double-float
    // subtraction per axis.
    auto separation_df = [&](int f, df* r) {
        const int e = sm.fe[f], il = (e >> 5) & 31, jl = e & 31;
        df r2{0.0f, 0.0f};
#pragma unroll
        for (int a = 0; a < D; ++a) {
            df xjv{sm.xjf[jl][a], sm.xjl[jl][a]};
            if (s.pbc) {
                const float dd = sm.xif[il][a] - sm.xjf[jl][a];
                if (fabsf(dd) > halfLf) {
                    const int side = dd > 0.0f ? 1 : 0;
                    xjv = df{sm.u.img.h[side][jl][a], sm.u.img.l[side][jl][a]};
                }
            }
            const df d = dfl::add_sloppy(df{sm.xif[il][a], sm.xil[il][a]}, dfl::neg(xjv));
            r[a] = d;
            r2 = a == 0 ? dfl::sqr(d) : dfl::add_sloppy(r2, dfl::sqr(d));
        }
        return r2;
    };
    double ai[D], aj[D];
    df aid[D], ajd[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
        ai[a] = aj[a] = 0.0;
        aid[a] = ajd[a] = df{0.0f, 0.0f};
    }
    const unsigned lt = (1u << lane) - 1u;
    for (int c0 = 0; c0 < total; c0 += cap) {
        const int cend = min(total, c0 + cap), cn = cend - c0;
        auto store = [&](int f, double sc, const double* r) {
#pragma unroll
            for (int a = 0; a < D; ++a) {
                const double v = sc * r[a];  // grad V(r_i - r_j)
                if (kDf) {
                    const float h = (float)v;
                    gd[f - c0][a] = make_float2(h, (float)(v - f32_to_f64(h)));
                } else {
                    g[f - c0][a] = v;
                }
            }
        };
        // every entry of the chunk on the branch-free path
        if (kMixed) {
            const float cut2f32 = (float)cut2;
            const float paramf = (float)s.int_a;
            for (int k = lane; k < cn; k += 32) {
                const int e = sm.fe[c0 + k], il = (e >> 5) & 31, jl = e & 31;
                float r[D];
                float r2 = 0.0f;
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    float d = (sm.xif[il][a] - sm.xjf[jl][a]) + (sm.u.lo[0][il][a] - sm.u.lo[1][jl][a]);
                    if (s.pbc && fabsf(d) > halfLf) d -= copysignf(Lf, d);
                    r[a] = d;
                    r2 += d * d;
                }
                const float sc = r2 < cut2f32 ? pair_scale<float>(s.int_kind, r2, paramf) : 0.0f;
#pragma unroll
                for (int a = 0; a < D; ++a) g[k][a] = f32_to_f64(sc * r[a]);
            }
        } else if (kDf) {
            // every entry on the double-float far path, two independent ones
            // per lane and iteration (their chains of dependent FP32
            // operations interleave; four measured slower, with twice the
            // code); the entries marked in the screen are redone below
            constexpr int kIlp = 2;
            for (int k = lane; k < cn; k += 32 * kIlp) {
                df sc[kIlp], r[kIlp][D];
#pragma unroll
                for (int q = 0; q < kIlp; ++q) {
                    const int f = c0 + min(k + 32 * q, cn - 1);  // past the end: a repeat, not stored
                    sc[q] = aziz_far_scale_df(separation_df(f, r[q]), *etbl);
                }
#pragma unroll
                for (int q = 0; q < kIlp; ++q) {
                    if (k + 32 * q >= cn) break;
#pragma unroll
                    for (int a = 0; a < D; ++a) {
                        const df v = dfl::mul(sc[q], r[q][a]);
                        gd[k + 32 * q][a] = make_float2(v.hi, v.lo);
                    }
                }
            }
        } else if (aziz) {
            // two independent entries per lane and iteration; entries inside
            // the damping radius are redone below
            for (int k = lane; k < cn; k += 64) {
                const bool two = k + 32 < cn;
                const int f0 = c0 + k, f1 = two ? f0 + 32 : f0;
                double r0[D], r1[D];
                const double q0 = separation_far(f0, r0), q1 = separation_far(f1, r1);
                const double sc0 = aziz_far_scale(q0, tbl), sc1 = aziz_far_scale(q1, tbl);
                // r2 >= 0: the cutoff test compares bit patterns (integer unit)
                store(f0, __double_as_longlong(q0) < cut2_bits ? sc0 : 0.0, r0);
                if (two) store(f1, __double_as_longlong(q1) < cut2_bits ? sc1 : 0.0, r1);
            }
        } else {
            for (int k = lane; k < cn; k += 32) {
                double r[D];
                const double r2 = separation(c0 + k, r);
                store(c0 + k, r2 < cut2 ? pair_scale_d<true>(s.int_kind, r2, s.int_a, tbl) : 0.0, r);
            }
        }
        __syncwarp();
        // Aziz entries inside the damping radius on the general FP64 path,
        // gathered by ballot into passes of up to kCompactNear entries
        if (aziz) {
            int cnt = 0;
            for (int f0 = c0; f0 < cend; f0 += 32) {
                const int f = f0 + lane;
                const bool take = f < cend && (sm.fe[f] >> 15);
                const unsigned bal = __ballot_sync(0xffffffffu, take);
                if (take) sm.nl[cnt + __popc(bal & lt)] = (unsigned short)f;
                cnt += __popc(bal);
                if (cnt > kCompactNear - 32 || (f0 + 32 >= cend && cnt > 0)) {
                    __syncwarp();
                    for (int k = lane; k < cnt; k += 32) {
                        const int fn = sm.nl[k];
                        if (kMixed && !(sm.fe[fn] & 0x4000u)) {
                            // mixed precision inside the damping radius:
                            // double-float from the hi/lo positions, FP64 sums
                            const int e = sm.fe[fn], il = (e >> 5) & 31, jl = e & 31;
                            df r[D], q{0.0f, 0.0f};
#pragma unroll
                            for (int a = 0; a < D; ++a) {
                                df d = dfl::add_sloppy(df{sm.xif[il][a], sm.u.lo[0][il][a]},
                                                       df{-sm.xjf[jl][a], -sm.u.lo[1][jl][a]});
                                if (s.pbc && fabsf(d.hi) > halfLf) d = dfl::add(d, d.hi > 0.0f ? dfl::neg(Ldf) : Ldf);
                                r[a] = d;
                                q = a == 0 ? dfl::sqr(d) : dfl::add_sloppy(q, dfl::sqr(d));
                            }
                            if (q.hi >= (float)kAzizNearMinR2 && q.hi < shell2f) {
                                const df sc = aziz_is_far_df(q) ? aziz_far_scale_df(q, *etbl)
                                                                : aziz_near_scale_df(q, *etbl);
#pragma unroll
                                for (int a = 0; a < D; ++a) g[fn - c0][a] = dfl::to_double(dfl::mul(sc, r[a]));
                                continue;
                            }
                        }
                        if (kDf && !(sm.fe[fn] & 0x4000u)) {
                            // inside the damping radius, the image certain and
                            // the pair clearly inside the cutoff: double-float
                            df r[D];
                            const df q = separation_df(fn, r);
                            if (q.hi >= (float)kAzizNearMinR2) {
                                // the screen's margin lets entries just beyond the
                                // damping radius in, where F = 1 and dF = 0
                                const df sc = aziz_is_far_df(q) ? aziz_far_scale_df(q, *etbl)
                                                                : aziz_near_scale_df(q, *etbl);
#pragma unroll
                                for (int a = 0; a < D; ++a) {
                                    const df v = dfl::mul(sc, r[a]);
                                    gd[fn - c0][a] = make_float2(v.hi, v.lo);
                                }
                                continue;
                            }
                        }
                        double r[D];
                        const double r2 = separation(fn, r);
                        store(fn, r2 < cut2 ? pair_scale_exact(s.int_kind, r2, s.int_a, tbl) : 0.0, r);
                    }
                    __syncwarp();
                    cnt = 0;
                }
            }
        }
        // 3. deterministic sums: i side over its own (contiguous) entries, j
        //    side down its column in ascending i (chunk by chunk)
        for (int k = max(off, c0); k < min(off + icnt, cend); ++k)
#pragma unroll
            for (int a = 0; a < D; ++a) {
                if (kDf) {
                    const float2 v = gd[k - c0][a];
                    aid[a] = dfl::add_sloppy(aid[a], df{-v.x, -v.y});
                } else {
                    ai[a] -= g[k - c0][a];
                }
            }
        for (unsigned cm = col; cm; cm &= cm - 1u) {
            const int ii = __ffs(cm) - 1;
            const int f = sm.off[ii] + __popc(sm.mask[ii] & lt);
            if (cn == total || (f >= c0 && f < cend)) {
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    if (kDf) {
                        const float2 v = gd[f - c0][a];
                        ajd[a] = dfl::add_sloppy(ajd[a], df{v.x, v.y});
                    } else {
                        aj[a] += g[f - c0][a];
                    }
                }
            }
        }
        __syncwarp();  // the next chunk overwrites g
    }
    if (kDf) {
#pragma unroll
        for (int a = 0; a < D; ++a) {
            ai[a] = f32_to_f64(aid[a].hi) + f32_to_f64(aid[a].lo);
            aj[a] = f32_to_f64(ajd[a].hi) + f32_to_f64(ajd[a].lo);
        }
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

// Task order: every bead's off-diagonal tile pairs (it < jt) first, then
// the diagonal ones, which hold half the pairs.  With more tasks than
// resident warps the second round then takes the short tasks (the benchmark
// system: 1792 off-diagonal tiles for 1800 warps, then 512 diagonal ones).
// w is the tile pair's index in compact_tile's row-major order over
// it <= jt; results do not depend on the order (each tile has its slots).
__device__ __forceinline__ void tile_of_task(int task, int P, int T, int& b, int& w) {
    const int noff = T * (T - 1) / 2;
    int it, jt;
    if (task < P * noff) {
        b = task / noff;
        int r = task - b * noff;
        it = 0;
        while (r >= T - 1 - it) {  // row it holds jt = it + 1 .. T - 1
            r -= T - 1 - it;
            ++it;
        }
        jt = it + 1 + r;
    } else {
        const int d = task - P * noff;
        b = d / T;
        it = jt = d - b * T;
    }
    w = it * T - it * (it - 1) / 2 + (jt - it);
}

// Persistent warps take tile tasks from ctr[0] until none are
// left; the warp that finishes last resets both counters for the next
// launch (no waiting).  Blocks that land on one of the last s.reserve_sms of
// the nsm SMs take no task: those SMs stay free for the exchange's one-block
// passes (FP32 estimate, FP64 triangular solve) that run beside this kernel,
// whose sequential chains would otherwise share the FP64 pipe with the
// pair warps.  The scheduler may place every block of a small grid there on
// a busy GPU, so the warp that finishes last first takes whatever tasks are
// left: the forces never depend on where blocks run.
template <int D, bool kMixed, bool kDf>
__global__ void __launch_bounds__(32 * kCompactWarps) k_pair_tiles_compact(Sys s, double* __restrict__ part, int T,
                                                                          int npairs, int* ctr, int cap, int nsm) {
    extern __shared__ __align__(16) unsigned char csm_raw[];
    __shared__ double tbl[256];
    __shared__ dfl::ExpTable etbl;
    for (int j = threadIdx.x; j < 256; j += blockDim.x) {
        const double v = kExp2Table256[j];
        tbl[j] = v;
        if (kDf || kMixed) {  // 2^(j/256) as a double-float (47 bits or more; bit patterns, no FP64 work)
            float h, l;
            split_f32(v, h, l);
            const dfl::df n = dfl::fast_two_sum(h, l);
            etbl.hi[j] = n.hi;
            etbl.lo[j] = n.lo;
        }
    }
    __syncthreads();
    unsigned char* wbase = csm_raw + (threadIdx.x >> 5) * compact_warp_bytes<D>(cap);
    CompactSmem<D>& sm = *reinterpret_cast<CompactSmem<D>*>(wbase);
    auto g = reinterpret_cast<double (*)[D]>(wbase + sizeof(CompactSmem<D>));
    const int lane = threadIdx.x & 31;
    unsigned smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    const bool reserved = (int)smid >= nsm - s.reserve_sms;
    const int ntask = s.P * npairs;
    auto take_tasks = [&]() {
        for (;;) {
            int task = 0;
            if (lane == 0) task = atomicAdd(&ctr[0], 1);
            task = __shfl_sync(0xffffffffu, task, 0);
            if (task >= ntask) break;
            int b, w;
            tile_of_task(task, s.P, T, b, w);
            compact_tile<D, kMixed, kDf>(s, part, T, b, w, sm, g, cap, tbl, &etbl, lane);
            __syncwarp();
        }
    };
    if (!reserved) take_tasks();
    int last = 0;
    if (lane == 0) {
        __threadfence();
        last = atomicAdd(&ctr[1], 1) == (int)(gridDim.x * kCompactWarps) - 1;
    }
    if (__shfl_sync(0xffffffffu, last, 0)) {
        // every other warp has finished; where the scheduler placed every
        // block on a reserved SM (a small grid on a busy GPU) the tasks are
        // still untaken, and this warp evaluates them
        __threadfence();
        take_tasks();
        if (lane == 0) {
            ctr[0] = 0;
            ctr[1] = 0;
            __threadfence();
        }
    }
}

// f = springs + (-grad V_ext + sum of the pair slots), one thread per
// (bead, axis, particle).  T = 0 when there are no pair forces.
template <int D>
__global__ void k_bead_finish(Sys s, const double* __restrict__ part, int T, int write_phys, int add_fx) {
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
        // exterior springs from the exchange (fx, written beside the pair
        // forces) or, without add_fx, added by the exchange force kernel
        s.f[o] = add_fx ? acc + s.fx[((size_t)(b == 0 ? 0 : 1) * D + a) * s.ld + i] : acc;
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

// ---------------------------------------------------------------------------
// Cell lists for a periodic box whose cutoff is small against the box
// (nc = floor(L / rc) >= 4 cells per edge, each at least rc wide): every
// pair inside the cutoff lies in one of the 3^D cells around a particle's
// own, so each particle tests ~27 cells' worth of candidates instead of N.
//
// k_cell_bin (one block per bead) wraps the bead's positions into the box,
// bins them by cell and writes them cell-sorted, stably (particles of a
// cell in ascending index: the order of every later sum is fixed), with
// FP64 and FP32 hi/lo copies.  k_pair_cells (one thread per particle in
// sorted order) screens the candidates in FP32 into a per-thread list, then
// the warp evaluates the lists in lockstep (FP64 Aziz pairs in double-float
// on the FP32 pipe, other FP64 potentials in FP64, FP32 in the mixed path)
// and sums the pair gradient on its own particle only; the result is one
// partial-sum slot for k_bead_finish.  The hi/lo copies are the wrapped
// position's nearest float and the float of the remainder: a double-float.
constexpr int kCellBinThreads = 1024;
constexpr int kCellThreads = 128;
constexpr int kCellList = 64;

template <int D>
__device__ __forceinline__ int cell_of(const double* u, int nc, double L) {
    int c = 0;
#pragma unroll
    for (int a = D - 1; a >= 0; --a) {
        int k = (int)floor((u[a] + 0.5 * L) * (nc / L));
        k = min(max(k, 0), nc - 1);
        c = c * nc + k;
    }
    return c;
}

template <int D>
__global__ void __launch_bounds__(kCellBinThreads) k_cell_bin(Sys s, int nc, int* __restrict__ cstart,
                                                              int* __restrict__ clist, double* __restrict__ xw,
                                                              float* __restrict__ xh, float* __restrict__ xl) {
    extern __shared__ int cur[];  // ncell (+1)
    int ncell = 1;
    for (int a = 0; a < D; ++a) ncell *= nc;
    const int b = blockIdx.x, N = s.N;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    for (int c = tid; c <= ncell; c += blockDim.x) cur[c] = 0;
    __syncthreads();
    auto wrapped = [&](int i, double* u) {
#pragma unroll
        for (int a = 0; a < D; ++a) {
            const double x = s.x[idx<D>(s, b, a, i)];
            u[a] = x - s.L * rint(x * s.invL);
        }
    };
    for (int i = tid; i < N; i += blockDim.x) {
        double u[D];
        wrapped(i, u);
        atomicAdd(&cur[cell_of<D>(u, nc, s.L)], 1);
    }
    __syncthreads();
    // exclusive scan of the counts by warp 0 (each lane a contiguous range)
    int* cs = cstart + (size_t)b * (ncell + 1);
    if (warp == 0) {
        const int per = (ncell + 31) / 32, c0 = lane * per, c1 = min(ncell, c0 + per);
        int sum = 0;
        for (int c = c0; c < c1; ++c) sum += cur[c];
        int pre = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, pre, o);
            if (lane >= o) pre += y;
        }
        int run = pre - sum;
        for (int c = c0; c < c1; ++c) {
            const int n = cur[c];
            cs[c] = run;
            cur[c] = run;
            run += n;
        }
        if (lane == 31) cs[ncell] = pre;
    }
    __syncthreads();
    // stable scatter: chunks of blockDim particles in index order; inside a
    // chunk the warps take their turns and a group of lanes with the same
    // cell is placed by its lowest lane
    const unsigned lt = (1u << lane) - 1u;
    for (int i0 = 0; i0 < N; i0 += blockDim.x) {
        const int i = i0 + tid;
        const bool valid = i < N;
        double u[D];
        int c = -1;
        if (valid) {
            wrapped(i, u);
            c = cell_of<D>(u, nc, s.L);
        }
        const unsigned grp = __match_any_sync(0xffffffffu, c);
        const int leader = __ffs(grp) - 1;
        int base = 0;
        for (int w = 0; w < nw; ++w) {
            if (w == warp && valid && lane == leader) {
                base = cur[c];
                cur[c] = base + __popc(grp);
            }
            __syncthreads();
        }
        base = __shfl_sync(0xffffffffu, base, leader);
        if (valid) {
            const int pos = base + __popc(grp & lt);
            clist[(size_t)b * N + pos] = i;
#pragma unroll
            for (int a = 0; a < D; ++a) {
                const size_t o = ((size_t)b * D + a) * N + pos;
                xw[o] = u[a];
                const float h = (float)u[a];
                xh[o] = h;
                xl[o] = (float)(u[a] - (double)h);
            }
        }
    }
}

template <int D, typename R>
__global__ void __launch_bounds__(kCellThreads) k_pair_cells(Sys s, int nc, const int* __restrict__ cstart,
                                                             const int* __restrict__ clist,
                                                             const double* __restrict__ xw,
                                                             const float* __restrict__ xh,
                                                             const float* __restrict__ xl, double* __restrict__ fpair) {
    __shared__ double tbl[256];
    __shared__ dfl::ExpTable etbl;
    extern __shared__ int lists[];  // kCellList x kCellThreads
    // FP64 with the Aziz potential: the pairs in double-float on the FP32
    // pipe (as the pair tiles), the few at the cutoff or closer than 0.01 r_m
    // on the exact FP64 path
    constexpr bool kFp64 = sizeof(R) == 8;
    const bool dfp = kFp64 && s.int_kind == POT_AZIZ;
    // mixed precision: the Aziz pairs inside the damping radius in
    // double-float too (FP32 would lose the cancelling terms' difference)
    const bool dfnear = s.int_kind == POT_AZIZ;
    for (int j = threadIdx.x; j < 256; j += blockDim.x) {
        const double v = kExp2Table256[j];
        tbl[j] = v;
        if (dfnear) {
            float h, l;
            split_f32(v, h, l);
            const dfl::df n = dfl::fast_two_sum(h, l);
            etbl.hi[j] = n.hi;
            etbl.lo[j] = n.lo;
        }
    }
    __syncthreads();
    int ncell = 1;
    for (int a = 0; a < D; ++a) ncell *= nc;
    const int b = blockIdx.y, N = s.N;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = k < N;
    const int kk = active ? k : 0;
    const int* cs = cstart + (size_t)b * (ncell + 1);
    const double* Xw = xw + (size_t)b * D * N;
    const float* Xh = xh + (size_t)b * D * N;
    const float* Xl = xl + (size_t)b * D * N;
    int* my = lists + threadIdx.x;
    const double cut = s.cutoff, cut2 = cut * cut;
    const float cut2f = (float)cut2 * 1.0001f;
    // FP32 r^2 below which a mixed-precision Aziz pair is evaluated in FP64
    const float near2f = (float)((Aziz::D * Aziz::rm) * (Aziz::D * Aziz::rm)) * 1.0001f;
    const float Lf = (float)s.L, halfLf = 0.5f * (float)s.L;
    const long long half_bits = __double_as_longlong(0.5 * s.L);
    double xi[D];
    float hi[D], lo[D];
    int cc[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
        xi[a] = Xw[(size_t)a * N + kk];
        hi[a] = Xh[(size_t)a * N + kk];
        lo[a] = Xl[(size_t)a * N + kk];
        cc[a] = min(max((int)floor((xi[a] + 0.5 * s.L) * (nc / s.L)), 0), nc - 1);
    }
    double acc[D];
    dfl::df accd[D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
        acc[a] = 0.0;
        accd[a] = dfl::df{0.0f, 0.0f};
    }
    const dfl::df Ldf{(float)s.L, (float)(s.L - f32_to_f64((float)s.L))};
    const float shell2f = (float)cut2 * (1.0f - 1e-5f);
    // the double-float gradient of candidate q; false: take the FP64 path
    auto eval_df = [&](int q) {
        dfl::df d[D], r2{0.0f, 0.0f};
#pragma unroll
        for (int a = 0; a < D; ++a) {
            dfl::df v = dfl::add_sloppy(dfl::df{hi[a], lo[a]},
                                        dfl::df{-Xh[(size_t)a * N + q], -Xl[(size_t)a * N + q]});
            if (fabsf(v.hi) > halfLf) v = dfl::add(v, v.hi > 0.0f ? dfl::neg(Ldf) : Ldf);
            d[a] = v;
            r2 = a == 0 ? dfl::sqr(v) : dfl::add_sloppy(r2, dfl::sqr(v));
        }
        // at the cutoff the in/out decision must be the FP64 one
        if (r2.hi >= shell2f || r2.hi < (float)kAzizNearMinR2) return false;
        const dfl::df sc = aziz_is_far_df(r2) ? aziz_far_scale_df(r2, etbl) : aziz_near_scale_df(r2, etbl);
#pragma unroll
        for (int a = 0; a < D; ++a) accd[a] = dfl::add_sloppy(accd[a], dfl::neg(dfl::mul(sc, d[a])));
        return true;
    };
    // gradient of one candidate q (sorted index), subtracted from acc
    auto eval = [&](int q) {
        if (dfp && eval_df(q)) return;
        R r[D];
        R r2 = (R)0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            R d;
            if constexpr (sizeof(R) == 8) {
                d = min_image_wrapped(xi[a] - Xw[(size_t)a * N + q], s.L, half_bits);
            } else {
                d = (hi[a] - Xh[(size_t)a * N + q]) + (lo[a] - Xl[(size_t)a * N + q]);
                if (fabsf(d) > halfLf) d -= copysignf(Lf, d);
            }
            r[a] = d;
            r2 += d * d;
        }
        if (!(r2 < (R)cut2)) return;
        R sc;
        if constexpr (sizeof(R) == 8) {
            sc = (s.int_kind == POT_AZIZ && aziz_is_far(r2)) ? aziz_far_scale(r2, tbl)
                                                              : pair_scale_d<true>(s.int_kind, r2, s.int_a, tbl);
        } else {
            if (s.int_kind == POT_AZIZ && r2 < near2f) {
                // inside the damping radius the repulsive and attractive
                // terms nearly cancel: double-float, or FP64 from the FP64
                // positions at the cutoff shell
                if (eval_df(q)) return;
                double rd[D];
                double q2 = 0.0;
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    rd[a] = min_image_wrapped(xi[a] - Xw[(size_t)a * N + q], s.L, half_bits);
                    q2 += rd[a] * rd[a];
                }
                if (!(q2 < cut2)) return;
                const double scd = pair_scale_d<true>(s.int_kind, q2, s.int_a, tbl);
#pragma unroll
                for (int a = 0; a < D; ++a) acc[a] -= scd * rd[a];
                return;
            }
            sc = pair_scale<float>(s.int_kind, r2, (float)s.int_a);
        }
#pragma unroll
        for (int a = 0; a < D; ++a) acc[a] -= (double)(sc * r[a]);
    };
    // 1. FP32 screen of the 3^D neighbour cells into the per-thread list
    int cnt = 0;
    if (active) {
        int ncand = 1;
        for (int a = 0; a < D; ++a) ncand *= 3;
        for (int t = 0; t < ncand; ++t) {
            int c = 0, tt = t;
            int code[D];
#pragma unroll
            for (int a = 0; a < D; ++a) {
                code[a] = tt % 3 - 1;
                tt /= 3;
            }
#pragma unroll
            for (int a = D - 1; a >= 0; --a) c = c * nc + (cc[a] + code[a] + nc) % nc;
            for (int q = cs[c]; q < cs[c + 1]; ++q) {
                if (q == k) continue;
                float r2 = 0.0f;
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    float d = hi[a] - Xh[(size_t)a * N + q];
                    if (fabsf(d) > halfLf) d -= copysignf(Lf, d);
                    r2 += d * d;
                }
                if (r2 <= cut2f) {
                    if (cnt < kCellList) my[cnt * kCellThreads] = q;
                    else eval(q);  // rare overflow: evaluated on the spot
                    ++cnt;
                }
            }
        }
    }
    // 2. lockstep evaluation of the lists
    const int mine = min(cnt, kCellList);
    const int most = __reduce_max_sync(0xffffffffu, mine);
    for (int e = 0; e < most; ++e)
        if (e < mine) eval(my[e * kCellThreads]);
    if (active) {
        const int i = clist[(size_t)b * N + k];
#pragma unroll
        for (int a = 0; a < D; ++a)
            fpair[idx<D>(s, b, a, i)] = dfnear ? acc[a] + (f32_to_f64(accd[a].hi) + f32_to_f64(accd[a].lo)) : acc[a];
    }
}

// Cell-list geometry: cells per edge (0 when cell lists do not apply).
int cell_grid(const Sys& s, int D) {
    if (!s.pbc || !(s.cutoff > 0.0) || s.int_kind == POT_FREE) return 0;
    int nc = (int)std::floor(s.L / (s.cutoff * 1.000001));
    if (nc < 4) return 0;
    const int cap = D == 3 ? 16 : (D == 2 ? 64 : 4096);
    return std::min(nc, cap);
}

size_t cell_buffer_bytes(const Sys& s, int D, int nc) {
    size_t ncell = 1;
    for (int a = 0; a < D; ++a) ncell *= nc;
    const size_t n = (size_t)s.P * s.N;
    return s.P * (ncell + 1) * sizeof(int) + n * sizeof(int) + n * D * (sizeof(double) + 2 * sizeof(float)) +
           (size_t)s.P * D * s.ld * sizeof(double) + 256 * 6;
}

template <int D>
static void cells_launch(const Sys& s, int nc, int mixed, int write_phys, unsigned char* buf, cudaEvent_t before_finish,
                         int add_fx, cudaStream_t st) {
    size_t ncell = 1;
    for (int a = 0; a < D; ++a) ncell *= nc;
    const size_t n = (size_t)s.P * s.N;
    auto carve = [&](size_t bytes) {
        unsigned char* p = buf;
        buf += (bytes + 255) / 256 * 256;
        return p;
    };
    int* cstart = reinterpret_cast<int*>(carve(s.P * (ncell + 1) * sizeof(int)));
    int* clist = reinterpret_cast<int*>(carve(n * sizeof(int)));
    double* xw = reinterpret_cast<double*>(carve(n * D * sizeof(double)));
    float* xh = reinterpret_cast<float*>(carve(n * D * sizeof(float)));
    float* xl = reinterpret_cast<float*>(carve(n * D * sizeof(float)));
    double* fpair = reinterpret_cast<double*>(carve((size_t)s.P * D * s.ld * sizeof(double)));
    const size_t bin_smem = (ncell + 1) * sizeof(int);
    if (bin_smem > 48 * 1024) cudaFuncSetAttribute(k_cell_bin<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bin_smem);
    k_cell_bin<D><<<s.P, kCellBinThreads, bin_smem, st>>>(s, nc, cstart, clist, xw, xh, xl);
    const size_t list_smem = sizeof(int) * kCellList * kCellThreads;
    dim3 grid((s.N + kCellThreads - 1) / kCellThreads, s.P);
    if (mixed) k_pair_cells<D, float><<<grid, kCellThreads, list_smem, st>>>(s, nc, cstart, clist, xw, xh, xl, fpair);
    else k_pair_cells<D, double><<<grid, kCellThreads, list_smem, st>>>(s, nc, cstart, clist, xw, xh, xl, fpair);
    const size_t ne = (size_t)s.P * D * s.ld;
    if (before_finish) cudaStreamWaitEvent(st, before_finish, 0);
    k_bead_finish<D><<<(unsigned)((ne + 255) / 256), 256, 0, st>>>(s, fpair, 1, write_phys, add_fx);
}

void launch_pair_cells_and_finish(const Sys& s, int D, int nc, int mixed, int write_phys, void* buf,
                                  cudaEvent_t before_finish, int add_fx, cudaStream_t st) {
    unsigned char* b = reinterpret_cast<unsigned char*>(buf);
    if (D == 1) cells_launch<1>(s, nc, mixed, write_phys, b, before_finish, add_fx, st);
    else if (D == 2) cells_launch<2>(s, nc, mixed, write_phys, b, before_finish, add_fx, st);
    else cells_launch<3>(s, nc, mixed, write_phys, b, before_finish, add_fx, st);
}

// The partial sums plus one trailing double that holds the compact kernel's
// two task counters (zero between launches).
size_t pair_partial_doubles(const Sys& s, int D) {
    const int T = (s.N + kTile - 1) / kTile;
    return (size_t)s.P * T * D * s.ld + 1;
}

template <int D>
static void tiles_launch(const Sys& s, int mixed, int write_phys, double* part, cudaEvent_t before_finish, int add_fx,
                         cudaStream_t st) {
    const bool pairs = s.int_kind != POT_FREE && s.cutoff != 0.0;
    const int T = pairs ? (s.N + kTile - 1) / kTile : 0;
    if (pairs) {
        const int np = T * (T + 1) / 2;
        if (s.cutoff > 0.0) {
            const int cap = s.pair_cap > 0 ? std::min(s.pair_cap, kCompactMaxCap) : kCompactDefaultCap;
            const size_t smem = compact_warp_bytes<D>(cap) * kCompactWarps;
            // occupancy per device and precision, measured again when the
            // entry cap changes (the attribute is set on the current device)
            struct Occ {
                int resident, cap, sms;
            };
            static Occ occ[64][3] = {};
            static std::mutex occ_mu;
            // FP64 with the Aziz potential: the double-float far path
            const bool dfp = !mixed && s.int_kind == POT_AZIZ;
            auto kern = mixed ? k_pair_tiles_compact<D, true, false>
                              : (dfp ? k_pair_tiles_compact<D, false, true> : k_pair_tiles_compact<D, false, false>);
            const int variant = mixed ? 1 : (dfp ? 2 : 0);
            int dev = 0;
            cudaGetDevice(&dev);
            Occ o{};
            {
                std::lock_guard<std::mutex> lock(occ_mu);
                Occ& slot = occ[(dev >= 0 && dev < 64) ? dev : 0][variant];
                if (slot.cap != cap || dev < 0 || dev >= 64) {
                    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(compact_warp_bytes<D>(kCompactMaxCap) * kCompactWarps));
                    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&slot.resident, kern, 32 * kCompactWarps, smem);
                    cudaDeviceGetAttribute(&slot.sms, cudaDevAttrMultiProcessorCount, dev);
                    if (slot.resident < 1) slot.resident = 1;
                    slot.cap = cap;
                }
                o = slot;
            }
            const int sms = o.sms;
            const int ntask = s.P * np;
            const int blocks = std::min((ntask + kCompactWarps - 1) / kCompactWarps, o.resident * sms);
            int* ctr = reinterpret_cast<int*>(part + (pair_partial_doubles(s, D) - 1));
            Sys sr = s;
            if (sms <= 16) sr.reserve_sms = 0;
            kern<<<blocks, 32 * kCompactWarps, smem, st>>>(sr, part, T, np, ctr, cap, sms);
        } else {
            dim3 grid((np + 3) / 4, s.P);
            if (mixed) k_pair_tiles<D, float><<<grid, 128, 0, st>>>(s, part, T, np);
            else k_pair_tiles<D, double><<<grid, 128, 0, st>>>(s, part, T, np);
        }
    }
    const size_t n = (size_t)s.P * D * s.ld;
    if (before_finish) cudaStreamWaitEvent(st, before_finish, 0);
    k_bead_finish<D><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s, part, T, write_phys, add_fx);
}

// pimdb_math_check: CUDA's exp and rsqrt beside exp_tang, exp_tang256 and
// rsqrt_newton on the same inputs.
__global__ void k_math_check(const double* __restrict__ x, int n, double* __restrict__ out) {
    __shared__ double t32[32], t256[256];
    for (int j = threadIdx.x; j < 256; j += blockDim.x) t256[j] = kExp2Table256[j];
    if (threadIdx.x < 32) t32[threadIdx.x] = kExp2Table[threadIdx.x];
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double v = x[i], r = fabs(v) + 1e-3;
        double* o = out + 8 * (size_t)i;
        o[0] = exp(v);
        o[1] = exp_tang(v, t32);
        o[2] = exp_tang256(v, t256);
        o[3] = rsqrt(r);
        o[4] = rsqrt_newton(r);
        float hi, lo;
        split_f32(v, hi, lo);
        o[5] = (double)hi;
        o[6] = (double)lo;
        o[7] = f32_to_f64((float)v);
    }
}
void launch_math_check(const double* x, int n, double* out, cudaStream_t st) {
    k_math_check<<<(n + 255) / 256, 256, 0, st>>>(x, n, out);
}

void launch_pair_tiles_and_finish(const Sys& s, int D, int mixed, int write_phys, double* part,
                                  cudaEvent_t before_finish, int add_fx, cudaStream_t st) {
    if (D == 1) tiles_launch<1>(s, mixed, write_phys, part, before_finish, add_fx, st);
    else if (D == 2) tiles_launch<2>(s, mixed, write_phys, part, before_finish, add_fx, st);
    else tiles_launch<3>(s, mixed, write_phys, part, before_finish, add_fx, st);
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

// Per-bead terms of the reference's observables (src/observables/*.cpp),
// thread per particle i of bead b:
//   [0] sum p^2            [1] |x_{b-1} - x_b|^2 (minimum image)
//   [2] V_ext(x_i)         [3] x_i . grad V_ext(x_i)
//   [4] V(r_ij), j > i     [5] x_i . grad V(r_ij), j > i   (energy.cpp:82-96:
//                              only the first particle's coordinate enters)
//   [6] |grad_i (V_ext + sum_j V(r_ij))|^2 (the GSF force term)
// part[((b * gridDim.x + block) * kObsTerms + k]
constexpr int kObsTerms = 7;

template <int D>
__global__ void __launch_bounds__(kEnergyThreads) k_observable_terms(Sys s, double* __restrict__ part) {
    __shared__ double xs[D][kEnergyThreads];
    __shared__ double red[kObsTerms * 32];
    const int b = blockIdx.y;
    const int i = blockIdx.x * kEnergyThreads + threadIdx.x;
    const bool active = i < s.N;
    double xi[D], t[kObsTerms] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, g[D];
#pragma unroll
    for (int a = 0; a < D; ++a) xi[a] = active ? s.x[idx<D>(s, b, a, i)] : 0.0;
    if (active) {
        const int bp = (b - 1 + s.P) % s.P;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            const double pv = s.p[idx<D>(s, b, a, i)];
            t[0] += pv * pv;
            double d = s.x[idx<D>(s, bp, a, i)] - xi[a];
            if (s.pbc) d = min_image(d, s.L, s.invL);
            t[1] += d * d;
        }
        t[2] = ext_value<D>(s, xi);
        double fe[D];
        ext_force<D>(s, xi, fe);
#pragma unroll
        for (int a = 0; a < D; ++a) {
            g[a] = -fe[a];
            t[3] += xi[a] * g[a];
        }
    }
    const bool pairs = s.int_kind != POT_FREE && s.cutoff != 0.0;
    if (pairs) {
        for (int j0 = 0; j0 < s.N; j0 += kEnergyThreads) {
            __syncthreads();
            const int jl = j0 + threadIdx.x;
#pragma unroll
            for (int a = 0; a < D; ++a) xs[a][threadIdx.x] = jl < s.N ? s.x[idx<D>(s, b, a, jl)] : 0.0;
            __syncthreads();
            if (!active) continue;
            const int jn = min(kEnergyThreads, s.N - j0);
            for (int jj = 0; jj < jn; ++jj) {
                const int j = j0 + jj;
                if (j == i) continue;
                double r[D], r2 = 0.0;
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    double d = xi[a] - xs[a][jj];
                    if (s.pbc) d = min_image(d, s.L, s.invL);
                    r[a] = d;
                    r2 += d * d;
                }
                if (s.cutoff > 0.0 && !(sqrt(r2) < s.cutoff)) continue;
                const double sc = pair_scale<double>(s.int_kind, r2, s.int_a);
#pragma unroll
                for (int a = 0; a < D; ++a) g[a] += sc * r[a];
                if (j > i) {
                    t[4] += pair_value(s.int_kind, r2, s.int_a);
#pragma unroll
                    for (int a = 0; a < D; ++a) t[5] += xi[a] * (sc * r[a]);
                }
            }
        }
    }
    if (active) {
#pragma unroll
        for (int a = 0; a < D; ++a) t[6] += g[a] * g[a];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < kObsTerms; ++k) {
        const double v = warp_sum(t[k]);
        if (lane == 0) red[k * 32 + w] = v;
    }
    __syncthreads();
    if (threadIdx.x < kObsTerms) {
        double v = 0.0;
        for (int q = 0; q < nw; ++q) v += red[threadIdx.x * 32 + q];
        part[((size_t)b * gridDim.x + blockIdx.x) * kObsTerms + threadIdx.x] = v;
    }
}

void launch_observable_terms(const Sys& s, int D, double* part, cudaStream_t st) {
    dim3 grid((s.N + kEnergyThreads - 1) / kEnergyThreads, s.P);
    if (D == 1) k_observable_terms<1><<<grid, kEnergyThreads, 0, st>>>(s, part);
    else if (D == 2) k_observable_terms<2><<<grid, kEnergyThreads, 0, st>>>(s, part);
    else k_observable_terms<3><<<grid, kEnergyThreads, 0, st>>>(s, part);
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

// Feldman-Hirshberg bosonic exchange on the first and last beads.
//
// Reference: BosonicExchange (src/bosonic_exchange/quadratic_bosonic_exchange.cpp)
//   evaluateCycleEnergies :34-61            -> k_exch_energies_rows (below 512
//                                              particles), k_exch_energies_flat
//   evaluateVBn :73-99, evaluateVBackwards :101-128
//                                           -> estimate + weights + solve (below)
//   evaluateConnectionProbabilities :142-157,
//   springForceLastBead / springForceFirstBead :159-215
//                                           -> k_exch_forces (probabilities formed on the fly)
//   primEstimator :250-279, getDistinctProbability :222-229,
//   getLongestProbability :238-240          -> k_exch_estimators
//
// Cycle energies are stored packed by row: the reference's E(m, k) (cycle of
// particles m-k+1..m, 1-based) lives at row v = m-1, column u = m-k, offset
// v(v+1)/2 + u, which is exactly the reference's E_kn[m(m+1)/2 - k].
//
// How the recursions are evaluated.  The reference's forward recursion
//   V[m] = -1/beta log( 1/m sum_{u<m} exp(-beta (E[m-1][u] + V[u])) )
// is sequential in m and costs one FP64 exponential per term, which on one
// streaming multiprocessor is far too slow (GB300 runs FP64 at 1/64 of FP32).
// It is evaluated in three passes with the same result in FP64:
//   1. k_exch_estimate: the recursion in FP32 (hardware exp2), one block,
//      one barrier per level ("wavefront": when V[j] is final every later
//      level adds its term u = j to a running log-sum-exp).  Gives Vh.
//   2. k_exch_weights: every FP64 exponential at once, spread over the GPU:
//      Wf[m-1][u] = exp(-beta (E[m-1][u] + Vh[u] - Vh[m])) / m.
//   3. k_exch_solve: y_0 = 1, y_m = sum_u Wf[m-1][u] y_u (an FP64 triangular
//      solve, multiply-adds only) and V[m] = Vh[m] - log(y_m)/beta exactly.
// Because Vh is within FP32 accuracy of V, every y stays near 1, no term
// over- or underflows and the FP64 result carries the reference's precision.
// If the estimate is ever off by more than 200 kT (not expected; e.g. for
// non-finite input), the solve kernel recomputes the level-by-level FP64
// log-sum-exp in the reference's own order instead.  The backward recursion
// is handled the same way by the second block of each kernel.
// Usually the previous evaluations' potentials (extrapolated linearly) serve
// as Vh and pass 1 is skipped; a solve that fails with them is retried from
// a fresh estimate, in the solving block below the multi-SM solve's size and
// by the phase-1 launches from there on.
// Launches per evaluation below 512 particles: k_exch_energies_rows (the
// energies, a due estimate in its last block, the weights), then
// k_exch_solve_band (pass 3 whole: banded or dense solve, post-processing,
// retry, finish), then k_exch_forces.  From 512 particles the passes run as
// the separate kernels named above, the solve across SMs from 768
// (k_exch_solve_grid) unless the weights are banded.
#include <algorithm>
#include <atomic>

#include "exchange_dev.cuh"
#include "kernels.h"

namespace pimdb {

// Cycle energies: one warp per row.
template <int D>
__global__ void k_exch_energies(Sys s) {
    const int lane = threadIdx.x & 31;
    const int v = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (v >= s.N) return;
    energy_row<D>(s, v, lane);
}

// Cycle energies below the flat form's size, one block per row: the row's
// 32-entry chunks (u = v - 1 - 32 k - lane) are independent but for the
// running carry, so every warp scans its chunks at once; thread 0 then
// forms each chunk's carry from E[v][v] and the chunk totals in the order
// energy_row adds them, and the warps add it.  The terms, the scans and the
// carries are energy_row's, operation for operation: the same bits.  The
// critical path of a row is one chunk instead of all of them.
// The weights follow in the same launch (k_exch_weights' phase-0 work, with
// its band measurement).  With the previous potentials as the estimate, each
// block forms its own row's weights (exch_weight, FP64) from the energies it
// just wrote.  When a fresh estimate is due, the block that finishes last
// runs it (both directions in turn) and then forms every weight in
// double-float on the FP32 pipe (weights_df_block; on one SM the FP64
// exponentials would take a quarter of a millisecond).  Four blocks per SM
// bound the registers (the rare estimate's arrays would otherwise set them
// for every row).
constexpr int kEnergyRowThreads = 256;
static_assert(kEnergyRowThreads == kWaveThreads, "the estimate runs with the energy kernel's block");
template <int D>
__global__ void __launch_bounds__(kEnergyRowThreads, 4) k_exch_energies_rows(Sys s) {
    extern __shared__ double rsm[];  // scans [N], then the chunks' totals and carries
    __shared__ double wtbl[32];      // exp_tang's table
    const int v = blockIdx.x, N = s.N;
    if (threadIdx.x < 32) wtbl[threadIdx.x] = kExp2Table[threadIdx.x];
    const int fresh = ((volatile int*)s.xflags)[3];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int first = 0, last = s.P - 1;
    const double hk = 0.5 * s.kappa;
    const int nch = (v + 31) / 32;  // chunks of u = v-1 .. 0
    double* scan = rsm;
    double* tot = rsm + N;
    double* carry = tot + nch;
    double xv[D];
#pragma unroll
    for (int a = 0; a < D; ++a) xv[a] = s.x[idx<D>(s, last, a, v)];
    auto dist_to_v = [&](int u) {  // |xP_v - x1_u|^2
        double d2 = 0.0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            double d = xv[a] - s.x[idx<D>(s, first, a, u)];
            if (s.pbc) d = min_image(d, s.L, s.invL);
            d2 += d * d;
        }
        return d2;
    };
    for (int k = warp; k < nch; k += nw) {
        const int base = v - 1 - 32 * k, u = base - lane;
        const double c = u >= 0 ? dist_to_v(u) : 0.0;
        double cu1 = __shfl_up_sync(0xffffffffu, c, 1);
        if (lane == 0) cu1 = dist_to_v(base + 1);  // the previous chunk's last distance
        double term = 0.0;
        if (u >= 0) term = hk * (sepsq<D>(s, last, u, first, u + 1) - cu1 + c);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, term, o);
            if (lane >= o) term += y;
        }
        if (u >= 0) scan[32 * k + lane] = term;
        const double tk = __shfl_sync(0xffffffffu, term, 31);
        if (lane == 0) tot[k] = tk;
    }
    __syncthreads();
    double* row = s.E + tri(v);
    if (threadIdx.x == 0) {
        double cr = hk * dist_to_v(v);
        row[v] = cr;
        if (v >= 1) s.Et[tri(N - v - 1) + (N - 1 - v)] = cr;
        for (int k = 0; k < nch; ++k) {
            carry[k] = cr;
            cr += tot[k];
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < v; e += blockDim.x) {
        const int k = e >> 5, u = v - 1 - e;
        const double val = carry[k] + scan[e];
        row[u] = val;
        // backward node r = N - u depends on node r' = N - 1 - v
        if (u >= 1) s.Et[tri(N - u - 1) + (N - 1 - v)] = val;
    }
    if (!fresh) {
        __syncthreads();  // this row's energies, written by the block
        const double inv = recip_row(v);
        int band = 0;
        for (int u = threadIdx.x; u <= v; u += blockDim.x)
            if (exch_weight(s, v, u, inv, wtbl)) band = max(band, v + 1 - u);
        band = __reduce_max_sync(0xffffffffu, band);
        if ((threadIdx.x & 31) == 0 && band > 0) atomicMax(&s.xflags[kExchBand], band);
    }
    __shared__ int is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) is_last = atomicAdd(&s.xflags[kExchRowsCount], 1) == (int)gridDim.x - 1;
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    if (threadIdx.x == 0) {
        s.xflags[kExchRowsCount] = 0;
        s.xflags[7] = !fresh;
        if (fresh) atomicAdd(&s.xflags[kExchFreshCount], 1);
    }
    if (!fresh) return;
    estimate_direction(s, 0, reinterpret_cast<float*>(rsm));
    __syncthreads();
    estimate_direction(s, 1, reinterpret_cast<float*>(rsm));
    __syncthreads();
    __shared__ dfl::ExpTable etbl;
    fill_exp_table_df(etbl);
    __syncthreads();
    int band = weights_df_block(s, etbl, reinterpret_cast<float*>(rsm));
    band = __reduce_max_sync(0xffffffffu, band);
    if ((threadIdx.x & 31) == 0 && band > 0) atomicMax(&s.xflags[kExchBand], band);
}

// Whether the cycle energies of s come from k_exch_energies_rows (which then
// also runs the phase-0 estimate and weights).
static size_t energies_rows_smem(const Sys& s) {
    return std::max(sizeof(double) * ((size_t)s.N + 2 * (((size_t)s.N + 31) / 32) + 2),
                    sizeof(float) * 4 * ((size_t)s.N + 1));
}
// The kernel's static shared memory (exp_tang's table, the double-float
// exponential table, the last-block flag) counts against the 48 KB that a
// launch gets without opting in to more.
constexpr size_t kRowsStaticSmem = 32 * sizeof(double) + sizeof(dfl::ExpTable) + 64;
static bool energies_by_rows(const Sys& s, const double* work) {
    return !(work && s.eflat) && energies_rows_smem(s) + kRowsStaticSmem <= 48 * 1024;
}

// Cycle energies for large N without a scan per row.  The row recursion
// telescopes: E[v][u] = k/2 (L[v] - L[u] + |xP_v - x1_u|^2) with the prefix
// sums L[w] = sum_{t<w} |x1_{t+1} - xP_t|^2 of the interior links, so every
// entry is independent.  L is kept in double-double (hi, lo): the difference
// of two long prefix sums then keeps the accuracy of the direct sum.
// k_link_prefix (one block) builds L and the beads' positions wrapped into
// the box; k_exch_energies_flat (one block per row) writes E and Et.
__device__ __forceinline__ void dd_add(double ah, double al, double bh, double bl, double& h, double& l) {
    const double s = ah + bh;
    const double bb = s - ah;
    double e = (ah - (s - bb)) + (bh - bb);
    e += al + bl;
    h = s + e;
    l = e - (h - s);
}

template <int D>
__global__ void __launch_bounds__(1024) k_link_prefix(Sys s, double* __restrict__ Lh, double* __restrict__ Ll,
                                                       double* __restrict__ wrap) {
    __shared__ double sh[32], sl[32];
    const int N = s.N, tid = threadIdx.x, nt = blockDim.x;
    const int first = 0, last = s.P - 1;
    // positions of beads 1 and P wrapped into [-L/2, L/2): wrap[side][a][N]
    for (int i = tid; i < N; i += nt)
#pragma unroll
        for (int a = 0; a < D; ++a) {
            double x1 = s.x[idx<D>(s, first, a, i)], xP = s.x[idx<D>(s, last, a, i)];
            if (s.pbc) {
                x1 -= s.L * rint(x1 * s.invL);
                xP -= s.L * rint(xP * s.invL);
            }
            wrap[(size_t)a * N + i] = x1;
            wrap[(size_t)(D + a) * N + i] = xP;
        }
    // contiguous chunk per thread, double-double sums, then a scan of the chunks
    const int chunk = (N + nt - 1) / nt;
    const int w0 = tid * chunk, w1 = min(N, w0 + chunk);
    double th = 0.0, tl = 0.0;
    for (int w = w0; w < w1 && w + 1 <= N - 1; ++w) {
        double d2 = sepsq<D>(s, last, w, first, w + 1);
        dd_add(th, tl, d2, 0.0, th, tl);
    }
    // inclusive warp scan, then across warps
    const int lane = tid & 31, warp = tid >> 5;
    double ih = th, il = tl;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double yh = __shfl_up_sync(0xffffffffu, ih, o), yl = __shfl_up_sync(0xffffffffu, il, o);
        if (lane >= o) dd_add(yh, yl, ih, il, ih, il);
    }
    if (lane == 31) {
        sh[warp] = ih;
        sl[warp] = il;
    }
    __syncthreads();
    if (warp == 0) {
        double wh = lane < nt / 32 ? sh[lane] : 0.0, wl = lane < nt / 32 ? sl[lane] : 0.0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double yh = __shfl_up_sync(0xffffffffu, wh, o), yl = __shfl_up_sync(0xffffffffu, wl, o);
            if (lane >= o) dd_add(yh, yl, wh, wl, wh, wl);
        }
        sh[lane] = wh;
        sl[lane] = wl;
    }
    __syncthreads();
    // exclusive prefix of this thread's chunk
    double ph = 0.0, pl = 0.0;
    if (warp > 0) {
        ph = sh[warp - 1];
        pl = sl[warp - 1];
    }
    const double xh = __shfl_up_sync(0xffffffffu, ih, 1), xl = __shfl_up_sync(0xffffffffu, il, 1);
    if (lane > 0) dd_add(ph, pl, xh, xl, ph, pl);
    for (int w = w0; w < w1; ++w) {
        Lh[w] = ph;
        Ll[w] = pl;
        if (w + 1 <= N - 1) {
            const double d2 = sepsq<D>(s, last, w, first, w + 1);
            dd_add(ph, pl, d2, 0.0, ph, pl);
        }
    }
}

template <int D>
__global__ void __launch_bounds__(256) k_exch_energies_flat(Sys s, const double* __restrict__ Lh,
                                                            const double* __restrict__ Ll,
                                                            const double* __restrict__ wrap) {
    const int N = s.N, v = blockIdx.x;
    const double hk = 0.5 * s.kappa;
    const long long half_bits = __double_as_longlong(0.5 * s.L);
    double xv[D];
#pragma unroll
    for (int a = 0; a < D; ++a) xv[a] = wrap[(size_t)(D + a) * N + v];
    const double lvh = Lh[v], lvl = Ll[v];
    double* row = s.E + tri(v);
    for (int u = threadIdx.x; u <= v; u += blockDim.x) {
        double c = 0.0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            double d = xv[a] - wrap[(size_t)a * N + u];
            if (s.pbc) {
                const long long bits = __double_as_longlong(d);
                if ((bits & 0x7fffffffffffffffLL) > half_bits) d -= copysign(s.L, d);
            }
            c = fma(d, d, c);
        }
        const double e = hk * (((lvh - Lh[u]) + (lvl - Ll[u])) + c);
        row[u] = e;
        // backward node r = N - u depends on node r' = N - 1 - v
        if (u >= 1) s.Et[tri(N - u - 1) + (N - 1 - v)] = e;
    }
}

// Pass 1: block 0 forward, block 1 backward.  Phase 0 skips (early exit)
// when the previous evaluation's exact potentials are still a good estimate
// (xflags[3] == 0) and records in xflags[7] that they were reused; phase 1
// (the retry) runs only when the solve asked for it (xflags[6]).
__global__ void __launch_bounds__(kWaveThreads) k_exch_estimate(Sys s, int phase) {
    if (phase == 0) {
        const int fresh = ((volatile int*)s.xflags)[3];
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            s.xflags[7] = !fresh;
            if (fresh) atomicAdd(&s.xflags[kExchFreshCount], 1);
        }
        if (!fresh) return;
    } else if (((volatile int*)s.xflags)[6] == 0) {
        return;
    }
    extern __shared__ float fsm[];  // 3 (N+1)
    estimate_direction(s, blockIdx.x, fsm);
}

// Pass 2: every FP64 exponential at once, one thread per packed entry
// (grid-stride over rows; phase 1 runs only on a retry).
// Also records the band of the weights (kExchBand: the largest p + 1 - u of
// a nonzero weight) for the banded solve; one atomic per warp.
__global__ void k_exch_weights(Sys s, int phase) {
    if (phase == 1 && ((volatile int*)s.xflags)[6] == 0) return;
    __shared__ double tbl[32];
    if (threadIdx.x < 32) tbl[threadIdx.x] = kExp2Table[threadIdx.x];
    __syncthreads();
    int band = 0;
    for (int p = blockIdx.y; p < s.N; p += gridDim.y) {
        const double inv = recip_row(p);
        for (int u = blockIdx.x * blockDim.x + threadIdx.x; u <= p; u += gridDim.x * blockDim.x)
            if (exch_weight(s, p, u, inv, tbl)) band = max(band, p + 1 - u);
    }
    band = __reduce_max_sync(0xffffffffu, band);
    if ((threadIdx.x & 31) == 0 && band > 0) atomicMax(&s.xflags[kExchBand], band);
}

// Pass 3: block 0 forward, block 1 backward.  Phase 0 may not fall back to
// the exact recursion when it reused the previous potentials (xflags[7]); a
// failed solve then leaves xflags[6] set and the phase-1 kernels redo the
// evaluation from a fresh estimate.  With `inline_retry` (smaller systems,
// where the retry's three launches would cost more than its work) the block
// whose solve failed redoes its direction itself: FP32 estimate, weights,
// solve; no phase 1 is launched.  No static shared memory beyond a flag:
// the block has to fit beside the pair kernel's resident blocks.
__global__ void __launch_bounds__(kWaveThreads) k_exch_solve(Sys s, int force_exact, int phase,
                                                             const double* __restrict__ pre, int inline_retry) {
    extern __shared__ double ys[];  // y: N+1, acc: N+1, then 32 for reductions
    __shared__ int last_block;
    __shared__ dfl::ExpTable etbl;  // log y and the row exponentials in double-float
    if (phase == 1 && ((volatile int*)s.xflags)[6] == 0) return;
    if (phase == 0) {
        // k_exch_solve_band post-processed both directions and finished: it
        // set the flag to 2, and each of the two blocks takes one off
        if (threadIdx.x == 0) {
            last_block = ((volatile int*)s.xflags)[kExchBandDone] > 0;
            if (last_block) atomicSub(&s.xflags[kExchBandDone], 1);
        }
        __syncthreads();
        if (last_block) return;
    }
    fill_exp_table_df(etbl);
    __syncthreads();
    if (phase == 1 && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&s.xflags[kExchRetryCount], 1);
    const int allow_exact = force_exact || phase == 1 || !((volatile int*)s.xflags)[7];
    const int dir = blockIdx.x;
    const int gave_up = solve_direction(s, dir, force_exact, ys, allow_exact,
                                        pre ? pre + (size_t)dir * (s.N + 1) : nullptr, !inline_retry, &etbl);
    if (gave_up && inline_retry) {
        if (threadIdx.x == 0) atomicAdd(&s.xflags[kExchRetryCount], 1);
        estimate_direction(s, dir, reinterpret_cast<float*>(ys));  // 3 (N+1) floats fit in ys
        __syncthreads();
        weights_direction(s, dir, nullptr);  // CUDA's exp (a rare path)
        __syncthreads();
        solve_direction(s, dir, 0, ys, 1, nullptr, 1, &etbl);
    }
    // The block that finishes second runs solve_finish (threadFenceReduction
    // pattern; no waiting).
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last_block = (atomicAdd(&s.xflags[2], 1) == 1);
    __syncthreads();
    if (!last_block) return;
    __threadfence();
    if (phase == 0 && ((volatile int*)s.xflags)[6]) {
        if (threadIdx.x == 0) s.xflags[2] = 0;  // retry pending: phase 1 finishes
        return;
    }
    solve_finish(s, !force_exact, &etbl);
    if (threadIdx.x == 0) {
        s.xflags[6] = 0;
        s.xflags[kExchBand] = 0;  // the next evaluation's weights measure it anew
        s.xflags[kExchBandLast] = 0;  // not the banded solve's evaluation: full rows
    }
}

// ---------------------------------------------------------------------------
// Pass 3 across SMs for large N.  The triangular solve y_n = sum_{u<n}
// W[n-1][u] y_u costs N^2/2 FP64 multiply-adds per direction, which on the
// one block of k_exch_solve is bound by a single SM's FP64 pipe.  Here 32-row
// blocks go round-robin to `nct` CTAs per direction (all resident: cooperative
// launch).  Block j's owner resolves its diagonal block with warp shuffles
// (its rows then hold the contributions of blocks < j) and publishes y_j
// behind a fence and a flag.  Once y_j is out, the owner of block j + 1 adds
// W[rows of j + 1][block j] y_j to those rows first, from weights loaded
// while it waited, resolves block j + 1 and publishes it; only then does it
// fold y_j into its other rows, as every other CTA does meanwhile (8 threads
// per row, shuffle sums: a fixed order).  The critical path per block is a
// flag, one 32x32 fold and one diagonal block.  Waits give up after a
// bounded number of polls (ERRB_TIMEOUT).  k_exch_solve then post-processes
// y as usual.
__global__ void __launch_bounds__(kGridSolveThreads) k_exch_solve_grid(Sys s, int phase, double* ysol,
                                                                      unsigned* gflags, int nct, int banded) {
    if (phase == 1 && ((volatile int*)s.xflags)[6] == 0) return;
    if (banded && ((volatile int*)s.xflags)[kExchBand] <= kBandMax) return;  // k_exch_solve_band solved it
    extern __shared__ double gsm[];
    __shared__ int abort_solve;
    const int dir = blockIdx.x / nct, c = blockIdx.x % nct;
    const int nn = dir == 0 ? s.N + 1 : s.N;
    const double* __restrict__ W = dir == 0 ? s.Wf : s.Wb;
    double* y = ysol + (size_t)dir * (s.N + 1);
    const int nbmax = (s.N + 1 + 31) / 32;
    unsigned* flags = gflags + (size_t)dir * nbmax;
    const int nb = (nn + 31) / 32;
    const int nown = (nb - c + nct - 1) / nct;  // blocks c, c + nct, ...
    double* acc = gsm;                           // [nown][32]
    double* yj = gsm + (size_t)nown * 32;        // [32]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int e = tid; e < nown * 32; e += blockDim.x) acc[e] = 0.0;
    if (tid == 0) abort_solve = 0;
    __syncthreads();
    const int i = tid >> 3, part = tid & 7;  // fold role: row of the block, quarter of the columns
    // weights of the block this CTA resolves next, loaded ahead: its
    // diagonal block (warp 0) and W[rows of b][block b - 1]
    double wd[32], wn[4];
    auto prefetch = [&](int b) {
        if (warp == 0) {
            const int n = 32 * b + lane;
#pragma unroll
            for (int t = 0; t < 32; ++t) wd[t] = (n < nn && n >= 1 && t < lane) ? W[tri(n - 1) + 32 * b + t] : 0.0;
        }
        const int n = 32 * b + i;
#pragma unroll
        for (int q = 0; q < 4; ++q) wn[q] = (b >= 1 && n < nn) ? W[tri(n - 1) + 32 * (b - 1) + 4 * part + q] : 0.0;
    };
    auto diag_publish = [&](int b) {  // warp 0 of the owner of block b
        const int n = 32 * b + lane;
        double a = n == 0 ? 1.0 : (n < nn ? acc[(b / nct) * 32 + lane] : 0.0);
#pragma unroll
        for (int t = 0; t < 32; ++t) {
            const double yt = __shfl_sync(0xffffffffu, a, t);
            if (lane > t) a = fma(wd[t], yt, a);
        }
        if (n < nn) y[n] = a;
        __threadfence();
        __syncwarp();
        if (lane == 0) atomicExch(&flags[b], 1u);
    };
    auto fold = [&](int r, int j, bool pre) {  // owned block r += W[rows of r][block j] y_j
        const int n = 32 * r + i;
        double sum = 0.0;
        if (n < nn) {
            if (pre) {
#pragma unroll
                for (int q = 0; q < 4; ++q) sum = fma(wn[q], yj[4 * part + q], sum);
            } else {
                const double* row = W + tri(n - 1) + 32 * j + 4 * part;
#pragma unroll
                for (int q = 0; q < 4; ++q) sum = fma(row[q], yj[4 * part + q], sum);
            }
        }
        sum += __shfl_xor_sync(0xffffffffu, sum, 1);
        sum += __shfl_xor_sync(0xffffffffu, sum, 2);
        sum += __shfl_xor_sync(0xffffffffu, sum, 4);
        if (part == 0 && n < nn) acc[(r / nct) * 32 + i] += sum;
    };
    if (c == 0) {
        prefetch(0);
        if (warp == 0) diag_publish(0);
    }
    if (nb > 1 && 1 % nct == c) prefetch(1);
    for (int j = 0; j + 1 < nb; ++j) {
        if (j % nct != c && tid == 0) {  // the owner of block j has y_j already
            unsigned it = 0;
            while (((volatile unsigned*)flags)[j] == 0u) {
                if (++it > (1u << 22)) {
                    atomicOr(s.err, ERRB_TIMEOUT);
                    abort_solve = 1;
                    break;
                }
                if (it > 64) __nanosleep(32);
            }
            __threadfence();
        }
        __syncthreads();
        if (abort_solve) break;
        if (tid < 32) {
            const int n = 32 * j + tid;
            yj[tid] = n < nn ? ((volatile double*)y)[n] : 0.0;
        }
        __syncthreads();
        const int jn = j + 1;
        const bool mine = jn % nct == c;
        if (mine) {  // the critical path: the next diagonal block's rows, then that block
            fold(jn, j, true);
            __syncthreads();
            if (warp == 0) diag_publish(jn);
        }
        for (int r = jn + (c - jn % nct + nct) % nct; r < nb; r += nct) {
            if (r == jn) continue;
            fold(r, j, false);
        }
        // weights for the next block this CTA resolves, while others work
        if (jn + 1 < nb && (jn + 1) % nct == c) prefetch(jn + 1);
        __syncthreads();
    }
    // the CTA that finishes last clears the flags for the next launch
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&gflags[2 * nbmax], 1u) == gridDim.x - 1) {
            for (int e = 0; e < 2 * nbmax; ++e) gflags[e] = 0u;
            gflags[2 * nbmax] = 0u;
            __threadfence();
        }
    }
}

// ---------------------------------------------------------------------------
// Pass 3 when the weights are banded.  A weight is exactly zero when its
// cycle costs beta_ex E > 700 (the exponential's result is returned as 0):
// at liquid-helium densities and temperatures every cycle of more than a
// dozen or so particles, so node n depends only on nodes n - band .. n - 1
// with a band far below N.  k_exch_weights records the band of the current
// evaluation; when it is at most kBandMax (two 32-row blocks) this kernel
// solves each direction on one CTA: block b's rows take the two previous
// blocks' y from shared memory (all threads, 8 columns each), then warp 0
// resolves the diagonal block by shuffles, while warps 1-7 stage the next
// block's weights into the other half of a double buffer.  No flags and no
// inter-CTA waits; y lands in ysol as from the dense solves, which step
// aside (their `banded` argument) and stay the general path.
// `standalone` (below the multi-SM solve's size): this kernel is the whole
// pass 3.  A band above kBandMax is solved densely on the same CTA
// (blocked_solve), a reused estimate that fails is redone from a fresh one
// in the block (k_exch_solve's in-block retry), and the CTA that finishes
// second runs solve_finish; no other solve kernel is launched.
__device__ __noinline__ void band_standalone_tail(const Sys& s, int dir, double* ys, const dfl::ExpTable& etbl,
                                                  int band, bool dense, int* last_band) {
    const int tid = threadIdx.x;
    const int allow_exact = !((volatile int*)s.xflags)[7];  // the estimate was fresh
    int retried = 0;
    if (solve_direction(s, dir, 0, ys, allow_exact, ys, 0, &etbl)) {
        if (tid == 0) atomicAdd(&s.xflags[kExchRetryCount], 1);
        estimate_direction(s, dir, reinterpret_cast<float*>(ys));  // 3 (N+1) floats fit in ys
        __syncthreads();
        weights_direction(s, dir, nullptr);  // CUDA's exp (a rare path)
        __syncthreads();
        solve_direction(s, dir, 0, ys, 1, nullptr, 1, &etbl);
        retried = 1;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) {
        // 1 per direction, 16 per direction that was redone
        const int mine = retried ? 16 : 1;
        const int prev = atomicAdd(&s.xflags[kExchBandCount], mine);
        *last_band = prev == 0 ? 0 : 1 + (((prev + mine) >> 4) ? 2 : 0);
    }
    __syncthreads();
    if (*last_band == 0) return;
    __threadfence();
    solve_finish(s, 1, &etbl);
    if (tid == 0) {
        s.xflags[6] = 0;
        // full exterior-force rows after a dense solve or a redone direction
        s.xflags[kExchBandLast] = (dense || *last_band == 3) ? 0 : band;
        s.xflags[kExchBand] = 0;  // the next evaluation's weights measure it anew
        s.xflags[kExchBandCount] = 0;
    }
}

__global__ void __launch_bounds__(kBandThreads) k_exch_solve_band(Sys s, int phase, double* ysol, int standalone) {
    if (phase == 1 && ((volatile int*)s.xflags)[6] == 0) return;
    const int band = ((volatile int*)s.xflags)[kExchBand];
    const bool dense = band > kBandMax;
    if (dense && !standalone) return;  // the dense solve runs instead
    extern __shared__ double bsm[];
    __shared__ double accb[32];
    __shared__ dfl::ExpTable etbl;
    __shared__ int last_band;
    const int dir = blockIdx.x;
    const int nn = dir == 0 ? s.N + 1 : s.N;
    const double* __restrict__ W = dir == 0 ? s.Wf : s.Wb;
    double* y = ysol + (size_t)dir * (s.N + 1);
    const int nnpad = (nn + 1) & ~1;
    double* ys = bsm;                    // [nn]
    double* wdiag = bsm + nnpad;         // [2][32][32]: block b's diagonal block, row-major
    double* wfold = wdiag + 2 * 1024;    // [2][32][64]: block b's rows, columns 32b - 64 .. 32b - 1
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nb = (nn + 31) / 32;
    // Threads t0.. stage block b's weights: row r of the block needs columns
    // 32b - 64 .. 32b + r - 1 of its packed row (contiguous), taken as one
    // row-major index e = 96 r + q (q < 64: fold, else diagonal) so that a
    // warp's loads are coalesced.  Every load of a thread is issued before
    // any store: one L2 round trip per block rather than one per element.
    constexpr int kStagePer = (32 * 96 + (kBandThreads - 32) - 1) / (kBandThreads - 32);
    auto stage = [&](int b, int t0, int nt) {
        double* d = wdiag + (b & 1) * 1024;
        double* f = wfold + (b & 1) * 2048;
        double v[kStagePer];
#pragma unroll
        for (int k = 0; k < kStagePer; ++k) {
            const int e = tid - t0 + k * nt;
            const int r = e / 96, q = e - 96 * r, m = 32 * b + r;
            const int c = q < 64 ? 32 * b - 64 + q : 32 * b + (q - 64);
            const bool in = e < 32 * 96 && m < nn && m >= 1 && (q < 64 ? c >= 0 : q - 64 < r);
            v[k] = in ? W[tri(m - 1) + c] : 0.0;
        }
#pragma unroll
        for (int k = 0; k < kStagePer; ++k) {
            const int e = tid - t0 + k * nt;
            if (e < 32 * 96) {
                const int r = e / 96, q = e - 96 * r;
                if (q < 64) f[r * 64 + q] = v[k];
                else d[r * 32 + (q - 64)] = v[k];
            }
        }
    };
    if (dense) {
        blocked_solve(W, nn, ys, wdiag);  // accumulators in the (unused) staging buffers
        for (int m = tid; m < nn; m += blockDim.x) y[m] = ys[m];
        __syncthreads();
    }
    if (!dense) stage(0, 0, blockDim.x);
    __syncthreads();
    const int i = tid >> 3, part = tid & 7;  // fold role: row of the block, 8 of its 64 columns
    const int dband = dense ? 32 : band;  // the diagonal chain's reach
    for (int b = 0; b < (dense ? 0 : nb); ++b) {
        const double* f = wfold + (b & 1) * 2048;
        double sum = 0.0;
        // columns more than `band` before the block's first row hold exact
        // zero weights: no multiply-add for them
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int col = 8 * part + q, c = 32 * b - 64 + col;
            if (c >= 0 && col >= 64 - band) sum = fma(f[i * 64 + col], ys[c], sum);
        }
        sum += __shfl_xor_sync(0xffffffffu, sum, 1);
        sum += __shfl_xor_sync(0xffffffffu, sum, 2);
        sum += __shfl_xor_sync(0xffffffffu, sum, 4);
        if (part == 0) accb[i] = sum;
        __syncthreads();
        if (warp == 0) {
            const double* d = wdiag + (b & 1) * 1024;
            const int m = 32 * b + lane;
            double a = m == 0 ? 1.0 : (m < nn ? accb[lane] : 0.0);
            // lanes more than `band` below t hold exact zero weights for t:
            // only the band's lanes issue the multiply-add
#pragma unroll
            for (int t = 0; t < 32; ++t) {
                const double yt = __shfl_sync(0xffffffffu, a, t);
                if (lane > t && lane - t <= dband) a = fma(d[lane * 32 + t], yt, a);
            }
            if (m < nn) {
                ys[m] = a;
                y[m] = a;
            }
        } else if (b + 1 < nb) {
            stage(b + 1, 32, blockDim.x - 32);
        }
        __syncthreads();
    }
    // The post-processing of k_exch_solve for this direction, from y in
    // shared memory (no exact fallback here: a direction that would need one
    // or a fresh estimate leaves the whole evaluation to k_exch_solve).  The
    // CTA that finishes second runs solve_finish when both directions
    // succeeded and marks the evaluation done.
    if (phase != 0) return;
    fill_exp_table_df(etbl);
    __syncthreads();
    if (standalone) {
        band_standalone_tail(s, dir, ys, etbl, band, dense, &last_band);
        return;
    }
    const int gave_up = solve_direction(s, dir, 0, ys, 0, ys, 0, &etbl);
    __threadfence();
    __syncthreads();
    if (tid == 0) {
        // count 2 per direction that succeeded, 1 per direction that gave up
        const int prev = atomicAdd(&s.xflags[kExchBandCount], gave_up ? 1 : 2);
        last_band = prev > 0 ? (prev + (gave_up ? 1 : 2)) : 0;
    }
    __syncthreads();
    if (last_band == 0) return;
    __threadfence();
    if (last_band == 4) {
        solve_finish(s, 1, &etbl);
        if (tid == 0) {
            s.xflags[kExchBandLast] = s.xflags[kExchBand];
            s.xflags[kExchBand] = 0;  // the next evaluation's weights measure it anew
            s.xflags[kExchBandDone] = 2;  // one for each block of k_exch_solve
        }
    }
    if (tid == 0) s.xflags[kExchBandCount] = 0;
}

bool banded_solve_fits(const Sys& s) { return s.N + 1 <= kBandMaxN; }

size_t banded_solve_smem(const Sys& s) {
    return sizeof(double) * ((((size_t)s.N + 2) & ~(size_t)1) + 2 * 1024 + 2 * 2048);
}


// Exterior spring forces: one warp per row (bead P) or column (bead 1).
template <int D>
__global__ void k_exch_forces(Sys s, int accumulate, int adjoint, double vb_bar) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (w >= 2 * s.N) return;
    exch_force_row<D>(s, w, lane, accumulate, nullptr, adjoint, vb_bar, ((volatile int*)s.xflags)[kExchBandLast]);
}

__global__ void k_exch_estimators(Sys s, int nbeads) {
    extern __shared__ double sh[];
    estimators_block(s, nbeads, sh);
}

// Every exchange kernel takes the largest shared-memory carveout.  An SM runs
// all its resident blocks under one carveout, so a kernel that prefers a
// smaller one (more L1) could start only on SMs without pair-tile blocks,
// and the pair tiles' blocks could not start beside it: launched first in a
// step graph, the exchange would hold back part of the pair kernel.
// Attributes belong to the current device: they are set once per device (a
// bit per device id below 64, every call above), and two host threads that
// set them at once only repeat the same cheap calls.
static std::atomic<unsigned long long> g_carveout_devices{0};

static void exchange_carveouts() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    const unsigned long long bit = dev >= 0 && dev < 64 ? 1ull << dev : 0ull;
    if (bit && (g_carveout_devices.load(std::memory_order_acquire) & bit)) return;
    const void* k[] = {(const void*)k_exch_energies<1>, (const void*)k_exch_energies<2>,
                       (const void*)k_exch_energies<3>, (const void*)k_exch_energies_rows<1>,
                       (const void*)k_exch_energies_rows<2>, (const void*)k_exch_energies_rows<3>, (const void*)k_link_prefix<1>,
                       (const void*)k_link_prefix<2>, (const void*)k_link_prefix<3>,
                       (const void*)k_exch_energies_flat<1>, (const void*)k_exch_energies_flat<2>,
                       (const void*)k_exch_energies_flat<3>, (const void*)k_exch_estimate,
                       (const void*)k_exch_weights, (const void*)k_exch_solve, (const void*)k_exch_solve_grid,
                       (const void*)k_exch_forces<1>, (const void*)k_exch_forces<2>, (const void*)k_exch_forces<3>};
    for (const void* f : k)
        cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (bit) g_carveout_devices.fetch_or(bit, std::memory_order_acq_rel);
}

int exchange_flat_default(int N) { return N >= kFlatEnergiesMinN ? 1 : 0; }

// A launch gets 48 KB of shared memory without opting in, static and
// dynamic together.  The kernels here hold up to about 2.3 KB of static
// shared memory (their exponential tables), so a dynamic size within
// kSmemOptInMargin of 48 KB opts in as well; opting in when the default
// would have done is harmless.
constexpr size_t kSmemOptInMargin = 8 * 1024;
static void opt_in_smem(const void* k, size_t dyn) {
    if (dyn + kSmemOptInMargin > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
}

// The work array of the prefix-sum energies (any N: Sys::eflat chooses).
size_t exchange_energy_doubles(const Sys& s, int D) { return (size_t)(2 + 2 * D) * s.N; }

int launch_exchange_energies(const Sys& s, int D, cudaStream_t st, double* work) {
    exchange_carveouts();
    if (work && s.eflat) {
        double* Lh = work;
        double* Ll = work + s.N;
        double* wrap = work + 2 * (size_t)s.N;
        if (D == 1) {
            k_link_prefix<1><<<1, 1024, 0, st>>>(s, Lh, Ll, wrap);
            k_exch_energies_flat<1><<<s.N, 256, 0, st>>>(s, Lh, Ll, wrap);
        } else if (D == 2) {
            k_link_prefix<2><<<1, 1024, 0, st>>>(s, Lh, Ll, wrap);
            k_exch_energies_flat<2><<<s.N, 256, 0, st>>>(s, Lh, Ll, wrap);
        } else {
            k_link_prefix<3><<<1, 1024, 0, st>>>(s, Lh, Ll, wrap);
            k_exch_energies_flat<3><<<s.N, 256, 0, st>>>(s, Lh, Ll, wrap);
        }
        return 0;
    }
    // one block per row; scans [N] and two chunk arrays in shared memory
    // (or the estimate's 3 (N + 1) floats)
    const size_t rs = energies_rows_smem(s);
    if (energies_by_rows(s, work)) {
        if (D == 1) k_exch_energies_rows<1><<<s.N, kEnergyRowThreads, rs, st>>>(s);
        else if (D == 2) k_exch_energies_rows<2><<<s.N, kEnergyRowThreads, rs, st>>>(s);
        else k_exch_energies_rows<3><<<s.N, kEnergyRowThreads, rs, st>>>(s);
        return 1;
    }
    const int warps = 2;
    dim3 grid((s.N + warps - 1) / warps);
    if (D == 1) k_exch_energies<1><<<grid, warps * 32, 0, st>>>(s);
    else if (D == 2) k_exch_energies<2><<<grid, warps * 32, 0, st>>>(s);
    else k_exch_energies<3><<<grid, warps * 32, 0, st>>>(s);
    return 0;
}

// y of both directions for the banded solve and the multi-SM solve;
// publication flags for the latter.
size_t exchange_grid_doubles(const Sys& s) { return 2 * ((size_t)s.N + 1); }
size_t exchange_grid_flags(const Sys& s) {
    return s.N >= kGridSolveMinN ? 2 * (((size_t)s.N + 1 + 31) / 32) + 1 : 1;
}

// The cooperative solve if every CTA can be resident; false otherwise.
static bool grid_solve(const Sys& s, int phase, double* ysol, unsigned* gflags, int banded, cudaStream_t st) {
    const int nb = (s.N + 1 + 31) / 32;
    const int nct = nb < kGridSolveCtas ? nb : kGridSolveCtas;
    const size_t smem = sizeof(double) * (((size_t)(nb + nct - 1) / nct) * 32 + 32);
    // resident CTAs of the whole GPU, per device (0 = not measured yet)
    static std::atomic<int> per_dev[64];
    int dev = 0;
    cudaGetDevice(&dev);
    int per = (dev >= 0 && dev < 64) ? per_dev[dev].load(std::memory_order_relaxed) - 1 : -1;
    if (per < 0) {
        int sms = 0, b = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_exch_solve_grid, kGridSolveThreads, 4096) != cudaSuccess)
            b = 0;
        per = b * sms;
        if (dev >= 0 && dev < 64) per_dev[dev].store(per + 1, std::memory_order_relaxed);
    }
    if (2 * nct > per) return false;
    Sys sc = s;
    int ph = phase, n = nct, bd = banded;
    void* args[] = {&sc, &ph, &ysol, &gflags, &n, &bd};
    return cudaLaunchCooperativeKernel((void*)k_exch_solve_grid, dim3(2 * nct), dim3(kGridSolveThreads), args, smem,
                                      st) == cudaSuccess;
}

// SMs the pair tiles leave free while this exchange runs beside them: its
// one-block passes (below the multi-SM solve's size) then run alone on an SM.
int exchange_reserved_sms(const Sys& s) { return s.N < kGridSolveMinN ? 2 : 0; }

int launch_exchange_recursions(const Sys& s, int exact, cudaStream_t st, double* ysol, unsigned* gflags,
                               int estimate_done) {
    exchange_carveouts();
    // With reserved SMs the one-block passes ask for 116 KB of shared memory,
    // whatever they use: more than an SM holding pair-tile blocks has left
    // and more than half an SM, so each lands alone on a reserved SM.
    const size_t least = s.reserve_sms ? 116 * 1024 : 0;
    const size_t esmem = std::max(sizeof(float) * 3 * (size_t)(s.N + 1), least);
    const size_t smem = std::max(sizeof(double) * (2 * (size_t)(s.N + 1) + 32), least);
    opt_in_smem((const void*)k_exch_estimate, esmem);
    opt_in_smem((const void*)k_exch_solve, smem);
    if (exact) {
        k_exch_solve<<<2, kWaveThreads, smem, st>>>(s, 1, 0, nullptr, 0);
        return 1;
    }
    const dim3 wgrid((s.N + 255) / 256, s.N < 65535 ? s.N : 65535);
    const dim3 rgrid(1, s.N < 256 ? s.N : 256);  // the retry's weights: a small grid-stride launch
    // below the multi-SM solve's size a failed solve is retried inside
    // k_exch_solve (phase 0 only)
    const int inline_retry = s.N < kGridSolveMinN;
    // below the multi-SM solve's size the banded kernel is the whole pass 3
    const int standalone = inline_retry && ysol && banded_solve_fits(s);
    int n = 0;
    for (int phase = 0; phase < (inline_retry ? 1 : 2); ++phase) {
        if (!(phase == 0 && estimate_done)) {  // else the energy kernel ran it
            k_exch_estimate<<<2, kWaveThreads, esmem, st>>>(s, phase);
            ++n;
        }
        if (!(phase == 0 && estimate_done)) {  // else the energy kernel formed them
            k_exch_weights<<<phase ? rgrid : wgrid, 256, 0, st>>>(s, phase);
            ++n;
        }
        // the banded kernel (one CTA per direction): below the multi-SM
        // solve's size the whole pass 3, from it the banded case only
        int banded = 0;
        if (ysol && banded_solve_fits(s)) {
            const size_t bs = std::max(banded_solve_smem(s), least);
            opt_in_smem((const void*)k_exch_solve_band, bs);
            k_exch_solve_band<<<2, kBandThreads, bs, st>>>(s, phase, ysol, standalone);
            banded = 1;
            ++n;
        }
        if (standalone) continue;
        // from kGridSolveMinN the dense solve runs across SMs; below it (no
        // ysol) k_exch_solve solves on its own block
        const bool dense = ysol && !inline_retry && gflags && grid_solve(s, phase, ysol, gflags, banded, st);
        const bool pre = banded || dense;
        k_exch_solve<<<2, kWaveThreads, smem, st>>>(s, 0, phase, pre ? ysol : nullptr, inline_retry);
        n += dense ? 2 : 1;
    }
    return n;
}

static void exchange_rows(const Sys& s, int D, int accumulate, int adjoint, double vb_bar, cudaStream_t st) {
    exchange_carveouts();
    const int warps = 2;  // small blocks: the 2N rows spread over every SM
    dim3 grid((2 * s.N + warps - 1) / warps);
    if (D == 1) k_exch_forces<1><<<grid, warps * 32, 0, st>>>(s, accumulate, adjoint, vb_bar);
    else if (D == 2) k_exch_forces<2><<<grid, warps * 32, 0, st>>>(s, accumulate, adjoint, vb_bar);
    else k_exch_forces<3><<<grid, warps * 32, 0, st>>>(s, accumulate, adjoint, vb_bar);
}

void launch_exchange_forces_mode(const Sys& s, int D, int accumulate, cudaStream_t st) {
    exchange_rows(s, D, accumulate, 0, 0.0, st);
}

void launch_exchange_adjoint(const Sys& s, int D, double vb_bar, cudaStream_t st) {
    exchange_rows(s, D, 0, 1, vb_bar, st);
}

void launch_exchange_estimators(const Sys& s, cudaStream_t st) {
    const size_t smem = sizeof(double) * (size_t)(s.N + 1 + 32);
    int t = ((s.N + 31) / 32) * 32;
    t = t > 512 ? 512 : (t < 32 ? 32 : t);
    opt_in_smem((const void*)k_exch_estimators, smem);
    k_exch_estimators<<<1, t, smem, st>>>(s, s.P);
}

}  // namespace pimdb

// Feldman-Hirshberg bosonic exchange on the first and last beads.
//
// Reference: BosonicExchange (src/bosonic_exchange/quadratic_bosonic_exchange.cpp)
//   evaluateCycleEnergies :34-61            -> k_exch_energies
//   evaluateVBn :73-99, evaluateVBackwards :101-128
//                                           -> k_exch_estimate + k_exch_weights + k_exch_solve
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

// Pass 1: block 0 forward, block 1 backward.  Phase 0 skips (early exit)
// when the previous evaluation's exact potentials are still a good estimate
// (xflags[3] == 0) and records in xflags[7] that they were reused; phase 1
// (the retry) runs only when the solve asked for it (xflags[6]).
__global__ void __launch_bounds__(kWaveThreads) k_exch_estimate(Sys s, int phase) {
    if (phase == 0) {
        const int fresh = ((volatile int*)s.xflags)[3];
        if (blockIdx.x == 0 && threadIdx.x == 0) s.xflags[7] = !fresh;
        if (!fresh) return;
    } else if (((volatile int*)s.xflags)[6] == 0) {
        return;
    }
    extern __shared__ float fsm[];  // 3 (N+1)
    estimate_direction(s, blockIdx.x, fsm);
}

// Pass 2: every FP64 exponential at once, one thread per packed entry
// (grid-stride over rows; phase 1 runs only on a retry).
__global__ void k_exch_weights(Sys s, int phase) {
    if (phase == 1 && ((volatile int*)s.xflags)[6] == 0) return;
    for (int p = blockIdx.y; p < s.N; p += gridDim.y)
        for (int u = blockIdx.x * blockDim.x + threadIdx.x; u <= p; u += gridDim.x * blockDim.x) exch_weight(s, p, u);
}

// Pass 3: block 0 forward, block 1 backward.  Phase 0 may not fall back to
// the exact recursion when it reused the previous potentials (xflags[7]); a
// failed solve then leaves xflags[6] set and the phase-1 kernels redo the
// evaluation from a fresh estimate.
__global__ void __launch_bounds__(kWaveThreads) k_exch_solve(Sys s, int force_exact, int phase) {
    extern __shared__ double ys[];  // y: N+1, acc: N+1, then 32 for reductions
    __shared__ int last_block;
    if (phase == 1 && ((volatile int*)s.xflags)[6] == 0) return;
    const int allow_exact = force_exact || phase == 1 || !((volatile int*)s.xflags)[7];
    solve_direction(s, blockIdx.x, force_exact, ys, allow_exact);
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
    solve_finish(s);
    if (threadIdx.x == 0) s.xflags[6] = 0;
}

// Exterior spring forces: one warp per row (bead P) or column (bead 1).
template <int D>
__global__ void k_exch_forces(Sys s, int accumulate) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (w >= 2 * s.N) return;
    exch_force_row<D>(s, w, lane, accumulate);
}

__global__ void k_exch_estimators(Sys s, int nbeads) {
    extern __shared__ double sh[];
    estimators_block(s, nbeads, sh);
}

void launch_exchange_energies(const Sys& s, int D, cudaStream_t st) {
    const int warps = 2;
    dim3 grid((s.N + warps - 1) / warps);
    if (D == 1) k_exch_energies<1><<<grid, warps * 32, 0, st>>>(s);
    else if (D == 2) k_exch_energies<2><<<grid, warps * 32, 0, st>>>(s);
    else k_exch_energies<3><<<grid, warps * 32, 0, st>>>(s);
}

int launch_exchange_recursions(const Sys& s, int exact, cudaStream_t st) {
    const size_t esmem = sizeof(float) * 3 * (size_t)(s.N + 1);
    const size_t smem = sizeof(double) * (2 * (size_t)(s.N + 1) + 32);
    if (esmem + 1024 > 48 * 1024)
        cudaFuncSetAttribute(k_exch_estimate, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)esmem);
    if (smem + 1024 > 48 * 1024) cudaFuncSetAttribute(k_exch_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (exact) {
        k_exch_solve<<<2, kWaveThreads, smem, st>>>(s, 1, 0);
        return 1;
    }
    const dim3 wgrid((s.N + 255) / 256, s.N < 65535 ? s.N : 65535);
    const dim3 rgrid(1, s.N < 256 ? s.N : 256);  // the retry's weights: a small grid-stride launch
    for (int phase = 0; phase < 2; ++phase) {
        k_exch_estimate<<<2, kWaveThreads, esmem, st>>>(s, phase);
        k_exch_weights<<<phase ? rgrid : wgrid, 256, 0, st>>>(s, phase);
        k_exch_solve<<<2, kWaveThreads, smem, st>>>(s, 0, phase);
    }
    return 6;
}

void launch_exchange_forces_mode(const Sys& s, int D, int accumulate, cudaStream_t st) {
    const int warps = 8;
    dim3 grid((2 * s.N + warps - 1) / warps);
    if (D == 1) k_exch_forces<1><<<grid, warps * 32, 0, st>>>(s, accumulate);
    else if (D == 2) k_exch_forces<2><<<grid, warps * 32, 0, st>>>(s, accumulate);
    else k_exch_forces<3><<<grid, warps * 32, 0, st>>>(s, accumulate);
}

void launch_exchange_estimators(const Sys& s, cudaStream_t st) {
    const size_t smem = sizeof(double) * (size_t)(s.N + 1 + 32);
    int t = ((s.N + 31) / 32) * 32;
    t = t > 512 ? 512 : (t < 32 ? 32 : t);
    if (smem + 1024 > 48 * 1024) cudaFuncSetAttribute(k_exch_estimators, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_exch_estimators<<<1, t, smem, st>>>(s, s.P);
}

}  // namespace pimdb

// Feldman-Hirshberg bosonic exchange on the first and last beads.
//
// Reference: BosonicExchange (src/bosonic_exchange/quadratic_bosonic_exchange.cpp)
//   evaluateCycleEnergies :34-61   -> k_exch_energies
//   evaluateVBn :73-99             -> k_exch_recursions (block 0)
//   evaluateVBackwards :101-128    -> k_exch_recursions (block 1)
//   evaluateConnectionProbabilities :142-157 and
//   springForceLastBead / springForceFirstBead :159-215
//                                  -> k_exch_forces (probabilities are formed
//                                     on the fly; the N x N matrix is never stored)
//   primEstimator :250-279, getDistinctProbability :222-229,
//   getLongestProbability :238-240 -> k_exch_estimators
// Everything is FP64.
//
// Cycle energies are stored packed by row: E(m, k) of the reference (the
// cycle of particles m-k+1..m, 1-based) lives at row v = m-1, column
// u = m-k, offset v(v+1)/2 + u.  Row v is contiguous, which is what the
// forward recursion reads at level m = v+1.
#include "common.cuh"
#include "kernels.h"

namespace pimdb {

__device__ __forceinline__ size_t tri(int v) { return (size_t)v * (size_t)(v + 1) / 2; }

template <int D>
__device__ __forceinline__ double sepsq(const Sys& s, int ba, int ia, int bb, int ib) {
    // |x_bb[ib] - x_ba[ia]|^2 with the minimum image (bosonic_exchange_base.cpp:30-64)
    double d2 = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
        double d = s.x[idx<D>(s, bb, a, ib)] - s.x[idx<D>(s, ba, a, ia)];
        if (s.pbc) d = min_image(d, s.L, s.invL);
        d2 += d * d;
    }
    return d2;
}

// One warp per row v: E[v][v] = k/2 |xP_v - x1_v|^2, then
// E[v][u] = E[v][u+1] + k/2 (|x1_{u+1} - xP_u|^2 - |xP_v - x1_{u+1}|^2 + |xP_v - x1_u|^2)
// for u = v-1 .. 0, evaluated as a warp-wide suffix scan over u.
template <int D>
__global__ void k_exch_energies(Sys s) {
    const int lane = threadIdx.x & 31;
    const int v = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (v >= s.N) return;
    const int first = 0, last = s.P - 1;
    const double hk = 0.5 * s.kappa;
    double* row = s.E + tri(v);
    double carry = hk * sepsq<D>(s, first, v, last, v);
    if (lane == 0) row[v] = carry;
    for (int base = v - 1; base >= 0; base -= 32) {
        const int u = base - lane;
        double term = 0.0;
        if (u >= 0) {
            term = hk * (sepsq<D>(s, last, u, first, u + 1) - sepsq<D>(s, first, u + 1, last, v) +
                         sepsq<D>(s, first, u, last, v));
        }
        // inclusive scan over lanes (lane 0 holds the largest u)
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, term, o);
            if (lane >= o) term += y;
        }
        if (u >= 0) row[u] = carry + term;
        carry += __shfl_sync(0xffffffffu, term, 31);
    }
}

// Block 0: forward recursion V[m] (:73-99).  Block 1: backward recursion
// V_backwards[l] (:101-128).  Each level is a block-wide log-sum-exp with
// the reference's minimum shift.
__global__ void k_exch_recursions(Sys s) {
    extern __shared__ double sh[];
    double* Vs = sh;              // N+1
    double* red = sh + s.N + 1;   // 32
    const int N = s.N;
    const double beta = s.beta_ex;
    const int tid = threadIdx.x, bd = blockDim.x;
    if (blockIdx.x == 0) {
        if (tid == 0) Vs[0] = 0.0;
        __syncthreads();
        for (int m = 1; m <= N; ++m) {
            const double* row = s.E + tri(m - 1);
            double lmin = 1.79769313486231570815e308;
            for (int u = tid; u < m; u += bd) lmin = fmin(lmin, row[u] + Vs[u]);
            const double shift = block_min(lmin, red);
            double ls = 0.0;
            for (int u = tid; u < m; u += bd) ls += exp(-beta * (row[u] + Vs[u] - shift));
            const double tot = block_sum(ls, red);
            if (tid == 0) {
                const double v = shift - (1.0 / beta) * log(tot / (double)m);
                Vs[m] = v;
                if (!isfinite(v)) atomicOr(s.err, ERRB_NONFINITE_VB);
            }
            __syncthreads();
        }
        for (int m = tid; m <= N; m += bd) s.V[m] = Vs[m];
    } else {
        if (tid == 0) Vs[N] = 0.0;
        __syncthreads();
        for (int l = N - 1; l > 0; --l) {
            double lmin = 1.79769313486231570815e308;
            for (int p = l + tid; p < N; p += bd) lmin = fmin(lmin, s.E[tri(p) + l] + Vs[p + 1]);
            const double shift = block_min(lmin, red);
            double ls = 0.0;
            for (int p = l + tid; p < N; p += bd) ls += exp(-beta * (s.E[tri(p) + l] + Vs[p + 1] - shift)) / (p + 1);
            const double tot = block_sum(ls, red);
            if (tid == 0) {
                const double v = shift - log(tot) / beta;
                Vs[l] = v;
                if (!isfinite(v)) atomicOr(s.err, ERRB_NONFINITE_VB);
            }
            __syncthreads();
        }
        for (int l = tid + 1; l <= N; l += bd) s.Vb[l] = Vs[l];
    }
}

// Exterior spring forces (:159-215).  Warps [0, N) handle bead P (row l of
// the connection-probability matrix), warps [N, 2N) bead 1 (column l).
// f on those beads already holds the physical forces; the spring part is
// added (simulation.cpp:363-373) and also kept in fx.
template <int D>
__global__ void k_exch_forces(Sys s, int accumulate) {
    const int lane = threadIdx.x & 31;
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int N = s.N;
    if (w >= 2 * N) return;
    const double beta = s.beta_ex;
    const double VN = s.V[N];
    const int first = 0, last = s.P - 1;
    double sum[D];
#pragma unroll
    for (int a = 0; a < D; ++a) sum[a] = 0.0;
    int bead, nb, l;
    if (w < N) {  // last bead, particle l: sum over n <= l+1
        l = w;
        bead = last;
        nb = (s.P - 2 + s.P) % s.P;
        const double vbl = s.Vb[l + 1];
        const size_t r = tri(l);
        const int nmax = min(l + 1, N - 1);
        for (int n = lane; n <= nmax; n += 32) {
            double pr;
            if (n <= l) pr = exp(-beta * (s.V[n] + s.E[r + n] + vbl - VN)) / (l + 1);
            else pr = 1.0 - exp(-beta * (s.V[l + 1] + vbl - VN));
#pragma unroll
            for (int a = 0; a < D; ++a) {
                double d = s.x[idx<D>(s, first, a, n)] - s.x[idx<D>(s, last, a, l)];
                if (s.pbc) d = min_image(d, s.L, s.invL);
                sum[a] += pr * d;
            }
        }
    } else {  // first bead, particle l: sum over q >= l-1
        l = w - N;
        bead = first;
        nb = 1 % s.P;
        for (int q = max(0, l - 1) + lane; q < N; q += 32) {
            double pr;
            if (q >= l) pr = exp(-beta * (s.V[l] + s.E[tri(q) + l] + s.Vb[q + 1] - VN)) / (q + 1);
            else pr = 1.0 - exp(-beta * (s.V[q + 1] + s.Vb[q + 1] - VN));
#pragma unroll
            for (int a = 0; a < D; ++a) {
                double d = s.x[idx<D>(s, last, a, q)] - s.x[idx<D>(s, first, a, l)];
                if (s.pbc) d = min_image(d, s.L, s.invL);
                sum[a] += pr * d;
            }
        }
    }
#pragma unroll
    for (int a = 0; a < D; ++a) sum[a] = warp_sum(sum[a]);
    if (lane == 0) {
        const int side = (bead == first) ? 0 : 1;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            double d = s.x[idx<D>(s, nb, a, l)] - s.x[idx<D>(s, bead, a, l)];
            if (s.pbc) d = min_image(d, s.L, s.invL);
            const double fs = (sum[a] + d) * s.kappa;
            s.fx[((size_t)side * D + a) * s.ld + l] = fs;
            if (accumulate) {
                const size_t o = idx<D>(s, bead, a, l);
                s.f[o] = fs + s.f[o];
            }
        }
    }
    if (w == 0 && lane == 0) {
        s.Vb[0] = VN;
        s.scal[0] = VN;
    }
}

// primEstimator (:250-279), getDistinctProbability (:222-229) and
// getLongestProbability (:238-240); one block.
__global__ void k_exch_estimators(Sys s, int nbeads) {
    extern __shared__ double sh[];
    double* G = sh;             // N+1
    double* red = sh + s.N + 1; // 32
    const int N = s.N;
    const double beta = s.beta_ex;
    const int tid = threadIdx.x, bd = blockDim.x;
    if (tid == 0) G[0] = 0.0;
    __syncthreads();
    for (int m = 1; m <= N; ++m) {
        const double* row = s.E + tri(m - 1);
        double lmin = 1.79769313486231570815e308;
        for (int u = tid; u < m; u += bd) lmin = fmin(lmin, row[u] + s.V[u]);
        const double shift = block_min(lmin, red);
        double ls = 0.0;
        for (int u = tid; u < m; u += bd) ls += (G[u] - row[u]) * exp(-beta * (row[u] + s.V[u] - shift));
        const double tot = block_sum(ls, red);
        if (tid == 0) G[m] = tot / (m * exp(-beta * (s.V[m] - shift)));
        __syncthreads();
    }
    double diag = 0.0;
    for (int m = tid; m < N; m += bd) diag += s.E[tri(m) + m];
    diag = block_sum(diag, red);
    if (tid == 0) {
        const double VN = s.V[N];
        s.scal[1] = G[N] / nbeads;
        s.scal[2] = exp(-beta * (diag - VN) - lgamma((double)(N + 1)));
        s.scal[3] = exp(-beta * (s.E[tri(N - 1)] - VN));
    }
}

static int recursion_threads(int N) {
    int t = ((N + 31) / 32) * 32;
    if (t > 512) t = 512;
    if (t < 32) t = 32;
    return t;
}

void launch_exchange_energies(const Sys& s, int D, cudaStream_t st) {
    const int warps = 8;
    dim3 grid((s.N + warps - 1) / warps);
    if (D == 1) k_exch_energies<1><<<grid, warps * 32, 0, st>>>(s);
    else if (D == 2) k_exch_energies<2><<<grid, warps * 32, 0, st>>>(s);
    else k_exch_energies<3><<<grid, warps * 32, 0, st>>>(s);
}

void launch_exchange_recursions(const Sys& s, cudaStream_t st) {
    const size_t smem = sizeof(double) * (size_t)(s.N + 1 + 32);
    k_exch_recursions<<<2, recursion_threads(s.N), smem, st>>>(s);
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
    k_exch_estimators<<<1, recursion_threads(s.N), smem, st>>>(s, s.P);
}

}  // namespace pimdb

// Factorial bosonic exchange: the sum over all N! permutations of the
// exterior links between beads P and 1 (the reference's build with
// FACTORIAL_BOSONIC_ALGORITHM, CMakeLists.txt:49-54).
//
// Reference: FactorialBosonicExchange (src/bosonic_exchange/factorial_bosonic_exchange.cpp)
//   prepare / getMinExteriorSpringEnergy :19-21, :58-82   -> k_fact_min
//   effectivePotential :91-114, springForceLastBead :121-172,
//   springForceFirstBead :179-230, primEstimator :259-293 -> k_fact_sums + k_fact_finish
//   getDistinctProbability :237-240, getLongestProbability :249-252 return 0
//
// For a given configuration this is a different potential from the
// Feldman-Hirshberg recursion (which keeps one representative cycle per set
// of exchanged particles); the two agree only after the interior beads are
// integrated out.
//
// The reference enumerates the permutations once per quantity and per bead,
// with O(N D) work per permutation each time.  Here one enumeration gives
// every quantity.  With d2[l][m] = |x_1[m] - x_P[l]|^2 (minimum image),
// E(s) = k/2 sum_l d2[l][s(l)] and w(s) = exp(-beta_ex (E(s) - E_min)):
//   S = sum_s w,  SE = sum_s w E,  M[l][m] = sum_{s(l) = m} w(s),
//   f_P[l] = k (x_{P-1}[l] - x_P[l] + sum_m M[l][m]/S (x_1[m] - x_P[l]))
//   f_1[m] = k (x_2[m] - x_1[m] + sum_l M[l][m]/S (x_P[l] - x_1[m]))
// (each difference under the minimum image), V_B = E_min - log(S/N!)/beta_ex
// and primEstimator = -(SE/S)/P.  effectivePotential's unshifted weights
// (:106-110) underflow to V_B = inf where these stay finite.
//
// Parallel layout.  Lexicographic order splits the permutations into runs of
// T! (T = min(N, 4)) that share their first N-T entries.  One thread takes
// one run: it decodes the prefix from the run index, keeps the T x T block of
// d2 that the suffixes use in registers and walks the T! suffixes fully
// unrolled, so one permutation costs T adds, one exponential and T+2 adds
// into registers.  Block totals are formed in a fixed order: every thread
// stages its run's sums in shared memory and one owner thread per entry of M
// adds them up, run by run; k_fact_finish adds the blocks' totals in block
// order.  The results are deterministic for a given N.
#include "forces_dev.cuh"
#include "kernels.h"

namespace pimdb {

namespace {

constexpr int kFactThreads = 256;
constexpr int kFactMaxBlocks = 152 * 4;
constexpr int kFactRecStride = kFactThreads + 1;  // staging rows: conflict-free owner reads

__host__ __device__ constexpr long long factorial_ll(int n) {
    long long r = 1;
    for (int i = 2; i <= n; ++i) r *= i;
    return r;
}
template <int T>
struct SuffixCount {
    static constexpr int value = (int)factorial_ll(T);
};

// d2[l * N + m] = |x_1[m] - x_P[l]|^2, minimum image per axis.
template <int D>
__device__ void fact_load_d2(const Sys& s, double* d2) {
    const int N = s.N;
    for (int e = threadIdx.x; e < N * N; e += blockDim.x) {
        const int l = e / N, m = e % N;
        double acc = 0.0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            double d = s.x[idx<D>(s, 0, a, m)] - s.x[idx<D>(s, s.P - 1, a, l)];
            if (s.pbc) d = min_image(d, s.L, s.invL);
            acc += d * d;
        }
        d2[e] = acc;
    }
}

// One run of T! permutations: prefix values written to pre[0 .. N-T) (when
// pre is not null), the remaining values ascending, the prefix's d2 sum and
// the T x T block sub[i][j] = d2[N-T+i][rem[j]].
template <int T>
struct Run {
    double epre;
    double sub[T][T];
    int rem[T];
};

template <int T>
__device__ __forceinline__ void fact_decode(int N, long long g, const double* d2, Run<T>& run, unsigned char* pre) {
    const int Lp = N - T;
    unsigned used = 0;
    double ep = 0.0;
    long long radix = factorial_ll(N - 1) / factorial_ll(T);  // runs per choice at position 0
    for (int p = 0; p < Lp; ++p) {
        int k = (int)(g / radix);
        g -= (long long)k * radix;
        if (p + 1 < Lp) radix /= (N - 1 - p);
        unsigned avail = ~used & ((1u << N) - 1u);
        for (; k > 0; --k) avail &= avail - 1u;  // drop the k smallest free values
        const int v = __ffs(avail) - 1;
        used |= 1u << v;
        ep += d2[p * N + v];
        if (pre) pre[p] = (unsigned char)v;
    }
    unsigned avail = ~used & ((1u << N) - 1u);
#pragma unroll
    for (int j = 0; j < T; ++j) {
        run.rem[j] = __ffs(avail) - 1;
        avail &= avail - 1u;
    }
#pragma unroll
    for (int i = 0; i < T; ++i)
#pragma unroll
        for (int j = 0; j < T; ++j) run.sub[i][j] = d2[(Lp + i) * N + run.rem[j]];
    run.epre = ep;
}

// pick[i] = position (in rem) of the value that suffix position i takes in
// the k-th permutation of T elements, lexicographic.  k is a compile-time
// constant in the fully unrolled loops below, so this folds away.
template <int T>
__device__ __forceinline__ void suffix_pick(int k, int (&pick)[T]) {
    int avail = (1 << T) - 1;
#pragma unroll
    for (int i = 0; i < T; ++i) {
        const int f = (int)factorial_ll(T - 1 - i);
        int q = k / f;
        k -= q * f;
        int chosen = 0;
#pragma unroll
        for (int j = T - 1; j >= 0; --j) {
            // the q-th set bit of avail, counted from the lowest
            if ((avail >> j) & 1) {
                if (__popc(avail & ((1 << j) - 1)) == q) chosen = j;
            }
        }
        pick[i] = chosen;
        avail &= ~(1 << chosen);
    }
}

template <int D, int T>
__global__ void __launch_bounds__(kFactThreads) k_fact_min(Sys s, double* work, long long runs) {
    __shared__ double d2[kFactMaxN * kFactMaxN];
    __shared__ double red[32];
    fact_load_d2<D>(s, d2);
    __syncthreads();
    double dmin = 1.79769313486231570815e308;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < runs; g += stride) {
        Run<T> run;
        fact_decode<T>(s.N, g, d2, run, nullptr);
#pragma unroll
        for (int k = 0; k < SuffixCount<T>::value; ++k) {
            int pick[T];
            suffix_pick<T>(k, pick);
            double d = run.epre;
#pragma unroll
            for (int i = 0; i < T; ++i) d += run.sub[i][pick[i]];
            dmin = fmin(dmin, d);
        }
    }
    dmin = block_min(dmin, red);
    if (threadIdx.x == 0) work[blockIdx.x] = dmin;
}

template <int D, int T>
__global__ void __launch_bounds__(kFactThreads) k_fact_sums(Sys s, double* work, long long runs, int nblocks) {
    __shared__ double d2[kFactMaxN * kFactMaxN];
    __shared__ double tbl[32];
    __shared__ double red[32];
    __shared__ double recS[kFactThreads];
    __shared__ double recM[T * T][kFactRecStride];
    __shared__ unsigned char recPre[kFactThreads][kFactMaxN];
    __shared__ unsigned char recRem[kFactThreads][4];
    const int tid = threadIdx.x, N = s.N, Lp = N - T, NN = N * N;
    fact_load_d2<D>(s, d2);
    if (tid < 32) tbl[tid] = kExp2Table[tid];
    double dmin = 1.79769313486231570815e308;
    for (int b = tid; b < nblocks; b += blockDim.x) dmin = fmin(dmin, work[b]);
    dmin = block_min(dmin, red);  // also orders d2 and tbl before their use
    const double half_k = 0.5 * s.kappa, beta = s.beta_ex;
    const double emin = half_k * dmin;
    double S = 0.0, SE = 0.0, own = 0.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < runs; base += stride) {
        const long long g = base + tid;
        double acc[T][T];
#pragma unroll
        for (int i = 0; i < T; ++i)
#pragma unroll
            for (int j = 0; j < T; ++j) acc[i][j] = 0.0;
        double Sg = 0.0;
        if (g < runs) {
            Run<T> run;
            fact_decode<T>(N, g, d2, run, recPre[tid]);
#pragma unroll
            for (int k = 0; k < SuffixCount<T>::value; ++k) {
                int pick[T];
                suffix_pick<T>(k, pick);
                double d = run.epre;
#pragma unroll
                for (int i = 0; i < T; ++i) d += run.sub[i][pick[i]];
                const double e = half_k * d;
                const double w = exp_tang(-beta * (e - emin), tbl);
                Sg += w;
                SE = fma(w, e, SE);
#pragma unroll
                for (int i = 0; i < T; ++i) acc[i][pick[i]] += w;
            }
#pragma unroll
            for (int j = 0; j < T; ++j) recRem[tid][j] = (unsigned char)run.rem[j];
        } else {
            for (int p = 0; p < Lp; ++p) recPre[tid][p] = 0xFF;
#pragma unroll
            for (int j = 0; j < T; ++j) recRem[tid][j] = 0xFF;
        }
        S += Sg;
        recS[tid] = Sg;
#pragma unroll
        for (int i = 0; i < T; ++i)
#pragma unroll
            for (int j = 0; j < T; ++j) recM[i * T + j][tid] = acc[i][j];
        __syncthreads();
        if (tid < NN) {
            const int l = tid / N, m = tid % N;
            if (l < Lp) {
                for (int r = 0; r < kFactThreads; ++r)
                    if (recPre[r][l] == m) own += recS[r];
            } else {
                const int i = l - Lp;
                for (int r = 0; r < kFactThreads; ++r) {
#pragma unroll
                    for (int j = 0; j < T; ++j)
                        if (recRem[r][j] == m) own += recM[i * T + j][r];
                }
            }
        }
        __syncthreads();
    }
    S = block_sum(S, red);
    SE = block_sum(SE, red);
    double* part = work + kFactMaxBlocks + (size_t)blockIdx.x * (2 + NN);
    if (tid == 0) {
        part[0] = S;
        part[1] = SE;
    }
    if (tid < NN) part[2 + tid] = own;
}

// Totals over the blocks, scalars, and the exterior spring forces of beads 1
// and P into fx (and added into f with `accumulate`).  One block.
template <int D>
__global__ void __launch_bounds__(kFactThreads) k_fact_finish(Sys s, const double* work, int nblocks, int accumulate) {
    __shared__ double M[kFactMaxN * kFactMaxN];
    __shared__ double red[32];
    const int tid = threadIdx.x, N = s.N, NN = N * N;
    const double* part = work + kFactMaxBlocks;
    const size_t rec = 2 + NN;
    double dmin = 1.79769313486231570815e308, S = 0.0, SE = 0.0;
    for (int b = tid; b < nblocks; b += blockDim.x) {
        dmin = fmin(dmin, work[b]);
        S += part[b * rec];
        SE += part[b * rec + 1];
    }
    if (tid < NN) {
        double a = 0.0;
        for (int b = 0; b < nblocks; ++b) a += part[b * rec + 2 + tid];
        M[tid] = a;
    }
    dmin = block_min(dmin, red);
    S = block_sum(S, red);
    SE = block_sum(SE, red);
    const double emin = 0.5 * s.kappa * dmin;
    if (tid == 0) {
        if (!(dmin < 1.79769313486231570815e308) || !(S >= 1.0) || !isfinite(S) || !isfinite(SE))
            atomicOr(s.err, ERRB_NONFINITE_VB);
        s.scal[0] = emin - log(S / (double)factorial_ll(N)) / s.beta_ex;
        s.scal[1] = -(SE / S) / s.P;
        s.scal[2] = 0.0;
        s.scal[3] = 0.0;
    }
    const double invS = 1.0 / S;
    const int first = 0, last = s.P - 1;
    for (int w = tid; w < 2 * N; w += blockDim.x) {
        const bool is_last = w < N;
        const int l = is_last ? w : w - N;
        const int bead = is_last ? last : first;
        const int other = is_last ? first : last;
        const int nb = is_last ? (s.P - 2 + s.P) % s.P : 1 % s.P;
        const int side = is_last ? 1 : 0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            const double xl = s.x[idx<D>(s, bead, a, l)];
            double sum = 0.0;
            for (int q = 0; q < N; ++q) {
                double d = s.x[idx<D>(s, other, a, q)] - xl;
                if (s.pbc) d = min_image(d, s.L, s.invL);
                sum += (is_last ? M[l * N + q] : M[q * N + l]) * d;
            }
            double di = s.x[idx<D>(s, nb, a, l)] - xl;
            if (s.pbc) di = min_image(di, s.L, s.invL);
            const double fs = (sum * invS + di) * s.kappa;
            s.fx[((size_t)side * D + a) * s.ld + l] = fs;
            if (accumulate) {
                const size_t o = idx<D>(s, bead, a, l);
                s.f[o] = fs + s.f[o];
            }
        }
    }
}

int fact_tail(int N) { return N < 4 ? N : 4; }

int fact_grid(int N) {
    const long long runs = factorial_ll(N) / factorial_ll(fact_tail(N));
    const long long g = (runs + kFactThreads - 1) / kFactThreads;
    return (int)(g < kFactMaxBlocks ? g : kFactMaxBlocks);
}

template <int D, int T>
void fact_front(const Sys& s, double* work, cudaStream_t st) {
    const long long runs = factorial_ll(s.N) / factorial_ll(T);
    const int grid = fact_grid(s.N);
    k_fact_min<D, T><<<grid, kFactThreads, 0, st>>>(s, work, runs);
    k_fact_sums<D, T><<<grid, kFactThreads, 0, st>>>(s, work, runs, grid);
}

template <int D>
void fact_front_d(const Sys& s, double* work, cudaStream_t st) {
    switch (fact_tail(s.N)) {
        case 1: fact_front<D, 1>(s, work, st); break;
        case 2: fact_front<D, 2>(s, work, st); break;
        case 3: fact_front<D, 3>(s, work, st); break;
        default: fact_front<D, 4>(s, work, st); break;
    }
}

}  // namespace

size_t factorial_work_doubles(int N) { return (size_t)kFactMaxBlocks * (3 + (size_t)N * N); }

int launch_factorial_sums(const Sys& s, int D, double* work, cudaStream_t st) {
    if (D == 1) fact_front_d<1>(s, work, st);
    else if (D == 2) fact_front_d<2>(s, work, st);
    else fact_front_d<3>(s, work, st);
    return 2;
}

void launch_factorial_finish(const Sys& s, int D, double* work, int accumulate, cudaStream_t st) {
    const int grid = fact_grid(s.N);
    if (D == 1) k_fact_finish<1><<<1, kFactThreads, 0, st>>>(s, work, grid, accumulate);
    else if (D == 2) k_fact_finish<2><<<1, kFactThreads, 0, st>>>(s, work, grid, accumulate);
    else k_fact_finish<3><<<1, kFactThreads, 0, st>>>(s, work, grid, accumulate);
}

}  // namespace pimdb

// Block- and warp-level pieces of the Feldman-Hirshberg exchange, shared by
// the one-system kernels (exchange.cu) and the batched-replica kernel
// (batch.cu).  Each function works on one system given by a Sys; the caller
// chooses which block or warp runs it.
#pragma once

#include <math_constants.h>

#include "common.cuh"
#include "forces_dev.cuh"  // exp_tang

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
// for u = v-1 .. 0, evaluated as a warp-wide suffix scan over u.  The middle
// distance of entry u is the last distance of entry u+1, so each entry costs
// two distance evaluations (passed between lanes by a shuffle), or one with
// `link` (link[u] = |x1_{u+1} - xP_u|^2, computed once per u by the caller).
template <int D>
__device__ inline void energy_row(const Sys& s, int v, int lane, const double* link = nullptr) {
    const int first = 0, last = s.P - 1;
    const double hk = 0.5 * s.kappa;
    double* row = s.E + tri(v);
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
    double cnext = dist_to_v(v);  // |xP_v - x1_{u+1}|^2 for the lane holding u = base
    double carry = hk * cnext;
    if (lane == 0) row[v] = carry;
    for (int base = v - 1; base >= 0; base -= 32) {
        const int u = base - lane;
        const double c = u >= 0 ? dist_to_v(u) : 0.0;
        double cu1 = __shfl_up_sync(0xffffffffu, c, 1);
        if (lane == 0) cu1 = cnext;
        double term = 0.0;
        if (u >= 0) term = hk * ((link ? link[u] : sepsq<D>(s, last, u, first, u + 1)) - cu1 + c);
        cnext = __shfl_sync(0xffffffffu, c, 31);
        // inclusive scan over lanes (lane 0 holds the largest u)
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, term, o);
            if (lane >= o) term += y;
        }
        if (u >= 0) {
            const double e = carry + term;
            row[u] = e;
            // backward node r = N - u depends on node r' = N - 1 - v
            if (u >= 1) s.Et[tri(s.N - u - 1) + (s.N - 1 - v)] = e;
        }
        carry += __shfl_sync(0xffffffffu, term, 31);
    }
    if (lane == 0 && v >= 1) s.Et[tri(s.N - v - 1) + (s.N - 1 - v)] = row[v];
}
__device__ __forceinline__ void lse_add(float& mx, float& sm, float t) {
    if (t > mx) {
        sm = sm * __expf(mx - t) + 1.0f;
        mx = t;
    } else {
        sm += __expf(t - mx);
    }
}
// The recursions as "node" recursions.  Forward: node n = level m = n,
// node 0 known (V = 0), node n depends on nodes u < n through the packed row
// E[n-1][u].  Backward: node r = N - l, node 0 (l = N) known, node r depends
// on nodes r' < r through Et[r-1][r'] = E[p][l] with p = N - 1 - r' (so
// p + 1 = N - r').  Both are evaluated by the same blocked scheme: nodes are
// taken 32 at a time; warp 0 resolves the 32 nodes of a block one after the
// other with shuffles (no barrier), then every thread folds the finished
// block into the accumulators of all later nodes (one barrier pair per 32
// nodes instead of one barrier per node).
constexpr int kWaveThreads = 256;
// FP32 log-sum-exp node recursion.  fwd: value(n) = -(LSE - log n)/beta;
// bwd: terms carry -log(N - r') and value(r) = -LSE/beta.
__device__ inline void blocked_estimate(const double* __restrict__ Eg, int nn, int N, float beta, bool fwd, float* val,
                                 float* amx, float* asm_) {
    const int tid = threadIdx.x, bd = blockDim.x, lane = tid & 31, warp = tid >> 5;
    for (int n = tid; n < nn; n += bd) {
        amx[n] = -CUDART_INF_F;
        asm_[n] = 0.0f;
    }
    __syncthreads();
    const int nb = (nn + 31) / 32;
    for (int b = 0; b < nb; ++b) {
        const int base = 32 * b;
        if (warp == 0) {
            const int n = base + lane;
            float mx = n < nn ? amx[n] : -CUDART_INF_F, sm = n < nn ? asm_[n] : 0.0f;
            float e[32];
#pragma unroll
            for (int t = 0; t < 32; ++t) e[t] = (n < nn && n >= 1 && t < lane) ? (float)Eg[tri(n - 1) + base + t] : 0.0f;
            float v = 0.0f;
#pragma unroll
            for (int t = 0; t < 32; ++t) {
                if (lane == t && n < nn && n >= 1)
                    v = -(mx + __logf(sm) - (fwd ? __logf((float)n) : 0.0f)) / beta;
                const float vt = __shfl_sync(0xffffffffu, v, t);
                if (lane > t && n < nn) {
                    const int u = base + t;
                    lse_add(mx, sm, -beta * (e[t] + vt) - (fwd ? 0.0f : __logf((float)(N - u))));
                }
            }
            if (n < nn) val[n] = v;
        }
        __syncthreads();
        for (int m = base + 32 + tid; m < nn; m += bd) {
            float t[32];
            float lmx = -CUDART_INF_F;
#pragma unroll
            for (int q = 0; q < 32; ++q) {
                const int u = base + q;
                t[q] = -beta * ((float)Eg[tri(m - 1) + u] + val[u]) - (fwd ? 0.0f : __logf((float)(N - u)));
                lmx = fmaxf(lmx, t[q]);
            }
            float ls = 0.0f;
#pragma unroll
            for (int q = 0; q < 32; ++q) ls += __expf(t[q] - lmx);
            float mx = amx[m], sm = asm_[m];
            if (lmx > mx) {
                sm = sm * __expf(mx - lmx) + ls;
                mx = lmx;
            } else {
                sm += ls * __expf(lmx - mx);
            }
            amx[m] = mx;
            asm_[m] = sm;
        }
        __syncthreads();
    }
}
// FP64 triangular node solve: y(0) = 1, y(n) = sum_{u<n} W[n-1][u] y(u).
__device__ inline void blocked_solve(const double* __restrict__ W, int nn, double* y, double* acc) {
    const int tid = threadIdx.x, bd = blockDim.x, lane = tid & 31, warp = tid >> 5;
    for (int n = tid; n < nn; n += bd) acc[n] = 0.0;
    __syncthreads();
    const int nb = (nn + 31) / 32;
    for (int b = 0; b < nb; ++b) {
        const int base = 32 * b;
        if (warp == 0) {
            const int n = base + lane;
            double a = n == 0 ? 1.0 : (n < nn ? acc[n] : 0.0);
            double w[32];
#pragma unroll
            for (int t = 0; t < 32; ++t) w[t] = (n < nn && n >= 1 && t < lane) ? W[tri(n - 1) + base + t] : 0.0;
#pragma unroll
            for (int t = 0; t < 32; ++t) {
                const double yt = __shfl_sync(0xffffffffu, a, t);
                if (lane > t) a = fma(w[t], yt, a);
            }
            if (n < nn) y[n] = a;
        }
        __syncthreads();
        for (int m = base + 32 + tid; m < nn; m += bd) {
            const double* row = W + tri(m - 1) + base;
            double sacc = acc[m];
#pragma unroll 8
            for (int q = 0; q < 32; ++q) sacc = fma(row[q], y[base + q], sacc);
            acc[m] = sacc;
        }
        __syncthreads();
    }
}
// Pass 1: the FP32 estimate of one direction (0 forward, 1 backward) by the
// whole block; `fsm` holds 3 (N+1) floats.
__device__ inline void estimate_direction(const Sys& s, int dir, float* fsm) {
    const int N = s.N;
    float* val = fsm;
    float* amx = fsm + (N + 1);
    float* asm_ = fsm + 2 * (N + 1);
    const float beta = (float)s.beta_ex;
    if (dir == 0) {
        blocked_estimate(s.E, N + 1, N, beta, true, val, amx, asm_);
        for (int m = threadIdx.x; m <= N; m += blockDim.x) s.Vh[m] = (double)val[m];
    } else {
        // nodes r = 0..N-1 <-> l = N..1
        blocked_estimate(s.Et, N, N, beta, false, val, amx, asm_);
        for (int l = threadIdx.x; l <= N; l += blockDim.x) s.Vbh[l] = (l >= 1) ? (double)val[N - l] : 0.0;
    }
}
// Pass 2: the FP64 weights of packed entry (row p, column u), both directions
// (dir 0 forward only, 1 backward only, -1 both); `inv` = 1/(p+1), once per
// row.  `tbl`: the exp_tang table (32 entries: a weights block then still
// fits beside the pair kernel's resident blocks) in shared memory (null:
// CUDA's exp).  Arguments of 709 and more give infinity either way (the
// solve then retries).
// 1/(p+1) for p < 4096, evaluated by the compiler (IEEE division, the
// device's own result) into constant memory: the weights read it once per row
// (a uniform index, one broadcast) instead of dividing.
struct RecipTable {
    double v[4096];
    constexpr RecipTable() : v() {
        for (int i = 0; i < 4096; ++i) v[i] = 1.0 / (i + 1);
    }
};
static __constant__ RecipTable kRecip = RecipTable();
__device__ __forceinline__ double recip_row(int p) { return p < 4096 ? kRecip.v[p] : 1.0 / (p + 1); }

__device__ __forceinline__ double weight_exp(double x, const double* tbl) {
    if (!tbl) return exp(x);
    return x < 709.0 ? exp_tang(x, tbl) : (double)INFINITY;
}
// Returns whether either weight it wrote is nonzero (the solve's band: node
// p + 1 depends on node u, backward node N - u on node N - 1 - p, both at
// distance p + 1 - u).
__device__ __forceinline__ bool exch_weight(const Sys& s, int p, int u, double inv, const double* tbl = nullptr,
                                            int dir = -1) {
    const double beta = s.beta_ex;
    const size_t e = tri(p) + u;
    const double E = s.E[e];
    bool nz = false;
    if (dir <= 0) {
        const double w = weight_exp(-beta * (E + s.Vh[u] - s.Vh[p + 1]), tbl) * inv;
        s.Wf[e] = w;
        nz = w != 0.0;
    }
    // backward node r = N - u from node r' = N - 1 - p (u >= 1)
    if (dir != 0 && u >= 1) {
        const double w = weight_exp(-beta * (E + s.Vbh[p + 1] - s.Vbh[u]), tbl) * inv;
        s.Wb[tri(s.N - u - 1) + (s.N - 1 - p)] = w;
        nz = nz || w != 0.0;
    }
    return nz;
}
// One direction's weights by the whole block (the in-block retry).
__device__ inline void weights_direction(const Sys& s, int dir, const double* tbl) {
    for (int p = 0; p < s.N; ++p) {
        const double inv = recip_row(p);
        for (int u = threadIdx.x; u <= p; u += blockDim.x) exch_weight(s, p, u, inv, tbl, dir);
    }
}
// The weights of every packed entry (row p, column u), both directions, as
// exch_weight computes them, in double-float on the FP32 pipe, by one block
// (the batched engine's mixed path; the one block that ran a fresh
// estimate): w = exp(-beta (E + Vh_u - Vh_{p+1})) / (p + 1) forward,
// exp(-beta (E + Vbh_{p+1} - Vbh_u)) / (p + 1) backward.  Arguments above 88 give infinity (the solve then retries with a
// fresh estimate or the exact recursion), below -88 zero (a weight under
// 1e-38 of the ones that normalise the row).  `vsm` holds 4 (N + 1) floats.
// Returns this thread's band: the largest p + 1 - u of a nonzero weight.
__device__ inline int weights_df_block(const Sys& s, const dfl::ExpTable& etbl, float* vsm) {
    using dfl::df;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int N = s.N;
    float* vh = vsm;               // Vh hi, lo
    float* vbh = vsm + 2 * (N + 1);  // Vbh hi, lo
    for (int m = threadIdx.x; m <= N; m += blockDim.x) {
        split_f32(s.Vh[m], vh[m], vh[N + 1 + m]);
        split_f32(s.Vbh[m], vbh[m], vbh[N + 1 + m]);
    }
    __syncthreads();
    const df nbeta = dfl::neg(split_df(s.beta_ex));
    int band = 0;
    for (int p = warp; p < N; p += nw) {
        const df inv = split_df(recip_row(p));
        const df vp = dfl::fast_two_sum(vh[p + 1], vh[N + 2 + p]);
        const df vbp = dfl::fast_two_sum(vbh[p + 1], vbh[N + 2 + p]);
        const size_t r = tri(p);
        for (int u = lane; u <= p; u += 32) {
            const df E = split_df(s.E[r + u]);
            const df vu = dfl::fast_two_sum(vh[u], vh[N + 1 + u]);
            const df tf = dfl::add(dfl::add(E, vu), dfl::neg(vp));
            const double wf = df_to_f64(dfl::mul(dfl::exp(dfl::mul(nbeta, tf), etbl), inv));
            s.Wf[r + u] = wf;
            bool nz = !f64_is_zero(wf);
            if (u >= 1) {
                const df vbu = dfl::fast_two_sum(vbh[u], vbh[N + 1 + u]);
                const df tb = dfl::add(dfl::add(E, vbp), dfl::neg(vbu));
                const double wb = df_to_f64(dfl::mul(dfl::exp(dfl::mul(nbeta, tb), etbl), inv));
                s.Wb[tri(N - u - 1) + (N - 1 - p)] = wb;
                nz = nz || !f64_is_zero(wb);
            }
            if (nz) band = max(band, p + 1 - u);
        }
    }
    return band;
}

// Exact level-by-level FP64 log-sum-exp in the reference's order (used only
// when the estimate is unusable, or on request).  `vs` holds N+1 doubles,
// `red` 32.
__device__ inline void exact_forward(const Sys& s, double* vs, double* red) {
    const int N = s.N, tid = threadIdx.x, bd = blockDim.x;
    const double beta = s.beta_ex;
    if (tid == 0) vs[0] = 0.0;
    __syncthreads();
    for (int m = 1; m <= N; ++m) {
        const double* row = s.E + tri(m - 1);
        double lmin = 1.79769313486231570815e308;
        for (int u = tid; u < m; u += bd) lmin = fmin(lmin, row[u] + vs[u]);
        const double shift = block_min(lmin, red);
        double ls = 0.0;
        for (int u = tid; u < m; u += bd) ls += exp(-beta * (row[u] + vs[u] - shift));
        const double tot = block_sum(ls, red);
        if (tid == 0) vs[m] = shift - (1.0 / beta) * log(tot / (double)m);
        __syncthreads();
    }
}
__device__ inline void exact_backward(const Sys& s, double* vs, double* red) {
    const int N = s.N, tid = threadIdx.x, bd = blockDim.x;
    const double beta = s.beta_ex;
    if (tid == 0) vs[N] = 0.0;
    __syncthreads();
    for (int l = N - 1; l > 0; --l) {
        double lmin = 1.79769313486231570815e308;
        for (int p = l + tid; p < N; p += bd) lmin = fmin(lmin, s.E[tri(p) + l] + vs[p + 1]);
        const double shift = block_min(lmin, red);
        double ls = 0.0;
        for (int p = l + tid; p < N; p += bd) ls += exp(-beta * (s.E[tri(p) + l] + vs[p + 1] - shift)) / (p + 1);
        const double tot = block_sum(ls, red);
        if (tid == 0) vs[l] = shift - log(tot) / beta;
        __syncthreads();
    }
}
// |log y| above which the next evaluation computes a fresh FP32 estimate
// instead of reusing the current potentials, and above which the present
// evaluation switches to the exact level-by-level recursion.
constexpr int kGridSolveMinN = 768;     // from here the solve runs across SMs
constexpr int kFlatEnergiesMinN = 512;  // from here the cycle energies come from link prefix sums
constexpr int kGridSolveCtas = 64;      // CTAs per direction
constexpr int kGridSolveThreads = 256;
constexpr double kRefreshLogY = 30.0;
constexpr double kExactLogY = 200.0;
// Pass 3, one direction (0 forward, 1 backward) by the whole block: the y
// solve and the exact V / V_backwards.  `ys` holds 2 (N+1) + 32 doubles.
// When the solve is unusable (|log y| >= 200) and `allow_exact` is 0 (the
// estimate was the previous evaluation's potentials, not a fresh FP32
// recursion), no exact recursion is run: xflags[6] asks the caller to
// retry with a fresh estimate instead.
// `pre`: y of this direction already solved (k_exch_solve_grid), or null.
// Returns 1 when it gave up that way (block-uniform); with `flag_retry` 0
// xflags[6] is left alone (the caller retries in the same block).
// `et` (2^(j/256) as double-floats in shared memory): log y in double-float
// on the FP32 pipe (log_df); null: CUDA's FP64 log.
__device__ inline int solve_direction(const Sys& s, int dir, int force_exact, double* ys, int allow_exact = 1,
                                      const double* pre = nullptr, int flag_retry = 1,
                                      const dfl::ExpTable* et = nullptr) {
    double* acc = ys + s.N + 1;
    double* red = ys + 2 * (s.N + 1);
    const int N = s.N, tid = threadIdx.x, bd = blockDim.x;
    int bad = force_exact, stale = 0;
    if (dir == 0) {
        if (!force_exact) {
            if (pre) {
                for (int m = tid; m <= N; m += bd) ys[m] = ((volatile const double*)pre)[m];
                __syncthreads();
            } else {
                blocked_solve(s.Wf, N + 1, ys, acc);
            }
            for (int m = tid; m <= N; m += bd) {
                const double y = ys[m];
                const double ly = et ? log_df(y, *et) : log(y);
                if (!(y > 0.0) || !(fabs(ly) < kExactLogY)) bad = 1;
                if (!(fabs(ly) < kRefreshLogY)) stale = 1;
                s.yf[m] = y;
                s.V[m] = s.Vh[m] - ly * s.inv_beta_ex;
            }
        }
        bad = __syncthreads_or(bad);
        if (bad && !allow_exact) {
            if (tid == 0 && flag_retry) s.xflags[6] = 1;
            return 1;
        }
        if (bad) {
            exact_forward(s, ys, red);
            for (int m = tid; m <= N; m += bd) s.V[m] = ys[m];
        }
        int nonfinite = 0;
        __syncthreads();
        for (int m = tid; m <= N; m += bd)
            if (!isfinite(s.V[m])) nonfinite = 1;
        nonfinite = __syncthreads_or(nonfinite);
        stale = __syncthreads_or(stale);
        if (tid == 0) {
            s.xflags[0] = bad;
            s.xflags[4] = stale | nonfinite;
            if (nonfinite) atomicOr(s.err, ERRB_NONFINITE_VB);
        }
    } else {
        if (!force_exact) {
            // nodes r = 0..N-1 <-> levels l = N..1
            if (pre) {
                for (int r = tid; r < N; r += bd) ys[r] = ((volatile const double*)pre)[r];
                __syncthreads();
            } else {
                blocked_solve(s.Wb, N, ys, acc);
            }
            for (int l = tid + 1; l < N; l += bd) {
                const double y = ys[N - l];
                const double ly = et ? log_df(y, *et) : log(y);
                if (!(y > 0.0) || !(fabs(ly) < kExactLogY)) bad = 1;
                if (!(fabs(ly) < kRefreshLogY)) stale = 1;
                s.yb[l] = y;
                s.Vb[l] = s.Vbh[l] - ly * s.inv_beta_ex;
            }
        }
        if (tid == 0) {
            s.Vb[N] = 0.0;
            s.yb[N] = 1.0;
        }
        bad = __syncthreads_or(bad);
        if (bad && !allow_exact) {
            if (tid == 0 && flag_retry) s.xflags[6] = 1;
            return 1;
        }
        if (bad) {
            exact_backward(s, ys, red);
            for (int l = tid + 1; l <= N; l += bd) s.Vb[l] = ys[l];
        }
        int nonfinite = 0;
        __syncthreads();
        for (int l = tid + 1; l <= N; l += bd)
            if (!isfinite(s.Vb[l])) nonfinite = 1;
        nonfinite = __syncthreads_or(nonfinite);
        stale = __syncthreads_or(stale);
        if (tid == 0) {
            s.xflags[1] = bad;
            s.xflags[5] = stale | nonfinite;
            if (nonfinite) atomicOr(s.err, ERRB_NONFINITE_VB);
        }
    }
    return 0;
}
// After both directions (one block): the per-row factors of the connection
// probabilities, which need both V and V_backwards, and the estimates of the
// next evaluation: V, V_backwards themselves or, with `extrapolate` and a
// previous result in s.Vp (NaN until there is one), the linear extrapolation
// 2 V(t) - V(t - dt), which smooth dynamics keep much closer.  With `et` the
// row exponentials in double-float (exp_df).
__device__ inline void solve_finish(const Sys& s, int extrapolate = 0, const dfl::ExpTable* et = nullptr) {
    const int N = s.N, tid = threadIdx.x, bd = blockDim.x;
    const double beta = s.beta_ex;
    volatile double* V = s.V;
    volatile double* Vb = s.Vb;
    const double VN = V[N];
    for (int l = tid; l < N; l += bd) {
        const double vbl = Vb[l + 1];
        const double aR = -beta * (s.Vh[l + 1] + vbl - VN), aC = -beta * (V[l + 1] + vbl - VN);
        s.rowR[l] = et ? exp_df(aR, *et) : exp(aR);
        s.rowC[l] = et ? exp_df(aC, *et) : exp(aC);
    }
    __syncthreads();
    const int need = ((volatile int*)s.xflags)[4] | ((volatile int*)s.xflags)[5];
    for (int m = tid; m <= N; m += bd) {
        const double v = V[m], vb = m >= 1 ? Vb[m] : 0.0;
        if (s.Vp && extrapolate && isfinite(s.Vp[m]) && isfinite(s.Vp[N + 1 + m])) {
            s.Vh[m] = 2.0 * v - s.Vp[m];
            s.Vbh[m] = 2.0 * vb - s.Vp[N + 1 + m];
        } else {
            s.Vh[m] = v;
            s.Vbh[m] = vb;
        }
        if (s.Vp) {
            s.Vp[m] = v;
            s.Vp[N + 1 + m] = vb;
        }
    }
    if (tid == 0) {
        s.xflags[2] = 0;
        s.xflags[3] = need;
        s.Vb[0] = VN;  // V_backwards[0] = V[N] (:127)
        s.scal[0] = VN;
    }
}
// Exterior spring forces (:159-215).  Warps [0, N) handle bead P (row l of
// the connection-probability matrix), warps [N, 2N) bead 1 (column l).
// Probabilities: close-cycle P[l][u] = Wf[l][u] y_u R_l (u <= l), direct
// link P[l][l+1] = 1 - C_l; with the exact fallback they are evaluated
// from their defining exponentials.  When `accumulate`, the spring force is
// added to f (which holds the physical forces; simulation.cpp:363-373).
// `xs` (optional): the positions of beads 1 and P staged in shared memory,
// xs[(side * D + a) * N + i] with side 0 = bead 1, 1 = bead P.
template <int D>
// With `adjoint` set, the row writes the cotangent of the exchange potential
// instead of the force: fx = vb_bar * dV_B/dx = -vb_bar * kappa * sum, with
// neither the interior neighbour spring nor the accumulation into f.
// `band` > 0: every weight beyond that distance from the diagonal is exactly
// zero (the banded solve's measurement); the rows skip the 32-entry chunks
// that hold only such entries, each lane keeping its own entries (the same
// sums, bit for bit).
__device__ inline void exch_force_row(const Sys& s, int w, int lane, int accumulate, const double* xs = nullptr,
                                      int adjoint = 0, double vb_bar = 0.0, int band = 0) {
    const int N = s.N;
    const double beta = s.beta_ex;
    const double VN = s.V[N];
    const bool exact = s.xflags[0] != 0;
    const int first = 0, last = s.P - 1;
    double sum[D];
#pragma unroll
    for (int a = 0; a < D; ++a) sum[a] = 0.0;
    int bead, nb, l;
    if (w < N) {  // last bead, particle l: sum over n <= l+1
        l = w;
        bead = last;
        nb = (s.P - 2 + s.P) % s.P;
        const size_t r = tri(l);
        const double Rl = s.rowR[l];
        const double vbl = s.Vb[l + 1];
        const int nmax = min(l + 1, N - 1);
        double xl[D];
#pragma unroll
        for (int a = 0; a < D; ++a) xl[a] = s.x[idx<D>(s, last, a, l)];
        const int n0 = (band > 0 && !exact) ? max(0, l + 1 - band) / 32 * 32 : 0;
        for (int n = n0 + lane; n <= nmax; n += 32) {
            double pr;
            if (n <= l) {
                // a zero weight (a cycle too costly to contribute) adds exactly 0
                if (!exact && s.Wf[r + n] == 0.0) continue;
                pr = exact ? exp(-beta * (s.V[n] + s.E[r + n] + vbl - VN)) / (l + 1) : s.Wf[r + n] * s.yf[n] * Rl;
            } else {
                pr = 1.0 - s.rowC[l];
            }
#pragma unroll
            for (int a = 0; a < D; ++a) {
                double d = (xs ? xs[(size_t)a * N + n] : s.x[idx<D>(s, first, a, n)]) - xl[a];
                if (s.pbc) d = min_image(d, s.L, s.invL);
                sum[a] += pr * d;
            }
        }
    } else {  // first bead, particle l: sum over q >= l-1
        l = w - N;
        bead = first;
        nb = 1 % s.P;
        const double yl = s.yf[l];
        const double vl = s.V[l];
        double xl[D];
#pragma unroll
        for (int a = 0; a < D; ++a) xl[a] = s.x[idx<D>(s, first, a, l)];
        const int qend = (band > 0 && !exact) ? min(N, l + band) : N;  // q + 1 - l <= band
        for (int q = max(0, l - 1) + lane; q < qend; q += 32) {
            double pr;
            if (q >= l) {
                if (!exact && s.Wf[tri(q) + l] == 0.0) continue;
                pr = exact ? exp(-beta * (vl + s.E[tri(q) + l] + s.Vb[q + 1] - VN)) / (q + 1)
                           : s.Wf[tri(q) + l] * yl * s.rowR[q];
            } else {
                pr = 1.0 - s.rowC[q];
            }
#pragma unroll
            for (int a = 0; a < D; ++a) {
                double d = (xs ? xs[((size_t)D + a) * N + q] : s.x[idx<D>(s, last, a, q)]) - xl[a];
                if (s.pbc) d = min_image(d, s.L, s.invL);
                sum[a] += pr * d;
            }
        }
    }
#pragma unroll
    for (int a = 0; a < D; ++a) sum[a] = warp_sum(sum[a]);
    if (lane == 0 && adjoint) {
        const int side = (bead == first) ? 0 : 1;
        const double c = -vb_bar * s.kappa;
#pragma unroll
        for (int a = 0; a < D; ++a) s.fx[((size_t)side * D + a) * s.ld + l] = c * sum[a];
    } else if (lane == 0) {
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
}
// primEstimator (:250-279), getDistinctProbability (:222-229) and
// getLongestProbability (:238-240); one block, evaluated on request.
// `sh` holds N+1+32 doubles.
__device__ inline void estimators_block(const Sys& s, int nbeads, double* sh) {
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

}  // namespace pimdb

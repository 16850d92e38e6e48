/*
 * pimdb_oracle — CPU restatement of the PIMD-B++ per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker for the GPU kernels; see the header).
 * Compile with -ffp-contract=off: every expression below keeps the
 * reference's evaluation order so that, with the same libm, the results are
 * bit-identical to the compiled reference.
 */
#include "pimdb_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.14159265358979323846
#define ORC_EPS 1.0E-7 /* include/common.h:45 */

/* ------------------------------------------------------------------------ */
/* system constants                                                          */

void orc_system_init(orc_system* s, double temperature, double raw_cutoff) {
    /* simulation.cpp:37,41-52 (IPI convention, kB = hbar = 1) */
    s->beta = 1.0 / (1.0 * temperature);
    s->thermo_beta = s->beta / s->nbeads;
    s->omega_p = s->nbeads / (s->beta * 1.0);
    s->spring_constant = s->mass * s->omega_p * s->omega_p;
    /* bosonic_exchange_base.cpp:16-18 */
    s->beta_ex = s->beta / s->nbeads;
    /* simulation.cpp:690 */
    s->bosonic = s->bosonic && (s->nbeads > 1);
    /* simulation.cpp:84-90 */
    double cut = (s->int_kind == ORC_INT_FREE) ? 0.0 : raw_cutoff;
    if (s->pbc && 0.5 * s->size < cut) cut = 0.5 * s->size;
    s->cutoff = cut;
}

/* common.cpp:41-43 (applyMinimumImage) */
double orc_min_image(double dx, double L) { return dx - L * floor(dx / L + 0.5); }

static inline double sep(const orc_system* s, const double* a, const double* b, int axis) {
    /* difference b - a with the optional minimum image:
     * bosonic_exchange_base.cpp:30-42 */
    double dx = b[axis] - a[axis];
    if (s->pbc) dx = orc_min_image(dx, s->size);
    return dx;
}

static inline double sepsq(const orc_system* s, const double* a, const double* b) {
    /* bosonic_exchange_base.cpp:53-64 */
    double d2 = 0.0;
    for (int ax = 0; ax < s->ndim; ++ax) {
        double d = sep(s, a, b, ax);
        d2 += d * d;
    }
    return d2;
}

/* ------------------------------------------------------------------------ */
/* potentials (src/potentials, one file each)                                        */

void orc_ext_grad(const orc_system* s, const double* x, int n, double* g) {
    const int D = s->ndim;
    switch (s->ext_kind) {
    case ORC_EXT_HARMONIC: { /* harmonic.cpp:3-5,21-23 */
        const double k = s->mass * s->ext_p[0] * s->ext_p[0];
        for (int i = 0; i < n * D; ++i) g[i] = x[i] * k;
        break;
    }
    case ORC_EXT_DOUBLE_WELL: { /* double_well.cpp:22-40 */
        const double loc2 = s->ext_p[1] * s->ext_p[1];
        for (int i = 0; i < n; ++i) {
            double pre = 0;
            for (int a = 0; a < D; ++a) pre += x[i * D + a] * x[i * D + a];
            pre = 4 * s->mass * s->ext_p[0] * (pre - loc2);
            for (int a = 0; a < D; ++a) g[i * D + a] = pre * x[i * D + a];
        }
        break;
    }
    case ORC_EXT_COSINE: { /* cosine.cpp:4-6,23-35 */
        const double k = 2 * ORC_PI / s->size;
        const double pre = -s->ext_p[0] * k;
        for (int i = 0; i < n * D; ++i) g[i] = pre * sin(k * x[i] + s->ext_p[1]);
        break;
    }
    default:
        for (int i = 0; i < n * D; ++i) g[i] = 0.0;
    }
}

double orc_ext_value(const orc_system* s, const double* x, int n) {
    const int D = s->ndim;
    double v = 0.0;
    switch (s->ext_kind) {
    case ORC_EXT_HARMONIC: { /* harmonic.cpp:7-19 */
        const double k = s->mass * s->ext_p[0] * s->ext_p[0];
        for (int i = 0; i < n; ++i)
            for (int a = 0; a < D; ++a) v += x[i * D + a] * x[i * D + a];
        v *= 0.5 * k;
        break;
    }
    case ORC_EXT_DOUBLE_WELL: { /* double_well.cpp:6-20 */
        const double loc2 = s->ext_p[1] * s->ext_p[1];
        for (int i = 0; i < n; ++i)
            for (int a = 0; a < D; ++a)
                v += (x[i * D + a] * x[i * D + a] - loc2) * (x[i * D + a] * x[i * D + a] - loc2);
        v *= s->mass * s->ext_p[0];
        break;
    }
    case ORC_EXT_COSINE: { /* cosine.cpp:9-21 */
        const double k = 2 * ORC_PI / s->size;
        for (int i = 0; i < n; ++i)
            for (int a = 0; a < D; ++a) v += cos(k * x[i * D + a] + s->ext_p[1]);
        v *= s->ext_p[0];
        break;
    }
    default:
        break;
    }
    return v;
}

/* Aziz HFDHE2 constants (aziz.cpp:6-13) */
static const double AZ_RM = 5.60738, AZ_A = 0.5448504e6, AZ_EPSILON = 3.42016E-5, AZ_ALPHA = 13.353384,
                    AZ_D = 1.241314, AZ_C6 = 1.3732412, AZ_C8 = 0.4253785, AZ_C10 = 0.1781;

static inline double az_F(double x) { /* aziz.h:25-27 */
    return (x < AZ_D ? exp(-(AZ_D / x - 1.0) * (AZ_D / x - 1.0)) : 1.0);
}
static inline double az_dF(double x) { /* aziz.h:30-34 */
    double ix = 1.0 / x;
    double r = 2.0 * AZ_D * ix * ix * (AZ_D * ix - 1.0) * exp(-(AZ_D * ix - 1.0) * (AZ_D * ix - 1.0));
    return (x < AZ_D ? r : 0.0);
}

static inline double vnorm(const double* r, int D) { /* common.h:121-127 */
    double n2 = 0.0;
    for (int a = 0; a < D; ++a) n2 += r[a] * r[a];
    return sqrt(n2);
}

void orc_pair_grad(const orc_system* s, const double* r, double* g) {
    const int D = s->ndim;
    switch (s->int_kind) {
    case ORC_INT_HARMONIC: { /* harmonic.cpp:21-23 */
        const double k = s->mass * s->int_p[0] * s->int_p[0];
        for (int a = 0; a < D; ++a) g[a] = r[a] * k;
        break;
    }
    case ORC_INT_DIPOLE: { /* dipole.cpp:24-45 */
        const double norm = vnorm(r, D);
        const double pre = -3.0 * s->int_p[0] / (norm * norm * norm * norm * norm);
        for (int a = 0; a < D; ++a) g[a] = pre * r[a];
        break;
    }
    case ORC_INT_AZIZ: { /* aziz.cpp:56-106 */
        const double norm = vnorm(r, D);
        const double r_scaled = norm / AZ_RM;
        const double T1 = -AZ_A * AZ_ALPHA * exp(-AZ_ALPHA * r_scaled);
        double grad;
        if (r_scaled > ORC_EPS && r_scaled < 0.01) {
            grad = T1 * (AZ_EPSILON / AZ_RM);
        } else {
            const double ix = 1.0 / r_scaled;
            const double ix2 = ix * ix;
            const double ix6 = ix2 * ix2 * ix2;
            const double ix7 = ix6 * ix;
            const double ix8 = ix6 * ix2;
            const double ix9 = ix8 * ix;
            const double ix10 = ix8 * ix2;
            const double ix11 = ix10 * ix;
            const double T2 = (6.0 * AZ_C6 * ix7 + 8.0 * AZ_C8 * ix9 + 10.0 * AZ_C10 * ix11) * az_F(r_scaled);
            const double T3 = -(AZ_C6 * ix6 + AZ_C8 * ix8 + AZ_C10 * ix10) * az_dF(r_scaled);
            grad = (AZ_EPSILON / AZ_RM) * (T1 + T2 + T3);
        }
        grad /= norm;
        for (int a = 0; a < D; ++a) g[a] = grad * r[a];
        break;
    }
    default:
        for (int a = 0; a < D; ++a) g[a] = 0.0;
    }
}

double orc_pair_value(const orc_system* s, const double* r) {
    const int D = s->ndim;
    switch (s->int_kind) {
    case ORC_INT_HARMONIC: { /* harmonic.cpp:7-19 */
        const double k = s->mass * s->int_p[0] * s->int_p[0];
        double v = 0.0;
        for (int a = 0; a < D; ++a) v += r[a] * r[a];
        return v * (0.5 * k);
    }
    case ORC_INT_DIPOLE: { /* dipole.cpp:5-22 */
        const double norm = vnorm(r, D);
        return 0.0 + s->int_p[0] / (norm * norm * norm);
    }
    case ORC_INT_AZIZ: { /* aziz.cpp:18-54 */
        const double r_scaled = vnorm(r, D) / AZ_RM;
        const double Urep = AZ_A * exp(-AZ_ALPHA * r_scaled);
        if (r_scaled > ORC_EPS && r_scaled < 0.01) return 0.0 + AZ_EPSILON * Urep;
        const double ix2 = 1.0 / (r_scaled * r_scaled);
        const double ix6 = ix2 * ix2 * ix2;
        const double ix8 = ix6 * ix2;
        const double ix10 = ix8 * ix2;
        const double Uatt = -(AZ_C6 * ix6 + AZ_C8 * ix8 + AZ_C10 * ix10) * az_F(r_scaled);
        return 0.0 + AZ_EPSILON * (Urep + Uatt);
    }
    default:
        return 0.0;
    }
}

/* ------------------------------------------------------------------------ */
/* bosonic exchange (quadratic_bosonic_exchange.cpp)                          */

static inline long enk_index(int m, int k) { return (long)m * (m + 1) / 2 - k; } /* :63-71 */

void orc_cycle_energies(const orc_system* s, const double* x1, const double* xP, double* E) {
    /* :34-61 with x_first_bead = bead 1 and x_last_bead = bead P (:86-94) */
    const int N = s->natoms, D = s->ndim;
    const double kap = s->spring_constant;
    double* self = (double*)malloc(sizeof(double) * (size_t)N);
    for (int i = 0; i < N; ++i) self[i] = sepsq(s, x1 + (long)i * D, xP + (long)i * D);
    for (int v = 0; v < N; ++v) {
        E[enk_index(v + 1, 1)] = 0.5 * kap * self[v];
        for (int u = v - 1; u >= 0; --u) {
            double val = E[enk_index(v + 1, v - u)] +
                         0.5 * kap *
                             (+sepsq(s, xP + (long)u * D, x1 + (long)(u + 1) * D) -
                              sepsq(s, x1 + (long)(u + 1) * D, xP + (long)v * D) +
                              sepsq(s, x1 + (long)u * D, xP + (long)v * D));
            E[enk_index(v + 1, v - u + 1)] = val;
        }
    }
    free(self);
}

int orc_vb_forward(const orc_system* s, const double* E, double* V) {
    /* :73-99 */
    const int N = s->natoms;
    const double beta = s->beta_ex;
    double* tmp = (double*)malloc(sizeof(double) * (size_t)(N + 1));
    int st = 0;
    V[0] = 0.0;
    for (int m = 1; m < N + 1; ++m) {
        double e_shift = DBL_MAX;
        for (int k = m; k > 0; --k) {
            double val = E[enk_index(m, k)] + V[m - k];
            e_shift = (val < e_shift) ? val : e_shift;
            tmp[k - 1] = val;
        }
        double sig = 0.0;
        for (int k = m; k > 0; --k) sig += exp(-beta * (tmp[k - 1] - e_shift));
        V[m] = e_shift - (1.0 / beta) * log(sig / (double)m);
        if (!isfinite(V[m])) st = 2;
    }
    free(tmp);
    return st;
}

int orc_vb_backward(const orc_system* s, const double* E, const double* V, double* Vb) {
    /* :101-128 */
    const int N = s->natoms;
    const double beta = s->beta_ex;
    double* tmp = (double*)malloc(sizeof(double) * (size_t)(N + 1));
    int st = 0;
    Vb[N] = 0.0;
    for (int l = N - 1; l > 0; --l) {
        double e_shift = DBL_MAX;
        for (int p = l; p < N; ++p) {
            double val = E[enk_index(p + 1, p - l + 1)] + Vb[p + 1];
            e_shift = (val < e_shift) ? val : e_shift;
            tmp[p] = val;
        }
        double sig = 0.0;
        for (int p = l; p < N; ++p) sig += 1.0 / (p + 1) * exp(-beta * (tmp[p] - e_shift));
        Vb[l] = e_shift - log(sig) / beta;
        if (!isfinite(Vb[l])) st = 2;
    }
    Vb[0] = V[N];
    free(tmp);
    return st;
}

void orc_connection_probabilities(const orc_system* s, const double* E, const double* V, const double* Vb,
                                  double* prob) {
    /* :142-157; entries above the first super-diagonal stay zero */
    const int N = s->natoms;
    const double beta = s->beta_ex;
    memset(prob, 0, sizeof(double) * (size_t)N * (size_t)N);
    for (int l = 0; l < N - 1; ++l)
        prob[(long)N * l + (l + 1)] = 1.0 - (exp(-beta * (V[l + 1] + Vb[l + 1] - V[N])));
    for (int u = 0; u < N; ++u)
        for (int l = u; l < N; ++l)
            prob[(long)N * l + u] =
                1.0 / (l + 1) * exp(-beta * (V[u] + E[enk_index(l + 1, l - u + 1)] + Vb[l + 1] - V[N]));
}

void orc_spring_force_last_bead(const orc_system* s, const double* prob, const double* x, const double* x_prev,
                                const double* x_next, double* f) {
    /* :159-186 (this bead = P; x_next = bead 1, x_prev = bead P-1) */
    const int N = s->natoms, D = s->ndim;
    for (int l = 0; l < N; ++l) {
        double sums[3] = {0.0, 0.0, 0.0};
        for (int nl = 0; nl <= l + 1 && nl < N; ++nl) {
            const double pr = prob[(long)N * l + nl];
            for (int a = 0; a < D; ++a) sums[a] += pr * sep(s, x + (long)l * D, x_next + (long)nl * D, a);
        }
        for (int a = 0; a < D; ++a) sums[a] += sep(s, x + (long)l * D, x_prev + (long)l * D, a);
        for (int a = 0; a < D; ++a) f[(long)l * D + a] = sums[a] * s->spring_constant;
    }
}

void orc_spring_force_first_bead(const orc_system* s, const double* prob, const double* x, const double* x_prev,
                                 const double* x_next, double* f) {
    /* :188-215 (this bead = 1; x_prev = bead P, x_next = bead 2) */
    const int N = s->natoms, D = s->ndim;
    for (int l = 0; l < N; ++l) {
        double sums[3] = {0.0, 0.0, 0.0};
        for (int pl = (l - 1 > 0 ? l - 1 : 0); pl < N; ++pl) {
            const double pr = prob[(long)N * pl + l];
            for (int a = 0; a < D; ++a) sums[a] += pr * sep(s, x + (long)l * D, x_prev + (long)pl * D, a);
        }
        for (int a = 0; a < D; ++a) sums[a] += sep(s, x + (long)l * D, x_next + (long)l * D, a);
        for (int a = 0; a < D; ++a) f[(long)l * D + a] = sums[a] * s->spring_constant;
    }
}

double orc_prim_estimator(const orc_system* s, const double* E, const double* V) {
    /* :250-279 */
    const int N = s->natoms;
    const double beta = s->beta_ex;
    double* G = (double*)malloc(sizeof(double) * (size_t)(N + 1));
    G[0] = 0.0;
    for (int m = 1; m < N + 1; ++m) {
        double sig = 0.0;
        double e_shift = DBL_MAX;
        for (int k = m; k > 0; --k) {
            double val = E[enk_index(m, k)] + V[m - k];
            e_shift = (val < e_shift) ? val : e_shift;
        }
        for (int k = m; k > 0; --k) {
            const double ekn = E[enk_index(m, k)];
            sig += (G[m - k] - ekn) * exp(-beta * (ekn + V[m - k] - e_shift));
        }
        const double denom = m * exp(-beta * (V[m] - e_shift));
        G[m] = sig / denom;
    }
    double out = G[N] / s->nbeads;
    free(G);
    return out;
}

double orc_distinct_probability(const orc_system* s, const double* E, const double* V) {
    /* :222-229 */
    const int N = s->natoms;
    double sum = 0.0;
    for (int m = 1; m < N + 1; ++m) sum += E[enk_index(m, 1)];
    return exp(-s->beta_ex * (sum - V[N]) - lgamma(N + 1));
}

double orc_longest_probability(const orc_system* s, const double* E, const double* V) {
    /* :238-240 */
    const int N = s->natoms;
    return exp(-s->beta_ex * (E[enk_index(N, N)] - V[N]));
}

/* ------------------------------------------------------------------------ */
/* factorial exchange (src/bosonic_exchange/factorial_bosonic_exchange.cpp)   */

/* std::ranges::next_permutation: the next arrangement in lexicographic order;
 * returns 0 (and restores ascending order) after the last one. */
static int orc_next_permutation(int* a, int n) {
    int i = n - 2;
    while (i >= 0 && !(a[i] < a[i + 1])) --i;
    if (i < 0) {
        for (int l = 0, r = n - 1; l < r; ++l, --r) {
            int t = a[l];
            a[l] = a[r];
            a[r] = t;
        }
        return 0;
    }
    int j = n - 1;
    while (!(a[i] < a[j])) --j;
    int t = a[i];
    a[i] = a[j];
    a[j] = t;
    for (int l = i + 1, r = n - 1; l < r; ++l, --r) {
        t = a[l];
        a[l] = a[r];
        a[r] = t;
    }
    return 1;
}

/* labels[] holds the bottom line of the permutation's two-line notation
 * (:9-12): the last bead of particle l links to the first bead of
 * labels[l] (lastBeadNeighbor, :47-49); the first bead of particle l links to
 * the last bead of the particle at l's position (firstBeadNeighbor, :33-35). */
static void orc_inverse(const int* labels, int n, int* inv) {
    for (int l = 0; l < n; ++l) inv[labels[l]] = l;
}

/* getMinExteriorSpringEnergy (:58-82) */
double orc_factorial_min_energy(const orc_system* s, const double* x_first, const double* x_last) {
    const int N = s->natoms, D = s->ndim;
    int* labels = (int*)malloc(sizeof(int) * (size_t)N);
    for (int l = 0; l < N; ++l) labels[l] = l;
    double min_delta = DBL_MAX;
    do {
        double diff2 = 0.0;
        for (int l = 0; l < N; ++l) diff2 += sepsq(s, x_first + (long)l * D, x_last + (long)labels[l] * D);
        const double e = 0.5 * s->spring_constant * diff2;
        if (e < min_delta) min_delta = e; /* std::min(min_delta, e) */
    } while (orc_next_permutation(labels, N));
    free(labels);
    return min_delta;
}

/* effectivePotential (:91-114) */
static double orc_factorial_potential(const orc_system* s, const double* x_first, const double* x_last) {
    const int N = s->natoms, D = s->ndim;
    const double beta_half_k = s->thermo_beta * 0.5 * s->spring_constant; /* simulation.cpp:52 */
    int* labels = (int*)malloc(sizeof(int) * (size_t)N);
    for (int l = 0; l < N; ++l) labels[l] = l;
    long counter = 0;
    double weights_sum = 0.0;
    do {
        counter++;
        double diff2 = 0.0;
        for (int l = 0; l < N; ++l) diff2 += sepsq(s, x_first + (long)l * D, x_last + (long)labels[l] * D);
        weights_sum += exp(-beta_half_k * diff2);
    } while (orc_next_permutation(labels, N));
    free(labels);
    return (-1.0 / s->beta_ex) * log(weights_sum / (double)counter);
}

/* springForceLastBead (:121-172, first == 0) and springForceFirstBead
 * (:179-230, first == 1).  x is the exchange bead, x_prev / x_next its
 * neighbours in the reference's bead order; f is overwritten. */
static void orc_factorial_force(const orc_system* s, int first, const double* x, const double* x_prev,
                                const double* x_next, double e_shift, double* f) {
    const int N = s->natoms, D = s->ndim;
    const double k = s->spring_constant, beta = s->beta_ex;
    const double* x_first_bead = first ? x : x_next;
    const double* x_last_bead = first ? x_prev : x;
    int* labels = (int*)malloc(sizeof(int) * (size_t)N * 2);
    int* inv = labels + N;
    double* temp = (double*)malloc(sizeof(double) * (size_t)N * D);
    for (int l = 0; l < N; ++l) labels[l] = l;
    for (long i = 0; i < (long)N * D; ++i) f[i] = 0.0;
    double denom_weight = 0.0;
    do {
        orc_inverse(labels, N, inv);
        double weight = 0.0;
        for (int l = 0; l < N; ++l) {
            double sums[3] = {0.0, 0.0, 0.0};
            double d_ext[3], d_int[3];
            const double* xl = (first ? x_first_bead : x_last_bead) + (long)l * D;
            for (int a = 0; a < D; ++a) {
                if (first) /* last bead of the particle at l's position minus first bead of l */
                    d_ext[a] = sep(s, xl, x_last_bead + (long)inv[l] * D, a);
                else /* first bead of labels[l] minus last bead of l */
                    d_ext[a] = sep(s, xl, x_first_bead + (long)labels[l] * D, a);
                weight += d_ext[a] * d_ext[a];
            }
            for (int a = 0; a < D; ++a) d_int[a] = sep(s, xl, (first ? x_next : x_prev) + (long)l * D, a);
            for (int a = 0; a < D; ++a) {
                /* sums += diff_prev + diff_next, each in the reference's roles */
                sums[a] += first ? d_ext[a] + d_int[a] : d_int[a] + d_ext[a];
                temp[(long)l * D + a] = sums[a] * k;
            }
        }
        weight = exp(-beta * (0.5 * k * weight - e_shift));
        for (long i = 0; i < (long)N * D; ++i) f[i] += weight * temp[i];
        denom_weight += weight;
    } while (orc_next_permutation(labels, N));
    for (long i = 0; i < (long)N * D; ++i) f[i] = f[i] / denom_weight;
    free(labels);
    free(temp);
}

/* primEstimator (:259-293) */
static double orc_factorial_prim(const orc_system* s, const double* x_first, const double* x_last, double e_shift) {
    const int N = s->natoms, D = s->ndim;
    const double k = s->spring_constant, beta = s->beta_ex;
    int* labels = (int*)malloc(sizeof(int) * (size_t)N * 2);
    int* inv = labels + N;
    for (int l = 0; l < N; ++l) labels[l] = l;
    double numerator = 0.0, denom_weight = 0.0;
    do {
        orc_inverse(labels, N, inv);
        double weight = 0.0;
        for (int l = 0; l < N; ++l) weight += sepsq(s, x_first + (long)l * D, x_last + (long)inv[l] * D);
        const double delta = 0.5 * k * weight;
        weight = exp(-beta * (delta - e_shift));
        numerator += delta * weight;
        denom_weight += weight;
    } while (orc_next_permutation(labels, N));
    free(labels);
    double e = numerator / denom_weight;
    e /= s->nbeads; /* IPI_CONVENTION */
    return (-1.0) * e;
}

int orc_factorial_exchange(const orc_system* s, const double* x_all, double* f1, double* fP, double* scalars) {
    const int N = s->natoms, D = s->ndim, P = s->nbeads;
    const long bead = (long)N * D;
    const double* x1 = x_all;
    const double* xP = x_all + (long)(P - 1) * bead;
    /* prepare() (:19-21): the shift of the weights, from beads 1 and P */
    const double e_shift = orc_factorial_min_energy(s, x1, xP);
    if (fP) orc_factorial_force(s, 0, xP, x_all + (long)(P - 2) * bead, x1, e_shift, fP);
    if (f1) orc_factorial_force(s, 1, x1, xP, x_all + (long)(P > 1 ? 1 : 0) * bead, e_shift, f1);
    if (scalars) {
        scalars[0] = orc_factorial_potential(s, x1, xP);
        scalars[1] = orc_factorial_prim(s, x1, xP, e_shift);
        scalars[2] = 0.0; /* getDistinctProbability (:237-240): not implemented there */
        scalars[3] = 0.0; /* getLongestProbability (:249-252) */
    }
    return isfinite(e_shift) ? 0 : 2;
}

int orc_exchange(const orc_system* s, const double* x_all, double* f1, double* fP, double* scalars, double* E_out,
                 double* V_out, double* Vb_out, double* prob_out) {
    const int N = s->natoms, D = s->ndim, P = s->nbeads;
    const long bead = (long)N * D;
    const double* x1 = x_all;
    const double* xP = x_all + (long)(P - 1) * bead;
    if (s->factorial) return orc_factorial_exchange(s, x_all, f1, fP, scalars);
    double* E = (double*)malloc(sizeof(double) * (size_t)((long)N * (N + 1) / 2 + 1));
    double* V = (double*)malloc(sizeof(double) * (size_t)(N + 1));
    double* Vb = (double*)malloc(sizeof(double) * (size_t)(N + 1));
    double* prob = (double*)malloc(sizeof(double) * (size_t)N * (size_t)N);
    orc_cycle_energies(s, x1, xP, E);
    int st = orc_vb_forward(s, E, V);
    st |= orc_vb_backward(s, E, V, Vb);
    orc_connection_probabilities(s, E, V, Vb, prob);
    if (fP) orc_spring_force_last_bead(s, prob, xP, x_all + (long)(P - 2) * bead, x1, fP);
    if (f1) orc_spring_force_first_bead(s, prob, x1, xP, x_all + (long)(P > 1 ? 1 : 0) * bead, f1);
    if (scalars) {
        scalars[0] = V[N];
        scalars[1] = orc_prim_estimator(s, E, V);
        scalars[2] = orc_distinct_probability(s, E, V);
        scalars[3] = orc_longest_probability(s, E, V);
    }
    if (E_out) memcpy(E_out, E, sizeof(double) * (size_t)((long)N * (N + 1) / 2));
    if (V_out) memcpy(V_out, V, sizeof(double) * (size_t)(N + 1));
    if (Vb_out) memcpy(Vb_out, Vb, sizeof(double) * (size_t)(N + 1));
    if (prob_out) memcpy(prob_out, prob, sizeof(double) * (size_t)N * (size_t)N);
    free(E);
    free(V);
    free(Vb);
    free(prob);
    return st;
}

/* ------------------------------------------------------------------------ */
/* forces on every bead (simulation.cpp:353-455)                              */

void orc_spring_forces_interior(const orc_system* s, const double* x_prev, const double* x, const double* x_next,
                                double* f) {
    /* simulation.cpp:405-419 */
    const int n = s->natoms * s->ndim;
    for (int i = 0; i < n; ++i) {
        double dp = x_prev[i] - x[i];
        double dn = x_next[i] - x[i];
        if (s->pbc) {
            dp = orc_min_image(dp, s->size);
            dn = orc_min_image(dn, s->size);
        }
        f[i] = s->spring_constant * (dp + dn);
    }
}

void orc_physical_forces(const orc_system* s, const double* x, double* f) {
    /* simulation.cpp:428-455 */
    const int N = s->natoms, D = s->ndim;
    orc_ext_grad(s, x, N, f);
    for (int i = 0; i < N * D; ++i) f[i] = f[i] * (-1.0);
    if (s->cutoff != 0.0) {
        double r[3], g[3];
        for (int i = 0; i < N; ++i) {
            for (int j = i + 1; j < N; ++j) {
                for (int a = 0; a < D; ++a) {
                    double d = x[(long)i * D + a] - x[(long)j * D + a]; /* simulation.cpp:499-512 */
                    if (s->pbc) d = orc_min_image(d, s->size);
                    r[a] = d;
                }
                const double dist = vnorm(r, D);
                if (dist < s->cutoff || s->cutoff < 0.0) {
                    orc_pair_grad(s, r, g);
                    for (int a = 0; a < D; ++a) {
                        const double fo = g[a] * (-1.0);
                        f[(long)i * D + a] += fo;
                        f[(long)j * D + a] -= fo;
                    }
                }
            }
        }
    }
}

/* Potential energy of the ring polymer, the function whose negative gradient
 * orc_update_forces returns: terms[0] external V over beads (the potentials'
 * V(), src/potentials/[*].cpp), terms[1] pair V over beads (each pair once,
 * cutoff and minimum image as simulation.cpp:428-455), terms[2] the springs
 * outside the exchange (classicalSpringEnergy, simulation.cpp:464-486: every
 * link when distinguishable, the interior links when bosonic), terms[3]
 * V_B (effectivePotential, quadratic_bosonic_exchange.cpp:130-132). */
int orc_potential_energy(const orc_system* s, const double* x_all, double* terms) {
    const int N = s->natoms, D = s->ndim, P = s->nbeads;
    const long bead = (long)N * D;
    const int bosonic = s->bosonic && P > 1;
    terms[0] = terms[1] = terms[2] = terms[3] = 0.0;
    for (int b = 0; b < P; ++b) {
        const double* x = x_all + (long)b * bead;
        terms[0] += orc_ext_value(s, x, N);
        if (s->cutoff != 0.0) {
            double r[3];
            for (int i = 0; i < N; ++i)
                for (int j = i + 1; j < N; ++j) {
                    for (int a = 0; a < D; ++a) {
                        double d = x[(long)i * D + a] - x[(long)j * D + a];
                        if (s->pbc) d = orc_min_image(d, s->size);
                        r[a] = d;
                    }
                    const double dist = vnorm(r, D);
                    if (dist < s->cutoff || s->cutoff < 0.0) terms[1] += orc_pair_value(s, r);
                }
        }
        if (P > 1 && (!bosonic || b > 0)) {
            const double* xp = x_all + (long)((b - 1 + P) % P) * bead;
            double e = 0.0;
            for (long k = 0; k < bead; ++k) {
                double diff = xp[k] - x[k];
                if (s->pbc) diff = orc_min_image(diff, s->size);
                e += diff * diff;
            }
            terms[2] += e * (0.5 * s->spring_constant);
        }
    }
    if (bosonic) {
        double sc[4];
        const int st = orc_exchange(s, x_all, NULL, NULL, sc, NULL, NULL, NULL, NULL);
        terms[3] = sc[0];
        return st;
    }
    return 0;
}

/* Observables of one state (src/observables/{energy,classical,bosonic,
 * gsf_action}.cpp), each bead's value as the reference computes it on that
 * bead's rank, summed over beads as ObservablesLogger::log does
 * (observable.cpp:82-116).  Atomic units, except temperature in kelvin as
 * classical.cpp:60 always reports it:
 *   out[0] kinetic (primitive)  out[1] potential  out[2] ext_pot
 *   out[3] int_pot              out[4] virial     out[5] temperature
 *   out[6] cl_kinetic           out[7] cl_spring  out[8] prob_dist
 *   out[9] prob_all             out[10] w_gsf     out[11] pot_gsf
 * The GSF force term uses the total gradient on each particle; the
 * reference's gsf_action.cpp:34 adds a one-vector array to an N-vector one,
 * which reads past the end of the smaller array when N > 1 and an
 * interaction is present. */
int orc_observables(const orc_system* s, const double* x_all, const double* p_all, double* out) {
    const int N = s->natoms, D = s->ndim, P = s->nbeads;
    const long bead = (long)N * D;
    const int bosonic = s->bosonic && P > 1;
    double sc[4] = {0.0, 0.0, 0.0, 0.0};
    int st = 0;
    if (bosonic) st = orc_exchange(s, x_all, NULL, NULL, sc, NULL, NULL, NULL, NULL);
    for (int k = 0; k < 12; ++k) out[k] = 0.0;
    double* g = (double*)malloc(sizeof(double) * (size_t)bead);
    double* fe = (double*)malloc(sizeof(double) * (size_t)bead);
    for (int b = 0; b < P; ++b) {
        const double* x = x_all + (long)b * bead;
        const double* p = p_all + (long)b * bead;
        const double* xp = x_all + (long)((b - 1 + P) % P) * bead;
        /* classicalSpringEnergy (simulation.cpp:464-486) */
        double spring = 0.0;
        for (long k = 0; k < bead; ++k) {
            double diff = xp[k] - x[k];
            if (s->pbc) diff = orc_min_image(diff, s->size);
            spring += diff * diff;
        }
        spring *= 0.5 * s->spring_constant;
        /* energy.cpp:30-51 */
        double kinetic = 0.5 * D * N / s->beta;
        if (b == 0 && bosonic) kinetic += sc[1];
        else kinetic -= spring / P;
        /* energy.cpp:59-110 */
        double ext = 0.0, inter = 0.0, virial = 0.0;
        ext = orc_ext_value(s, x, N);
        orc_ext_grad(s, x, N, fe);
        for (long k = 0; k < bead; ++k) {
            g[k] = fe[k];
            virial -= x[k] * (-fe[k]);
        }
        if (s->cutoff != 0.0) {
            double r[3], gr[3];
            for (int i = 0; i < N; ++i)
                for (int j = i + 1; j < N; ++j) {
                    for (int a = 0; a < D; ++a) {
                        double d = x[(long)i * D + a] - x[(long)j * D + a];
                        if (s->pbc) d = orc_min_image(d, s->size);
                        r[a] = d;
                    }
                    const double dist = vnorm(r, D);
                    if (dist < s->cutoff || s->cutoff < 0.0) {
                        orc_pair_grad(s, r, gr);
                        const double v = orc_pair_value(s, r);
                        inter += v;
                        for (int a = 0; a < D; ++a) {
                            virial -= x[(long)i * D + a] * (-gr[a]);
                            g[(long)i * D + a] += gr[a];
                            g[(long)j * D + a] -= gr[a];
                        }
                    }
                }
        }
        out[1] += (ext + inter) / P;
        out[2] += ext / P;
        out[3] += inter / P;
        out[4] += virial * (0.5 / P);
        out[0] += kinetic;
        /* classical.cpp:32-78 */
        double ke = 0.0;
        for (long k = 0; k < bead; ++k) ke += p[k] * p[k];
        ke *= 0.5 / s->mass;
        const double dof = (double)D * N * P;
        out[5] += 2.0 * ke / (dof * 1.0) / P / 3.1668152e-06; /* units.h: kelvin */
        out[6] += ke;
        out[7] += (b == 0 && bosonic) ? sc[0] : spring;
        /* bosonic.cpp:17-22 */
        if (b == 0 && bosonic) {
            out[8] += sc[2];
            out[9] += sc[3];
        }
        /* gsf_action.cpp:21-73 (alpha = 0) */
        double f2 = 0.0;
        for (long k = 0; k < bead; ++k) f2 += g[k] * g[k];
        const double sp = s->spring_constant / P;
        const double pot_term = (ext + inter) / (3 * P);
        const double f2_term = f2 / (9 * sp * P * P);
        double w = (b % 2 != 0) ? -pot_term : pot_term + f2_term;
        out[10] += w * (-s->beta);
        if (b % 2 != 0) out[11] += (ext + inter) / (0.5 * P);
    }
    free(g);
    free(fe);
    return st;
}

/* ---- a tiny parallel-for over POSIX threads ---- */
typedef void (*orc_body)(void* ctx, int i);
typedef struct {
    orc_body fn;
    void* ctx;
    int begin, end, step;
} orc_chunk;

static void* orc_chunk_run(void* arg) {
    orc_chunk* c = (orc_chunk*)arg;
    for (int i = c->begin; i < c->end; i += c->step) c->fn(c->ctx, i);
    return NULL;
}

static void orc_parallel_for(int nthreads, int n, orc_body fn, void* ctx) {
    if (nthreads <= 1 || n <= 1) {
        for (int i = 0; i < n; ++i) fn(ctx, i);
        return;
    }
    if (nthreads > n) nthreads = n;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    orc_chunk ch[256];
    for (int t = 0; t < nthreads; ++t) {
        ch[t].fn = fn;
        ch[t].ctx = ctx;
        ch[t].begin = t;
        ch[t].end = n;
        ch[t].step = nthreads;
        if (t > 0) pthread_create(&th[t], NULL, orc_chunk_run, &ch[t]);
    }
    orc_chunk_run(&ch[0]);
    for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
}

typedef struct {
    const orc_system* s;
    const double* x;
    double* f;
    double* spring;
    double* phys;
    const double* exch1;
    const double* exchP;
} orc_force_ctx;

static void orc_force_bead(void* vctx, int b) {
    orc_force_ctx* c = (orc_force_ctx*)vctx;
    const orc_system* s = c->s;
    const int P = s->nbeads;
    const long nb = (long)s->natoms * s->ndim;
    double* sp = c->spring + b * nb;
    double* ph = c->phys + b * nb;
    if (s->bosonic && (b == 0 || b == P - 1)) {
        memcpy(sp, b == 0 ? c->exch1 : c->exchP, sizeof(double) * (size_t)nb);
    } else {
        const int bp = (b - 1 + P) % P, bn = (b + 1) % P;
        orc_spring_forces_interior(s, c->x + bp * nb, c->x + b * nb, c->x + bn * nb, sp);
    }
    orc_physical_forces(s, c->x + b * nb, ph);
    for (long i = 0; i < nb; ++i) c->f[b * nb + i] = sp[i] + ph[i]; /* simulation.cpp:363-373 */
}

int orc_update_forces(const orc_system* s, const double* x_all, double* f_all, double* spring_out, double* phys_out,
                      int nthreads) {
    const int P = s->nbeads;
    const long nb = (long)s->natoms * s->ndim;
    double* spring = spring_out ? spring_out : (double*)malloc(sizeof(double) * (size_t)(P * nb));
    double* phys = phys_out ? phys_out : (double*)malloc(sizeof(double) * (size_t)(P * nb));
    double* e1 = NULL;
    double* eP = NULL;
    int st = 0;
    if (s->bosonic) {
        /* BosonicExchange::prepare + exteriorSpringForce, simulation.cpp:395-400.
         * Ranks 0 and P-1 evaluate the same recursion; it is evaluated once here. */
        e1 = (double*)malloc(sizeof(double) * (size_t)nb);
        eP = (double*)malloc(sizeof(double) * (size_t)nb);
        st = orc_exchange(s, x_all, e1, eP, NULL, NULL, NULL, NULL, NULL);
    }
    orc_force_ctx c = {s, x_all, f_all, spring, phys, e1, eP};
    orc_parallel_for(nthreads, P, orc_force_bead, &c);
    free(e1);
    free(eP);
    if (!spring_out) free(spring);
    if (!phys_out) free(phys);
    return st;
}

/* ------------------------------------------------------------------------ */
/* integrator                                                                 */

void orc_zero_momentum(const orc_system* s, double* p) {
    /* simulation.cpp:581-603; the MPI_Allreduce sums bead contributions in
     * rank order */
    const int N = s->natoms, D = s->ndim, P = s->nbeads;
    double cm[3] = {0.0, 0.0, 0.0};
    for (int b = 0; b < P; ++b) {
        double per[3] = {0.0, 0.0, 0.0};
        for (int i = 0; i < N; ++i)
            for (int a = 0; a < D; ++a) per[a] += p[((long)b * N + i) * D + a];
        for (int a = 0; a < D; ++a) per[a] /= (N * P);
        for (int a = 0; a < D; ++a) cm[a] += per[a];
    }
    for (long i = 0; i < (long)P * N; ++i)
        for (int a = 0; a < D; ++a) p[i * D + a] -= cm[a];
}

static double langevin_c1(const orc_system* s) { return exp(-0.5 * s->gamma * s->dt); } /* langevin.cpp:11 */
static double langevin_c2(const orc_system* s) {                                   /* langevin.cpp:12 */
    const double c1 = langevin_c1(s);
    return sqrt((1 - c1 * c1) * s->mass / s->thermo_beta);
}

void orc_langevin(const orc_system* s, double* p, const double* xi) {
    /* langevin.cpp:15-27 with CartesianCoupling (thermostat_coupling.cpp:11-25) */
    const double c1 = langevin_c1(s), c2 = langevin_c2(s);
    const long n = (long)s->natoms * s->ndim * s->nbeads;
    for (long i = 0; i < n; ++i) p[i] = c1 * p[i] + c2 * xi[i];
}

void orc_nm_matrices(const orc_system* s, double* c2nm, double* nm2c) {
    /* normal_modes.cpp:48-79: row k of cart_to_nm is rank k's row; row j of
     * nm_to_cart is rank j's row */
    const int P = s->nbeads;
    for (int k = 0; k < P; ++k) {
        double* row = c2nm + (long)k * P;
        const double fund = 2 * ORC_PI / P * k;
        double pref;
        if (k == 0) {
            pref = 1 / sqrt(P);
            for (int i = 0; i < P; ++i) row[i] = pref;
        } else if (k < 0.5 * P) {
            pref = sqrt(2.0 / P);
            for (int i = 0; i < P; ++i) row[i] = pref * cos(fund * i);
        } else if (k == 0.5 * P) {
            pref = 1 / sqrt(P);
            for (int i = 0; i < P; ++i) row[i] = pref * (i % 2 == 0 ? 1.0 : -1.0);
        } else {
            pref = sqrt(2.0 / P);
            for (int i = 0; i < P; ++i) row[i] = -pref * sin(fund * i);
        }
    }
    for (int j = 0; j < P; ++j) {
        double* row = nm2c + (long)j * P;
        const double fund = 2 * ORC_PI / P * j;
        const double pref = sqrt(2.0 / P);
        for (int i = 0; i < P; ++i) row[i] = 0.0;
        row[0] = 1 / sqrt(P);
        for (int i = 1; i < 0.5 * P; ++i) row[i] = pref * cos(fund * i);
        if (P % 2 == 0) row[P / 2] = 1 / sqrt(P) * (j % 2 == 0 ? 1.0 : -1.0);
        for (int i = (int)ceil(0.5 * (P + 1)); i < P; ++i) row[i] = -pref * sin(fund * i);
    }
}

/* y[j][dof] = sum_k M[j][k] v[k][dof] in the reference's loop order (k
 * ascending, accumulator starting at 0). */
static void orc_bead_transform(const orc_system* s, const double* M, const double* v, double* y) {
    const int P = s->nbeads;
    const long nb = (long)s->natoms * s->ndim;
    for (int j = 0; j < P; ++j)
        for (long d = 0; d < nb; ++d) {
            double acc = 0;
            for (int k = 0; k < P; ++k) acc += M[(long)j * P + k] * v[(long)k * nb + d];
            y[(long)j * nb + d] = acc;
        }
}

/* ---- Nose-Hoover chains (src/thermostats/nose_hoover.cpp) ---- */
long orc_nh_chains(const orc_system* s) {
    const long P = s->nbeads, N = s->natoms, D = s->ndim;
    switch (s->thermostat) {
    case ORC_THERMO_NOSE_HOOVER: return P;
    case ORC_THERMO_NOSE_HOOVER_NP: return P * N;
    case ORC_THERMO_NOSE_HOOVER_NP_DIM: return P * N * D;
    default: return 0;
    }
}

typedef struct {
    double Q1, Qi, required, dt2, dt4, dt8;
    int nchains;
} orc_nh_par;

static orc_nh_par nh_par(const orc_system* s) {
    /* constructors, nose_hoover.cpp:9-33, :149-158, :196-206 */
    orc_nh_par q;
    const int N = s->natoms, D = s->ndim;
    q.nchains = s->nchains;
    q.Qi = 1.0 * 1.0 * s->beta / s->nbeads;
    if (s->thermostat == ORC_THERMO_NOSE_HOOVER) {
        q.Q1 = D * N * q.Qi;
        q.required = D * N / s->thermo_beta;
    } else if (s->thermostat == ORC_THERMO_NOSE_HOOVER_NP) {
        q.Q1 = D * q.Qi;
        q.required = D / s->thermo_beta;
    } else {
        q.Q1 = q.Qi;
        q.required = 1 / s->thermo_beta;
    }
    q.dt2 = 0.5 * s->dt;
    q.dt4 = 0.25 * s->dt;
    q.dt8 = 0.125 * s->dt;
    return q;
}

/* singleChainStep (nose_hoover.cpp:98-144) on one chain; returns the scale */
static double nh_chain_step(const orc_system* s, const orc_nh_par* q, double current_energy, double* eta,
                            double* eta_dot, double* eta_dd) {
    const int M = q->nchains;
    double exp_factor = 0.0;
    eta_dd[0] = (current_energy - q->required) / q->Q1;
    eta_dot[M - 1] += eta_dd[M - 1] * q->dt4;
    for (int i = M - 2; i >= 0; i--) {
        exp_factor = exp(-q->dt8 * eta_dot[i + 1]);
        eta_dot[i] *= exp_factor;
        eta_dot[i] += eta_dd[i] * q->dt4;
        eta_dot[i] *= exp_factor;
    }
    double scale = exp(-q->dt2 * eta_dot[0]);
    for (int i = 0; i < M; i++) eta[i] += q->dt2 * eta_dot[i];
    eta_dd[0] = (current_energy * scale * scale - q->required) / q->Q1;
    eta_dot[0] *= exp_factor;
    eta_dot[0] += eta_dd[0] * q->dt4;
    eta_dot[0] *= exp_factor;
    double Q_former = q->Q1;
    for (int i = 1; i < M - 1; i++) {
        exp_factor = exp(-q->dt8 * eta_dot[i + 1]);
        eta_dot[i] *= exp_factor;
        eta_dd[i] = (Q_former * eta_dot[i - 1] * eta_dot[i - 1] - 1 / s->thermo_beta) / q->Qi;
        eta_dot[i] += eta_dd[i] * q->dt4;
        eta_dot[i] *= exp_factor;
        Q_former = q->Qi;
    }
    eta_dd[M - 1] = (q->Qi * eta_dot[M - 2] * eta_dot[M - 2] - 1 / s->thermo_beta) / q->Qi;
    eta_dot[M - 1] += eta_dd[M - 1] * q->dt4;
    return scale;
}

/* momentaUpdate of the three variants (nose_hoover.cpp:68-96, :160-184,
 * :208-221) on every bead (or normal mode) of `p`. */
static void orc_nose_hoover(const orc_system* s, double* p, double* nh) {
    const int N = s->natoms, D = s->ndim, P = s->nbeads, M = s->nchains;
    const orc_nh_par q = nh_par(s);
    const long nch = orc_nh_chains(s);
    double* eta = nh;
    double* eta_dot = nh + nch * M;
    double* eta_dd = nh + 2 * nch * M;
    for (int b = 0; b < P; ++b) {
        double* pb = p + (long)b * N * D;
        if (s->thermostat == ORC_THERMO_NOSE_HOOVER) {
            double e = 0.0;
            for (int i = 0; i < N; ++i)
                for (int a = 0; a < D; ++a) e += pb[i * D + a] * pb[i * D + a];
            e /= s->mass;
            const long c = (long)b * M;
            const double scale = nh_chain_step(s, &q, e, eta + c, eta_dot + c, eta_dd + c);
            for (int i = 0; i < N; ++i)
                for (int a = 0; a < D; ++a) pb[i * D + a] = pb[i * D + a] * scale;
        } else if (s->thermostat == ORC_THERMO_NOSE_HOOVER_NP) {
            for (int i = 0; i < N; ++i) {
                double e = 0.0;
                for (int a = 0; a < D; ++a) e += pb[i * D + a] * pb[i * D + a];
                e /= s->mass;
                const long c = ((long)b * N + i) * M;
                const double scale = nh_chain_step(s, &q, e, eta + c, eta_dot + c, eta_dd + c);
                for (int a = 0; a < D; ++a) pb[i * D + a] = pb[i * D + a] * scale;
            }
        } else {
            for (int i = 0; i < N; ++i)
                for (int a = 0; a < D; ++a) {
                    const double e = pb[i * D + a] * pb[i * D + a] / s->mass;
                    const long c = (((long)b * N + i) * D + a) * M;
                    const double scale = nh_chain_step(s, &q, e, eta + c, eta_dot + c, eta_dd + c);
                    pb[i * D + a] = pb[i * D + a] * scale;
                }
        }
    }
}

double orc_nh_energy(const orc_system* s, const double* nh) {
    const long nch = orc_nh_chains(s);
    if (!nch || !nh) return 0.0;
    const int M = s->nchains;
    const orc_nh_par q = nh_par(s);
    const double* eta = nh;
    const double* eta_dot = nh + nch * M;
    const int ndof = s->thermostat == ORC_THERMO_NOSE_HOOVER ? s->ndim * s->natoms
                     : s->thermostat == ORC_THERMO_NOSE_HOOVER_NP ? s->ndim : 1;
    double total = 0.0;
    for (long c = 0; c < nch; ++c) {
        const double* e = eta + c * M;
        const double* ed = eta_dot + c * M;
        /* singleChainGetAdditionToH (nose_hoover.cpp:51-66) */
        double h = 0.5 * q.Q1 * ed[0] * ed[0];
        h += ndof * e[0] / s->thermo_beta;
        for (int i = 1; i < M; i++) {
            h += 0.5 * q.Qi * ed[i] * ed[i];
            h += e[i] / s->thermo_beta;
        }
        total += h;
    }
    return total;
}

static void orc_thermostat_step(const orc_system* s, double* p, const double* xi, const double* c2nm,
                                const double* nm2c, double* work, double* nh) {
    /* thermostat.cpp:15-19 */
    if (orc_nh_chains(s)) {
        if (!s->nmthermostat) {
            orc_nose_hoover(s, p, nh);
            return;
        }
        /* NMCoupling (thermostat_coupling.cpp:29-47): chains per normal mode */
        orc_bead_transform(s, c2nm, p, work);
        orc_nose_hoover(s, work, nh);
        orc_bead_transform(s, nm2c, work, p);
        return;
    }
    if (s->thermostat != ORC_THERMO_LANGEVIN) return;
    if (!s->nmthermostat) {
        orc_langevin(s, p, xi);
        return;
    }
    /* NMCoupling (thermostat_coupling.cpp:29-47): p_nm = C p; Langevin on
     * p_nm; p = C^T p_nm (normal_modes.cpp:131-139) */
    const double c1 = langevin_c1(s), c2 = langevin_c2(s);
    const long n = (long)s->natoms * s->ndim * s->nbeads;
    orc_bead_transform(s, c2nm, p, work);
    for (long i = 0; i < n; ++i) work[i] = c1 * work[i] + c2 * xi[i];
    orc_bead_transform(s, nm2c, work, p);
}

static void orc_momentum_step(const orc_system* s, double* p, const double* f) {
    /* velocity_verlet.cpp:24-30 */
    const long n = (long)s->natoms * s->ndim * s->nbeads;
    for (long i = 0; i < n; ++i) p[i] += 0.5 * s->dt * f[i];
}

static void orc_coords_step(const orc_system* s, double* x, const double* p) {
    /* velocity_verlet.cpp:32-38 */
    const long n = (long)s->natoms * s->ndim * s->nbeads;
    for (long i = 0; i < n; ++i) x[i] += s->dt * p[i] / s->mass;
}

static void orc_nm_external_kick(const orc_system* s, orc_state* st) {
    /* normal_modes_propagator.cpp:73-103 */
    const int N = s->natoms, D = s->ndim, P = s->nbeads;
    const long nb = (long)N * D;
    for (int b = 0; b < P; ++b) {
        double* p = st->p + b * nb;
        const double* ef = st->ext_f + b * nb;
        if (s->bosonic && (b == 0 || b == P - 1)) {
            const double* x = st->x + b * nb;
            const double* xp = st->x + (long)((b - 1 + P) % P) * nb;
            const double* xn = st->x + (long)((b + 1) % P) * nb;
            const double* sf = st->spring_f + b * nb;
            for (long i = 0; i < nb; ++i) {
                const double inner = -s->spring_constant * (2 * x[i] - xp[i] - xn[i]);
                p[i] += 0.5 * s->dt * (ef[i] + sf[i] - inner);
            }
        } else {
            for (long i = 0; i < nb; ++i) p[i] += 0.5 * s->dt * ef[i];
        }
    }
}

static int orc_nm_propagate(const orc_system* s, orc_state* st, const double* c2nm, const double* nm2c,
                            double* w1, double* w2, int nthreads) {
    /* normal_modes_propagator.cpp:19-71 */
    const int P = s->nbeads;
    const long nb = (long)s->natoms * s->ndim;
    orc_nm_external_kick(s, st);
    orc_bead_transform(s, c2nm, st->x, w1);
    orc_bead_transform(s, c2nm, st->p, w2);
    for (int k = 0; k < P; ++k) {
        const double freq = 2 * s->omega_p * sin(k * ORC_PI / P); /* :13-16 */
        const double c = cos(freq * s->dt), sn = sin(freq * s->dt), mw = s->mass * freq;
        for (long d = 0; d < nb; ++d) {
            const double q = w1[k * nb + d], pm = w2[k * nb + d];
            if (freq == 0) {
                w1[k * nb + d] = q + s->dt / s->mass * pm;
                w2[k * nb + d] = pm;
            } else {
                w1[k * nb + d] = c * q + sn / mw * pm;
                w2[k * nb + d] = (-1) * mw * sn * q + c * pm;
            }
        }
    }
    orc_bead_transform(s, nm2c, w1, st->x);
    orc_bead_transform(s, nm2c, w2, st->p);
    /* :64-67: updateForces, then the physical and spring forces are stored */
    int rc = orc_update_forces(s, st->x, st->f, st->spring_f, st->ext_f, nthreads);
    orc_nm_external_kick(s, st);
    return rc;
}

int orc_md_step(const orc_system* s, orc_state* st, const double* xi, int nthreads) {
    /* simulation.cpp:236-260 */
    const int P = s->nbeads;
    const long n = (long)s->natoms * s->ndim * P;
    double* c2nm = NULL;
    double* nm2c = NULL;
    double* w1 = (double*)malloc(sizeof(double) * (size_t)n);
    double* w2 = (double*)malloc(sizeof(double) * (size_t)n);
    if (s->nmthermostat || s->propagator == ORC_PROP_NORMAL_MODES) {
        c2nm = (double*)malloc(sizeof(double) * (size_t)P * P);
        nm2c = (double*)malloc(sizeof(double) * (size_t)P * P);
        orc_nm_matrices(s, c2nm, nm2c);
    }
    int rc = 0;
    orc_thermostat_step(s, st->p, xi, c2nm, nm2c, w1, st->nh);
    if (s->fixcom) orc_zero_momentum(s, st->p);
    if (s->propagator == ORC_PROP_NORMAL_MODES) {
        rc = orc_nm_propagate(s, st, c2nm, nm2c, w1, w2, nthreads);
    } else {
        orc_momentum_step(s, st->p, st->f);
        orc_coords_step(s, st->x, st->p);
        rc = orc_update_forces(s, st->x, st->f, NULL, NULL, nthreads);
        orc_momentum_step(s, st->p, st->f);
    }
    orc_thermostat_step(s, st->p, xi + n, c2nm, nm2c, w1, st->nh);
    if (s->fixcom) orc_zero_momentum(s, st->p);
    free(w1);
    free(w2);
    free(c2nm);
    free(nm2c);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* noise                                                                      */

static inline void philox_round(uint32_t* c, const uint32_t* k) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c[1] ^ k[0];
    const uint32_t n2 = hi0 ^ c[3] ^ k[1];
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
}

static void philox4x32_10(uint32_t* c, uint64_t seed) {
    uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k[0] += 0x9E3779B9u;
            k[1] += 0xBB67AE85u;
        }
        philox_round(c, k);
    }
}

/* Box-Muller on FP32 with its own log, sin and cos from their series,
 * correctly rounded operations only (fmaf, no contraction): the GPU's
 * bm_log / bm_sincos_2pi / philox_normal_pair_f32 in the same order, so both
 * draw bit-identical numbers.  log u = e ln2 + 2 atanh((m-1)/(m+1)) to s^9;
 * sin to phi^13 and cos to phi^14 on a quadrant. */
static float bm_log(float u) {
    uint32_t bits;
    memcpy(&bits, &u, sizeof bits);
    int e = (int)((bits >> 23) & 0xffu) - 127;
    const uint32_t mb = (bits & 0x7fffffu) | 0x3f800000u;
    float m;
    memcpy(&m, &mb, sizeof m);
    if (m > 1.41421354f) {
        m = m * 0.5f;
        e += 1;
    }
    const float sv = (m - 1.0f) / (m + 1.0f);
    const float s2 = sv * sv;
    float q = fmaf(0.111111112f, s2, 0.142857149f);
    q = fmaf(q, s2, 0.2f);
    q = fmaf(q, s2, 0.333333343f);
    q = fmaf(q, s2, 1.0f);
    const float lm = (2.0f * sv) * q;
    const float ef = (float)e;
    return fmaf(ef, 0.693145752f, fmaf(ef, 1.42860677e-06f, lm));
}

static void bm_sincos_2pi(uint32_t w, float* sn, float* cs) {
    const uint32_t quad = w >> 30;
    const float ph = ((float)((w >> 6) & 0xffffffu) * 5.96046448e-08f) * 1.57079637f;
    const float p2 = ph * ph;
    float sp = fmaf(1.60590444e-10f, p2, -2.50521079e-08f);
    sp = fmaf(sp, p2, 2.75573188e-06f);
    sp = fmaf(sp, p2, -1.98412701e-04f);
    sp = fmaf(sp, p2, 8.33333377e-03f);
    sp = fmaf(sp, p2, -0.166666672f);
    sp = fmaf(sp * p2, ph, ph);
    float cp = fmaf(-1.14707454e-11f, p2, 2.08767559e-09f);
    cp = fmaf(cp, p2, -2.75573188e-07f);
    cp = fmaf(cp, p2, 2.48015876e-05f);
    cp = fmaf(cp, p2, -1.38888892e-03f);
    cp = fmaf(cp, p2, 4.16666679e-02f);
    cp = fmaf(cp, p2, -0.5f);
    cp = fmaf(cp, p2, 1.0f);
    const float a = (quad & 1u) ? cp : sp, b = (quad & 1u) ? sp : cp;
    *sn = (quad & 2u) ? -a : a;
    *cs = ((quad + 1u) & 2u) ? -b : b;
}

void orc_philox_normals(uint64_t seed, uint32_t replica, uint64_t step, int substep, int64_t ndof, double* out) {
    const uint64_t t = 2 * step + (uint64_t)substep;
    for (int64_t pair = 0; 2 * pair < ndof; ++pair) {
        uint32_t c[4] = {(uint32_t)pair, replica, (uint32_t)t, (uint32_t)(t >> 32)};
        philox4x32_10(c, seed);
        const float u1 = (float)((c[0] >> 8) + 1u) * 5.96046448e-08f; /* exact */
        const float r = sqrtf(-2.0f * bm_log(u1));
        float sn, cs;
        bm_sincos_2pi(c[2], &sn, &cs);
        out[2 * pair] = (double)(r * cs);
        if (2 * pair + 1 < ndof) out[2 * pair + 1] = (double)(r * sn);
    }
}

struct orc_ranmars {
    double u[98];
    double c, cd, cm;
    int i97, j97;
    int save;
    double second;
};

orc_ranmars* orc_ranmars_new(int seed) {
    if (seed <= 0 || seed > 900000000) return NULL;
    orc_ranmars* r = (orc_ranmars*)calloc(1, sizeof(orc_ranmars));
    /* RANMAR initialisation: two seeds (ij, kl) drive a 3-lag multiplicative
     * generator mod 179 and a linear congruential generator mod 169; 24 bits
     * of their combination fill each of the 97 lagged-Fibonacci seeds. */
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
        r->u[n] = acc;
    }
    r->c = 362436.0 / 16777216.0;
    r->cd = 7654321.0 / 16777216.0;
    r->cm = 16777213.0 / 16777216.0;
    r->i97 = 97;
    r->j97 = 33;
    orc_ranmars_uniform(r);
    return r;
}

void orc_ranmars_free(orc_ranmars* r) { free(r); }

double orc_ranmars_uniform(orc_ranmars* r) {
    /* lagged Fibonacci difference (lags 97, 33) combined with an arithmetic
     * sequence mod cm */
    double uni = r->u[r->i97] - r->u[r->j97];
    if (uni < 0.0) uni += 1.0;
    r->u[r->i97] = uni;
    if (--r->i97 == 0) r->i97 = 97;
    if (--r->j97 == 0) r->j97 = 97;
    r->c -= r->cd;
    if (r->c < 0.0) r->c += r->cm;
    uni -= r->c;
    if (uni < 0.0) uni += 1.0;
    return uni;
}

double orc_ranmars_gaussian(orc_ranmars* r) {
    /* Marsaglia polar method; the second variate of each pair is cached */
    if (r->save) {
        r->save = 0;
        return r->second;
    }
    double v1, v2, rsq;
    do {
        v1 = 2.0 * orc_ranmars_uniform(r) - 1.0;
        v2 = 2.0 * orc_ranmars_uniform(r) - 1.0;
        rsq = v1 * v1 + v2 * v2;
    } while (rsq >= 1.0 || rsq == 0.0);
    const double fac = sqrt(-2.0 * log(rsq) / rsq);
    r->second = v1 * fac;
    r->save = 1;
    return v2 * fac;
}

void orc_ranmars_gaussians(orc_ranmars* r, int64_t n, double* out) {
    for (int64_t i = 0; i < n; ++i) out[i] = orc_ranmars_gaussian(r);
}

/* Test harness with no counterpart in the reference: a thermostatted run for
 * estimator statistics.  Langevin noise comes from one RanMars stream per
 * bead seeded seed+bead, drawn in the reference's order (each O-step draws
 * N*D normals per bead, langevin.cpp:18-25).  Every `every` steps (after
 * step k, k = every-1, 2*every-1, ...) the 12 values of orc_observables are
 * appended to out. */
int orc_sample_run(const orc_system* s, orc_state* st, int seed, long nsteps, long every, double* out) {
    const int P = s->nbeads;
    const long bead = (long)s->natoms * s->ndim;
    orc_ranmars** rs = (orc_ranmars**)calloc((size_t)P, sizeof(orc_ranmars*));
    double* xi = (double*)malloc(sizeof(double) * 2 * (size_t)P * (size_t)bead);
    int status = 0;
    for (int b = 0; b < P; ++b) {
        rs[b] = orc_ranmars_new(seed + b);
        if (!rs[b]) status = 1;
    }
    long row = 0;
    for (long k = 0; k < nsteps && status == 0; ++k) {
        for (int o = 0; o < 2; ++o)
            for (int b = 0; b < P; ++b) orc_ranmars_gaussians(rs[b], bead, xi + ((long)o * P + b) * bead);
        status = orc_md_step(s, st, xi, 1);
        if (status == 0 && every > 0 && (k + 1) % every == 0) {
            status = orc_observables(s, st->x, st->p, out + 12 * row);
            ++row;
        }
    }
    for (int b = 0; b < P; ++b) orc_ranmars_free(rs[b]);
    free(rs);
    free(xi);
    return status;
}

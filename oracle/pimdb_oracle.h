/*
 * pimdb_oracle — CPU restatement of the PIMD-B++ per-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU path:
 * only the tests, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * reference legs may load it.  The GPU product never links or calls it.
 *
 * Every routine follows the reference's arithmetic in the reference's
 * operation order (plain FP64, compiled with -ffp-contract=off), so with the
 * same libm it reproduces the compiled reference bit for bit.  Each function
 * cites the reference file:line it restates.
 *
 * Layouts follow the reference's per-rank dVec (include/common.h:79-248):
 * one bead is [particle][axis]; all beads are stacked [bead][particle][axis].
 */
#ifndef PIMDB_ORACLE_H
#define PIMDB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_EXT_FREE = 0, ORC_EXT_HARMONIC = 1, ORC_EXT_DOUBLE_WELL = 2, ORC_EXT_COSINE = 3 };
enum { ORC_INT_FREE = 0, ORC_INT_HARMONIC = 1, ORC_INT_AZIZ = 2, ORC_INT_DIPOLE = 3 };
enum { ORC_PROP_CARTESIAN = 0, ORC_PROP_NORMAL_MODES = 1 };
enum { ORC_THERMO_NONE = 0, ORC_THERMO_LANGEVIN = 1, ORC_THERMO_NOSE_HOOVER = 2, ORC_THERMO_NOSE_HOOVER_NP = 3,
       ORC_THERMO_NOSE_HOOVER_NP_DIM = 4 };

typedef struct {
    int ndim;
    int natoms;
    int nbeads;
    int bosonic;      /* already combined with nbeads > 1 (simulation.cpp:690) */
    int pbc;
    int fixcom;
    int propagator;
    int thermostat;
    int nmthermostat;
    double size;            /* L, bohr */
    double mass;            /* electron masses */
    double dt;              /* atomic time units */
    double gamma;           /* Langevin friction */
    double beta;            /* physical 1/(kB T) */
    double thermo_beta;     /* beta/P (IPI convention, simulation.cpp:41-44) */
    double omega_p;         /* P/(beta hbar) */
    double spring_constant; /* m omega_p^2 */
    double beta_ex;         /* exchange beta: beta/P (bosonic_exchange_base.cpp:16-18) */
    int ext_kind;
    double ext_p[3];        /* harmonic: omega | double_well: strength, location | cosine: amplitude, phase */
    int int_kind;
    double int_p[3];        /* harmonic: omega | dipole: strength */
    double cutoff;          /* effective cutoff (simulation.cpp:84-90): 0 = no pairs, <0 = all pairs */
    int nchains;            /* Nose-Hoover chain length (params.cpp nchains) */
    int factorial;          /* exchange by the sum over all N! permutations
                               (factorial_bosonic_exchange.cpp, the reference's
                               compile-time FACTORIAL_BOSONIC_ALGORITHM) */
} orc_system;

/* Fills the derived constants of `s` from T (atomic units), P, mass, ... and
 * the raw interaction cutoff, following simulation.cpp:37-52,84-90. */
void orc_system_init(orc_system* s, double temperature, double raw_cutoff);

/* ---- elementary pieces ---- */
double orc_min_image(double dx, double L);                                   /* common.cpp:41-43 */
void orc_ext_grad(const orc_system* s, const double* x, int n, double* g);  /* src/potentials: gradV */
double orc_ext_value(const orc_system* s, const double* x, int n);          /* src/potentials: V */
void orc_pair_grad(const orc_system* s, const double* r, double* g);        /* one separation vector */
double orc_pair_value(const orc_system* s, const double* r);

/* ---- bosonic exchange (quadratic_bosonic_exchange.cpp) on one ring ---- */
/* x1 = coordinates of bead 1 (index 0), xP = bead P (index P-1).  Arrays:
 * E[N(N+1)/2], V[N+1], Vb[N+1], prob[N*N] (row = last-bead particle l,
 * column = first-bead particle u).  Return 0, or 2 when V or V_backwards is
 * non-finite (the reference throws std::overflow_error). */
void orc_cycle_energies(const orc_system* s, const double* x1, const double* xP, double* E);
int orc_vb_forward(const orc_system* s, const double* E, double* V);
int orc_vb_backward(const orc_system* s, const double* E, const double* V, double* Vb);
void orc_connection_probabilities(const orc_system* s, const double* E, const double* V, const double* Vb,
                                  double* prob);
void orc_spring_force_last_bead(const orc_system* s, const double* prob, const double* x, const double* x_prev,
                                const double* x_next, double* f);
void orc_spring_force_first_bead(const orc_system* s, const double* prob, const double* x, const double* x_prev,
                                 const double* x_next, double* f);
double orc_prim_estimator(const orc_system* s, const double* E, const double* V);
double orc_distinct_probability(const orc_system* s, const double* E, const double* V);
double orc_longest_probability(const orc_system* s, const double* E, const double* V);

/* Convenience: the whole exchange for one ring.  Any output pointer may be
 * NULL.  With s->factorial set it is orc_factorial_exchange (E_out, V_out,
 * Vb_out and prob_out are then left untouched).  f1/fP are the exterior spring forces on beads 1 and P including the
 * interior neighbour spring (quadratic_bosonic_exchange.cpp:159-215).
 * scalars = {V_B, primEstimator, P_distinct, P_longest}. */
int orc_exchange(const orc_system* s, const double* x_all, double* f1, double* fP, double* scalars, double* E_out,
                 double* V_out, double* Vb_out, double* prob_out);

/* ---- factorial exchange (factorial_bosonic_exchange.cpp) on one ring ----
 * The permutation sum the Feldman-Hirshberg recursion replaces.  For a given
 * configuration the two are different potentials: the recursion keeps one
 * representative cycle per particle set, which equals the full sum only after
 * the interior beads are integrated out.  Same outputs as orc_exchange;
 * P_distinct and P_longest are 0 as in the reference (:237-252). */
double orc_factorial_min_energy(const orc_system* s, const double* x_first, const double* x_last);
int orc_factorial_exchange(const orc_system* s, const double* x_all, double* f1, double* fP, double* scalars);

/* ---- forces on all beads (simulation.cpp:353-455) ---- */
void orc_spring_forces_interior(const orc_system* s, const double* x_prev, const double* x, const double* x_next,
                                double* f);
void orc_physical_forces(const orc_system* s, const double* x, double* f);
/* spring_out / phys_out may be NULL.  Returns the exchange status. */
/* External, pair, non-exchange spring energies and V_B (terms[4]). */
int orc_potential_energy(const orc_system* s, const double* x_all, double* terms);
/* Observables (energy, classical, bosonic, gsf), summed over beads, out[12]. */
int orc_observables(const orc_system* s, const double* x_all, const double* p_all, double* out);
int orc_update_forces(const orc_system* s, const double* x_all, double* f_all, double* spring_out, double* phys_out,
                      int nthreads);

/* ---- integrator state for whole-ring-polymer steps ---- */
typedef struct {
    double* x;          /* [P][N][D] */
    double* p;          /* [P][N][D] */
    double* f;          /* [P][N][D] forces as stored by Simulation::forces */
    double* ext_f;      /* NM propagator: physical forces member (normal_modes_propagator.h:16) */
    double* spring_f;   /* NM propagator: spring forces member */
    double* nh;         /* Nose-Hoover chains: eta, eta_dot, eta_dot_dot, each [nh_chains(s)][nchains] */
} orc_state;

/* Number of Nose-Hoover chains of the whole ring polymer: one per bead
 * (nose_hoover), per bead and particle (_np) or per degree of freedom
 * (_np_dim); 0 for the other thermostats. */
long orc_nh_chains(const orc_system* s);
/* Sum over beads of NoseHooverThermostat::getAdditionToH
 * (nose_hoover.cpp:41-66, :186-192, :223-231). */
double orc_nh_energy(const orc_system* s, const double* nh);

/* Applies one full MD step of Simulation::run (simulation.cpp:236-260):
 * O, [COM], propagator, O, [COM].  xi holds the Gaussian noise of both
 * O-steps: xi[2][P][N][D] (for the NM coupling, index [mode][particle][axis]).
 * nthreads > 1 splits the per-bead loops over POSIX threads (results are
 * identical).  Returns the exchange status. */
int orc_md_step(const orc_system* s, orc_state* st, const double* xi, int nthreads);

/* Test harness (no counterpart in the reference): nsteps MD steps with
 * Langevin noise from RanMars streams seeded seed+bead, storing the 12
 * orc_observables values after every `every`-th step in out[row][12].
 * Returns 0, 1 for an invalid seed, or the exchange status. */
int orc_sample_run(const orc_system* s, orc_state* st, int seed, long nsteps, long every, double* out);

/* Individual pieces of the step, exposed for unit tests. */
void orc_zero_momentum(const orc_system* s, double* p);                       /* simulation.cpp:581-603 */
void orc_langevin(const orc_system* s, double* p, const double* xi);          /* langevin.cpp:15-27 */
void orc_nm_matrices(const orc_system* s, double* cart_to_nm, double* nm_to_cart); /* normal_modes.cpp:48-79 */

/* ---- noise sources ---- */
/* Counter-based Philox4x32-10 (Salmon et al., SC'11) + Box-Muller on FP32
 * with series log, sin and cos (correctly rounded operations only, so the GPU
 * draws bit-identical numbers).  This is the project's noise definition
 * shared with the GPU kernels: normal number of degree of freedom `dof` at
 * (replica, step, substep). */
void orc_philox_normals(uint64_t seed, uint32_t replica, uint64_t step, int substep, int64_t ndof, double* out);
/* RANMAR (Marsaglia, Zaman & Tsang 1990; F. James, Comp. Phys. Comm. 60, 329)
 * with the polar Gaussian, one stream per bead seeded seed+bead, as the
 * reference draws Langevin noise (libs/random_mars.cpp:11-103). */
typedef struct orc_ranmars orc_ranmars;
orc_ranmars* orc_ranmars_new(int seed);
void orc_ranmars_free(orc_ranmars* r);
double orc_ranmars_uniform(orc_ranmars* r);
double orc_ranmars_gaussian(orc_ranmars* r);
void orc_ranmars_gaussians(orc_ranmars* r, int64_t n, double* out);

#ifdef __cplusplus
}
#endif

#endif

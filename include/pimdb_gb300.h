/*
 * pimdb_gb300 — C ABI of the GB300-native PIMD-B++ per-step hot path.
 *
 * One handle holds every bead of one ring-polymer system on one GPU (the
 * reference spreads the beads over MPI ranks, one bead per rank).  All
 * arrays crossing this boundary are plain FP64 in the reference's per-bead
 * dVec order, stacked over beads: [bead][particle][axis]
 * (include/common.h:79-248 of the reference), in Hartree atomic units.
 * Every entry point returns a pimdb_status.  No pointer passed in is kept
 * after the call returns.
 *
 * Which reference interface each entry point stands in for is noted beside
 * it (paths are within the PIMD-B++ source tree).
 */
#ifndef PIMDB_GB300_H
#define PIMDB_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define PIMDB_ABI_VERSION 1

/* Status codes.  The reference throws std::invalid_argument for configuration
 * errors (src/params.cpp:11-260) and std::overflow_error for a non-finite
 * exchange potential (src/bosonic_exchange/quadratic_bosonic_exchange.cpp:92-97,119-124). */
typedef enum pimdb_status {
    PIMDB_OK = 0,
    PIMDB_ERR_CONFIG = 1,        /* invalid configuration (std::invalid_argument) */
    PIMDB_ERR_NONFINITE_VB = 2,  /* V or V_backwards not finite (std::overflow_error) */
    PIMDB_ERR_CUDA = 3,          /* CUDA runtime error; see pimdb_last_error */
    PIMDB_ERR_TIMEOUT = 4,       /* a bounded device-side wait gave up */
    PIMDB_ERR_BOUNDS = 5,        /* a device-side index check failed */
    PIMDB_ERR_ARG = 6,           /* NULL handle or invalid argument */
    PIMDB_ERR_NO_DEVICE = 7,     /* no CUDA device visible */
    PIMDB_ERR_PARSE = 8          /* config.ini could not be read */
} pimdb_status;

/* Potentials (src/simulation.cpp:612-645; names as in config.ini). */
enum pimdb_potential {
    PIMDB_POT_FREE = 0,
    PIMDB_POT_HARMONIC = 1,    /* params: omega */
    PIMDB_POT_DOUBLE_WELL = 2, /* params: strength, location (external only) */
    PIMDB_POT_COSINE = 3,      /* params: amplitude, phase (external only) */
    PIMDB_POT_AZIZ = 4,        /* HFDHE2 (interaction only) */
    PIMDB_POT_DIPOLE = 5       /* params: strength in Hartree bohr^3 (interaction only) */
};
enum pimdb_propagator { PIMDB_PROP_CARTESIAN = 0, PIMDB_PROP_NORMAL_MODES = 1 };
/* none, langevin, and the Nose-Hoover chains nose_hoover (one chain per
 * bead), nose_hoover_np (per bead and particle), nose_hoover_np_dim (per
 * degree of freedom) of src/thermostats/nose_hoover.cpp. */
enum pimdb_thermostat {
    PIMDB_THERMO_NONE = 0,
    PIMDB_THERMO_LANGEVIN = 1,
    PIMDB_THERMO_NOSE_HOOVER = 2,
    PIMDB_THERMO_NOSE_HOOVER_NP = 3,
    PIMDB_THERMO_NOSE_HOOVER_NP_DIM = 4
};
/* Bosonic exchange algorithm (the reference chooses at compile time with
 * FACTORIAL_BOSONIC_ALGORITHM, CMakeLists.txt:49-54, include/common.h:26-28):
 * the Feldman-Hirshberg recursion (src/bosonic_exchange/quadratic_bosonic_exchange.cpp),
 * or the sum over all N! permutations
 * (src/bosonic_exchange/factorial_bosonic_exchange.cpp; natoms <= 12).  The
 * two are different potentials for a given configuration with the same
 * partition function.  The factorial sum is FP64 in both precisions and
 * reports P_distinct = P_longest = 0 as the reference does. */
enum pimdb_exchange_algorithm { PIMDB_EXCHANGE_FELDMAN_HIRSHBERG = 0, PIMDB_EXCHANGE_FACTORIAL = 1 };
/* Langevin noise.  PIMDB_RNG_PHILOX: counter-based Philox4x32-10 normals,
 * a pure function of (seed, replica, step, degree of freedom), so any step
 * can be replayed (pimdb_set_step) and graphs need no state.
 * PIMDB_RNG_RANMAR: the reference's own streams, one RanMars per bead seeded
 * seed + bead (src/simulation.cpp:54-59, libs/random_mars.cpp), drawn in the
 * reference's order (src/thermostats/langevin.cpp:15-27), so trajectories
 * follow the reference's from the same initial state.  The streams advance
 * with every MD step and are not rewound by pimdb_set_step or
 * pimdb_set_state; each bead's seed must lie in 1..900000000 as the
 * reference requires.  Drawing is sequential per bead: a parity mode, not a
 * fast path. */
enum pimdb_rng { PIMDB_RNG_PHILOX = 0, PIMDB_RNG_RANMAR = 1 };
/* Arithmetic of the pair forces: FP64 throughout, or FP32 pair arithmetic
 * with FP64 per-atom accumulation.  Exchange and integrator are FP64 in both. */
enum pimdb_precision { PIMDB_FP64 = 0, PIMDB_MIXED = 1 };

/* The hot-path subset of the reference's Params (src/params.cpp:8-260),
 * already converted to atomic units. */
typedef struct pimdb_config {
    int ndim;            /* 1, 2 or 3 (the reference's compile-time NDIM) */
    int natoms;          /* [system] natoms */
    int nbeads;          /* [simulation] nbeads */
    int bosonic;         /* [simulation] bosonic (ignored when nbeads == 1) */
    int pbc;             /* [simulation] pbc */
    int fixcom;          /* [simulation] fixcom */
    int propagator;      /* enum pimdb_propagator */
    int thermostat;      /* enum pimdb_thermostat */
    int nmthermostat;    /* [simulation] nmthermostat */
    int precision;       /* enum pimdb_precision */
    double temperature;  /* kB T in Hartree */
    double mass;         /* electron masses */
    double size;         /* box edge L, bohr */
    double dt;           /* atomic time units */
    double gamma;        /* Langevin friction; < 0 selects 1/(100 dt) */
    int ext_kind;        /* enum pimdb_potential */
    double ext_params[3];
    int int_kind;        /* enum pimdb_potential */
    double int_params[3];
    double cutoff;       /* interaction cutoff before min(cutoff, L/2) under PBC; < 0 = all pairs */
    unsigned long long seed;  /* Langevin noise key */
    unsigned int replica;     /* folded into the noise counter */
    int nchains;              /* [simulation] nchains: Nose-Hoover chain length */
    int exchange;             /* enum pimdb_exchange_algorithm */
    int rng;                  /* enum pimdb_rng */
} pimdb_config;

typedef struct pimdb_handle pimdb_handle;

/* Reference defaults (src/params.cpp:15-259) for a 3-dimensional system. */
int pimdb_config_default(pimdb_config* cfg);

/* Reads a reference config.ini (schema, defaults, units and validation of
 * src/params.cpp:8-260 and src/units.cpp).  `ndim` stands for the reference's
 * compile-time NDIM.  On failure returns PIMDB_ERR_PARSE or PIMDB_ERR_CONFIG
 * and writes the reference's message into err (if err_len > 0). */
int pimdb_config_from_ini(const char* path, int ndim, pimdb_config* cfg, char* err, int err_len);

/* Simulation::Simulation (src/simulation.cpp:16-101) minus initial
 * conditions: allocates the device state of all beads.  `cuda_stream` is a
 * cudaStream_t to run on, or NULL for a stream owned by the handle.  A
 * configuration the reference would reject, a bosonic ring polymer of more
 * than 14000 particles (the largest whose exchange solve fits one block's
 * shared memory) or normal modes with more than 1536 beads (likewise for
 * the matrix-transform step) returns PIMDB_ERR_CONFIG before any GPU work. */
int pimdb_create(const pimdb_config* cfg, void* cuda_stream, pimdb_handle** out);
int pimdb_destroy(pimdb_handle* h);

/* Sets coordinates and momenta of every bead (host arrays
 * [bead][particle][axis]); either may be NULL to keep the current values.
 * Forces are reset to zero, as after the reference's constructor
 * (src/simulation.cpp:16-101 never evaluates them). */
int pimdb_set_state(pimdb_handle* h, const double* x, const double* p);
/* Same with device pointers in the same layout. */
int pimdb_set_state_device(pimdb_handle* h, const double* x, const double* p);
/* Copies coordinates, momenta and forces (Simulation::forces) to host arrays;
 * any may be NULL. */
int pimdb_get_state(pimdb_handle* h, double* x, double* p, double* f);
int pimdb_get_state_device(pimdb_handle* h, double* x, double* p, double* f);

/* MD step index used as the Langevin noise counter. */
int pimdb_set_step(pimdb_handle* h, long long step);
int pimdb_get_step(pimdb_handle* h, long long* step);

/* Simulation::updateForces on every bead (src/simulation.cpp:353-374):
 * exchange springs on beads 1 and P, interior springs, external and pair
 * forces. */
int pimdb_compute_forces(pimdb_handle* h);

/* `nsteps` iterations of the body of Simulation::run
 * (src/simulation.cpp:246-259): thermostat O-step, COM removal, propagator
 * (VelocityVerletPropagator::step, src/propagators/velocity_verlet.cpp:7-22,
 * or NormalModesPropagator::step, src/propagators/normal_modes_propagator.cpp:19-71),
 * thermostat O-step, COM removal.  Synchronous: returns after the GPU is done
 * and reports a non-finite exchange potential.  The last operations of the
 * last step (with the fused normal-mode kernel: its kick, O-step and COM
 * removal; otherwise a COM correction) are deferred and folded into the next
 * step; every call that reads or changes the state (get/set_state, forces,
 * exchange, energies, the plugin calls) completes them first, so the state
 * seen by the caller is always that at the end of the step.  Runs of steps
 * are captured once per step count and replayed as CUDA graphs. */
int pimdb_step(pimdb_handle* h, int nsteps);
/* Same, only enqueued on the handle's stream; errors surface at the next
 * pimdb_synchronize or synchronous call. */
int pimdb_step_async(pimdb_handle* h, int nsteps);
int pimdb_synchronize(pimdb_handle* h);
/* For callers that keep the state on the host: pimdb_set_state (x_in, p_in;
 * both NULL keeps the device state), pimdb_step(nsteps) and pimdb_get_state
 * (x_out, p_out, f_out; any may be NULL) in one call with one
 * synchronisation.  The host arrays may be pinned or pageable and may
 * alias (x_in == x_out).  Page-locked arrays are read and written by the
 * state kernels directly, and then the whole call (state in, steps, state
 * out) is captured once per (nsteps, arrays) and replayed as one CUDA graph. */
int pimdb_step_io(pimdb_handle* h, const double* x_in, const double* p_in, int nsteps, double* x_out, double* p_out,
                  double* f_out);

/* The step's pieces one by one, for hosts that mirror the reference's
 * plugin calls (Simulation::run, src/simulation.cpp:246-259).  Together,
 *   thermostat_step(0); zero_momentum(); propagate(); thermostat_step(1);
 *   zero_momentum(); set_step(step + 1)
 * give the same state as pimdb_step(h, 1) (the fused normal-mode kernel
 * aside, which reorders the same linear operations).
 *   pimdb_thermostat_step  Thermostat::step (src/thermostats/thermostat.cpp:15-19);
 *                          `substep` 0 / 1 selects the first / second O-step's
 *                          noise of the current MD step;
 *   pimdb_zero_momentum    Simulation::zeroMomentum (src/simulation.cpp:581-603);
 *   pimdb_propagate        Propagator::step (velocity_verlet.cpp:7-22 or
 *                          normal_modes_propagator.cpp:19-71); synchronous. */
int pimdb_thermostat_step(pimdb_handle* h, int substep);
int pimdb_zero_momentum(pimdb_handle* h);
int pimdb_propagate(pimdb_handle* h);

/* BosonicExchange on the current coordinates
 * (src/bosonic_exchange/quadratic_bosonic_exchange.cpp:30-279; with
 * PIMDB_EXCHANGE_FACTORIAL FactorialBosonicExchange,
 * src/bosonic_exchange/factorial_bosonic_exchange.cpp:19-293, whose
 * scalars[2] and [3] are 0):
 *   scalars[0] = effectivePotential()      V_B = V[N]
 *   scalars[1] = primEstimator()           -d(beta_ex V_B)/d(beta_ex) / P at fixed E
 *   scalars[2] = getDistinctProbability()
 *   scalars[3] = getLongestProbability()
 *   f_first    = exterior spring force on bead 1 (springForceFirstBead), [particle][axis]
 *   f_last     = exterior spring force on bead P (springForceLastBead)
 * Any output may be NULL.  Requires a bosonic configuration. */
int pimdb_exchange(pimdb_handle* h, double* scalars, double* f_first, double* f_last);
/* The same exchange as a forward function and its adjoint, for callers that
 * compose V_B with something else (BosonicExchangeBase's split into
 * prepare / effectivePotential / exteriorSpringForce / primEstimator,
 * include/bosonic_exchange/bosonic_exchange_base.h:16-54; Feldman-Hirshberg
 * exchange only, PIMDB_ERR_CONFIG with the factorial one).
 *
 * pimdb_exchange_forward: prepare() + effectivePotential() on the current
 * coordinates (quadratic_bosonic_exchange.cpp:30-132): cycle energies, the
 * V and V_backwards recursions, and V_B = V[N] into *VB (may be NULL).  The
 * arrays stay on the device for the two calls below.
 *
 * pimdb_exchange_adjoint: the vector-Jacobian product of V_B with an
 * incoming cotangent vb_bar = dL/dV_B: x1_bar = vb_bar * dV_B/dx_1 and
 * xP_bar = vb_bar * dV_B/dx_P, [particle][axis] (either may be NULL).  With
 * vb_bar = 1 these are minus the exchange part of springForceFirstBead /
 * springForceLastBead (:159-215), without their interior neighbour spring.
 *
 * pimdb_exchange_dbeta: primEstimator() (:250-279), -d(beta_ex V_B)/d(beta_ex)
 * / P at fixed cycle energies, the bosonic term of the primitive energy.
 *
 * The adjoint and dbeta read the last forward evaluation; they return
 * PIMDB_ERR_ARG when the coordinates changed since (a state set, a step). */
int pimdb_exchange_forward(pimdb_handle* h, double* VB);
/* Diagnostic (no counterpart in the reference): how many exchange
 * evaluations since creation found the reused estimate of V (the previous
 * evaluations' potentials, extrapolated) unusable and were redone from a
 * fresh FP32 estimate, per direction for the in-block retry below 768
 * particles and per evaluation above.  Smooth dynamics keep it near 0; each
 * retry costs a slower evaluation, not accuracy. */
int pimdb_exchange_retries(pimdb_handle* h, long long* count);
/* Diagnostic (no counterpart in the reference): how many exchange
 * evaluations since creation began with a fresh FP32 estimate of V (the
 * first one, and those after a solve found the reused potentials more than
 * 30 kT off), counted below 768 particles by the estimate kernel of the
 * first pass only (not the in-block retries pimdb_exchange_retries counts). */
int pimdb_exchange_fresh_estimates(pimdb_handle* h, long long* count);
int pimdb_exchange_adjoint(pimdb_handle* h, double vb_bar, double* x1_bar, double* xP_bar);
int pimdb_exchange_dbeta(pimdb_handle* h, double* dbeta);

/* Intermediate arrays of the last pimdb_exchange / force evaluation:
 * E (N(N+1)/2, the reference's E_kn order, getEnk(m,k) = E[m(m+1)/2 - k]),
 * V (N+1), V_backwards (N+1).  Any may be NULL.  PIMDB_ERR_CONFIG with the
 * factorial exchange, which has none of them. */
int pimdb_exchange_arrays(pimdb_handle* h, double* E_kn, double* V, double* V_backwards);

/* The forward function of pimdb_compute_forces: the potential energy U of
 * the ring polymer at the current coordinates, whose negative gradient the
 * force kernels return (the adjoint).  Terms, from the potentials' V()
 * (src/potentials/{harmonic,aziz,dipole,double_well,cosine}.cpp) and
 * classicalSpringEnergy (src/simulation.cpp:464-486):
 *   terms[0]  external V summed over beads and particles
 *   terms[1]  pair V summed over beads, each pair once (same cutoff and
 *             minimum image as the forces)
 *   terms[2]  ring springs outside the exchange: all P links when
 *             distinguishable, links b -> b+1 (b < P-1) when bosonic
 *   terms[3]  V_B = effectivePotential() when bosonic, else 0
 * U = terms[0] + terms[1] + terms[2] + terms[3].  (The reference's double
 * well gradV uses |x|^2 of all axes while its V sums per axis, so for ndim > 1
 * its force is not -dU/dx; everything else is.) */
int pimdb_potential_energy(pimdb_handle* h, double* terms);
/* Energy of every term of U that involves particle i of bead b, for n items
 * items[2k] = b, items[2k+1] = i: external V, pair V with every other
 * particle of bead b, and the adjacent springs outside the exchange.  Its
 * derivative with respect to x_bi, plus that of V_B on bosonic beads 1 and
 * P, is -f_bi; finite differences of it stay accurate at any N. */
int pimdb_local_energy(pimdb_handle* h, int n, const int* items, double* out);

/* The reference's observables of the current state (src/observables/
 * energy.cpp, classical.cpp, bosonic.cpp, gsf_action.cpp), each bead's
 * value as the reference computes it on that bead's rank, summed over beads
 * as ObservablesLogger::log does (src/observables/observable.cpp:82-116).
 * Atomic units, except temperature in kelvin (classical.cpp:60).  The GSF
 * force term uses the total gradient on each particle (the reference's
 * gsf_action.cpp:34 adds arrays of different lengths when an interaction is
 * present). */
typedef struct pimdb_observables {
    double kinetic, potential, ext_pot, int_pot, virial;  /* energy */
    double temperature, cl_kinetic, cl_spring;            /* classical */
    double prob_dist, prob_all;                           /* bosonic */
    double w_gsf, pot_gsf;                                /* gsf */
    double nh_energy;  /* classical, Nose-Hoover: getAdditionToH summed over beads */
} pimdb_observables;
int pimdb_compute_observables(pimdb_handle* h, pimdb_observables* out);

/* Instrumentation (no counterpart in the reference, which only reports the
 * wall time per step, src/simulation.cpp:517-572).  Kernel classes: */
enum pimdb_kernel_class {
    PIMDB_K_BEAD_FORCES = 0,      /* external + pair forces + interior springs */
    PIMDB_K_EXCH_ENERGIES = 1,    /* cycle energies E */
    PIMDB_K_EXCH_RECURSIONS = 2,  /* V and V_backwards recursions */
    PIMDB_K_EXCH_FORCES = 3,      /* connection probabilities -> forces on beads 1 and P */
    PIMDB_K_EXCH_ESTIMATORS = 4,  /* primEstimator and topology probabilities */
    PIMDB_K_CART_UPDATE = 5,      /* B / A / Langevin / COM on Cartesian momenta */
    PIMDB_K_NM_PROPAGATE = 6,     /* normal-mode free ring-polymer propagation (fused with the
                                     normal-mode thermostat when both are selected) */
    PIMDB_K_NM_THERMO = 7,        /* normal-mode Langevin O-step */
    PIMDB_NUM_KERNEL_CLASSES = 8
};
/* Reads the accumulated per-class device milliseconds and launch counts and
 * the total number of kernels launched since the last reset (any output may
 * be NULL).  enable = 1 / 0 resets the counters and turns the per-launch
 * event timing on / off (timing synchronises after every launch); enable = -1
 * only reads. */
int pimdb_profile(pimdb_handle* h, int enable, double* ms, long long* counts, long long* launches);

/* Execution options (no counterpart in the reference):
 *   "exact_exchange" 1: evaluate V and V_backwards level by level with the
 *                    FP64 log-sum-exp in the reference's own order
 *                    (evaluateVBn / evaluateVBackwards, :73-128) instead of
 *                    the estimate + triangular-solve evaluation (default 0);
 *   "newton3"        0: all-pairs pair kernel (each pair evaluated from both
 *                    sides) instead of the pair-tile kernel (default 1);
 *   "fused_normal_modes" 0: with the normal-mode propagator and thermostat,
 *                    run the thermostat and the propagator as separate
 *                    kernels in the reference's order instead of the fused
 *                    normal-mode-frame kernel (default 1 when all its blocks
 *                    fit on the GPU at once);
 *   "fft_normal_modes" 0: in the fused kernel, transform with the P x P
 *                    matrices instead of FFTs (FFTs are used when P is a
 *                    power of two; default 1);
 *   "cell_lists"     1 / 0 / -1: pair forces from cell lists (periodic box
 *                    with at least 4 cutoff-wide cells per edge) on / off /
 *                    automatic (default: on from 512 particles);
 *   "cuda_graphs"    0: enqueue every step's kernels instead of replaying a
 *                    captured graph (default 1);
 *   "flat_energies"  1 / 0 / -1: cycle energies from prefix sums of the
 *                    interior links (one independent entry per thread) /
 *                    from a scan per row / automatic (default: prefix sums
 *                    from 512 particles);
 *   "pair_entry_cap" pair-tile kernel: gradients held in shared memory per
 *                    warp (a multiple of 32 up to 1024; 0 = default).  Fewer
 *                    let more warps share an SM; a tile with more pairs
 *                    inside the cutoff is summed in chunks (same result up to
 *                    the order of its j-side additions);
 *   "reserved_sms"   pair-tile kernel beside the bosonic exchange: how many
 *                    SMs (the highest ids) its blocks leave to the
 *                    exchange's one-block passes (-1 = automatic: 2 below 768
 *                    particles, else 0).  Blocks placed there take no tile;
 *                    the warp that finishes last takes any tile still left,
 *                    so any value gives the same forces. */
int pimdb_set_option(pimdb_handle* h, const char* name, int value);

/* Bosonic exchange without any allocation (no counterpart in the reference).
 * For callers that may not call cudaMalloc while they need the exchange: a
 * program whose device memory belongs to another allocator or a fixed budget
 * (an allocation behind its back fails or breaks its accounting), or a loop
 * that cannot afford cudaMalloc's implicit device synchronisation.
 * Inputs and outputs are device memory supplied by the caller:
 *   ring       x[bead][particle][axis] of all `nbeads` beads (only beads 1, 2,
 *              P-1 and P are read), atomic units;
 *   scalars    4 doubles: V_B, primEstimator, P_distinct, P_longest (as
 *              pimdb_exchange);
 *   f_first, f_last  exterior spring forces on beads 1 and P, [particle][axis]
 *              (either may be NULL).
 * spring_constant = m omega_P^2 and beta_ex = beta/P as in the reference.
 * All intermediate arrays live in one fixed __device__ array of about 1.1 MB
 * that every GPU loading the library keeps until the process exits; hence at
 * most 256 particles (larger natoms returns PIMDB_ERR_ARG and a message in
 * err).  The first call on a device looks up that array's device address, so
 * make it before any stream capture.  Calls share the array: calls that
 * overlap on the GPU (different streams or host threads) race.  The call runs
 * on `cuda_stream` (NULL = legacy default stream), which must belong to the
 * current device (PIMDB_ERR_ARG otherwise); it synchronises that stream and
 * returns after the work is done, reporting a non-finite V_B as
 * PIMDB_ERR_NONFINITE_VB. */
int pimdb_exchange_noalloc(const double* ring, int nbeads, int natoms, int ndim, double spring_constant,
                           double beta_ex, int pbc, double box, double* scalars, double* f_first, double* f_last,
                           void* cuda_stream, char* err, int err_len);

/* ------------------------------------------------------------------------
 * Batched replicas (no counterpart in the reference, which runs one system
 * per MPI job: src/pimdb.cpp:31-68).  A batch is many independent systems,
 * each with its own pimdb_config (natoms, nbeads, temperature, potentials,
 * seed, replica), advanced together: one launch per MD step, and a run of
 * steps is replayed as one CUDA graph.  Each step is the body of
 * Simulation::run (src/simulation.cpp:246-259) with, per replica, the
 * cartesian propagator (VelocityVerletPropagator::step,
 * src/propagators/velocity_verlet.cpp:7-22) or the normal-mode one
 * (NormalModesPropagator::step, src/propagators/normal_modes_propagator.cpp:
 * 19-71; nbeads <= 256), and the Langevin thermostat in the cartesian or the
 * normal-mode frame, or none (Nose-Hoover chains: one system at a time).
 * Every replica must share ndim and precision; natoms <= 2048; at most 65535
 * replicas.  Blocks are 256 threads unless every warp's staged copy of the
 * largest replica needs smaller ones (above about 900 particles); a block
 * shape that cannot hold it returns PIMDB_ERR_CONFIG.  With PIMDB_MIXED the pair forces are FP32 with FP64
 * accumulation, the exchange weights double-float and its exterior spring
 * forces FP32 with compensated sums; potentials, triangular solve, cycle
 * energies and integrator stay FP64.  The Langevin normals are the
 * one-system path's in both precisions.
 * Host arrays of the batch are the replicas' [bead][particle][axis] arrays
 * concatenated in replica order (pimdb_batch_size gives the total length).
 */
typedef struct pimdb_batch pimdb_batch;
int pimdb_batch_create(const pimdb_config* cfgs, int nreplicas, void* cuda_stream, pimdb_batch** out);
int pimdb_batch_destroy(pimdb_batch* b);
int pimdb_batch_size(const pimdb_batch* b, int* nreplicas, long long* host_doubles);
/* As pimdb_set_state / pimdb_get_state for every replica at once. */
int pimdb_batch_set_states(pimdb_batch* b, const double* x, const double* p);
int pimdb_batch_get_states(pimdb_batch* b, double* x, double* p, double* f);
/* MD step index shared by the replicas (the Langevin noise counter). */
int pimdb_batch_set_step(pimdb_batch* b, long long step);
int pimdb_batch_get_step(pimdb_batch* b, long long* step);
/* Simulation::updateForces (src/simulation.cpp:353-374) on every replica. */
int pimdb_batch_compute_forces(pimdb_batch* b);
/* `nsteps` MD steps of every replica; synchronous, reports a non-finite V_B
 * of any replica (the message names it).  _async only enqueues. */
int pimdb_batch_step(pimdb_batch* b, int nsteps);
int pimdb_batch_step_async(pimdb_batch* b, int nsteps);
int pimdb_batch_synchronize(pimdb_batch* b);
/* pimdb_exchange's four scalars for every replica, scalars[nreplicas][4]
 * (zeros for distinguishable replicas); evaluates the forces first. */
int pimdb_batch_exchange(pimdb_batch* b, double* scalars);
/* "threads" (32..512 per CTA), "ctas_per_sm" (resident CTAs per SM the grid
 * is sized for), "graph" (0: plain launches instead of a CUDA graph). */
int pimdb_batch_set_option(pimdb_batch* b, const char* name, int value);
int pimdb_batch_get_launch(pimdb_batch* b, int* threads, int* ctas_per_sm, int* grid, long long* launches);
/* Chooses threads per CTA and CTAs per SM by timing `steps` steps of each
 * candidate from a copy of the current state; the state is restored. */
int pimdb_batch_autotune(pimdb_batch* b, int steps, int* threads, int* ctas_per_sm);
int pimdb_batch_last_error(const pimdb_batch* b, char* buf, int len);

/* Measures the FP64 fused-multiply-add throughput of the current device in
 * TFLOP/s (the roofline denominator of the FP64 kernels). */
int pimdb_measure_fp64_peak(double* tflops);
/* The same for FP32 fused multiply-adds (the mixed paths' pair forces). */
int pimdb_measure_fp32_peak(double* tflops);

/* Diagnostics of the hand-written FP64 functions against CUDA's own, on n
 * host values x (no counterpart in the reference).  out (8 n doubles, host):
 * per value, exp(x), exp_tang(x) (32-entry table) and exp_tang256(x)
 * (256-entry table), then rsqrt(r) and rsqrt_newton(r) for r = |x| + 1e-3,
 * then the bit-pattern conversions: hi and lo of split_f32(x) and
 * f32_to_f64((float)x). */
int pimdb_math_check(const double* x, int n, double* out);

/* Human-readable text of the last error on this handle (or a global one if
 * h is NULL). */
int pimdb_last_error(const pimdb_handle* h, char* buf, int len);
const char* pimdb_status_string(int status);

#ifdef __cplusplus
}
#endif

#endif

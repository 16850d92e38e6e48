// Host-side launch wrappers for the device kernels (one system per call).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "common.cuh"

namespace pimdb {

// The reference's normal-mode rows C (row k: mode k over beads), their
// inverse T (row j: bead j over modes) and per mode {cos(w_k dt),
// sin(w_k dt), m w_k, sin(w_k dt) / (m w_k)} (normal_modes.cpp:48-79,
// normal_modes_propagator.cpp:13-16); host code.
void nm_tables(int P, double omega_p, double mass, double dt, std::vector<double>& C, std::vector<double>& T,
               std::vector<double>& rot);

// Flags of the momentum-update kernels.  Within one launch the operations
// run in this order: COM correction from the pending partial sums, B
// half-kick, Langevin O-step, A drift, partial sums for the next COM removal.
enum StepFlags : int {
    SF_COM_APPLY = 1,
    SF_LANGEVIN = 2,
    SF_COM_PARTIAL = 4,
    SF_KICK = 8,
    SF_DRIFT = 16,
};

// forces.cu: external + pair forces and distinguishable springs on every
// bead; on bosonic beads 0 and P-1 only the physical part is stored in f.
void launch_bead_forces(const Sys& s, int D, int mixed, int write_phys, cudaStream_t st);
// Same result with Newton's third law: pair tiles write partial sums into
// `part` (pair_partial_doubles doubles), a second kernel adds them in order.
// With add_fx the finishing kernel also adds the exchange's exterior spring
// forces (fx) on beads 1 and P, after waiting for `before_finish` (may be
// null) that marks them done.
size_t pair_partial_doubles(const Sys& s, int D);
// pimdb_math_check's kernel (device arrays; out holds 8 n doubles).
void launch_math_check(const double* x, int n, double* out, cudaStream_t st);
void launch_pair_tiles_and_finish(const Sys& s, int D, int mixed, int write_phys, double* part,
                                  cudaEvent_t before_finish, int add_fx, cudaStream_t st);
// Cell lists for a periodic box with a short cutoff: cells per edge (0 when
// they do not apply), the work buffer they need, and the force evaluation
// (binning, pair forces, finish) into that buffer.
int cell_grid(const Sys& s, int D);
size_t cell_buffer_bytes(const Sys& s, int D, int nc);
void launch_pair_cells_and_finish(const Sys& s, int D, int nc, int mixed, int write_phys, void* buf,
                                  cudaEvent_t before_finish, int add_fx, cudaStream_t st);

// Potential energy: per-bead partial sums of the external, pair and
// non-exchange spring energies, part[(b * energy_blocks + blk) * 3 + term];
// and the local energy of listed (bead, particle) items ([n][2] ints).
int energy_blocks(const Sys& s);
// Per-bead observable terms, part[(b * energy_blocks + blk) * 7 + term]
// (see k_observable_terms).
void launch_observable_terms(const Sys& s, int D, double* part, cudaStream_t st);
void launch_energy_terms(const Sys& s, int D, double* part, cudaStream_t st);
void launch_local_energy(const Sys& s, int D, int n, const int* items, double* out, cudaStream_t st);

// exchange.cu: Feldman-Hirshberg exchange on beads 1 and P.
// For N >= 512 with `work` (exchange_energy_doubles) the energies come from
// the links' prefix sums, one independent entry per thread.
// Returns 1 when the per-row energy kernel ran, which also runs a due FP32
// estimate and forms the weights (pass `estimate_done` = 1 to
// launch_exchange_recursions).
int launch_exchange_energies(const Sys& s, int D, cudaStream_t st, double* work = nullptr);
size_t exchange_energy_doubles(const Sys& s, int D);
// Returns the number of kernels launched: the estimate and the weights
// (unless the energy kernel formed them) and the solve kernels (with their retry phase
// from 768 particles), or 1 with `exact` (the reference-order FP64
// log-sum-exp recursion only).  With `ysol` (exchange_grid_doubles) below 768
// particles the banded kernel is the whole solve; from 768 the solve runs
// across SMs when `gflags` (exchange_grid_flags, zeroed once) is given.
int launch_exchange_recursions(const Sys& s, int exact, cudaStream_t st, double* ysol = nullptr,
                               unsigned* gflags = nullptr, int estimate_done = 0);
size_t exchange_grid_doubles(const Sys& s);
// SMs the pair tiles should leave free (Sys::reserve_sms) while the exchange
// runs beside them on another stream.
int exchange_reserved_sms(const Sys& s);
size_t exchange_grid_flags(const Sys& s);
void launch_exchange_forces_mode(const Sys& s, int D, int accumulate, cudaStream_t st);
// Whether the cycle energies of a system of N particles come from link prefix
// sums by default (Sys::eflat; the option "flat_energies" overrides it).
int exchange_flat_default(int N);
// Index in Sys::xflags (16 ints) of the count of exchange evaluations redone
// from a fresh estimate after the reused one failed.
constexpr int kExchRetryCount = 10;
// Index in Sys::xflags of the solve's band: the largest node distance p + 1
// - u of a nonzero weight of the current evaluation (0 between evaluations).
constexpr int kExchBand = 11;
// Index in Sys::xflags of the count of evaluations whose first pass computed
// a fresh FP32 estimate (the previous potentials were not reusable).
constexpr int kExchFreshCount = 12;
// Indices in Sys::xflags of the banded solve's finishing handshake: its CTAs
// that post-processed their direction (count), and whether the evaluation is
// complete (2: each of k_exch_solve's two blocks takes one off and exits).
constexpr int kExchBandCount = 13;
constexpr int kExchBandDone = 14;
// Index in Sys::xflags of the band of the evaluation the banded solve
// completed (0 when another path solved it): the exterior-force rows skip
// the entries beyond it, all exact zeros.
constexpr int kExchBandLast = 15;
// Index in Sys::xflags of the count of finished blocks of the per-row energy
// kernel (its last block runs a due FP32 estimate).
constexpr int kExchRowsCount = 9;
// The banded solve: weights within kBandMax levels of the diagonal, one CTA
// of kBandThreads per direction, y of up to kBandMaxN nodes in shared memory.
constexpr int kBandMax = 64;
constexpr int kBandThreads = 256;
constexpr int kBandMaxN = 8192;
// The largest bosonic system: the one-block solve holds 2 (N + 1) + 32
// doubles of dynamic shared memory beside about 2 KB of static tables, and
// a block gets at most 227 KB (sm_103a), which allows N = 14382; 14000
// leaves room for the static part to grow.
constexpr int kExchangeMaxN = 14000;
static_assert(sizeof(double) * (2 * (kExchangeMaxN + 1) + 32) + 4096 <= 227 * 1024,
              "the one-block solve's shared memory at the largest bosonic system");
// The most beads with the normal-mode propagator or thermostat: the
// matrix-transform step (k_nm_propagate, the path for bead counts the
// register and fused kernels do not take) holds 4 P x 4 particles' doubles
// of shared memory, and a block gets at most 227 KB (sm_103a).
constexpr int kNmMaxBeads = 1536;
// The cotangent of V_B on beads 1 and P into fx: vb_bar * dV_B/dx (the
// exterior spring forces' exchange part times -vb_bar).
void launch_exchange_adjoint(const Sys& s, int D, double vb_bar, cudaStream_t st);
void launch_exchange_estimators(const Sys& s, cudaStream_t st);

// factorial.cu: the factorial exchange (sum over all N! permutations) on
// beads 1 and P, for at most kFactMaxN particles.  launch_factorial_sums
// (2 kernels) fills `work` (factorial_work_doubles(N) doubles);
// launch_factorial_finish then writes the scalars (V_B, primEstimator, 0, 0)
// and the exterior spring forces into fx (and adds them into f with
// `accumulate`).
constexpr int kFactMaxN = 12;
size_t factorial_work_doubles(int N);
int launch_factorial_sums(const Sys& s, int D, double* work, cudaStream_t st);
void launch_factorial_finish(const Sys& s, int D, double* work, int accumulate, cudaStream_t st);

// RanMars parity noise (integrator.cu): one RanMars stream per bead,
// seeded on the host (ranmars_seed: seed in 1..900000000), drawn on the
// device into Sys::noise at the start of each MD step.
struct RanMarsState {
    double u[98];
    double c, cd, cm, second;
    int i97, j97, save, pad;
};
static_assert(sizeof(RanMarsState) % sizeof(double) == 0, "RanMarsState is copied as doubles");
void ranmars_seed(int seed, RanMarsState& r);
void launch_ranmars_draw(const Sys& s, int D, RanMarsState* states, double* noise, StepRef step, cudaStream_t st);

// Nose-Hoover chains: parameters of one thermostat (constructors of
// src/thermostats/nose_hoover.cpp) and its chain state, [chains][nchains]
// each.  variant 0: a chain per bead, 1: per bead and particle, 2: per
// degree of freedom.
struct NHPar {
    int variant, nchains;
    double Q1, Qi, required, thermo_beta, dt2, dt4, dt8;
    double* eta;
    double* eta_dot;
    double* eta_dd;
};
// One thermostat step on s.p; with C (cart -> NM rows) and T (NM -> cart)
// the chains act on the normal-mode momenta, staged in pnm ([P][D][ld]).
// Returns the number of kernels launched.
int launch_nose_hoover(const Sys& s, int D, const NHPar& q, const double* C, const double* T, double* pnm,
                       cudaStream_t st);

// integrator.cu
void launch_pack(const Sys& s, int D, const double* src, double* dst, cudaStream_t st);
void launch_unpack(const Sys& s, int D, const double* src, double* dst, cudaStream_t st);
// The state crossing the boundary in one launch each way: k_state_in packs
// x and p (either may be null) from host-order arrays and zeroes the force
// arrays; k_state_out unpacks x, p, f (any may be null) into host-order
// arrays.  The arrays are device staging or page-locked host memory.
void launch_state_in(const Sys& s, int D, const double* sx, const double* sp, cudaStream_t st);
void launch_state_out(const Sys& s, int D, double* ox, double* op, double* of, cudaStream_t st);
int cart_update_blocks(const Sys& s, int D);
int nm_blocks(const Sys& s, int D);
void launch_cart_update(const Sys& s, int D, int flags, const double* red_in, int nred_in, double* red_out,
                        StepRef step, int substep, int kick_nm, cudaStream_t st);
void launch_nm_thermo(const Sys& s, int D, const double* C, const double* T, int flags, const double* red_in,
                      int nred_in, double* red_out, StepRef step, int substep, cudaStream_t st);
// With `tw` (FFT twiddles) and `cm` (3 doubles of scratch), P = 32, 64, 128
// run the register-transform kernel; returns the number of kernels launched.
int launch_nm_propagate(const Sys& s, int D, const double* C, const double* T, const double* rot, int com_apply,
                        const double* red_in, int nred_in, const double2* tw, double* cm, cudaStream_t st);

// Fused normal-mode step (normal-mode propagator + normal-mode Langevin):
// mode bit 0 = tail of step-1 (kick, O, COM), bit 1 = head of step (O, COM,
// kick, rotation).  Cooperative launch; nm_fused_fits tells whether every
// block can be resident.
bool nm_fused_fits(const Sys& s, int D);
// whether the block kernel (any P) can be resident; the warp kernel (P = 32,
// 64, 128, with the FFT twiddles) is used whenever it can be
bool nm_block_fits(const Sys& s, int D);
// doubles of COM partial sums the fused step needs (cmpart)
size_t nm_fused_partials(const Sys& s, int D);
// `tw` (P/2 twiddles exp(-2 pi i t/P)) selects the FFT transforms (P a power
// of two, logP = log2 P); NULL selects the P x P matrix products.
// `modes` (may be null): buffers for the normal modes of p and x
// (nm_mode_doubles doubles each).  With the three-warp register kernel a
// launch with the head stores the modes its rotation produced (written is
// set), and with `use` the next launch takes p's (and, with the head, x's)
// from them instead of transforming the Cartesian arrays: valid only while
// nothing else has changed x or p.
struct NmModes {
    double2* p;
    double2* x;
    int use;
    mutable bool written;
};
size_t nm_mode_doubles(const Sys& s, int D);
cudaError_t launch_nm_fused(const Sys& s, int D, const double* C, const double* T, const double* rot, double* cmpart,
                            unsigned* bar, int mode, StepRef step, int fixcom, const double2* tw, int logP,
                            cudaStream_t st, const NmModes* modes = nullptr);

}  // namespace pimdb

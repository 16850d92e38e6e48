"""Throughput benchmark of the GB300 PIMD-B++ hot path: bead-steps/s
(N * P * MD steps per second).

Default workload (the second benchmark system of the project): N = 256
He-4-mass bosons, P = 64 beads, NDIM = 3, T = 1.5 K, Aziz HFDHE2 pair
potential with cutoff L/2 and minimum image in a periodic cube at number
density 0.0218 A^-3 (L = 22.7297 A), no external potential, normal-mode
propagator with the normal-mode Langevin thermostat, dt = 2 fs, FP64.

One bench "step" is one MD step of the whole ring polymer.  Synthetic inputs:
particle centres on the reference's "grid" placement (uniformParticleGrid,
src/simulation.cpp:133-193: a cubic grid of ceil(L / rho^(-1/3)) cells per
edge filled in order), shared by all beads, plus a 0.05 A per-bead Gaussian
jitter (seed 12345); Maxwell-Boltzmann momenta at the ring-polymer
temperature.  (Random placement at liquid density leaves pairs on the Aziz
wall, and the N = 4096 system heated up by orders of magnitude within tens of
steps from it.)

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload cfg2|cfg1|cfg3|cfg5] [--precision fp64|mixed]
                  [--batch-steps K4] [--no-batched] [--no-others]

The same JSON line carries:
- "systems": the other benchmark systems on the plain single-system path
  (N = 16 trap; N = 1024 2D dipole; N = 4096, P = 128 in FP64 and mixed),
  each with its mixed-precision force error against the FP64 path;
- "batched" / "batched_fp64": the batched-replica engine on the ensemble
  workload (512 independent replicas from default_rng(12345): N ~ U{8..128},
  P ~ U{16,32,64}, T ~ U[0.5,4] K, 3D bosons of mass 1 Da in a 3 meV
  harmonic trap with a 1 meV harmonic pair interaction (all pairs),
  cartesian velocity Verlet + Langevin, dt = 1 fs, replica seed 12345+r),
  K4 steps replayed as one CUDA graph, in mixed precision and in FP64, each
  with its roofline;
- "plain_fp64_same_ensemble": the same 512 replicas run one by one through
  the plain FP64 single-system path, the denominator of the batched
  engine's speed-up on the same work.

For N > 1 (torchrun) every rank runs its own replica (replicas only: the
bead ring of one system is never split across GPUs); value = all ranks'
bead-steps / max time.  --impl reference times the CPU oracle port on the
host cores (the reference's own binaries cannot be built on the GPU host).
"""
from __future__ import annotations

import argparse
import importlib
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

ANG = 1.8897261
KELVIN = 3.1668152e-06
MEV = 0.036749326e-3
DALTON = 1822.8885
FS = 4.1341373e16 * 1e-15
METRIC = "bead-steps/s (N·P·steps/s): plain FP64 vs mixed+batched at stated force error"

WORKLOADS = {
    "cfg2": dict(desc="N=256 He-4 bosons, P=64, 3D PBC, Aziz cutoff L/2 (min image), rho=0.0218/A^3 "
                      "(L=22.7297 A), T=1.5 K, normal-mode propagator + normal-mode Langevin, dt=2 fs",
                 ndim=3, natoms=256, nbeads=64, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=22.7297,
                 inter="aziz", int_p=(0, 0, 0), cutoff_ang=11.36485, ext="free", ext_p=(0, 0, 0),
                 propagator="normal_modes", nmthermostat=True, dt_fs=2.0, placement="grid", jitter_ang=0.05),
    "cfg1": dict(desc="N=16 bosons, P=32, 3D, harmonic trap 3 meV, free pair, VV + Langevin, dt=1 fs",
                 ndim=3, natoms=16, nbeads=32, T_K=1.0, mass_amu=1.0, pbc=False, box_ang=10.0, inter="free",
                 int_p=(0, 0, 0), cutoff_ang=-1.0, ext="harmonic", ext_p=(3.0 * MEV, 0, 0), propagator="cartesian",
                 nmthermostat=False, dt_fs=1.0, placement="uniform", jitter_ang=0.0),
    "cfg3": dict(desc="N=1024 bosons, P=32, 2D, dipole D=1 meV A^3 (no cutoff), harmonic trap 1 meV, "
                      "VV + Langevin, dt=1 fs", ndim=2, natoms=1024, nbeads=32, T_K=2.0, mass_amu=1.0, pbc=False,
                 box_ang=60.0, inter="dipole", int_p=(2.4799673e-4, 0, 0), cutoff_ang=-1.0, ext="harmonic",
                 ext_p=(1.0 * MEV, 0, 0), propagator="cartesian", nmthermostat=False, dt_fs=1.0,
                 placement="separated", min_sep_ang=1.0, jitter_ang=0.3),
    "cfg5": dict(desc="N=4096 He-4 bosons, P=128, 3D PBC, Aziz cutoff 7 A + double well, rho=0.0218/A^3 "
                      "(L=57.2754 A), T=1 K, normal-mode propagator, dt=2 fs", ndim=3, natoms=4096, nbeads=128,
                 T_K=1.0, mass_amu=4.0026, pbc=True, box_ang=57.2754, inter="aziz", int_p=(0, 0, 0), cutoff_ang=7.0,
                 ext="double_well", ext_p=(1.32684e-7 * MEV, 3.0 * ANG, 0), propagator="normal_modes",
                 nmthermostat=False, dt_fs=2.0, placement="grid", jitter_ang=0.05),
}


def max_over_ranks(x, dist, device="cuda"):
    """The largest of each rank's `x` (the slowest rank's time); `x` itself
    without a process group."""
    if not dist:
        return x
    import torch
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_workload(w, precision, rank):
    """Rank r runs its own replica: replica id r in the noise counter and
    initial state seed 12345 + r (no data is shared between ranks)."""
    cfg = workload_config(w, precision)
    cfg.replica = rank
    return cfg, initial_state(w, seed=12345 + rank)


def batched_workload(precision, n=512, seed=12345):
    """The ensemble workload: configs and initial states of `n` replicas."""
    pk = importlib.import_module("pimd-b_gb300")
    rng = np.random.default_rng(seed)
    Ns = rng.integers(8, 129, n)
    Ps = rng.choice([16, 32, 64], n)
    Ts = rng.uniform(0.5, 4.0, n)
    cfgs, xs, ps = [], [], []
    mass = 1.0 * DALTON
    for r in range(n):
        N, P, T = int(Ns[r]), int(Ps[r]), float(Ts[r])
        cfgs.append(pk.make_config(
            ndim=3, natoms=N, nbeads=P, bosonic=1, pbc=0, fixcom=1, propagator="cartesian", thermostat="langevin",
            nmthermostat=0, precision=precision, temperature=T * KELVIN, mass=mass, size=10.0 * ANG, dt=1.0 * FS,
            gamma=-1.0, ext_kind="harmonic", ext_params=(3.0 * MEV, 0, 0), int_kind="harmonic",
            int_params=(1.0 * MEV, 0, 0), cutoff=-1.0, seed=seed + r, replica=r))
        c = rng.uniform(-5.0 * ANG, 5.0 * ANG, (N, 3))
        xs.append(c[None] + rng.normal(0.0, 0.05 * ANG, (P, N, 3)))
        thermo_beta = 1.0 / (T * KELVIN) / P
        ps.append(rng.normal(0.0, math.sqrt(mass / thermo_beta), (P, N, 3)))
    return cfgs, xs, ps

# FP32 operations per ordered pair evaluation of the FP64 batch's
# double-float all-pairs harmonic loop (bead_pairs_df, counted from the
# source; FMA = 1): the separation (3 AccurateDWPlusDW, 60) and the gradient
# sum (3 DWTimesDW + 3 AccurateDWPlusDW, 81).  The batch evaluates every
# ordered pair (each unique pair twice).
DF_OPS_PER_BATCH_PAIR = 141

# The exchange's FP64 accounting per evaluation: about 19 N^2 FLOPs and
# 1.5 N^2 exponentials (cycle energies, both recursions, the exterior
# forces).  The recursions are sequential in their levels (N + 1 forward, N
# backward, the two directions side by side, one SM each), so the chain is
# reported as time per level, a latency bound, beside its FP64 rate.
EXCH_FLOP_PER_N2 = 19.0
EXCH_EXP_PER_N2 = 1.5


def exchange_latency(per_class_ms, N, fp64_peak_tflops):
    """The exchange chain of one step from the event-timed kernel classes
    (ms per step): its classes, ns per recursion level and its FP64 rate
    against the FP64 peak.  None when the step ran no exchange."""
    keys = sorted(k for k in per_class_ms if k.startswith("exch_"))
    if not keys or N < 1:
        return None
    chain = sum(per_class_ms[k] for k in keys)
    rec = per_class_ms.get("exch_recursions", 0.0)
    flops = EXCH_FLOP_PER_N2 * N * N
    rate = flops / (chain * 1e-3) / 1e12
    return {"chain_ms_per_step": chain, "classes": {k: per_class_ms[k] for k in keys},
            "levels_per_direction": N + 1, "ns_per_level": rec * 1e6 / (N + 1),
            "fp64_flop_per_step": flops, "exp_per_step": EXCH_EXP_PER_N2 * N * N,
            "fp64_tflops": rate, "vs_fp64_peak": rate / fp64_peak_tflops,
            "bound": "latency: the recursions are sequential in their levels",
            "note": "each class event-timed on its own; in a step the chain overlaps the pair kernel"}


def batched_roofline(cfgs, t_step, precision, peaks):
    """The ensemble step against its roofline, by the accounting of the
    project: t_ideal = B / BW + t_pair + F_exch / peak_FP64 with B = 6 d 8
    bytes per bead-particle (x, p, f read and written) and F_exch = 19 N^2
    FP64 FLOPs per replica (its 1.5 N^2 + 0.5 N^2 exponentials are counted
    apart).  Pairs: mixed precision, 17 FLOPs per unique harmonic pair and
    bead (FMA = 2) against the FP32 FMA peak; FP64, the double-float loop's
    141 FP32 operations per ordered pair against the FP32 issue rate (half
    the FMA peak in FLOP/s), with the FP64-equivalent 17 FLOPs per unique
    pair against the FP64 peak beside it.  frac = t_ideal / t_measured."""
    units = sum(c.natoms * c.nbeads for c in cfgs)
    B = 6 * 3 * 8 * units
    F_pair = sum(17 * c.nbeads * c.natoms * (c.natoms - 1) // 2 for c in cfgs)
    ordered = sum(c.nbeads * c.natoms * (c.natoms - 1) for c in cfgs)
    F_exch = sum(19 * c.natoms ** 2 for c in cfgs)
    exps = sum(2 * c.natoms ** 2 for c in cfgs)
    bw = peaks["hbm_gbs"] * 1e9
    p64 = peaks["fp64_tflops"] * 1e12
    p32 = peaks["fp32_tflops"] * 1e12
    if precision == "mixed":
        t_pair, pair_bound = F_pair / p32, "fp32 pipe (pairs)"
    else:
        t_pair, pair_bound = ordered * DF_OPS_PER_BATCH_PAIR / (0.5 * p32), "fp32 pipe (double-float pairs)"
    t_ideal = B / bw + t_pair + F_exch / p64
    out = {"bound": "fp64 pipe (exchange) + " + pair_bound + " + hbm",
           "t_ideal_ms": 1e3 * t_ideal, "t_measured_ms": 1e3 * t_step, "frac": t_ideal / t_step,
           "streaming_bytes_per_step": B, "pair_flops_per_step": F_pair, "exchange_flops_per_step": F_exch,
           "exchange_exps_per_step": exps,
           "peaks": {"hbm_gbs": peaks["hbm_gbs"], "fp64_tflops": peaks["fp64_tflops"],
                     "fp32_tflops": peaks["fp32_tflops"]},
           "peak_source": "HBM: MEASURED_PEAKS.json; FP64 and FP32: FMA probes measured in this run "
                          "(MEASURED_PEAKS.json has neither)"}
    if precision != "mixed":
        out["pair_fp32_ops_per_step"] = ordered * DF_OPS_PER_BATCH_PAIR
        t_eq = B / bw + F_pair / p64 + F_exch / p64
        out["fp64_equivalent"] = {"t_ideal_ms": 1e3 * t_eq, "frac": t_eq / t_step,
                                  "accounting": "the same FLOPs with the pairs on the FP64 pipe; above 1: the "
                                                "pair arithmetic no longer runs there"}
    return out


def run_batched(pk, torch, stream, K, W, rank, world, dist, precision, peaks, e2e=True, ref_forces=None):
    """The batched ensemble: device-timed replay of one CUDA graph of K steps;
    for mixed precision also the force error against the FP64 batch and an
    end-to-end run through the C ABI."""
    cfgs, xs, ps = batched_workload(precision)
    units = sum(c.natoms * c.nbeads for c in cfgs)
    out = {}
    with pk.Batch(cfgs, stream=stream.cuda_stream) as b:
        b.set_states(xs, ps)
        b.compute_forces()
        f = b.get_states(flat=True)[2]
        if ref_forces is not None:
            errs = [float(np.linalg.norm(f[b.offsets[r]:b.offsets[r + 1]] - ref_forces[b.offsets[r]:b.offsets[r + 1]])
                          / np.linalg.norm(ref_forces[b.offsets[r]:b.offsets[r + 1]])) for r in range(len(cfgs))]
            out["force_error"] = {
                "max_norm_rel": max(errs), "median_norm_rel": float(np.median(errs)),
                "against": "the FP64 batch on the same coordinates; tests/test_baseline_sizes.py checks every "
                           "replica of both against the FP64 oracle (FP64 within 1e-10 per bead, mixed within 1e-6)"}
        threads, ctas = b.autotune(steps=3)
        b.step_async(max(W, 3))
        b.synchronize()
        b.step_async(K)  # instantiates the graph of K steps
        b.synchronize()
        launches0 = b.launch()["launches"]
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        b.step_async(K)
        ev1.record(stream)
        torch.cuda.synchronize()
        b.synchronize()
        t = max_over_ranks(ev0.elapsed_time(ev1) / 1e3, dist)
        launches = b.launch()["launches"] - launches0
        if e2e:
            # end to end: pinned host state in, one step, state and forces out
            n = int(b.offsets[-1])
            hx = torch.empty(n, dtype=torch.float64, pin_memory=True)
            hp = torch.empty(n, dtype=torch.float64, pin_memory=True)
            hf = torch.empty(n, dtype=torch.float64, pin_memory=True)
            hx.numpy()[:] = b.flatten(xs)
            hp.numpy()[:] = b.flatten(ps)
            Ke = 20
            lib = pk.lib()
            ptr = lambda a: pk.C.c_void_p(a.data_ptr())
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(Ke):
                b._c(lib.pimdb_batch_set_states(b._b, ptr(hx), ptr(hp)))
                b.step(1)
                b._c(lib.pimdb_batch_get_states(b._b, ptr(hx), ptr(hp), ptr(hf)))
            te = max_over_ranks(time.perf_counter() - t0, dist)
            out["e2e"] = {"value": world * units * Ke / te, "unit": "bead-steps/s", "h2d_bytes_per_step": 2 * n * 8,
                          "d2h_bytes_per_step": 3 * n * 8, "steps": Ke}
    out.update({
        "value": world * units * K / t, "unit": "bead-steps/s", "ms_per_step": 1e3 * t / K, "steps": K,
        "replicas": len(cfgs), "bead_particles": units,
        "precision": ("mixed (FP32 pair forces, FP64 accumulation, exchange and integrator)" if precision == "mixed"
                      else "fp64"),
        "launch": {"threads": threads, "ctas_per_sm": ctas, "graph": "one CUDA graph of K step launches",
                   "autotuned": True},
        "gpu_launches": launches, "l2": "not flushed inside the graph; working set 140+ MB > 129 MB L2",
        "workload": "512 replicas, N~U{8..128}, P~U{16,32,64}, T~U[0.5,4] K, 3D bosons, mass 1 Da, harmonic "
                    "trap 3 meV + harmonic pair 1 meV (all pairs), no PBC, cartesian VV + Langevin, dt=1 fs",
        "roofline": batched_roofline(cfgs, t / K, precision, peaks)})
    return out


def batched_fp64_forces(pk, stream):
    cfgs, xs, ps = batched_workload("fp64")
    with pk.Batch(cfgs, stream=stream.cuda_stream) as b:
        b.set_states(xs, ps)
        b.compute_forces()
        return b.get_states(flat=True)[2]


def run_ensemble_single(pk, torch, stream, K, W):
    """The plain FP64 single-system path on the ensemble workload: every
    replica through its own handle (pimdb_step), one after another, each a
    K-step graph replay timed with events after W warm-up steps.  value =
    all replicas' bead-steps / the summed device time."""
    cfgs, xs, ps = batched_workload("fp64")
    tot, units = 0.0, 0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches = 0
    for r, c in enumerate(cfgs):
        with pk.System(c, stream=stream.cuda_stream) as g:
            g.set_state(xs[r], ps[r])
            g.step_async(max(W, 1))
            g.step_async(K)  # captures the K-step graph
            g.synchronize()
            g.profile(0)
            torch.cuda.synchronize()
            ev0.record(stream)
            g.step_async(K)
            ev1.record(stream)
            torch.cuda.synchronize()
            g.synchronize()
            launches += g.profile(-1)["launches"]
            tot += ev0.elapsed_time(ev1) / 1e3
            units += c.natoms * c.nbeads * K
    return {"value": units / tot, "unit": "bead-steps/s", "ms_per_step": 1e3 * tot / K, "steps": K,
            "replicas": len(cfgs), "precision": "fp64", "gpu_launches": launches,
            "how": "each replica alone through pimdb_step (a K-step CUDA graph per handle), replicas one after "
                   "another; summed device time"}


def workload_config(w, precision):
    pk = importlib.import_module("pimd-b_gb300")
    return pk.make_config(
        ndim=w["ndim"], natoms=w["natoms"], nbeads=w["nbeads"], bosonic=1, pbc=int(w["pbc"]), fixcom=1,
        propagator=w["propagator"], thermostat="langevin", nmthermostat=int(w["nmthermostat"]), precision=precision,
        temperature=w["T_K"] * KELVIN, mass=w["mass_amu"] * DALTON, size=w["box_ang"] * ANG, dt=w["dt_fs"] * FS,
        gamma=-1.0, ext_kind=w["ext"], ext_params=w["ext_p"], int_kind=w["inter"], int_params=w["int_p"],
        cutoff=w["cutoff_ang"] * ANG, seed=12345, replica=0)


def grid_centres(N, D, L, pbc):
    """The reference's "grid" initial positions (Simulation::
    uniformParticleGrid, src/simulation.cpp:133-193): ceil(L / side - 1e-7)
    cells per edge with side = (N / L^D)^(-1/D), particles at the cell
    centres in row-major cell order, wrapped by the minimum image under PBC."""
    side = (N / L ** D) ** (-1.0 / D)
    n = max(int(math.ceil(L / side - 1.0e-7)), 1)
    if n ** D < N:
        raise ValueError("Number of grid boxes is less than the number of particles")
    cell = L / n
    idx = np.arange(N)
    out = np.empty((N, D))
    for a in range(D):
        out[:, a] = ((idx // n ** (D - 1 - a)) % n + 0.5) * cell - 0.5 * L
    if pbc:
        out -= L * np.floor(out / L + 0.5)
    return out


def initial_state(w, seed=12345):
    rng = np.random.default_rng(seed)
    N, P, D = w["natoms"], w["nbeads"], w["ndim"]
    L = w["box_ang"] * ANG
    if w["placement"] == "grid":
        centres = grid_centres(N, D, L, w["pbc"])
    else:
        # uniform in the box; "separated": random sequential addition keeping
        # centres min_sep apart (minimum image under PBC)
        dmin = w.get("min_sep_ang", 0.0) * ANG if w["placement"] == "separated" else 0.0
        pts = []
        while len(pts) < N:
            c = rng.uniform(-0.5 * L, 0.5 * L, D)
            if dmin > 0 and pts:
                d = np.asarray(pts) - c
                if w["pbc"]:
                    d -= L * np.floor(d / L + 0.5)
                if np.min(np.einsum("ij,ij->i", d, d)) < dmin * dmin:
                    continue
            pts.append(c)
        centres = np.asarray(pts)
    x = centres[None] + rng.normal(0.0, w["jitter_ang"] * ANG, (P, N, D))
    m = w["mass_amu"] * DALTON
    thermo_beta = 1.0 / (w["T_K"] * KELVIN) / P
    p = rng.normal(0.0, math.sqrt(m / thermo_beta), (P, N, D))
    return x, p

# FLOPs of one pair's force (FMA = 2): Aziz 63, dipole 16 (2D) or 20 (3D),
# harmonic 17, plus 9 for the minimum image under PBC; transcendentals
# (square root, reciprocal, exponential, division) counted apart.  A pair
# only tested against the cutoff costs 15 FLOPs with the minimum image, 6
# without.
PAIR_FLOPS = {"aziz": 63, "harmonic": 17, "free": 0}
PAIR_TRANSC = {"aziz": 4, "dipole": 1, "harmonic": 0, "free": 0}


def pair_work(w, x):
    """Algorithmic work of one pair-force evaluation (all beads) of
    workload w at positions x: unique pairs, pairs inside the cutoff, FLOPs
    with every unique pair priced at the full force (the project's
    accounting), FLOPs with only the pairs inside the cutoff priced at the
    force and the others at the test, and the transcendental count."""
    if w["inter"] == "free":
        return None
    per = PAIR_FLOPS.get(w["inter"], 16 if w["ndim"] == 2 else 20) + (9 if w["pbc"] else 0)
    tested = 15 if w["pbc"] else 6
    N, P = w["natoms"], w["nbeads"]
    L = w["box_ang"] * ANG
    cut = w["cutoff_ang"] * ANG
    inside = 0
    iu = np.triu_indices(N, 1)
    for b in range(P):
        d = x[b][iu[0]] - x[b][iu[1]]
        if w["pbc"]:
            d -= L * np.floor(d / L + 0.5)
        r2 = np.einsum("ij,ij->i", d, d)
        inside += int(np.sum(r2 < cut * cut)) if cut > 0 else len(r2)
    pairs = P * N * (N - 1) // 2
    return {"pairs": pairs, "inside": inside, "flops_all": float(pairs * per),
            "flops_in_cutoff": float(pairs * tested + inside * (per - (9 if w["pbc"] else 0))),
            "transcendentals_in_cutoff": inside * PAIR_TRANSC[w["inter"]], "per_pair": per}

# FP32 operations of the double-float Aziz pair evaluation, counted from the
# source (pimd-b_gb300/csrc/forces.cu compact_tile, aziz_df.cuh, dfloat.cuh):
# separation 76, gradient scale 248 (1/sqrt 21, |r| 9, exponent argument
# 29, exp 81, powers, polynomial and the two terms 108), gradient 27, the
# i- and j-side sums 66; the FP32 screen costs about 12 per tested pair.
DF_OPS_PER_PAIR = 417
SCREEN_OPS_PER_PAIR = 12
# One k_pair_tiles_compact launch on the benchmark system (ncu --set full,
# profiles/pair_tiles_compact_aziz_pbc_N256_P64_fp64.md): DRAM bytes read +
# written, pipe utilisation over active cycles, warps active and
# warp-instructions issued per SM cycle (of 4).
PAIR_NCU = {"dram_bytes": 475648, "fma_pipe_active": 0.320, "alu_pipe_active": 0.196, "warps_active": 0.164,
            "issue_per_sm_cycle": 1.98, "duration_us_cold": 62.5}


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.path = Path(tempfile.mkstemp(prefix="clocks_", suffix=".csv")[1])
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        rows = [ln.split(", ") for ln in self.path.read_text().splitlines() if ln.strip()]
        self.path.unlink(missing_ok=True)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if len(r) > 5 + k and r[5 + k].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(w, seconds=12.0, nthreads=None):
    """The oracle port (FP64, reference operation order) on the host cores,
    over a bounded sample of MD steps of the same workload."""
    from oracle import oracle as O
    nthreads = nthreads or os.cpu_count() or 1
    s = O.make_system(ndim=w["ndim"], natoms=w["natoms"], nbeads=w["nbeads"], temperature=w["T_K"] * KELVIN,
                      mass=w["mass_amu"] * DALTON, bosonic=True, pbc=w["pbc"], size=w["box_ang"] * ANG, fixcom=True,
                      propagator=w["propagator"], thermostat="langevin", nmthermostat=w["nmthermostat"],
                      dt=w["dt_fs"] * FS, ext=w["ext"], ext_p=w["ext_p"], interaction=w["inter"], int_p=w["int_p"],
                      cutoff=w["cutoff_ang"] * ANG)
    x, p = initial_state(w)
    tr = O.Trajectory(s, x, p)
    steps = 0
    t0 = time.perf_counter()
    while True:
        xi = O.philox_noise_device(12345, 0, steps, s.nbeads, s.natoms, s.ndim)
        tr.step(xi, nthreads=nthreads)
        steps += 1
        el = time.perf_counter() - t0
        if (el >= seconds and steps >= 2) or steps >= 100000:
            break
    value = w["natoms"] * w["nbeads"] * steps / el
    return {"value": value, "unit": "bead-steps/s", "cores": nthreads, "kind": "port", "cpu": host_cpu(),
            "sample": f"{steps} MD steps of the same workload ({el:.1f} s), FP64 oracle port with the "
                      f"per-bead force loops on {nthreads} POSIX threads"}


def run_reference(args, w, rank, world):
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    W = max(args.warmup, 0)
    K = max(args.steps, 1)
    nthreads = os.cpu_count() or 1
    s = O.make_system(ndim=w["ndim"], natoms=w["natoms"], nbeads=w["nbeads"], temperature=w["T_K"] * KELVIN,
                      mass=w["mass_amu"] * DALTON, bosonic=True, pbc=w["pbc"], size=w["box_ang"] * ANG, fixcom=True,
                      propagator=w["propagator"], thermostat="langevin", nmthermostat=w["nmthermostat"],
                      dt=w["dt_fs"] * FS, ext=w["ext"], ext_p=w["ext_p"], interaction=w["inter"], int_p=w["int_p"],
                      cutoff=w["cutoff_ang"] * ANG)
    x, p = initial_state(w)
    tr = O.Trajectory(s, x, p)
    for st in range(W):
        tr.step(O.philox_noise_device(12345, 0, st, s.nbeads, s.natoms, s.ndim), nthreads=nthreads)
    noise = [O.philox_noise_device(12345, 0, W + k, s.nbeads, s.natoms, s.ndim) for k in range(K)]
    t0 = time.perf_counter()
    for k in range(K):
        tr.step(noise[k], nthreads=nthreads)
    el = time.perf_counter() - t0
    value = w["natoms"] * w["nbeads"] * K / el
    line = {"metric": METRIC, "value": value, "unit": "bead-steps/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": 1e3 * el / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": w["desc"], "precision": "fp64"},
            "cpu_baseline": {"value": value, "unit": "bead-steps/s", "cores": nthreads, "kind": "port",
                             "cpu": host_cpu(),
                             "sample": f"{K} MD steps after {W} warm-up steps, FP64 oracle port of the reference "
                                       f"(the reference's own build needs its sources, absent on the GPU host)"},
            "e2e": {"value": value, "unit": "bead-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def time_single(pk, torch, stream, w, precision, K, W, dist, rank, world, sampler=None, profile=False):
    """One system of workload w through the plain single-system path: W
    warm-up steps, then K steps each bracketed by events on the library's
    stream (L2 flushed before each one when the working set fits in twice
    the L2).  Returns the timing, launch count and optionally per-kernel
    device times, plus the handle and initial state for further use."""
    cfg, (x0, p0) = rank_workload(w, precision, rank)
    N, P, D = w["natoms"], w["nbeads"], w["ndim"]
    sysm = pk.System(cfg, stream=stream.cuda_stream)
    sysm.set_state(x0, p0)
    # warm-up as single steps, like the timed loop: the step graphs are
    # captured here, outside the timed region
    for _ in range(W):
        sysm.step_async(1)
    sysm.synchronize()
    ld = (N + 31) // 32 * 32
    ws = 4 * P * D * ld * 8 + 4 * N * (N + 1) // 2 * 8
    do_flush = ws <= 2 * 129e6
    l2_note = ("flushed before every timed step (512 MiB write, outside the step's events)" if do_flush else
               f"not flushed: working set {ws / 1e6:.0f} MB (state and exchange arrays) > 2 x 129 MB L2")
    flush = torch.empty(512 * 1024 * 1024 // 4 if do_flush else 1, dtype=torch.float32, device="cuda")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    for k in range(K):
        if do_flush:
            flush.zero_()
        ev[k][0].record(stream)
        sysm.step_async(1)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    sysm.synchronize()
    clocks = sampler.stop() if sampler else None
    del flush
    step_ms = [a.elapsed_time(b) for a, b in ev]
    tot_s = max_over_ranks(sum(step_ms) / 1e3, dist)
    # kernel launches in the timed region: the same K steps, counted.  Each
    # untimed block restarts from the initial state, so no run goes far past
    # W + K steps (the 2D dipole system is not stable over thousands)
    sysm.set_state(x0, p0)
    sysm.profile(0)
    sysm.step_async(K)
    sysm.synchronize()
    launches = sysm.profile(-1)["launches"]
    prof = None
    if profile:
        # per-kernel device times (events around each launch on the library stream)
        sysm.set_state(x0, p0)
        sysm.profile(1)
        sysm.step_async(K)
        sysm.synchronize()
        prof = sysm.profile(-1)
        sysm.profile(0)
    res = {"value": world * N * P * K / tot_s, "unit": "bead-steps/s", "ms_per_step": 1e3 * tot_s / K, "steps": K,
           "warmup": W, "gpu_launches": launches, "l2": l2_note, "precision": precision, "workload": w["desc"]}
    return res, sysm, (x0, p0), prof, clocks


def forces_of(pk, stream, w, precision, x):
    cfg = workload_config(w, precision)
    with pk.System(cfg, stream=stream.cuda_stream) as g:
        g.set_state(x, np.zeros_like(x))
        g.compute_forces()
        return g.get_state()[2]


def run_other_systems(pk, torch, stream, K, W, dist, rank, world):
    """The other benchmark systems on the plain single-system path: the
    N = 16 trap, the N = 1024 2D dipole system and the N = 4096 system in
    FP64 and in mixed precision, each with its mixed-precision force error
    against the FP64 path on its initial state."""
    out = {}
    for name, precs in (("cfg1", ("fp64",)), ("cfg3", ("fp64",)), ("cfg5", ("fp64", "mixed"))):
        w = WORKLOADS[name]
        x0 = initial_state(w)[0]
        f64 = forces_of(pk, stream, w, "fp64", x0)
        fmx = forces_of(pk, stream, w, "mixed", x0)
        err = float(np.linalg.norm(fmx - f64) / np.linalg.norm(f64))
        for prec in precs:
            Ks = min(K, 100)
            res, sysm, _, prof, _ = time_single(pk, torch, stream, w, prec, Ks, W, dist, rank, world, profile=True)
            sysm.close()
            ms, cnt = prof["ms"], prof["counts"]
            res["per_class_ms_per_step"] = {k: v / Ks for k, v in ms.items() if v > 0}
            res["force_error_mixed_vs_fp64"] = err
            res["parity"] = ("FP64 forces, exchange and 5-step trajectories of this initial state match the oracle "
                             "within 1e-10 / 1e-9 (tests/test_baseline_sizes.py); mixed within 1e-6")
            out[f"{name}_{prec}"] = res
    return out


def host_cpu():
    model = ""
    try:
        for ln in Path("/proc/cpuinfo").read_text().splitlines():
            if ln.lower().startswith("model name"):
                model = ln.split(":", 1)[1].strip()
                break
        if not model:
            r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
            for ln in r.stdout.splitlines():
                if ln.startswith("Model name"):
                    model = ln.split(":", 1)[1].strip()
                    break
    except Exception:
        pass
    import platform
    return {"model": model or "unknown", "arch": platform.machine(), "logical_cpus": os.cpu_count()}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cfg2", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-only", action="store_true", help="short run for an ncu capture")
    ap.add_argument("--batch-steps", type=int, default=1000)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-others", action="store_true", help="skip the other benchmark systems")
    ap.add_argument("--profile-only-batched", action="store_true",
                    help="short run of the batched ensemble only (plain launches) for an ncu capture")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, w, rank, world)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    pk = importlib.import_module("pimd-b_gb300")
    # a dedicated stream: the library launches on it and the events below are
    # recorded on it (the legacy default stream has handle 0, which the C ABI
    # reads as "create your own stream")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    if args.profile_only_batched:
        cfgs, xs, ps = batched_workload("mixed")
        with pk.Batch(cfgs, stream=stream.cuda_stream) as b:
            b.set_option("graph", 0)
            b.set_states(xs, ps)
            b.step(max(args.warmup, 1) + max(args.steps, 1))
        return
    W = max(args.warmup, 3)
    K = max(args.steps, 1)
    if args.profile_only:
        cfg, (x0, p0) = rank_workload(w, args.precision, rank)
        with pk.System(cfg, stream=stream.cuda_stream) as sysm:
            sysm.set_state(x0, p0)
            for _ in range(W):
                sysm.step_async(1)
            sysm.step_async(K)
            sysm.synchronize()
        return

    N, P, D = w["natoms"], w["nbeads"], w["ndim"]
    units = N * P
    sampler = ClockSampler(local) if rank == 0 else None
    head, sysm, (x0, p0), prof, clocks = time_single(pk, torch, stream, w, args.precision, K, W, dist, rank, world,
                                                     sampler=sampler, profile=True)
    value = head["value"]

    # end to end through the C ABI (pimdb_step_io) with pinned host buffers
    shape = (P, N, D)
    hx = torch.empty(shape, dtype=torch.float64, pin_memory=True)
    hp = torch.empty(shape, dtype=torch.float64, pin_memory=True)
    hf = torch.empty(shape, dtype=torch.float64, pin_memory=True)
    sysm.set_state(x0, p0)
    sysm.step(W)
    sysm.get_state_ptr(hx.data_ptr(), hp.data_ptr(), None, device=False)
    Ke = max(1, min(K // 2, 200))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(Ke):
        # pimdb_step_io: x, p in; one step; x, p, f out; one synchronisation
        sysm.step_io_ptr(hx.data_ptr(), hp.data_ptr(), 1, hx.data_ptr(), hp.data_ptr(), hf.data_ptr())
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
    e2e = {"value": world * units * Ke / e2e_s, "unit": "bead-steps/s", "h2d_bytes_per_step": 2 * P * N * D * 8,
           "d2h_bytes_per_step": 3 * P * N * D * 8, "steps": Ke}
    sysm.close()

    fp64_peak = pk.measure_fp64_peak()
    fp32_peak = pk.measure_fp32_peak()
    peaks = {"hbm_gbs": 6800.0, "hbm_source": "fallback"}
    try:
        mp = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        peaks = {"hbm_gbs": float(mp["hbm_gbs"]), "hbm_source": "MEASURED_PEAKS.json"}
    except Exception:
        pass
    peaks.update(fp64_tflops=fp64_peak, fp32_tflops=fp32_peak)

    others = None if args.no_others else run_other_systems(pk, torch, stream, K, W, dist, rank, world)
    batched = batched64 = plain_ens = None
    if not args.no_batched:
        Kb = max(args.batch_steps, 1)
        f64 = batched_fp64_forces(pk, stream)
        batched = run_batched(pk, torch, stream, Kb, W, rank, world, dist, "mixed", peaks, ref_forces=f64)
        batched64 = run_batched(pk, torch, stream, Kb, W, rank, world, dist, "fp64", peaks, e2e=False)
        plain_ens = run_ensemble_single(pk, torch, stream, min(K, 20), W)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    # roofline of the dominant kernel class
    ms, cnt = prof["ms"], prof["counts"]
    dom = max(ms, key=lambda k: ms[k])
    dom_ms = ms[dom] / max(cnt[dom], 1)
    roof = {"kernel": dom, "kernel_share": ms[dom] / max(sum(ms.values()), 1e-30), "launch_ms": dom_ms,
            "per_class_ms_per_step": {k: v / K for k, v in ms.items() if v > 0}}
    work = pair_work(w, x0) if dom == "bead_forces" else None
    dfpath = work is not None and args.precision == "fp64" and w["inter"] == "aziz" and w["cutoff_ang"] > 0
    if work and dfpath:
        # The FP64 Aziz pair tiles evaluate in double-float on the FP32 pipe:
        # their roofline is the FP32 issue rate.  Algorithmic FP32 operations
        # per launch: DF_OPS_PER_PAIR per pair inside the cutoff (separation,
        # gradient scale, gradient and the two sums in double-float) plus
        # SCREEN_OPS_PER_PAIR per tested pair (the FP32 screen); the FP32
        # peak in operations is the FMA probe's FLOP rate / 2.
        t = dom_ms * 1e-3
        ops = work["inside"] * DF_OPS_PER_PAIR + work["pairs"] * SCREEN_OPS_PER_PAIR
        peak_ops = fp32_peak / 2.0
        ncu = PAIR_NCU if args.workload == "cfg2" else None
        roof.update({
            "bound": "fp32 pipe (double-float arithmetic)",
            "achieved": ops / t / 1e12, "peak": peak_ops, "unit": "T FP32 operations/s",
            "frac": ops / t / 1e12 / peak_ops,
            "algorithmic": (f"{ops:.4g} FP32 operations per launch: {work['inside']} pairs inside the cutoff x "
                            f"{DF_OPS_PER_PAIR} (double-float separation, Aziz gradient scale, gradient, i and j "
                            f"sums) + {work['pairs']} tested pairs x {SCREEN_OPS_PER_PAIR} (FP32 screen)"),
            "fp64_equivalent": {
                "achieved_tflops": work["flops_all"] / t / 1e12, "fp64_peak_tflops": fp64_peak,
                "vs_fp64_peak": work["flops_all"] / t / 1e12 / fp64_peak,
                "accounting": (f"{work['flops_all']:.4g} FLOP per launch: {work['pairs']} unique pairs x "
                               f"{work['per_pair']} FLOP (force with minimum image, FMA = 2); above 1: the "
                               f"arithmetic no longer runs on the FP64 pipe"),
                "in_cutoff_tflops": work["flops_in_cutoff"] / t / 1e12},
            "transcendentals_per_launch": work["transcendentals_in_cutoff"],
            "ncu": ncu,
            "traffic": ncu["dram_bytes"] if ncu else None,
            "traffic_unit": "DRAM bytes per launch (ncu capture)" if ncu else None,
            "peak_source": "FP32 FMA probe measured in this run (MEASURED_PEAKS.json has no FP32 entry)"})
    elif work:
        t = dom_ms * 1e-3
        peak = fp64_peak if args.precision == "fp64" else fp32_peak
        roof.update({
            "bound": "fp64" if args.precision == "fp64" else "fp32",
            "achieved": work["flops_all"] / t / 1e12, "peak": peak, "unit": "TFLOP/s",
            "frac": work["flops_all"] / t / 1e12 / peak,
            "algorithmic": (f"{work['flops_all']:.4g} FLOP per launch: {work['pairs']} unique pairs x "
                            f"{work['per_pair']} FLOP (force with minimum image, FMA = 2)"),
            "achieved_in_cutoff": work["flops_in_cutoff"] / t / 1e12,
            "frac_in_cutoff": work["flops_in_cutoff"] / t / 1e12 / peak,
            "transcendentals_per_launch": work["transcendentals_in_cutoff"], "traffic": None,
            "peak_source": ("FP64 FMA probe measured in this run (MEASURED_PEAKS.json has no FP64 entry)"
                            if args.precision == "fp64" else "FP32 FMA probe measured in this run")})
    else:
        bytes_per = 6 * 8 * units * D
        ach = bytes_per / (dom_ms * 1e-3) / 1e9
        roof.update({"bound": "hbm", "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": ach / peaks["hbm_gbs"], "traffic": None, "peak_source": peaks["hbm_source"]})
    line = {"metric": METRIC, "value": value, "unit": "bead-steps/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32 pair forces / f64 exchange and integrator",
            "data": "synthetic",
            "config": {"workload": w["desc"], "natoms": N, "nbeads": P, "ndim": D, "precision": args.precision,
                       "init": "grid placement (reference uniformParticleGrid) + 0.05 A jitter"
                       if w["placement"] == "grid" else w["placement"],
                       "parallelism": f"replicas x{world}" if world > 1 else "single system",
                       "l2": head["l2"]},
            "e2e": e2e, "roofline": roof, "gpu_launches": head["gpu_launches"], "clocks": clocks,
            "peaks": peaks}
    xl = exchange_latency(roof["per_class_ms_per_step"], N, fp64_peak)
    if xl:
        line["exchange"] = xl
    if others:
        line["systems"] = others
    if batched:
        batched["vs_batched_fp64"] = batched["value"] / batched64["value"]
        batched["vs_plain_fp64_same_ensemble"] = batched["value"] / plain_ens["value"]
        batched64["vs_plain_fp64_same_ensemble"] = batched64["value"] / plain_ens["value"]
        batched["vs_plain_fp64_benchmark_system"] = batched["value"] / value if args.precision == "fp64" else None
        line["batched"] = batched
        line["batched_fp64"] = batched64
        line["plain_fp64_same_ensemble"] = plain_ens
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, seconds=args.cpu_seconds)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

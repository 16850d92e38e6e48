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
                  [--batch-steps K4] [--no-batched]

The same JSON line carries a "batched" object: the batched-replica engine on
the ensemble workload (512 independent replicas from default_rng(12345):
N ~ U{8..128}, P ~ U{16,32,64}, T ~ U[0.5,4] K, 3D bosons of mass 1 Da in a
3 meV harmonic trap with a 1 meV harmonic pair interaction (all pairs),
cartesian velocity Verlet + Langevin, dt = 1 fs, replica seed 12345+r), in
mixed precision, K4 steps replayed as one CUDA graph; its force error is
measured against the engine's FP64 path on the same coordinates.

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


def run_batched(pk, torch, stream, K, W, rank, world, dist):
    """Mixed-precision batched ensemble: device-timed graph replay, force
    error against the FP64 path, and an end-to-end run through the C ABI."""
    cfgs, xs, ps = batched_workload("mixed")
    c64, _, _ = batched_workload("fp64")
    units = sum(c.natoms * c.nbeads for c in cfgs)
    with pk.Batch(c64, stream=stream.cuda_stream) as b64, pk.Batch(cfgs, stream=stream.cuda_stream) as b:
        b64.set_states(xs, ps)
        b64.compute_forces()
        f64 = b64.get_states(flat=True)[2]
        b.set_states(xs, ps)
        b.compute_forces()
        f32 = b.get_states(flat=True)[2]
        errs = []
        for r in range(len(cfgs)):
            lo, hi = b.offsets[r], b.offsets[r + 1]
            errs.append(float(np.linalg.norm(f32[lo:hi] - f64[lo:hi]) / np.linalg.norm(f64[lo:hi])))
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
    return {"value": world * units * K / t, "unit": "bead-steps/s", "ms_per_step": 1e3 * t / K, "steps": K,
            "replicas": len(cfgs), "bead_particles": units, "precision": "mixed (FP32 pair forces, FP64 accumulation, "
            "exchange and integrator)",
            "force_error": {"max_norm_rel": max(errs), "median_norm_rel": float(np.median(errs)),
                            "against": "the engine's FP64 path on the same coordinates (which matches the FP64 "
                                       "oracle within 1e-10)"},
            "launch": {"threads": threads, "ctas_per_sm": ctas, "graph": "one CUDA graph of K step launches",
                       "autotuned": True},
            "gpu_launches": launches, "l2": "not flushed inside the graph; working set 140+ MB > 129 MB L2",
            "e2e": {"value": world * units * Ke / te, "unit": "bead-steps/s", "h2d_bytes_per_step": 2 * n * 8,
                    "d2h_bytes_per_step": 3 * n * 8, "steps": Ke},
            "workload": "512 replicas, N~U{8..128}, P~U{16,32,64}, T~U[0.5,4] K, 3D bosons, mass 1 Da, harmonic "
                        "trap 3 meV + harmonic pair 1 meV (all pairs), no PBC, cartesian VV + Langevin, dt=1 fs"}


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


def pair_flops(w, x):
    """Algorithmic FLOPs of one evaluation of the pair kernel: every unique
    pair costs the separation test (15 FLOPs with the minimum image); pairs
    inside the cutoff add the gradient.  Aziz: 63 arithmetic + sqrt + 3
    divisions (10 each) + 2 exp (20 each) = 133; dipole: 8 + sqrt + div = 28;
    harmonic: 6."""
    per_in = {"aziz": 133, "dipole": 28, "harmonic": 6, "free": 0}[w["inter"]]
    if w["inter"] == "free":
        return 0.0, 0
    N, P = w["natoms"], w["nbeads"]
    L = w["box_ang"] * ANG
    cut = w["cutoff_ang"] * ANG
    inside = 0
    for b in range(P):
        d = x[b][:, None, :] - x[b][None, :, :]
        if w["pbc"]:
            d -= L * np.floor(d / L + 0.5)
        r = np.sqrt(np.einsum("ijk,ijk->ij", d, d))
        iu = np.triu_indices(N, 1)
        inside += int(np.sum(r[iu] < cut)) if cut > 0 else len(iu[0])
    pairs = P * N * (N - 1) // 2
    return float(pairs * 15 + inside * per_in), inside


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
    return {"value": value, "unit": "bead-steps/s", "cores": nthreads, "kind": "port",
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
                             "sample": f"{K} MD steps after {W} warm-up steps, FP64 oracle port of the reference "
                                       f"(the reference's own build needs its sources, absent on the GPU host)"},
            "e2e": {"value": value, "unit": "bead-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


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
    cfg, (x0, p0) = rank_workload(w, args.precision, rank)
    N, P, D = w["natoms"], w["nbeads"], w["ndim"]
    units = N * P
    sysm = pk.System(cfg, stream=stream.cuda_stream)
    sysm.set_state(x0, p0)
    W = max(args.warmup, 3)
    K = max(args.steps, 1)
    # warm-up as single steps, like the timed loop: the step graphs are
    # captured here, outside the timed region
    for _ in range(W):
        sysm.step_async(1)
    sysm.synchronize()
    if args.profile_only:
        sysm.step_async(K)
        sysm.synchronize()
        return

    # L2 between timed steps: flushed (a 512 MiB write) unless the step's own
    # working set is more than twice the 129 MB L2
    ld = (N + 31) // 32 * 32
    ws = 4 * P * D * ld * 8 + (4 * N * (N + 1) // 2 * 8 if w.get("bosonic", True) else 0)
    do_flush = ws <= 2 * 129e6
    l2_note = ("flushed before every timed step (512 MiB write, outside the step's events)" if do_flush else
               f"not flushed: working set {ws / 1e6:.0f} MB (state and exchange arrays) > 2 x 129 MB L2")
    flush = torch.empty(512 * 1024 * 1024 // 4 if do_flush else 1, dtype=torch.float32, device="cuda")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    sampler = ClockSampler(local) if rank == 0 else None
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
    step_ms = [a.elapsed_time(b) for a, b in ev]
    tot_s = max_over_ranks(sum(step_ms) / 1e3, dist)
    value = world * units * K / tot_s

    # kernel launches in the timed region: the same K steps, counted.  Each
    # untimed block restarts from the initial state, so no run goes far past
    # W + K steps (the 2D dipole system is not stable over thousands)
    sysm.set_state(x0, p0)
    prof = sysm.profile(0)
    sysm.step_async(K)
    sysm.synchronize()
    launches = sysm.profile(-1)["launches"]
    # per-kernel device times (events around each launch on the library stream)
    sysm.set_state(x0, p0)
    sysm.profile(1)
    sysm.step_async(K)
    sysm.synchronize()
    prof = sysm.profile(-1)
    sysm.profile(0)

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
    del flush
    batched = None if args.no_batched else run_batched(pk, torch, stream, max(args.batch_steps, 1), W, rank, world,
                                                      dist)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    # roofline of the dominant kernel class
    ms, cnt = prof["ms"], prof["counts"]
    dom = max(ms, key=lambda k: ms[k])
    dom_ms = ms[dom] / max(cnt[dom], 1)
    fp64_peak = pk.measure_fp64_peak()
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    roof = {"kernel": dom, "kernel_share": ms[dom] / max(sum(ms.values()), 1e-30), "launch_ms": dom_ms,
            "per_class_ms_per_step": {k: v / K for k, v in ms.items() if v > 0}}
    if dom == "bead_forces" and w["inter"] != "free":
        fl, inside = pair_flops(w, x0)
        ach = fl / (dom_ms * 1e-3) / 1e12
        peak = fp64_peak if args.precision == "fp64" else None
        # DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one
        # k_pair_tiles_compact launch on this workload, from an ncu capture
        # (ncu --set full -k regex:k_pair_tiles_compact -s 2 -c 1 of
        # --profile-only --steps 3 --warmup 3); the per-step state (2.4 MB)
        # stays in L2 between launches
        traffic = 458496 if (args.workload == "cfg2" and args.precision == "fp64") else None
        roof.update({"bound": "fp64" if args.precision == "fp64" else "fp32", "achieved": ach,
                     "peak": peak, "unit": "TFLOP/s", "frac": (ach / peak) if peak else None,
                     "traffic": traffic, "traffic_unit": "bytes per launch (ncu capture)" if traffic else None,
                     "peak_source": "measured in-run (FP64 FMA probe)",
                     "algorithmic": f"{fl:.4g} FLOP per launch ({inside} unique pairs inside the cutoff)"})
    else:
        bytes_per = 6 * 8 * units * D
        ach = bytes_per / (dom_ms * 1e-3) / 1e9
        peak = peaks.get("hbm_gbs", 6800.0)
        roof.update({"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                     "traffic": None, "peak_source": "MEASURED_PEAKS.json hbm_gbs"})
    line = {"metric": METRIC, "value": value, "unit": "bead-steps/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": 1e3 * tot_s / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32 pair forces / f64 exchange and integrator",
            "data": "synthetic",
            "config": {"workload": w["desc"], "natoms": N, "nbeads": P, "ndim": D, "precision": args.precision,
                       "parallelism": f"replicas x{world}" if world > 1 else "single system",
                       "l2": l2_note},
            "e2e": e2e, "roofline": roof, "gpu_launches": launches, "clocks": clocks,
            "fp64_peak_tflops": fp64_peak}
    if batched:
        batched["vs_plain_fp64"] = batched["value"] / value if args.precision == "fp64" else None
        line["batched"] = batched
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, seconds=args.cpu_seconds)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

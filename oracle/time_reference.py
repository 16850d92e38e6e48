"""Times the unmodified reference (``oracle/_ref``, built by ``build_ref.py``)
on the benchmark systems and, on the same cores, the oracle port, to
calibrate the port that stands in for the reference on the GPU host.

Measurement infrastructure only; it runs where the reference was built.

Each reference run is its own main, one process per bead through the MPI
shim (the reference's decomposition, ranks oversubscribed when P exceeds the
cores, as the reference's own test driver does), from the benchmark's
initial state (per-bead xyz files and velocity files), with every observable
off and no state dumps.  Time is the reference's own "Wall time per step"
from output/report.txt (src/simulation.cpp:565-569) and the wall clock
around the process.  The reference rejects bosons with the normal-mode
propagator (src/params.cpp:146-148), so the two normal-mode systems run as
the "cartesian substitute": cartesian velocity Verlet with the normal-mode
Langevin thermostat, the same force and exchange work.  The port is timed
on the same substitute (and on the normal-mode original) with
``os.cpu_count()`` POSIX threads over its per-bead loops, noise drawn
before the timed steps.

Usage: python oracle/time_reference.py [cfg1 cfg2 cfg3 cfg4 cfg5] [--out file.json]
"""
from __future__ import annotations

import json
import os
import re
import shutil
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
# run as a script, this directory would shadow the oracle package
sys.path[:] = [q for q in sys.path if Path(q or ".").resolve() != HERE]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle import refrun  # noqa: E402

# steps per timed run: enough for seconds of reference time, bounded
STEPS = {"cfg1": 2000, "cfg2": 40, "cfg3": 10, "cfg5": 2}


def sections_of(w, steps, substitute):
    prop = "cartesian" if substitute else w["propagator"]
    nmth = w["nmthermostat"] or (substitute and w["propagator"] == "normal_modes")
    sec = {
        "simulation": {"dt": f"{w['dt_fs']} femtosecond", "steps": steps, "sfreq": max(steps, 1), "threshold": 0.0,
                       "nbeads": w["nbeads"], "bosonic": "true", "fixcom": "true",
                       "pbc": "true" if w["pbc"] else "false", "seed": 12345, "thermostat": "langevin",
                       "nmthermostat": "true" if nmth else "false", "propagator": prop},
        "system": {"temperature": f"{w['T_K']} kelvin", "natoms": w["natoms"], "size": f"{w['box_ang']} angstrom",
                   "mass": f"{w['mass_amu']} dalton"},
        "observables": {"energy": "off", "classical": "off", "bosonic": "off", "gsf": "off"},
    }
    if w["inter"] == "aziz":
        sec["interaction_potential"] = {"name": "aziz", "cutoff": f"{w['cutoff_ang']} angstrom"}
    elif w["inter"] == "dipole":
        sec["interaction_potential"] = {"name": "dipole", "strength": repr(w["int_p"][0]), "cutoff": "-1.0 angstrom"}
    elif w["inter"] == "harmonic":
        sec["interaction_potential"] = {"name": "harmonic",
                                        "omega": f"{w['int_p'][0] / bench.MEV!r} millielectronvolt",
                                        "cutoff": "-1.0 angstrom"}
    else:
        sec["interaction_potential"] = {"name": "free"}
    if w["ext"] == "harmonic":
        sec["external_potential"] = {"name": "harmonic", "omega": f"{w['ext_p'][0] / bench.MEV!r} millielectronvolt"}
    elif w["ext"] == "double_well":
        sec["external_potential"] = {"name": "double_well",
                                     "strength": f"{w['ext_p'][0] / bench.MEV!r} millielectronvolt",
                                     "location": f"{w['ext_p'][1] / bench.ANG!r} angstrom"}
    else:
        sec["external_potential"] = {"name": "free"}
    return sec


def run_reference(w, x, p, steps, substitute=True, variant=None):
    """Runs the reference's main; returns (wall time per step from
    report.txt, external wall seconds)."""
    variant = variant or ("d2" if w["ndim"] == 2 else "d3")
    exe = refrun.REF / f"pimdb_{variant}"
    P, N, D = x.shape
    td = Path(tempfile.mkdtemp(prefix="pimdb_time_"))
    try:
        m = w["mass_amu"] * bench.DALTON
        for b in range(P):
            # NDIM numbers per row, as the reference's loaders read them
            refrun._write_xyz(td / f"pos_{b}.xyz", x[b] / bench.ANG)
            refrun._write_vel(td / f"vel_{b}.dat", p[b] / m / refrun.ANG_PER_PS)
        sec = sections_of(w, steps, substitute)
        sec["simulation"]["initial_position"] = "xyz(pos_{}.xyz)"
        sec["simulation"]["initial_velocity"] = "manual(vel_{}.dat)"
        refrun.write_ini(td / "c.ini", sec)
        env = dict(os.environ, PIMDB_SHIM_NP=str(P), PIMDB_SHIM_TIMEOUT="3600")
        t0 = time.perf_counter()
        r = subprocess.run([str(exe), "-in", "c.ini"], cwd=td, capture_output=True, text=True, env=env, timeout=7200)
        wall = time.perf_counter() - t0
        if r.returncode != 0 or "[X]" in r.stdout:
            raise RuntimeError(f"reference run failed: {r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        rep = (td / "output" / "report.txt").read_text()
        mm = re.search(r"Wall time per step \(sec\)\s*[:=]?\s*([0-9.eE+-]+)", rep)
        per = float(mm.group(1)) if mm else float("nan")
        return per, wall
    finally:
        shutil.rmtree(td, ignore_errors=True)


def oracle_system(w, substitute):
    prop = "cartesian" if substitute else w["propagator"]
    nmth = w["nmthermostat"] or (substitute and w["propagator"] == "normal_modes")
    return O.make_system(ndim=w["ndim"], natoms=w["natoms"], nbeads=w["nbeads"], temperature=w["T_K"] * bench.KELVIN,
                         mass=w["mass_amu"] * bench.DALTON, bosonic=True, pbc=w["pbc"], size=w["box_ang"] * bench.ANG,
                         fixcom=True, propagator=prop, thermostat="langevin", nmthermostat=nmth,
                         dt=w["dt_fs"] * bench.FS, ext=w["ext"], ext_p=w["ext_p"], interaction=w["inter"],
                         int_p=w["int_p"], cutoff=w["cutoff_ang"] * bench.ANG)


def time_port(w, x, p, steps, substitute=True, nthreads=None):
    nthreads = nthreads or os.cpu_count() or 1
    s = oracle_system(w, substitute)
    tr = O.Trajectory(s, x, p)
    noise = [O.philox_noise_device(12345, 0, k, s.nbeads, s.natoms, s.ndim) for k in range(steps)]
    t0 = time.perf_counter()
    for k in range(steps):
        tr.step(noise[k], nthreads=nthreads)
    return (time.perf_counter() - t0) / steps, nthreads


def measure(name):
    w = bench.WORKLOADS[name]
    x, p = bench.initial_state(w)
    steps = STEPS[name]
    units = w["natoms"] * w["nbeads"]
    substitute = w["propagator"] == "normal_modes"
    per, wall = run_reference(w, x, p, steps, substitute)
    port, nth = time_port(w, x, p, max(2, steps // 2), substitute)
    row = {"system": name, "workload": w["desc"], "steps": steps,
           "reference": {"wall_per_step_s": per, "bead_steps_per_s": units / per, "external_wall_s": wall,
                         "ranks": w["nbeads"], "run": "cartesian substitute" if substitute else "as specified"},
           "port": {"per_step_s": port, "bead_steps_per_s": units / port, "threads": nth,
                    "run": "cartesian substitute" if substitute else "as specified"},
           "port_over_reference": per / port}
    if substitute:
        port_nm, _ = time_port(w, x, p, max(2, steps // 2), False)
        row["port_normal_modes"] = {"per_step_s": port_nm, "bead_steps_per_s": units / port_nm}
    return row


def measure_ensemble(sample=16, steps=200):
    """The 512-replica ensemble: a stratified sample of replicas run one
    after another, extrapolated to all 512 by their bead-particle weights."""
    from tests.test_baseline_sizes import stratified_sample
    cfgs, xs, ps = bench.batched_workload("fp64")
    pick = stratified_sample(cfgs, sample)
    ref_t, port_t, units_sample = 0.0, 0.0, 0
    for r in pick:
        c = cfgs[r]
        w = dict(desc="", ndim=3, natoms=c.natoms, nbeads=c.nbeads, T_K=c.temperature / bench.KELVIN, mass_amu=1.0,
                 pbc=False, box_ang=10.0, inter="harmonic", int_p=(1.0 * bench.MEV, 0, 0), cutoff_ang=-1.0,
                 ext="harmonic", ext_p=(3.0 * bench.MEV, 0, 0), propagator="cartesian", nmthermostat=False,
                 dt_fs=1.0)
        per, _ = run_reference(w, xs[r], ps[r], steps, False)
        port, nth = time_port(w, xs[r], ps[r], steps, False)
        ref_t += per
        port_t += port
        units_sample += c.natoms * c.nbeads
    units_all = sum(c.natoms * c.nbeads for c in cfgs)
    # time per bead-particle step of the sample, applied to the whole ensemble
    return {"system": "cfg4", "workload": "512-replica ensemble, stratified sample of %d replicas" % len(pick),
            "steps": steps,
            "reference": {"bead_steps_per_s": units_sample / ref_t, "ranks": "P per replica",
                          "run": "sample run one replica after another; rate of the sample"},
            "port": {"bead_steps_per_s": units_sample / port_t, "threads": nth},
            "port_over_reference": ref_t / port_t, "ensemble_bead_particles": units_all}


def main(argv):
    out = None
    if "--out" in argv:
        i = argv.index("--out")
        out = Path(argv[i + 1])
        argv = argv[:i] + argv[i + 2:]
    names = argv or ["cfg1", "cfg2", "cfg3", "cfg4", "cfg5"]
    if not refrun.available("d3"):
        raise SystemExit("the reference is not built here (python oracle/build_ref.py)")
    import platform
    cpu = {"machine": platform.machine(), "logical_cpus": os.cpu_count(), "model": bench.host_cpu()["model"]}
    rows = []
    for n in names:
        row = measure_ensemble() if n == "cfg4" else measure(n)
        row["cpu"] = cpu
        print(json.dumps(row), flush=True)
        rows.append(row)
    if out:
        out.write_text(json.dumps(rows, indent=1))


if __name__ == "__main__":
    main(sys.argv[1:])

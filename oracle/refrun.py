"""Drives the compiled reference (``oracle/_ref``, built by ``build_ref.py``)
on chosen inputs.  Test infrastructure only; every helper returns None when
the reference binaries are not present (they are built only where the
reference checkout exists).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF = HERE / "_ref"

ANGSTROM = 1.8897261        # include/units.h:95
ANG_PER_PS = 4.5710289e-5   # include/units.h:110


def available(variant: str = "d3") -> bool:
    return (REF / f"pimdb_{variant}").exists() and (REF / f"ref_probe_{variant}").exists()


def write_ini(path: Path, sections: dict):
    with open(path, "w") as fh:
        for sec, kv in sections.items():
            fh.write(f"[{sec}]\n")
            for k, v in kv.items():
                fh.write(f"{k} = {v}\n")
            fh.write("\n")


def probe(sections: dict, coords: np.ndarray, variant: str = "d3"):
    """Runs ref_probe: per-bead reference forces and exchange scalars for the
    ring polymer `coords` [P][N][D] (atomic units)."""
    if not available(variant):
        return None
    P, N, D = coords.shape
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        write_ini(td / "c.ini", sections)
        np.ascontiguousarray(coords, dtype=np.float64).tofile(td / "x.bin")
        r = subprocess.run([str(REF / f"ref_probe_{variant}"), "c.ini", "x.bin", "o.bin"], cwd=td,
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"ref_probe failed: {r.stderr}")
        raw = np.fromfile(td / "o.bin")
    per = 3 * N * D + 8
    raw = raw.reshape(P, per)
    nd = N * D
    return dict(f=raw[:, :nd].reshape(P, N, D), spring=raw[:, nd:2 * nd].reshape(P, N, D),
                phys=raw[:, 2 * nd:3 * nd].reshape(P, N, D), scalars=raw[:, 3 * nd:])


def _write_xyz(path: Path, x_ang: np.ndarray):
    with open(path, "w") as fh:
        fh.write(f"{len(x_ang)}\ncomment\n")
        for row in x_ang:
            fh.write("1 " + " ".join(repr(float(v)) for v in row) + "\n")


def _write_vel(path: Path, v_angps: np.ndarray):
    with open(path, "w") as fh:
        fh.write(f"{len(v_angps)}\ncomment\n")
        for i, row in enumerate(v_angps):
            fh.write(f"{i + 1} 1 " + " ".join(repr(float(v)) for v in row) + "\n")


def read_frames(path: Path, natoms: int, ndim: int):
    """Frames of a reference state dump (position_k.xyz / velocity_k.dat /
    force_k.dat): the last `ndim` numbers of each particle row."""
    frames = []
    with open(path) as fh:
        lines = fh.read().split("\n")
    i = 0
    while i < len(lines) and lines[i].strip():
        n = int(lines[i].split()[0])
        rows = [list(map(float, lines[i + 2 + j].split()))[-3:] for j in range(n)]
        frames.append(np.array(rows)[:, :ndim])
        i += 2 + n
    return np.array(frames)


def run_trajectory(sections: dict, x_ang: np.ndarray, v_angps: np.ndarray, variant: str = "d3", timeout=600):
    """Runs the reference's own main (one process per bead through the MPI
    shim) from per-bead initial positions (angstrom) and velocities
    (angstrom/ps), with every state dumped in atomic units each `sfreq`.
    Returns dict of arrays [frame][bead][N][D] plus simulation.out text."""
    if not available(variant):
        return None
    P, N, D = x_ang.shape
    td = Path(tempfile.mkdtemp(prefix="pimdb_ref_"))
    try:
        for b in range(P):
            _write_xyz(td / f"pos_{b}.xyz", x_ang[b])
            _write_vel(td / f"vel_{b}.dat", v_angps[b])
        sec = {k: dict(v) for k, v in sections.items()}
        sec.setdefault("simulation", {})
        sec["simulation"]["initial_position"] = "xyz(pos_{}.xyz)"
        sec["simulation"]["initial_velocity"] = "manual(vel_{}.dat)"
        sec["output"] = {"positions": "atomic_unit", "velocities": "atomic_unit", "forces": "atomic_unit"}
        sec.setdefault("observables", {"energy": "off"})
        write_ini(td / "c.ini", sec)
        env = dict(os.environ, PIMDB_SHIM_NP=str(P), PIMDB_SHIM_TIMEOUT="120")
        r = subprocess.run([str(REF / f"pimdb_{variant}"), "-in", "c.ini"], cwd=td, capture_output=True, text=True,
                           env=env, timeout=timeout)
        if r.returncode != 0 or "[X]" in r.stdout:
            raise RuntimeError(f"reference run failed: {r.stdout}\n{r.stderr}")
        out = td / "output"
        res = {}
        for key, stem in (("x", "position_{}.xyz"), ("v", "velocity_{}.dat"), ("f", "force_{}.dat")):
            res[key] = np.stack([read_frames(out / stem.format(b), N, D) for b in range(P)], axis=1)
        res["simulation_out"] = (out / "simulation.out").read_text() if (out / "simulation.out").exists() else ""
        return res
    finally:
        shutil.rmtree(td, ignore_errors=True)

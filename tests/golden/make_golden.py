"""Extracts compact golden fixtures from the reference's own regression cases
(tests/cases/* in the PIMD-B++ checkout) into ``tests/golden/cases.npz``.

For every case it keeps the case's config.ini text and the first rows of its
golden ``simulation.out``; for the dynamics cases it also keeps a subset of the
per-bead position frames (angstrom) and force frames (eV/angstrom), read the
way the reference's tests/main.py:145-161 reads them (last three numbers of
each particle row).

Usage: python tests/golden/make_golden.py [reference_dir]
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent / "cases.npz"
MAX_FRAMES = 21
MAX_ROWS = 11


def read_frames(path: Path):
    lines = path.read_text().split("\n")
    frames, i = [], 0
    while i < len(lines) and lines[i].strip():
        n = int(lines[i].split()[0])
        frames.append([list(map(float, lines[i + 2 + j].split()))[-3:] for j in range(n)])
        i += 2 + n
    return np.array(frames)


def main(ref: Path):
    cases = sorted(p for p in (ref / "tests" / "cases").iterdir() if p.is_dir())
    arrays = {}
    index = {}
    for c in cases:
        ini = (c / f"{c.name}.ini").read_text()
        sim = (c / "simulation.out").read_text().split("\n")
        header = sim[0].split()
        rows = np.array([list(map(float, ln.split())) for ln in sim[1:1 + MAX_ROWS] if ln.strip()])
        entry = {"ini": ini, "columns": header, "dynamics": False}
        arrays[f"{c.name}/simulation_out"] = rows
        if (c / "force_0.dat").exists():
            P = len(list(c.glob("force_*.dat")))
            f0 = read_frames(c / "force_0.dat")
            nfr = f0.shape[0]
            stride = max(1, (nfr - 1) // (MAX_FRAMES - 1))
            sel = np.arange(0, nfr, stride)[:MAX_FRAMES]
            X = np.stack([read_frames(c / f"position_{b}.xyz")[sel] for b in range(P)], axis=1)
            F = np.stack([read_frames(c / f"force_{b}.dat")[sel] for b in range(P)], axis=1)
            V = np.stack([read_frames(c / f"velocity_{b}.dat")[sel] for b in range(P)], axis=1)
            arrays[f"{c.name}/frames"] = sel
            arrays[f"{c.name}/positions_angstrom"] = X
            arrays[f"{c.name}/forces_ev_per_angstrom"] = F
            arrays[f"{c.name}/velocities_angstrom_per_ps"] = V
            entry.update(dynamics=True, nbeads=P, frame_stride_steps=None)
        index[c.name] = entry
    arrays["index_json"] = np.frombuffer(json.dumps(index).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT} ({OUT.stat().st_size / 1024:.0f} KiB, {len(cases)} cases)")


if __name__ == "__main__":
    sys.path.insert(0, str(Path(__file__).resolve().parents[2]))
    from oracle.build_ref import DEFAULT_REF  # $PIMDB_REFERENCE_DIR or ../reference beside the repository
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_REF)

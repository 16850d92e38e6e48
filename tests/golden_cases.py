"""Loader for the golden fixtures extracted from the reference's own
regression cases (tests/golden/make_golden.py)."""
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden" / "cases.npz"
ANGSTROM = 1.8897261        # include/units.h:95
EV_PER_ANG = 0.019446904    # include/units.h:146
KELVIN = 3.1668152e-06      # include/units.h:64 (energy and temperature)


def load():
    z = np.load(GOLDEN)
    index = json.loads(bytes(z["index_json"]).decode())
    return z, index


def dynamics_cases(include_factorial=False):
    z, index = load()
    out = []
    for name, e in index.items():
        if e["dynamics"] and (include_factorial or "factorial" not in name):
            out.append(name)
    return out


def write_ini(name, tmp_path):
    z, index = load()
    p = Path(tmp_path) / f"{name}.ini"
    p.write_text(index[name]["ini"])
    return p

"""Writes tests/golden/cli/<case>/{config.ini,simulation.out}: the compiled
reference (oracle/_ref, built by oracle/build_ref.py from the reference
sources) run on small deterministic (NVE) configurations, for comparing the
pimdb_gb300 driver's simulation.out with the reference's.  Run here, where
the reference checkout exists:  python tests/golden/make_cli_golden.py"""
import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
from oracle import refrun as R  # noqa: E402

CASES = {
    "nve_bosons_trap_pairharm": {
        "simulation": {"dt": "1.0 femtosecond", "steps": 40, "sfreq": 5, "threshold": 0.0, "nbeads": 4,
                       "bosonic": "true", "fixcom": "true", "pbc": "false", "seed": 2024, "thermostat": "none",
                       "initial_position": "random", "initial_velocity": "random", "propagator": "cartesian"},
        "system": {"temperature": "3.0 kelvin", "natoms": 8, "size": "10 angstrom", "mass": "1.0 dalton"},
        "interaction_potential": {"name": "harmonic", "omega": "1.0 millielectronvolt"},
        "external_potential": {"name": "harmonic", "omega": "3.0 millielectronvolt"},
        "observables": {"energy": "kelvin", "classical": "kelvin", "bosonic": "on", "gsf": "off"},
    },
    "nve_dist_nm_trap_gsf": {
        "simulation": {"dt": "1.0 femtosecond", "steps": 30, "sfreq": 3, "threshold": 0.2, "nbeads": 6,
                       "bosonic": "false", "fixcom": "false", "pbc": "false", "seed": 77, "thermostat": "none",
                       "initial_position": "random", "initial_velocity": "random", "propagator": "normal_modes"},
        "system": {"temperature": "2.0 kelvin", "natoms": 5, "size": "8 angstrom", "mass": "4.0026 dalton"},
        "interaction_potential": {"name": "free"},
        "external_potential": {"name": "harmonic", "omega": "2.0 millielectronvolt"},
        "observables": {"energy": "millielectronvolt", "classical": "kelvin", "gsf": "kelvin"},
    },
    "nve_bosons_factorial_trap": {
        "simulation": {"dt": "1.0 femtosecond", "steps": 40, "sfreq": 5, "threshold": 0.0, "nbeads": 4,
                       "bosonic": "true", "fixcom": "true", "pbc": "false", "seed": 515, "thermostat": "none",
                       "initial_position": "random", "initial_velocity": "random", "propagator": "cartesian"},
        "system": {"temperature": "2.0 kelvin", "natoms": 5, "size": "8 angstrom", "mass": "1.0 dalton"},
        "interaction_potential": {"name": "harmonic", "omega": "1.0 millielectronvolt"},
        "external_potential": {"name": "harmonic", "omega": "3.0 millielectronvolt"},
        "observables": {"energy": "kelvin", "classical": "kelvin", "bosonic": "on"},
    },
}
# Cases run by another build of the reference, with the driver flags that
# select the same algorithm (written to <case>/args).
VARIANTS = {"nve_bosons_factorial_trap": ("d3_fact", ["--factorial"])}


def main():
    if not (R.available("d3") and R.available("d3_fact")):
        raise SystemExit("compiled reference not built (python oracle/build_ref.py)")
    for name, sec in CASES.items():
        variant, args = VARIANTS.get(name, ("d3", []))
        td = Path(tempfile.mkdtemp(prefix="pimdb_cli_golden_"))
        try:
            R.write_ini(td / "config.ini", sec)
            P = int(sec["simulation"]["nbeads"])
            env = dict(os.environ, PIMDB_SHIM_NP=str(P), PIMDB_SHIM_TIMEOUT="120")
            r = subprocess.run([str(R.REF / f"pimdb_{variant}"), "-in", "config.ini"], cwd=td, env=env,
                               capture_output=True, text=True, timeout=300)
            if r.returncode != 0 or "[X]" in r.stdout:
                raise SystemExit(f"{name}: reference run failed\n{r.stdout}\n{r.stderr}")
            out = HERE / "cli" / name
            out.mkdir(parents=True, exist_ok=True)
            shutil.copy(td / "config.ini", out / "config.ini")
            shutil.copy(td / "output" / "simulation.out", out / "simulation.out")
            if args:
                (out / "args").write_text(" ".join(args) + "\n")
            print(name, (out / "simulation.out").read_text().count("\n"), "lines")
        finally:
            shutil.rmtree(td, ignore_errors=True)


if __name__ == "__main__":
    main()

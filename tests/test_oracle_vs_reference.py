"""The oracle against the compiled, unmodified reference (oracle/_ref, built
from the reference sources by oracle/build_ref.py).  Skipped where the
reference checkout is absent.

* Probe cases: per-bead forces and exchange scalars on identical ring-polymer
  configurations must be bit-identical (same operation order, same libm).
* Trajectories: the reference's own main, one process per bead, from the same
  initial state; Langevin noise from RANMAR streams seeded seed+bead as the
  reference draws it.  The reference's state dumps carry 13 significant
  digits, which bounds the comparison.
* Fixture replays: the reference's regression cases, run for their first
  1000 steps, reproduce the golden simulation.out rows.
"""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import refrun as R
from tests import golden_cases as G

pytestmark = pytest.mark.skipif(not R.available("d3"), reason="compiled reference not built here")


def _sections(N, P, bosonic, pbc, inter, ext, size_ang, T="1.0 kelvin", cutoff="-1.0 angstrom"):
    sec = {"simulation": {"nbeads": P, "bosonic": str(bosonic).lower(), "pbc": str(pbc).lower(),
                          "thermostat": "langevin", "seed": 7},
           "system": {"temperature": T, "natoms": N, "size": f"{size_ang} angstrom", "mass": "4.0026 dalton"},
           "interaction_potential": {"name": inter, "cutoff": cutoff}, "external_potential": {"name": ext},
           "observables": {"energy": "off"}}
    if inter == "harmonic":
        sec["interaction_potential"]["omega"] = "1.0 millielectronvolt"
    if inter == "dipole":
        sec["interaction_potential"]["strength"] = "2.4799673e-4"
    if ext == "harmonic":
        sec["external_potential"]["omega"] = "3.0 millielectronvolt"
    if ext == "double_well":
        sec["external_potential"].update(strength="1.32684e-7 millielectronvolt", location="3 angstrom")
    if ext == "cosine":
        sec["external_potential"].update(amplitude="1.0 millielectronvolt", phase="0.3")
    return sec


PROBES = [
    # N, P, D, bosonic, pbc, interaction, external, box (angstrom), T, cutoff
    (8, 8, 3, True, False, "free", "harmonic", 10.0, "1.0 kelvin", "-1.0 angstrom"),
    (16, 32, 3, True, False, "free", "harmonic", 10.0, "1.0 kelvin", "-1.0 angstrom"),
    (32, 8, 3, True, True, "aziz", "free", 12.0, "1.5 kelvin", "6 angstrom"),
    (20, 6, 3, False, True, "aziz", "double_well", 12.0, "1.0 kelvin", "-1.0 angstrom"),
    (24, 5, 2, True, False, "dipole", "harmonic", 30.0, "2.0 kelvin", "-1.0 angstrom"),
    (12, 4, 3, True, False, "harmonic", "cosine", 10.0, "1.0 kelvin", "-1.0 angstrom"),
    (48, 16, 3, True, True, "aziz", "double_well", 14.0, "1.0 kelvin", "7 angstrom"),
    (6, 2, 3, True, False, "free", "harmonic", 10.0, "1.0 kelvin", "-1.0 angstrom"),
]


@pytest.mark.parametrize("case", PROBES)
def test_probe_bit_identical(case, tmp_path):
    N, P, D, bos, pbc, inter, ext, box, T, cut = case
    rng = np.random.default_rng(N * 1000 + P)
    L = box * R.ANGSTROM
    x = rng.uniform(-0.5 * L, 0.5 * L, (N, D))[None] + rng.normal(0, 0.3 * R.ANGSTROM, (P, N, D))
    sec = _sections(N, P, bos, pbc, inter, ext, box, T, cut)
    R.write_ini(tmp_path / "c.ini", sec)
    s, _ = O.system_from_ini(tmp_path / "c.ini", ndim=D)
    ref = R.probe(sec, x, variant="d3" if D == 3 else "d2")
    got = O.update_forces(s, x)
    assert np.array_equal(got["f"], ref["f"])
    assert np.array_equal(got["spring"], ref["spring"])
    assert np.array_equal(got["phys"], ref["phys"])
    if s.bosonic:
        ex = O.exchange(s, x)
        sc = ref["scalars"][0]
        assert [ex["VB"], ex["prim"], ex["p_distinct"], ex["p_longest"]] == list(sc[:4])
        assert ref["scalars"][P - 1][0] == ex["VB"]


TRAJ = [
    # N, P, D, bosonic, propagator, thermostat, nmthermostat, fixcom, interaction, external, pbc
    (8, 8, 3, True, "cartesian", "none", False, False, "free", "harmonic", False),
    (8, 8, 3, True, "cartesian", "langevin", True, True, "free", "harmonic", False),
    (8, 6, 3, False, "normal_modes", "langevin", True, True, "free", "harmonic", False),
    (7, 5, 3, False, "normal_modes", "none", False, True, "free", "harmonic", False),
    (10, 4, 3, True, "cartesian", "langevin", False, True, "aziz", "free", True),
    (9, 4, 2, True, "cartesian", "langevin", False, True, "free", "harmonic", False),
]


@pytest.mark.parametrize("case", TRAJ)
def test_trajectory_matches_reference(case, tmp_path):
    N, P, D, bos, prop, thermo, nmth, fixcom, inter, ext, pbc = case
    steps, seed = 15, 4242
    rng = np.random.default_rng(steps * N + P)
    box = 9.0
    x_ang = rng.uniform(-0.5 * box, 0.5 * box, (N, D))[None] + rng.normal(0, 0.2, (P, N, D))
    v = rng.normal(0, 2.0, (P, N, D))
    sec = _sections(N, P, bos, pbc, inter, ext, box, "2.0 kelvin", "5 angstrom")
    sec["simulation"].update(thermostat=thermo, nmthermostat=str(nmth).lower(), propagator=prop,
                             fixcom=str(fixcom).lower(), seed=seed, steps=steps, sfreq=1, dt="1.0 femtosecond")
    ref = R.run_trajectory(sec, x_ang, v, variant="d3" if D == 3 else "d2")
    R.write_ini(tmp_path / "c.ini", sec)
    s, _ = O.system_from_ini(tmp_path / "c.ini", ndim=D)
    tr = O.Trajectory(s, x_ang * R.ANGSTROM, s.mass * (v * R.ANG_PER_PS))
    streams = [O.RanMars(seed + b) for b in range(P)]
    for st in range(steps + 1):
        for got, want in ((tr.x, ref["x"][st]), (tr.p / s.mass, ref["v"][st]), (tr.f, ref["f"][st])):
            scale = max(np.abs(want).max(), 1e-300)
            assert np.abs(got - want).max() <= 2e-12 * scale
        xi = O.ranmars_noise(streams, N, D) if thermo == "langevin" else np.zeros((2, P, N, D))
        assert tr.step(xi) == 0


@pytest.mark.parametrize("case", sorted(G.load()[1]))
def test_fixture_replay_first_1000_steps(case, tmp_path):
    """The compiled reference through the MPI shim reproduces the reference's
    own golden simulation.out rows (9 significant digits)."""
    import os
    import subprocess
    z, index = G.load()
    ini = index[case]["ini"].replace("steps = 100000", "steps = 1000")
    (tmp_path / "c.ini").write_text(ini)
    variant = "d3_fact" if "factorial" in case else "d3"
    P = int(float([ln.split("=")[1] for ln in ini.splitlines() if ln.strip().startswith("nbeads")][0]))
    env = dict(os.environ, PIMDB_SHIM_NP=str(P), PIMDB_SHIM_TIMEOUT="120")
    r = subprocess.run([str(R.REF / f"pimdb_{variant}"), "-in", "c.ini"], cwd=tmp_path, env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "[X]" not in r.stdout, r.stdout + r.stderr
    lines = (tmp_path / "output" / "simulation.out").read_text().split("\n")
    cols = lines[0].split()
    got = np.array([list(map(float, ln.split())) for ln in lines[1:] if ln.strip()])
    want = z[f"{case}/simulation_out"]
    gold_cols = index[case]["columns"]
    n = min(len(got), len(want))
    assert n >= 2
    for j, c in enumerate(cols):
        k = gold_cols.index(c)
        assert np.allclose(got[:n, j], want[:n, k], rtol=1e-5), c


OBS_CASES = [
    # N, P, bosonic, pbc, interaction, external, box, T, cutoff, gsf
    (8, 6, True, False, "harmonic", "harmonic", 10.0, "3.0 kelvin", "-1.0 angstrom", "off"),
    (6, 4, True, False, "free", "harmonic", 10.0, "2.0 kelvin", "-1.0 angstrom", "atomic_unit"),
    (7, 5, False, False, "free", "double_well", 10.0, "1.0 kelvin", "-1.0 angstrom", "atomic_unit"),
    (20, 4, True, True, "aziz", "free", 9.0, "1.5 kelvin", "4 angstrom", "off"),
]


@pytest.mark.parametrize("case", OBS_CASES)
def test_observables_match_reference_simulation_out(case, tmp_path):
    """orc_observables on the state at the end of each step (the reference's
    state dump at the start of the next step) against the reference's own
    simulation.out row of that step (9 significant digits)."""
    N, P, bos, pbc, inter, ext, box, T, cut, gsf = case
    sec = _sections(N, P, bos, pbc, inter, ext, box, T, cut)
    sec["simulation"].update(steps=5, sfreq=1, threshold=0.0)
    sec["observables"] = {"energy": "atomic_unit", "classical": "atomic_unit", "bosonic": "atomic_unit", "gsf": gsf}
    rng = np.random.default_rng(N + P)
    if pbc:
        side = np.linspace(-box / 2, box / 2, 4, endpoint=False) + box / 8
        grid = np.array(np.meshgrid(side, side, side)).reshape(3, -1).T[:N]
        x = grid[None] + rng.normal(0, 0.05, (P, N, 3))
    else:
        x = rng.uniform(-3, 3, (N, 3))[None] + rng.normal(0, 0.3, (P, N, 3))
    v = rng.normal(0, 3.0, (P, N, 3))
    res = R.run_trajectory(sec, x, v)
    R.write_ini(tmp_path / "c.ini", sec)
    s, _ = O.system_from_ini(tmp_path / "c.ini")
    lines = res["simulation_out"].strip().split("\n")
    cols = lines[0].split()
    rows = np.array([list(map(float, ln.split())) for ln in lines[1:]])
    assert len(rows) >= 5
    for k in range(len(rows) - 1):
        ob = O.observables(s, res["x"][k + 1], res["v"][k + 1] * s.mass)
        for j, c in enumerate(cols[1:], start=1):
            assert abs(ob[c] - rows[k, j]) <= 1e-7 * abs(rows[k, j]) + 1e-300, (k, c, ob[c], rows[k, j])


# The factorial build of the reference (FACTORIAL_BOSONIC_ALGORITHM): the
# permutation sum over all N! exchanges.
FACT_PROBES = [
    # N, P, bosonic, pbc, interaction, external, box (angstrom)
    (1, 3, True, False, "free", "harmonic", 5.0),
    (3, 2, True, False, "harmonic", "cosine", 6.0),
    (4, 6, True, False, "free", "harmonic", 10.0),
    (5, 4, True, True, "aziz", "free", 8.0),
    (6, 8, True, True, "free", "double_well", 9.0),
    (7, 5, True, False, "dipole", "harmonic", 12.0),
]
needs_fact = pytest.mark.skipif(not R.available("d3_fact"), reason="factorial reference build absent")


@needs_fact
@pytest.mark.parametrize("case", FACT_PROBES)
def test_factorial_probe_bit_identical(case, tmp_path):
    N, P, bos, pbc, inter, ext, box = case
    rng = np.random.default_rng(N * 7 + P)
    L = box * R.ANGSTROM
    x = rng.uniform(-0.5 * L, 0.5 * L, (N, 3))[None] + rng.normal(0, 0.3 * R.ANGSTROM, (P, N, 3))
    sec = _sections(N, P, bos, pbc, inter, ext, box)
    R.write_ini(tmp_path / "c.ini", sec)
    s, _ = O.system_from_ini(tmp_path / "c.ini", factorial=True)
    ref = R.probe(sec, x, variant="d3_fact")
    got = O.update_forces(s, x)
    for k in ("f", "spring", "phys"):
        assert np.array_equal(got[k], ref[k]), k
    ex = O.exchange(s, x)
    assert [ex["VB"], ex["prim"], ex["p_distinct"], ex["p_longest"]] == list(ref["scalars"][0][:4])
    assert list(ref["scalars"][P - 1][:2]) == [ex["VB"], ex["prim"]]


@needs_fact
@pytest.mark.parametrize("thermo", ["langevin", "none"])
def test_factorial_trajectory_and_observables_match_reference(thermo, tmp_path):
    N, P, steps, seed = 4, 6, 12, 99
    rng = np.random.default_rng(41)
    x_ang = rng.uniform(-2.0, 2.0, (N, 3))[None] + rng.normal(0, 0.2, (P, N, 3))
    v = rng.normal(0, 2.0, (P, N, 3))
    sec = _sections(N, P, True, False, "harmonic", "harmonic", 9.0, "2.0 kelvin")
    sec["simulation"].update(thermostat=thermo, seed=seed, steps=steps, sfreq=1, dt="1.0 femtosecond",
                             threshold=0.0)
    sec["observables"] = {"energy": "atomic_unit", "classical": "atomic_unit", "bosonic": "atomic_unit"}
    ref = R.run_trajectory(sec, x_ang, v, variant="d3_fact")
    R.write_ini(tmp_path / "c.ini", sec)
    s, _ = O.system_from_ini(tmp_path / "c.ini", factorial=True)
    tr = O.Trajectory(s, x_ang * R.ANGSTROM, s.mass * (v * R.ANG_PER_PS))
    streams = [O.RanMars(seed + b) for b in range(P)]
    for st in range(steps + 1):
        for got, want in ((tr.x, ref["x"][st]), (tr.p / s.mass, ref["v"][st]), (tr.f, ref["f"][st])):
            assert np.abs(got - want).max() <= 2e-12 * max(np.abs(want).max(), 1e-300)
        xi = O.ranmars_noise(streams, N, 3) if thermo == "langevin" else np.zeros((2, P, N, 3))
        assert tr.step(xi) == 0
    lines = ref["simulation_out"].strip().split("\n")
    cols = lines[0].split()
    rows = np.array([list(map(float, ln.split())) for ln in lines[1:]])
    for k in range(len(rows) - 1):
        ob = O.observables(s, ref["x"][k + 1], ref["v"][k + 1] * s.mass)
        for j, c in enumerate(cols[1:], start=1):
            assert abs(ob[c] - rows[k, j]) <= 1e-7 * abs(rows[k, j]) + 1e-300, (k, c, ob[c], rows[k, j])

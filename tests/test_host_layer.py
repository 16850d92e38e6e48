"""The C++ host layer (pimd-b_gb300/host/pimdb_host.hpp) and the pimdb_gb300
command-line driver.

CPU: the driver parses config.ini like the reference's main
(src/pimdb.cpp:31-68), reports configuration errors the reference's way, and
draws the reference's initial state (src/simulation.cpp:58-217, :750-751):
compared with frame 0 of the compiled reference's own dumps.

GPU: one step through the plugin calls (thermostat, COM removal, propagator,
thermostat, COM removal as src/simulation.cpp:246-259) equals the fused step;
a full driver run from config.ini matches the oracle trajectory."""
import importlib
import os
import shutil
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from oracle import refrun as R
from tests.gpu_cases import case, momenta, rel_per_bead, ring

build = importlib.import_module("pimd-b_gb300.build")
pk = importlib.import_module("pimd-b_gb300")
CLI = build.CLI


def _need_cli():
    if not CLI.exists():
        pytest.skip("pimdb_gb300 driver not built")


def _sections(P=8, N=8, fixcom="true", steps=0, propagator="cartesian", thermostat="langevin",
              nmthermostat="false", init_pos="random", T="5.802 kelvin", bosonic="true"):
    return {
        "simulation": {"dt": "1.0 femtosecond", "steps": steps, "sfreq": 1, "nbeads": P, "fixcom": fixcom,
                       "bosonic": bosonic, "seed": 90846, "pbc": "false", "initial_position": init_pos,
                       "initial_velocity": "random", "thermostat": thermostat, "propagator": propagator,
                       "nmthermostat": nmthermostat},
        "system": {"temperature": T, "natoms": N, "size": "300.0 atomic_unit", "mass": "1.0 atomic_unit"},
        "interaction_potential": {"name": "free"},
        "external_potential": {"name": "harmonic", "omega": "3.0 millielectronvolt"},
        "output": {"positions": "atomic_unit", "velocities": "atomic_unit", "forces": "off"},
        "observables": {"energy": "off"},
    }


def _cli(args, cwd):
    return subprocess.run([str(CLI), *args], cwd=cwd, capture_output=True, text=True, timeout=600)


def _initial(tmp_path, sec, P, N, D=3):
    R.write_ini(tmp_path / "c.ini", sec)
    r = _cli(["-in", "c.ini", "--check", "--initial", "init.bin"], tmp_path)
    assert r.returncode == 0 and "[X]" not in r.stdout, r.stdout
    a = np.fromfile(tmp_path / "init.bin")
    n = a.size // 2
    return a[:n].reshape(P, N, D), a[n:].reshape(P, N, D)


def test_cli_check_reports_configuration(tmp_path):
    _need_cli()
    R.write_ini(tmp_path / "c.ini", _sections(P=4, N=6, steps=17))
    r = _cli(["-in", "c.ini", "--check"], tmp_path)
    assert r.returncode == 0
    assert "natoms=6 nbeads=4 ndim=3 bosonic=1 propagator=0 thermostat=1 steps=17" in r.stdout
    assert "exchange=feldman_hirshberg" in r.stdout
    r = _cli(["-in", "c.ini", "--check", "--factorial"], tmp_path)
    assert r.returncode == 0 and "exchange=factorial" in r.stdout


def test_cli_bosonic_alg_reports_the_selected_algorithm(tmp_path):
    # src/pimdb.cpp:12-17: print the algorithm and run nothing
    _need_cli()
    r = _cli(["--bosonic_alg"], tmp_path)
    assert r.returncode == 0 and r.stdout.strip() == "Running with quadratic bosonic algorithm."
    r = _cli(["--factorial", "--bosonic_alg"], tmp_path)
    assert r.returncode == 0 and r.stdout.strip() == "Running with naive bosonic algorithm."
    assert not (tmp_path / "output").exists()


@pytest.mark.parametrize("key,value,message",[("thermostat", "berendsen", "is not supported"),
                                               ("propagator", "normal_modes", "not available for bosons")])
def test_cli_configuration_error_is_reported_like_the_reference(key, value, message, tmp_path):
    _need_cli()
    sec = _sections()
    sec["simulation"][key] = value
    R.write_ini(tmp_path / "c.ini", sec)
    r = _cli(["-in", "c.ini", "--check"], tmp_path)
    assert r.returncode == 0          # src/pimdb.cpp catches and returns 0
    assert "[X] Invalid argument error:" in r.stdout and message in r.stdout


def test_cli_initial_state_grid_positions(tmp_path):
    _need_cli()
    x, p = _initial(tmp_path, _sections(P=2, N=27, init_pos="grid"), 2, 27)
    L = 300.0
    assert np.array_equal(x[0], x[1])
    assert set(np.round(np.unique(x[0]) / (L / 3), 9)) == {-1.0, 0.0, 1.0}
    assert abs(p.reshape(-1, 3).sum(0)).max() < 1e-12 * abs(p).max()


@pytest.mark.skipif(not R.available("d3"), reason="compiled reference not built here")
@pytest.mark.parametrize("P,N,init_pos", [(8, 8, "random"), (4, 27, "grid"), (3, 5, "random")])
def test_cli_initial_state_matches_reference(P, N, init_pos, tmp_path):
    _need_cli()
    sec = _sections(P=P, N=N, init_pos=init_pos)
    x, p = _initial(tmp_path, sec, P, N)
    # the reference's own main from the same config.ini, frame 0 of its dumps
    td = Path(tempfile.mkdtemp(prefix="pimdb_ref_init_"))
    try:
        R.write_ini(td / "c.ini", sec)
        env = dict(os.environ, PIMDB_SHIM_NP=str(P), PIMDB_SHIM_TIMEOUT="120")
        r = subprocess.run([str(R.REF / "pimdb_d3"), "-in", "c.ini"], cwd=td, capture_output=True, text=True,
                           env=env, timeout=300)
        assert r.returncode == 0 and "[X]" not in r.stdout, r.stdout
        X = np.stack([R.read_frames(td / "output" / f"position_{b}.xyz", N, 3)[0] for b in range(P)])
        V = np.stack([R.read_frames(td / "output" / f"velocity_{b}.dat", N, 3)[0] for b in range(P)])
    finally:
        shutil.rmtree(td, ignore_errors=True)
    # the dumps carry 13 significant digits
    assert np.abs(x - X).max() <= 1e-12 * np.abs(X).max()
    assert np.abs(p / 1.0 - V).max() <= 1e-12 * np.abs(V).max()


# ------------------------------------------------------------------------ GPU
PLUGIN_CASES = {
    "vv_langevin_fixcom": dict(natoms=16, nbeads=8, ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0)),
    "vv_nve": dict(natoms=10, nbeads=6, thermostat="none", fixcom=False, pbc=True, box_ang=9.0, mass_amu=4.0026,
                   inter="aziz", cutoff_ang=4.5),
    "nm_nmthermo_aziz": dict(natoms=16, nbeads=8, propagator="normal_modes", nmthermostat=True, T_K=1.5,
                             mass_amu=4.0026, pbc=True, box_ang=11.0, inter="aziz", cutoff_ang=5.5, dt_fs=2.0),
    "vv_nmthermo": dict(natoms=8, nbeads=8, nmthermostat=True, ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0)),
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(PLUGIN_CASES))
def test_plugin_calls_equal_fused_step(name):
    s, cfg = case(**PLUGIN_CASES[name])
    x = ring(s, seed=4, spread_ang=0.2)
    p = momenta(s, 4)
    with pk.System(cfg) as a, pk.System(cfg) as b:
        for g in (a, b):
            g.set_state(x, p)
            g.set_step(0)
        for st in range(5):
            a.step(1)
            b.thermostat_step(0)
            if cfg.fixcom:
                b.zero_momentum()
            b.propagate()
            b.thermostat_step(1)
            if cfg.fixcom:
                b.zero_momentum()
            b.set_step(st + 1)
            for u, v, label in zip(a.get_state(), b.get_state(), "xpf"):
                assert rel_per_bead(v, u) < 1e-12, (st, label)


@pytest.mark.gpu
@pytest.mark.parametrize("plugin", [False, True])
# the reference's reader rejects bosons with the normal-mode propagator
# (src/params.cpp:146-148), so that case runs distinguishable particles
@pytest.mark.parametrize("propagator,nmthermostat,bosonic", [("cartesian", "false", "true"),
                                                             ("cartesian", "true", "true"),
                                                             ("normal_modes", "true", "false")])
def test_cli_run_matches_oracle(plugin, propagator, nmthermostat, bosonic, tmp_path):
    _need_cli()
    steps = 6
    P, N = 8, 8
    sec = _sections(P=P, N=N, steps=steps, propagator=propagator, nmthermostat=nmthermostat, bosonic=bosonic)
    x0, p0 = _initial(tmp_path, sec, P, N)
    args = ["-in", "c.ini", "--positions", "final.xyz"] + (["--plugin-steps"] if plugin else [])
    r = _cli(args, tmp_path)
    assert r.returncode == 0 and "[X]" not in r.stdout, r.stdout + r.stderr
    got = np.stack([fr for fr in R.read_frames(tmp_path / "final.xyz", N, 3)]) * R.ANGSTROM
    s, _ = O.system_from_ini(tmp_path / "c.ini")
    cfg = pk.config_from_ini(tmp_path / "c.ini")
    tr = O.Trajectory(s, x0, p0)
    for st in range(steps + 1):
        xi = O.philox_noise_device(cfg.seed, cfg.replica, st, P, N, 3)
        assert tr.step(xi) == 0
    assert rel_per_bead(got, tr.x) < 1e-9


GOLDEN_CLI = Path(__file__).resolve().parent / "golden" / "cli"


def _read_out(path):
    lines = [ln for ln in Path(path).read_text().split("\n") if ln.strip()]
    return lines[0].split(), np.array([list(map(float, ln.split())) for ln in lines[1:]])


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(p.name for p in GOLDEN_CLI.iterdir()) if GOLDEN_CLI.exists() else [])
def test_cli_simulation_out_matches_reference(name, tmp_path):
    """The driver on a reference config.ini (NVE, random initial state as the
    reference draws it) writes the reference's simulation.out: same columns,
    same rows (tests/golden/make_cli_golden.py ran the compiled reference)."""
    _need_cli()
    shutil.copy(GOLDEN_CLI / name / "config.ini", tmp_path / "config.ini")
    extra = GOLDEN_CLI / name / "args"  # flags selecting the reference build's algorithm
    r = _cli(["-in", "config.ini", *(extra.read_text().split() if extra.exists() else [])], tmp_path)
    assert r.returncode == 0 and "[X]" not in r.stdout, r.stdout + r.stderr
    cols, got = _read_out(tmp_path / "output" / "simulation.out")
    want_cols, want = _read_out(GOLDEN_CLI / name / "simulation.out")
    assert cols == want_cols
    assert got.shape == want.shape
    np.testing.assert_allclose(got, want, rtol=1e-6, atol=1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["bosonic_quadratic_harmonic_nh_dynamics", "bosonic_quadratic_harmonic_nh_np_dynamics",
                                  "bosonic_quadratic_harmonic_nh_np_dim_dynamics"])
def test_cli_replays_nose_hoover_regression_cases(case, tmp_path):
    """The reference's own Nose-Hoover regression cases (deterministic), run
    from their config.ini for 5000 steps: the driver's simulation.out rows
    against the reference's golden rows (energy, classical with nh_energy)."""
    from tests import golden_cases as G
    _need_cli()
    z, index = G.load()
    ini = index[case]["ini"].replace("steps = 100000", "steps = 5000")
    (tmp_path / "config.ini").write_text(ini)
    r = _cli(["-in", "config.ini"], tmp_path)
    assert r.returncode == 0 and "[X]" not in r.stdout, r.stdout + r.stderr
    cols, got = _read_out(tmp_path / "output" / "simulation.out")
    assert cols == index[case]["columns"]
    want = z[f"{case}/simulation_out"][:len(got)]
    assert len(got) == 6
    np.testing.assert_allclose(got, want, rtol=1e-6, atol=1e-9)
    # the state dumps (src/states/*.cpp) at the golden frames (steps 0 and 5000)
    P, N = index[case]["nbeads"], z[f"{case}/positions_angstrom"].shape[2]
    for stem, key in (("position_{}.xyz", "positions_angstrom"), ("velocity_{}.dat", "velocities_angstrom_per_ps"),
                      ("force_{}.dat", "forces_ev_per_angstrom")):
        frames = np.stack([R.read_frames(tmp_path / "output" / stem.format(b), N, 3) for b in range(P)], axis=1)
        assert frames.shape[0] == 6
        gold = z[f"{case}/{key}"]
        for mine, k in ((frames[0], 0), (frames[5], 1)):
            scale = np.abs(gold[k]).max()
            assert np.abs(mine - gold[k]).max() <= 1e-6 * scale + (1e-300 if scale else 0.0), (stem, k)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["bosonic_factorial_harmonic", "bosonic_factorial_harmonic_dynamics",
                                  "bosonic_quadratic_harmonic", "bosonic_quadratic_harmonic_dynamics",
                                  "bosonic_quadratic_harmonic_gsf", "bosonic_quadratic_harmonic_nmthermostat_dynamics",
                                  "dist_harmonic", "dist_harmonic_dynamics", "dist_harmonic_nm_propagation_dynamics"])
def test_cli_replays_langevin_regression_cases_with_ranmars(case, tmp_path):
    """The reference's Langevin regression cases run from their config.ini
    for 5000 steps with the reference's own noise streams (--ranmars; the
    factorial build's cases with --factorial): simulation.out rows and the
    state dumps at the golden frames against the reference's golden files."""
    from tests import golden_cases as G
    _need_cli()
    z, index = G.load()
    ini = index[case]["ini"].replace("steps = 100000", "steps = 5000")
    (tmp_path / "config.ini").write_text(ini)
    args = ["-in", "config.ini", "--ranmars"] + (["--factorial"] if "factorial" in case else [])
    r = _cli(args, tmp_path)
    assert r.returncode == 0 and "[X]" not in r.stdout, r.stdout + r.stderr
    cols, got = _read_out(tmp_path / "output" / "simulation.out")
    # the fixtures come from a revision of the reference that also printed
    # ext_pot and int_pot with one potential free (energy.cpp:12-18 now
    # omits them): compare the columns by name
    gold_cols = index[case]["columns"]
    assert set(cols) <= set(gold_cols)
    want = z[f"{case}/simulation_out"][:, [gold_cols.index(c) for c in cols]]  # the run's first rows
    n = min(len(got), len(want))
    assert n >= 6 and np.array_equal(got[:n, 0], want[:n, 0])
    np.testing.assert_allclose(got[:n], want[:n], rtol=1e-6, atol=1e-9)
    if not index[case]["dynamics"]:
        return
    P, N = index[case]["nbeads"], z[f"{case}/positions_angstrom"].shape[2]
    gap = 100000 // (z[f"{case}/positions_angstrom"].shape[0] - 1)  # golden dumps keep every gap-th step
    for stem, key in (("position_{}.xyz", "positions_angstrom"), ("velocity_{}.dat", "velocities_angstrom_per_ps"),
                      ("force_{}.dat", "forces_ev_per_angstrom")):
        frames = np.stack([R.read_frames(tmp_path / "output" / stem.format(b), N, 3) for b in range(P)], axis=1)
        step_of = [k * (5000 // (frames.shape[0] - 1)) for k in range(frames.shape[0])]
        for k in (0, 1):
            mine = frames[step_of.index(k * gap)]
            gold = z[f"{case}/{key}"][k]
            scale = np.abs(gold).max()
            assert np.abs(mine - gold).max() <= 1e-8 * scale + (1e-300 if scale else 0.0), (stem, k)


@pytest.mark.skipif(not R.available("d3"), reason="compiled reference not built here")
@pytest.mark.parametrize("pos_spec,vel_spec", [("xyz(pos_{}.xyz)", "manual(vel_{}.dat)"),
                                               ("xyz(one.xyz)", "random"),
                                               ("random", "manual")])
def test_cli_initial_state_from_files_matches_reference(pos_spec, vel_spec, tmp_path):
    """xyz / velocity-file initialisation (src/common.cpp:49-136): the driver's
    initial state against frame 0 of the compiled reference's own dumps."""
    _need_cli()
    P, N = 4, 6
    rng = np.random.default_rng(9)
    xa = rng.uniform(-4, 4, (P, N, 3))
    va = rng.normal(0, 3.0, (P, N, 3))
    for d in (tmp_path, tmp_path / "ref"):
        d.mkdir(exist_ok=True)
        (d / "init").mkdir(exist_ok=True)
        for b in range(P):
            R._write_xyz(d / f"pos_{b}.xyz", xa[b])
            R._write_vel(d / f"vel_{b}.dat", va[b])
            R._write_vel(d / "init" / f"vel_{b + 1:02}.dat", va[b])
        R._write_xyz(d / "one.xyz", xa[0])
    sec = _sections(P=P, N=N, init_pos="random")
    sec["simulation"]["initial_position"] = pos_spec
    sec["simulation"]["initial_velocity"] = vel_spec
    x, p = _initial(tmp_path, sec, P, N)
    R.write_ini(tmp_path / "ref" / "c.ini", sec)
    env = dict(os.environ, PIMDB_SHIM_NP=str(P), PIMDB_SHIM_TIMEOUT="120")
    r = subprocess.run([str(R.REF / "pimdb_d3"), "-in", "c.ini"], cwd=tmp_path / "ref", capture_output=True, text=True,
                       env=env, timeout=300)
    assert r.returncode == 0 and "[X]" not in r.stdout, r.stdout
    X = np.stack([R.read_frames(tmp_path / "ref" / "output" / f"position_{b}.xyz", N, 3)[0] for b in range(P)])
    V = np.stack([R.read_frames(tmp_path / "ref" / "output" / f"velocity_{b}.dat", N, 3)[0] for b in range(P)])
    assert np.abs(x - X).max() <= 1e-12 * np.abs(X).max()
    assert np.abs(p / 1.0 - V).max() <= 1e-12 * np.abs(V).max()

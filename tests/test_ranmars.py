"""RanMars parity noise: Langevin normals from the reference's own streams
(RanMars(seed + bead), libs/random_mars.cpp, drawn per particle and axis as
src/thermostats/langevin.cpp:15-27 does), so that trajectories follow the
reference's.

CPU: the oracle, started from the driver's initial state (the reference's
mt19937 draws, pinned against the reference's frame-0 dumps in
test_host_layer.py) and fed RanMars noise, replays the reference's Langevin
regression cases: its positions after 5000 steps match the golden position
dumps (13 significant digits) within 1e-9 relative.  Seeds the reference
rejects are rejected.

GPU: trajectories in RanMars mode match the oracle fed the same streams
(1e-9 relative per bead) for every thermostat coupling and propagator, CUDA
graph replay equals plain launches, and the plugin calls equal the fused
step."""
import importlib
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G
from tests.gpu_cases import MEV, case, momenta, pk, rel_per_bead, ring

build = importlib.import_module("pimd-b_gb300.build")

LANGEVIN_CASES = ["bosonic_factorial_harmonic_dynamics", "bosonic_quadratic_harmonic_dynamics",
                  "bosonic_quadratic_harmonic_nmthermostat_dynamics", "dist_harmonic_dynamics",
                  "dist_harmonic_nm_propagation_dynamics"]


def reference_initial_state(ini, tmp_path, P, N):
    if not build.CLI.exists():
        pytest.skip("pimdb_gb300 driver not built")
    r = subprocess.run([str(build.CLI), "-in", str(ini), "--check", "--initial", "init.bin"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "[X]" not in r.stdout, r.stdout
    a = np.fromfile(tmp_path / "init.bin")
    n = a.size // 2
    return a[:n].reshape(P, N, 3), a[n:].reshape(P, N, 3)


# ------------------------------------------------------------------------ CPU
@pytest.mark.parametrize("case", LANGEVIN_CASES)
def test_oracle_with_ranmars_replays_golden_langevin_case(case, tmp_path):
    z, index = G.load()
    ini = G.write_ini(case, tmp_path)
    s, extra = O.system_from_ini(ini, factorial="factorial" in case)
    P, N = s.nbeads, s.natoms
    X = z[f"{case}/positions_angstrom"]
    gap = extra["steps"] // (X.shape[0] - 1)  # the golden dumps keep every gap-th step
    x, p = reference_initial_state(ini, tmp_path, P, N)
    tr = O.Trajectory(s, x, p)
    streams = [O.RanMars(extra["seed"] + b) for b in range(P)]
    for _ in range(gap):
        assert tr.step(O.ranmars_noise(streams, N, 3)) == 0
    # the dump at the start of step `gap` holds the state after `gap` steps
    got = tr.x / G.ANGSTROM
    assert np.abs(got - X[1]).max() <= 1e-9 * np.abs(X[1]).max()


def test_ranmars_rejects_the_seeds_the_reference_rejects():
    for seed, P in ((0, 4), (900000000 - 2, 4)):
        _, cfg = case(natoms=4, nbeads=P, seed=seed)
        cfg.rng = pk.RNG["ranmars"]
        with pytest.raises(pk.ConfigError, match="Invalid seed for Marsaglia"):
            pk.System(cfg)


def test_batch_rejects_ranmars_noise():
    _, cfg = case(natoms=4, nbeads=4)
    cfg.rng = pk.RNG["ranmars"]
    with pytest.raises(pk.ConfigError, match="Philox"):
        pk.Batch([cfg])


# ------------------------------------------------------------------------ GPU
TRAJ = {
    "vv_langevin_bosons": dict(natoms=7, nbeads=8, T_K=2.0, ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
    "vv_nmthermo_bosons": dict(natoms=6, nbeads=8, nmthermostat=True, ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
    "nm_langevin_dist": dict(natoms=5, nbeads=6, bosonic=False, propagator="normal_modes", ext="harmonic",
                             ext_p=(3.0 * MEV, 0, 0)),
    "nm_nmthermo_dist_odd_N": dict(natoms=9, nbeads=8, bosonic=False, propagator="normal_modes",
                                   nmthermostat=True, ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
    "vv_langevin_aziz_pbc_nofixcom": dict(natoms=10, nbeads=4, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=9.0,
                                          inter="aziz", cutoff_ang=4.5, fixcom=False),
    "vv_langevin_2d": dict(ndim=2, natoms=5, nbeads=4, T_K=2.0, ext="harmonic", ext_p=(1.0 * MEV, 0, 0)),
    "vv_factorial": dict(natoms=5, nbeads=6, T_K=2.0, ext="harmonic", ext_p=(3.0 * MEV, 0, 0),
                         exchange="factorial"),
}
OPTIONS = {"nm_nmthermo_dist_odd_N": [{}, {"fused_normal_modes": 0}]}


@pytest.mark.gpu
@pytest.mark.parametrize("name,options", [(n, o) for n in sorted(TRAJ) for o in OPTIONS.get(n, [{}])])
def test_ranmars_trajectory_matches_oracle(name, options):
    s, cfg = case(seed=4321, **TRAJ[name])
    cfg.rng = pk.RNG["ranmars"]
    x = ring(s, seed=11, spread_ang=0.2)
    p = momenta(s, 11)
    tr = O.Trajectory(s, x, p)
    streams = [O.RanMars(4321 + b) for b in range(s.nbeads)]
    with pk.System(cfg) as g:
        for k, v in options.items():
            g.set_option(k, v)
        g.set_state(x, p)
        g.set_step(0)
        st = 0
        while st < 12:
            n = 1 if st < 6 else 2  # then two-step calls (a deferred tail between the steps)
            for _ in range(n):
                assert tr.step(O.ranmars_noise(streams, s.natoms, s.ndim)) == 0
            g.step(n)
            st += n
            gx, gp, gf = g.get_state()
            for got, want, label in ((gx, tr.x, "x"), (gp, tr.p, "p"), (gf, tr.f, "f")):
                assert rel_per_bead(got, want) < 1e-9, (st, label, rel_per_bead(got, want))


@pytest.mark.gpu
def test_ranmars_graph_replay_equals_plain_launches():
    s, cfg = case(seed=99, **TRAJ["nm_nmthermo_dist_odd_N"])
    cfg.rng = pk.RNG["ranmars"]
    x = ring(s, seed=3, spread_ang=0.2)
    p = momenta(s, 3)
    out = []
    for graphs in (1, 0):
        with pk.System(cfg) as g:
            g.set_option("cuda_graphs", graphs)
            g.set_state(x, p)
            g.set_step(0)
            for _ in range(3):
                g.step(4)
            out.append(g.get_state())
    for u, v in zip(*out):
        assert np.array_equal(u, v)


@pytest.mark.gpu
def test_ranmars_plugin_calls_equal_fused_step():
    s, cfg = case(seed=77, **TRAJ["vv_langevin_bosons"])
    cfg.rng = pk.RNG["ranmars"]
    x = ring(s, seed=5, spread_ang=0.2)
    p = momenta(s, 5)
    with pk.System(cfg) as a, pk.System(cfg) as b:
        for g in (a, b):
            g.set_state(x, p)
            g.set_step(0)
        for st in range(3):
            a.step(1)
            # Simulation::run (src/simulation.cpp:246-259): O, COM, propagator, O, COM
            b.thermostat_step(0)
            b.zero_momentum()
            b.propagate()
            b.thermostat_step(1)
            b.zero_momentum()
            b.set_step(st + 1)
        for u, v in zip(a.get_state(), b.get_state()):
            assert rel_per_bead(u, v) < 1e-12

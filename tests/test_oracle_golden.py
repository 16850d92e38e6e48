"""The oracle against the reference's own golden regression fixtures.

The reference dumps forces at the top of every saved step, i.e. the forces of
the positions dumped in the same frame (src/simulation.cpp:243-245 before the
propagator).  Recomputing the forces from the golden positions pins the whole
force path (Feldman-Hirshberg exchange on beads 1 and P, interior springs,
external trap) without any random numbers.  The dumps carry 13 significant
digits (src/states/force.cpp:44), which bounds the achievable agreement.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G


@pytest.mark.parametrize("case", G.dynamics_cases())
def test_forces_match_golden_frames(case, tmp_path):
    z, index = G.load()
    s, _ = O.system_from_ini(G.write_ini(case, tmp_path))
    X = z[f"{case}/positions_angstrom"]
    F = z[f"{case}/forces_ev_per_angstrom"]
    assert X.shape[1] == s.nbeads and X.shape[2] == s.natoms
    worst = 0.0
    for fr in range(1, X.shape[0]):
        f = O.update_forces(s, X[fr] * G.ANGSTROM)["f"] / G.EV_PER_ANG
        # the reference's own comparison (tests/main.py:77-86)
        assert np.allclose(f, F[fr], rtol=1e-5)
        worst = max(worst, float(np.max(np.abs(f - F[fr])) / np.max(np.abs(F[fr]))))
    assert worst < 1e-9, worst


@pytest.mark.parametrize("case", G.dynamics_cases(include_factorial=True))
def test_forces_are_zero_in_the_first_frame(case):
    # Simulation's constructor never evaluates forces (src/simulation.cpp:16-101),
    # so the first half-kick uses zero forces.
    z, _ = G.load()
    assert np.all(z[f"{case}/forces_ev_per_angstrom"][0] == 0.0)


def test_factorial_exchange_matches_golden_frames(tmp_path):
    # The permutation sum over all N! exchanges (factorial_bosonic_exchange.cpp)
    # recomputed from the golden positions of the factorial build's fixture.
    z, _ = G.load()
    case = "bosonic_factorial_harmonic_dynamics"
    s, _ = O.system_from_ini(G.write_ini(case, tmp_path), factorial=True)
    X = z[f"{case}/positions_angstrom"]
    F = z[f"{case}/forces_ev_per_angstrom"]
    worst = 0.0
    for fr in range(1, X.shape[0]):
        f = O.update_forces(s, X[fr] * G.ANGSTROM)["f"] / G.EV_PER_ANG
        assert np.allclose(f, F[fr], rtol=1e-5)
        worst = max(worst, float(np.max(np.abs(f - F[fr])) / np.max(np.abs(F[fr]))))
    assert worst < 1e-9, worst


def test_factorial_and_quadratic_potentials_differ_configurationwise(tmp_path):
    # The factorial fixture cannot pin the FH forces: the FH recursion keeps
    # one representative cycle per set of exchanged particles and equals the
    # permutation sum only after integrating over the interior beads.
    z, _ = G.load()
    case = "bosonic_factorial_harmonic_dynamics"
    s, _ = O.system_from_ini(G.write_ini(case, tmp_path))
    f = O.update_forces(s, z[f"{case}/positions_angstrom"][3] * G.ANGSTROM)["f"] / G.EV_PER_ANG
    g = z[f"{case}/forces_ev_per_angstrom"][3]
    interior = slice(1, s.nbeads - 1)
    assert np.allclose(f[interior], g[interior], rtol=1e-8, atol=1e-12 * np.abs(g).max())
    assert not np.allclose(f[0], g[0], rtol=1e-5)


def test_philox_noise_is_deterministic_and_normal():
    a = O.philox_normals(12345, 3, 17, 1, 200001)
    b = O.philox_normals(12345, 3, 17, 1, 200001)
    c = O.philox_normals(12345, 3, 17, 0, 200001)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)
    assert abs(a.mean()) < 0.01 and abs(a.std() - 1) < 0.01
    # an odd count returns the leading part of the even one
    assert np.array_equal(O.philox_normals(1, 0, 0, 0, 7), O.philox_normals(1, 0, 0, 0, 8)[:7])


def test_ranmars_rejects_reference_invalid_seeds():
    # libs/random_mars.cpp:16-17
    with pytest.raises(ValueError):
        O.RanMars(0)
    with pytest.raises(ValueError):
        O.RanMars(900000001)
    g = O.RanMars(1234).gaussians(100000)
    assert abs(g.mean()) < 0.02 and abs(g.std() - 1) < 0.02


NH_CASES = ["bosonic_quadratic_harmonic_nh_dynamics", "bosonic_quadratic_harmonic_nh_np_dynamics",
            "bosonic_quadratic_harmonic_nh_np_dim_dynamics"]


def nh_initial_state(case, tmp_path):
    """The exact initial state of a regression case (initial_position and
    initial_velocity = random): the driver's draw, which is the reference's
    (tests/test_host_layer.py), or golden frame 0 when the driver is absent."""
    import importlib
    import subprocess
    z, index = G.load()
    s, _ = O.system_from_ini(G.write_ini(case, tmp_path))
    cli = importlib.import_module("pimd-b_gb300.build").CLI
    if cli.exists():
        ini = G.write_ini(case, tmp_path)
        r = subprocess.run([str(cli), "-in", str(ini), "--check", "--initial", str(tmp_path / "init.bin")],
                           capture_output=True, text=True, timeout=60)
        if r.returncode == 0 and (tmp_path / "init.bin").exists():
            a = np.fromfile(tmp_path / "init.bin")
            n = a.size // 2
            shp = (s.nbeads, s.natoms, s.ndim)
            return s, a[:n].reshape(shp), a[n:].reshape(shp)
    x = z[f"{case}/positions_angstrom"][0] * G.ANGSTROM
    v = z[f"{case}/velocities_angstrom_per_ps"][0] * 4.5710289e-5
    return s, x, v * s.mass


@pytest.mark.parametrize("case", NH_CASES)
def test_nose_hoover_replays_golden_trajectory(case, tmp_path):
    """Nose-Hoover chains are deterministic: the oracle replays the reference's
    regression run from its initial state for 5000 steps and meets its
    golden positions and simulation.out rows (energy, classical with nh_energy)."""
    z, index = G.load()
    s, x, p = nh_initial_state(case, tmp_path)
    assert O.lib().orc_nh_chains(O.C.byref(s)) > 0
    tr = O.Trajectory(s, x, p)
    rows = z[f"{case}/simulation_out"]
    cols = index[case]["columns"]
    noise = np.zeros((2,) + x.shape)
    X = z[f"{case}/positions_angstrom"]
    frames = list(z[f"{case}/frames"])
    checked = 0
    for step in range(5001):
        if step in (1000 * f for f in frames):
            k = frames.index(step // 1000)
            np.testing.assert_allclose(tr.x / G.ANGSTROM, X[k], rtol=1e-6, atol=1e-9 * np.abs(X[k]).max())
            checked += 1
        assert tr.step(noise) == 0
        if step % 1000 == 0:
            ob = O.observables(s, tr.x, tr.p)
            ob["nh_energy"] = tr.nh_energy()
            row = rows[list(rows[:, 0]).index(step)]
            for j, c in enumerate(cols[1:], start=1):
                val = ob[c] / G.KELVIN if c not in ("temperature",) else ob[c]
                assert abs(val - row[j]) <= 1e-6 * abs(row[j]) + 1e-9, (step, c, val, row[j])
    assert checked == 2

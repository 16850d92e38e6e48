"""GPU parity: the CUDA path through the C ABI against the oracle (which is
bit-identical to the compiled reference, see test_oracle_vs_reference.py) and
against the reference's own golden fixtures.

Tolerances: the FP64 path must agree within 1e-10 relative (forces per bead,
V_B, trajectories); the mixed path within 1e-6 norm-relative force error."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G
from tests.gpu_cases import case, momenta, pk, rel_per_bead, ring, ring_separated

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10

FORCE_CASES = {
    # name: (case kwargs, ring kwargs)
    "bosons_trap_N16_P32": (dict(natoms=16, nbeads=32, ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0)),
                            dict(spread_ang=0.5)),
    "bosons_aziz_pbc_N64_P8": (dict(natoms=64, nbeads=8, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=14.0,
                                    inter="aziz", cutoff_ang=7.0), dict(spread_ang=0.2)),
    "dist_aziz_allpairs_doublewell": (dict(natoms=40, nbeads=6, bosonic=False, pbc=True, box_ang=12.0,
                                           mass_amu=4.0026, inter="aziz", cutoff_ang=-1.0, ext="double_well",
                                           ext_p=(1.32684e-7 * 0.036749326e-3, 3.0 * 1.8897261, 0)),
                                      dict(spread_ang=0.2)),
    "bosons_dipole_2d": (dict(ndim=2, natoms=48, nbeads=5, T_K=2.0, inter="dipole", int_p=(2.4799673e-4, 0, 0),
                              ext="harmonic", ext_p=(1.0 * 0.036749326e-3, 0, 0), box_ang=60.0),
                         dict(spread_ang=0.3)),
    "bosons_pairharm_cosine": (dict(natoms=12, nbeads=4, inter="harmonic", int_p=(1.0 * 0.036749326e-3, 0, 0),
                                    ext="cosine", ext_p=(1.0 * 0.036749326e-3, 0.3, 0)), dict(spread_ang=0.3)),
    "bosons_1d": (dict(ndim=1, natoms=10, nbeads=3, ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0)),
                  dict(spread_ang=0.3)),
    "bosons_P2": (dict(natoms=6, nbeads=2, ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0)), dict()),
    "boson_N1": (dict(natoms=1, nbeads=4, ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0)), dict()),
    "dist_P1": (dict(natoms=9, nbeads=1, inter="harmonic", int_p=(1.0 * 0.036749326e-3, 0, 0)), dict()),
    "bosons_aziz_pbc_N300_P4": (dict(natoms=300, nbeads=4, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=24.0,
                                     inter="aziz", cutoff_ang=12.0), dict(spread_ang=0.2)),
    # every cycle contributes (all weights nonzero): the banded kernel's dense solve
    "bosons_trap_N100_P4_dense_weights": (dict(natoms=100, nbeads=4, ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0)),
                                          dict(spread_ang=0.05)),
    "bosons_trap_N1100_P3_far_from_equilibrium": (dict(natoms=1100, nbeads=3, ext="harmonic",
                                                       ext_p=(3.0 * 0.036749326e-3, 0, 0), box_ang=40.0),
                                                  dict(spread_ang=3.0)),
}


@pytest.mark.parametrize("newton3", [1, 0])
@pytest.mark.parametrize("name", sorted(FORCE_CASES))
def test_forces_match_oracle(name, newton3):
    kw, rk = FORCE_CASES[name]
    s, cfg = case(**kw)
    x = ring(s, seed=len(name), **rk)
    want = O.update_forces(s, x)["f"]
    with pk.System(cfg) as g:
        g.set_option("newton3", newton3)
        g.set_state(x, np.zeros_like(x))
        g.compute_forces()
        _, _, f = g.get_state()
    assert rel_per_bead(f, want) < FP64_TOL


@pytest.mark.parametrize("exact", [0, 1])
@pytest.mark.parametrize("name", [n for n in sorted(FORCE_CASES) if FORCE_CASES[n][0].get("bosonic", True)
                                  and FORCE_CASES[n][0].get("nbeads", 4) > 1])
def test_exchange_matches_oracle(name, exact):
    kw, rk = FORCE_CASES[name]
    s, cfg = case(**kw)
    x = ring(s, seed=len(name) + 7, **rk)
    ref = O.exchange(s, x)
    with pk.System(cfg) as g:
        g.set_option("exact_exchange", exact)
        g.set_state(x, np.zeros_like(x))
        got = g.exchange()
        arr = g.exchange_arrays()
    assert abs(got["VB"] - ref["VB"]) <= FP64_TOL * abs(ref["VB"])
    for key in ("prim", "p_distinct", "p_longest"):
        assert abs(got[key] - ref[key]) <= 1e-9 * abs(ref[key]) + 1e-300, key
    np.testing.assert_allclose(arr["E"], ref["E"], rtol=1e-12, atol=1e-14 * np.abs(ref["E"]).max())
    np.testing.assert_allclose(arr["V"], ref["V"], rtol=FP64_TOL, atol=1e-14 * np.abs(ref["V"]).max())
    np.testing.assert_allclose(arr["Vb"][1:], ref["Vb"][1:], rtol=FP64_TOL, atol=1e-14 * np.abs(ref["Vb"]).max())
    for key in ("f1", "fP"):
        assert np.abs(got[key] - ref[key]).max() <= FP64_TOL * np.abs(ref[key]).max(), key


TRAJ_CASES = {
    "vv_langevin_bosons_N16_P32": dict(natoms=16, nbeads=32, ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0)),
    "vv_nve_bosons_aziz": dict(natoms=10, nbeads=6, thermostat="none", fixcom=False, pbc=True, box_ang=9.0,
                               mass_amu=4.0026, inter="aziz", cutoff_ang=4.5),
    "vv_nmthermo_bosons": dict(natoms=8, nbeads=8, nmthermostat=True, ext="harmonic",
                               ext_p=(3.0 * 0.036749326e-3, 0, 0)),
    "nm_langevin_dist": dict(natoms=12, nbeads=8, bosonic=False, propagator="normal_modes",
                             ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0)),
    "nm_nmthermo_bosons_aziz": dict(natoms=16, nbeads=8, propagator="normal_modes", nmthermostat=True,
                                    T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=11.0, inter="aziz",
                                    cutoff_ang=5.5, dt_fs=2.0),
    "nm_none_dist_odd_P": dict(natoms=7, nbeads=5, bosonic=False, propagator="normal_modes", thermostat="none",
                               ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0)),
    "vv_langevin_dipole_2d": dict(ndim=2, natoms=20, nbeads=4, T_K=2.0, inter="dipole", int_p=(2.4799673e-4, 0, 0),
                                  ext="harmonic", ext_p=(1.0 * 0.036749326e-3, 0, 0), box_ang=40.0),
    "nm_nmthermo_dist_nofixcom_odd_N": dict(natoms=13, nbeads=6, bosonic=False, propagator="normal_modes",
                                            nmthermostat=True, fixcom=False, ext="harmonic",
                                            ext_p=(3.0 * 0.036749326e-3, 0, 0)),
    "nm_nmthermo_bosons_P16_2d": dict(ndim=2, natoms=24, nbeads=16, propagator="normal_modes", nmthermostat=True,
                                      inter="dipole", int_p=(2.4799673e-4, 0, 0), ext="harmonic",
                                      ext_p=(1.0 * 0.036749326e-3, 0, 0), box_ang=40.0),
    # P = 32, 64, 128: the fused step runs in registers, one warp per particle pair
    "nm_nmthermo_dist_P32_odd_N": dict(natoms=7, nbeads=32, bosonic=False, propagator="normal_modes",
                                       nmthermostat=True, ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0)),
    "nm_nmthermo_bosons_P64_aziz": dict(natoms=20, nbeads=64, propagator="normal_modes", nmthermostat=True,
                                        T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=11.0, inter="aziz",
                                        cutoff_ang=5.5, dt_fs=2.0),
    "nm_nmthermo_dist_P128_2d_nofixcom": dict(ndim=2, natoms=9, nbeads=128, bosonic=False, fixcom=False,
                                              propagator="normal_modes", nmthermostat=True, ext="harmonic",
                                              ext_p=(1.0 * 0.036749326e-3, 0, 0)),
    "nm_nmthermo_bosons_P32_1d": dict(ndim=1, natoms=6, nbeads=32, propagator="normal_modes", nmthermostat=True,
                                      ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0)),
    # the normal-mode propagator without the normal-mode thermostat, P = 32, 64, 128
    "nm_langevin_dist_P64": dict(natoms=9, nbeads=64, bosonic=False, propagator="normal_modes",
                                 ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0)),
    "nm_none_bosons_P32_nofixcom": dict(natoms=6, nbeads=32, propagator="normal_modes", thermostat="none",
                                        fixcom=False, ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0)),
    "nm_langevin_bosons_P128_2d": dict(ndim=2, natoms=5, nbeads=128, propagator="normal_modes",
                                       ext="harmonic", ext_p=(1.0 * 0.036749326e-3, 0, 0)),
    # too many pairs for three warps each to be resident at once: one warp each
    "nm_nmthermo_dist_P32_N2300": dict(natoms=2300, nbeads=32, bosonic=False, propagator="normal_modes",
                                       nmthermostat=True, ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0),
                                       box_ang=60.0),
}
# options applied to the GPU side only
TRAJ_OPTIONS = {"nm_nmthermo_bosons_aziz": [{}, {"fused_normal_modes": 0}, {"fft_normal_modes": 0}],
                "nm_nmthermo_bosons_P64_aziz": [{}, {"fft_normal_modes": 0}, {"fused_normal_modes": 0}],
                "nm_langevin_dist_P64": [{}, {"fft_normal_modes": 0}]}


def _run_pair(kw, steps, seed_state=3, options=None):
    s, cfg = case(**kw)
    x = ring(s, seed=seed_state, spread_ang=0.2)
    p = momenta(s, seed_state)
    tr = O.Trajectory(s, x, p)
    frames = []
    with pk.System(cfg) as g:
        for k, v in (options or {}).items():
            g.set_option(k, v)
        g.set_state(x, p)
        g.set_step(0)
        for st in range(steps):
            xi = O.philox_noise_device(cfg.seed, cfg.replica, st, s.nbeads, s.natoms, s.ndim)
            assert tr.step(xi) == 0
            g.step(1)
            frames.append(((tr.x.copy(), tr.p.copy(), tr.f.copy()), g.get_state()))
    return frames


@pytest.mark.parametrize("name,options", [(n, o) for n in sorted(TRAJ_CASES) for o in TRAJ_OPTIONS.get(n, [{}])])
def test_trajectory_matches_oracle(name, options):
    frames = _run_pair(TRAJ_CASES[name], steps=12, options=options)
    for k, (want, got) in enumerate(frames):
        for w, gq, label in zip(want, got, "xpf"):
            assert rel_per_bead(gq, w) < 1e-9, (k, label, rel_per_bead(gq, w))


@pytest.mark.parametrize("name", ["vv_langevin_bosons_N16_P32", "nm_nmthermo_bosons_aziz"])
def test_multi_step_call_equals_single_steps(name):
    kw = TRAJ_CASES[name]
    s, cfg = case(**kw)
    x = ring(s, seed=5, spread_ang=0.2)
    p = momenta(s, 5)
    with pk.System(cfg) as a, pk.System(cfg) as b:
        a.set_state(x, p)
        b.set_state(x, p)
        a.step(6)
        for _ in range(6):
            b.step(1)
        sa, sb = a.get_state(), b.get_state()
    for u, v in zip(sa, sb):
        assert rel_per_bead(u, v) < 1e-12


def test_deterministic():
    kw = TRAJ_CASES["nm_nmthermo_bosons_aziz"]
    s, cfg = case(**kw)
    x = ring(s, seed=9, spread_ang=0.2)
    p = momenta(s, 9)
    out = []
    for _ in range(2):
        with pk.System(cfg) as g:
            g.set_state(x, p)
            g.step(5)
            out.append(g.get_state())
    for u, v in zip(*out):
        assert np.array_equal(u, v)


@pytest.mark.parametrize("case_name", G.dynamics_cases())
def test_gpu_forces_match_golden_frames(case_name, tmp_path):
    z, _ = G.load()
    ini = G.write_ini(case_name, tmp_path)
    # forces do not depend on the thermostat; the Nose-Hoover cases are read as Langevin
    ini.write_text("\n".join("thermostat = langevin" if ln.strip().startswith("thermostat") else ln
                             for ln in ini.read_text().splitlines()))
    cfg = pk.config_from_ini(ini)
    X = z[f"{case_name}/positions_angstrom"]
    F = z[f"{case_name}/forces_ev_per_angstrom"]
    with pk.System(cfg) as g:
        for fr in range(1, X.shape[0], 4):
            g.set_state(X[fr] * G.ANGSTROM, np.zeros_like(X[fr]))
            g.compute_forces()
            f = g.get_state()[2] / G.EV_PER_ANG
            assert np.allclose(f, F[fr], rtol=1e-5)
            assert np.abs(f - F[fr]).max() <= 1e-9 * np.abs(F[fr]).max()


MIXED_CASES = ["bosons_aziz_pbc_N64_P8", "bosons_dipole_2d", "bosons_pairharm_cosine", "bosons_aziz_pbc_N300_P4"]


@pytest.mark.parametrize("name", MIXED_CASES)
def test_mixed_precision_force_error(name):
    kw, rk = FORCE_CASES[name]
    s, cfg = case(precision="mixed", **kw)
    x = ring(s, seed=len(name), **rk)
    want = O.update_forces(s, x)
    with pk.System(cfg) as g:
        g.set_state(x, np.zeros_like(x))
        g.compute_forces()
        f = g.get_state()[2]
    err = np.linalg.norm(f - want["f"]) / np.linalg.norm(want["f"])
    phys_err = np.linalg.norm(f - want["spring"] - want["phys"]) / np.linalg.norm(want["phys"])
    assert err <= 1e-6 and phys_err <= 1e-6, (err, phys_err)


def test_nonfinite_exchange_potential_is_reported():
    s, cfg = case(natoms=8, nbeads=4, ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0))
    x = ring(s, seed=1)
    x[0, 3, 1] = np.nan
    with pk.System(cfg) as g:
        g.set_state(x, np.zeros_like(x))
        with pytest.raises(pk.ExchangeOverflowError):
            g.compute_forces()
        # the handle stays usable after the error
        x[0, 3, 1] = 0.0
        g.set_state(x, np.zeros_like(x))
        g.compute_forces()


def _violent(seed=11):
    """Beads 1 and P thrown apart by 30 bohr per step: V moves by thousands
    of kT between steps, so the previous step's potentials fail as the
    estimate and the exchange takes its fresh-estimate retry every step."""
    s, cfg = case(natoms=24, nbeads=8, T_K=0.5, ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0),
                  thermostat="none", fixcom=False)
    x = ring(s, seed=seed, spread_ang=0.2)
    p = momenta(s, seed)
    p[0, :, 0] += s.mass * 30.0 / s.dt
    p[-1, :, 0] -= s.mass * 30.0 / s.dt
    return s, cfg, x, p


def test_exchange_retry_after_large_jump():
    s, cfg, x, p = _violent()
    tr = O.Trajectory(s, x, p)
    with pk.System(cfg) as g:
        g.set_state(x, p)
        g.set_step(0)
        for st in range(4):
            assert tr.step(np.zeros((2,) + x.shape)) == 0
            g.step(1)
            gx, gp, gf = g.get_state()
            for got, want, label in ((gx, tr.x, "x"), (gp, tr.p, "p"), (gf, tr.f, "f")):
                assert rel_per_bead(got, want) < 1e-9, (st, label, rel_per_bead(got, want))
        # the violent steps did take the retry
        assert g.exchange_retries() > 0


CELL_CASES = {
    # periodic boxes with at least 4 cutoff-wide cells per edge; centres at
    # least 2.2 A (Aziz) or 1 A (dipole) apart, beads jittered by 0.05 A
    "aziz_3d_N600_P4": (dict(natoms=600, nbeads=4, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=24.0, inter="aziz",
                             cutoff_ang=5.5), 2.2),
    "dipole_2d_N700_P3": (dict(ndim=2, natoms=700, nbeads=3, T_K=2.0, pbc=True, box_ang=60.0, inter="dipole",
                               int_p=(2.4799673e-4, 0, 0), cutoff_ang=9.0, ext="harmonic",
                               ext_p=(1.0 * 0.036749326e-3, 0, 0)), 1.0),
    "aziz_3d_dist_N300_P2": (dict(natoms=300, nbeads=2, bosonic=False, T_K=1.0, mass_amu=4.0026, pbc=True,
                                  box_ang=20.0, inter="aziz", cutoff_ang=4.8), 2.2),
}


@pytest.mark.parametrize("name", sorted(CELL_CASES))
def test_cell_list_forces_match_oracle_and_tiles(name):
    kw, dmin = CELL_CASES[name]
    s, cfg = case(**kw)
    x = ring_separated(s, seed=21, dmin_ang=dmin)
    want = O.update_forces(s, x)["f"]
    out = {}
    for opt in (1, 0):
        with pk.System(cfg) as g:
            g.set_option("cell_lists", opt)
            g.set_state(x, np.zeros_like(x))
            g.compute_forces()
            out[opt] = g.get_state()[2]
    assert rel_per_bead(out[1], want) < FP64_TOL
    assert rel_per_bead(out[1], out[0]) < 1e-12
    s2, cfg2 = case(precision="mixed", **kw)
    with pk.System(cfg2) as g:
        g.set_option("cell_lists", 1)
        g.set_state(x, np.zeros_like(x))
        g.compute_forces()
        f32 = g.get_state()[2]
    assert np.linalg.norm(f32 - want) / np.linalg.norm(want) <= 1e-6


def test_cell_list_trajectory_matches_oracle():
    kw, dmin = CELL_CASES["aziz_3d_N600_P4"]
    s, cfg = case(**kw)
    x = ring_separated(s, seed=22, dmin_ang=dmin)
    p = momenta(s, 22)
    tr = O.Trajectory(s, x, p)
    with pk.System(cfg) as g:
        g.set_option("cell_lists", 1)
        g.set_state(x, p)
        g.set_step(0)
        for st in range(4):
            tr.step(O.philox_noise_device(cfg.seed, cfg.replica, st, s.nbeads, s.natoms, s.ndim))
            g.step(1)
            gx, gp, gf = g.get_state()
            for got, want, label in ((gx, tr.x, "x"), (gp, tr.p, "p"), (gf, tr.f, "f")):
                assert rel_per_bead(got, want) < 1e-9, (st, label)


def test_cell_list_option_needs_cells():
    s, cfg = case(natoms=8, nbeads=2, pbc=True, box_ang=10.0, inter="aziz", cutoff_ang=4.0)
    with pk.System(cfg) as g:
        with pytest.raises(pk.ConfigError, match="cell lists"):
            g.set_option("cell_lists", 1)


@pytest.mark.parametrize("cells", [0, 1])
def test_mixed_precision_liquid_aziz(cells):
    """Mixed precision on a liquid-like Aziz configuration (centres >= 2.2 A
    apart at the benchmark density): FP32 beyond the damping radius, FP64
    inside it, force error <= 1e-6 norm-relative."""
    kw = dict(natoms=512, nbeads=4, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=28.6434, inter="aziz",
              cutoff_ang=5.5 if cells else 14.3217)
    s, cfg = case(precision="mixed", **kw)
    x = ring_separated(s, seed=31, dmin_ang=2.2)
    want = O.update_forces(s, x)
    with pk.System(cfg) as g:
        g.set_option("cell_lists", cells)
        g.set_state(x, np.zeros_like(x))
        g.compute_forces()
        f = g.get_state()[2]
    err = np.linalg.norm(f - want["f"]) / np.linalg.norm(want["f"])
    phys_err = np.linalg.norm(f - want["spring"] - want["phys"]) / np.linalg.norm(want["phys"])
    assert err <= 1e-6 and phys_err <= 1e-6, (err, phys_err)


@pytest.mark.parametrize("name", ["vv_langevin_bosons_N16_P32", "nm_nmthermo_bosons_aziz", "nm_langevin_dist",
                                  "vv_nve_bosons_aziz"])
def test_cuda_graph_steps_equal_plain_launches(name):
    """Replayed step graphs (with the device-side step counter) against plain
    launches, including a jump of the step index between calls."""
    kw = TRAJ_CASES[name]
    s, cfg = case(**kw)
    x = ring(s, seed=8, spread_ang=0.2)
    p = momenta(s, 8)
    out = []
    for graphs in (1, 0):
        with pk.System(cfg) as g:
            g.set_option("cuda_graphs", graphs)
            g.set_state(x, p)
            g.set_step(0)
            for _ in range(4):
                g.step(1)
            g.step(2)
            g.set_step(100)
            for _ in range(3):
                g.step(1)
            assert g.get_step() == 103
            out.append(g.get_state())
    for u, v in zip(*out):
        assert np.array_equal(u, v)


NH_TRAJ = {
    "nh_bosons_trap": dict(natoms=8, nbeads=4, thermostat="nose_hoover", fixcom=False, ext="harmonic",
                           ext_p=(3.0 * 0.036749326e-3, 0, 0), dt_fs=0.5),
    "nh_np_bosons_pairharm_fixcom": dict(natoms=10, nbeads=6, thermostat="nose_hoover_np", ext="harmonic",
                                         ext_p=(3.0 * 0.036749326e-3, 0, 0), inter="harmonic",
                                         int_p=(1.0 * 0.036749326e-3, 0, 0), dt_fs=0.5),
    "nh_np_dim_dist_2d": dict(ndim=2, natoms=12, nbeads=5, bosonic=False, thermostat="nose_hoover_np_dim",
                              ext="harmonic", ext_p=(1.0 * 0.036749326e-3, 0, 0), dt_fs=0.5),
    "nh_nmcoupling_bosons": dict(natoms=8, nbeads=8, thermostat="nose_hoover", nmthermostat=True, fixcom=False,
                                 ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0), dt_fs=0.5),
    "nh_np_nm_propagator_dist": dict(natoms=9, nbeads=4, bosonic=False, propagator="normal_modes",
                                     thermostat="nose_hoover_np", nmthermostat=True, ext="harmonic",
                                     ext_p=(3.0 * 0.036749326e-3, 0, 0), dt_fs=0.5),
}


@pytest.mark.parametrize("name", sorted(NH_TRAJ))
def test_nose_hoover_trajectory_matches_oracle(name):
    kw = NH_TRAJ[name]
    s, cfg = case(**kw)
    x = ring(s, seed=13, spread_ang=0.2)
    p = momenta(s, 13)
    tr = O.Trajectory(s, x, p)
    noise = np.zeros((2,) + x.shape)
    with pk.System(cfg) as g:
        g.set_state(x, p)
        for st in range(12):
            assert tr.step(noise) == 0
            g.step(1)
            gx, gp, gf = g.get_state()
            for got, want, label in ((gx, tr.x, "x"), (gp, tr.p, "p"), (gf, tr.f, "f")):
                assert rel_per_bead(got, want) < 1e-9, (st, label, rel_per_bead(got, want))
        ob = g.observables()
    assert abs(ob["nh_energy"] - tr.nh_energy()) <= 1e-9 * abs(tr.nh_energy())


@pytest.mark.parametrize("name", ["nm_nmthermo_bosons_aziz", "vv_langevin_bosons_N16_P32"])
def test_step_io_equals_separate_calls(name):
    """pimdb_step_io (state in, steps, state out, one synchronisation) gives
    bitwise the state of pimdb_set_state + pimdb_step + pimdb_get_state."""
    s, cfg = case(**TRAJ_CASES[name])
    x = ring(s, seed=8, spread_ang=0.2)
    p = momenta(s, 8)
    with pk.System(cfg) as a, pk.System(cfg) as b:
        for g in (a, b):
            g.set_step(0)
        xa, pa = x.copy(), p.copy()
        xb, pb = x.copy(), p.copy()
        for n in (1, 2, 1):
            a.set_state(xa, pa)
            a.step(n)
            xa, pa, fa = a.get_state()
            xb, pb, fb = b.step_io(xb, pb, n)
            for u, v in ((xa, xb), (pa, pb), (fa, fb)):
                assert np.array_equal(u, v)
        # absent inputs keep the device state; nsteps = 0 only reads it
        xc, pc, fc = b.step_io(None, None, 0)
        assert np.array_equal(xc, xb) and np.array_equal(pc, pb) and np.array_equal(fc, fb)
        a.step(1)
        xa, pa, fa = a.get_state()
        xc, pc, fc = b.step_io(None, None, 1)
        for u, v in ((xa, xc), (pa, pc), (fa, fc)):
            assert np.array_equal(u, v)


def test_step_io_reports_a_nonfinite_exchange():
    kw, rk = FORCE_CASES["bosons_trap_N16_P32"]
    s, cfg = case(**kw)
    x = ring(s, seed=2, **rk)
    x[0, 0, 0] = np.nan
    with pk.System(cfg) as g:
        with pytest.raises(pk.ExchangeOverflowError):
            g.step_io(x, np.zeros_like(x), 1)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("reserved", [0, 4096])
def test_pair_tiles_forces_do_not_depend_on_reserved_sms(reserved, precision):
    """Beside the bosonic exchange the pair-tile blocks that land on the
    reserved SMs take no tile; the warp that finishes last takes the tiles
    left.  With every SM reserved (4096: all blocks idle until that warp) and
    with none, the forces match the oracle and the automatic setting."""
    s, cfg = case(natoms=70, nbeads=4, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=14.0, inter="aziz",
                  cutoff_ang=7.0, precision=precision)
    x = ring_separated(s, seed=41, dmin_ang=2.2)
    want = O.update_forces(s, x)["f"]
    out = {}
    for opt in (-1, reserved):
        with pk.System(cfg) as g:
            g.set_option("cell_lists", 0)
            g.set_option("reserved_sms", opt)
            g.set_state(x, np.zeros_like(x))
            g.compute_forces()
            out[opt] = g.get_state()[2]
    if precision == "fp64":
        assert rel_per_bead(out[reserved], want) < FP64_TOL
    else:
        assert np.linalg.norm(out[reserved] - want) <= 1e-6 * np.linalg.norm(want)
    assert rel_per_bead(out[reserved], out[-1]) < 1e-12


def test_pair_tiles_half_box_edge_images():
    """Far-field pair separations take the image the FP32 screen chose; pairs
    whose FP32 test lies within 1e-6 L of the half-box edge take the exact
    FP64 minimum image.  Six pairs with the cutoff at L/2, each just inside
    it and with its separation along one axis 1e-9 .. 1e-5 L short of L/2
    (or past it, the other image), match the oracle (FP64 tolerance).  No
    two particles are closer than 2.8 A, so every pair's force counts."""
    L_ang = 22.7297
    eps_list = [1e-9, 1e-7, 5e-7, 2e-6, 1e-5, 3e-6]
    s, cfg = case(natoms=2 * len(eps_list), nbeads=2, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=L_ang,
                  inter="aziz", cutoff_ang=0.5 * L_ang)
    L = s.size
    pts = []
    for k, eps in enumerate(eps_list):
        axis = k % 3
        sign = 1.0 if (k // 3) % 2 == 0 else -1.0
        o1, o2 = (axis + 1) % 3, (axis + 2) % 3
        base = np.zeros(3)
        base[o1] = (k % 3 - 1) * 0.18 * L
        base[o2] = (k // 3 - 0.5) * 0.3 * L
        a, b = base.copy(), base.copy()
        a[axis] = -0.25 * L
        b[axis] = 0.25 * L - sign * eps * L
        b[o1] += 0.3 * np.sqrt(eps) * L  # r just inside L/2
        pts += [a, b]
    x = np.repeat(np.array(pts)[None], s.nbeads, axis=0)
    x[1] += np.random.default_rng(17).normal(0.0, 1e-4, x[1].shape)
    d = x[0][:, None] - x[0][None]
    d -= L * np.round(d / L)
    r = np.sqrt((d ** 2).sum(-1)) + 1e9 * np.eye(s.natoms)
    assert r.min() > 2.8 * 1.8897261
    want = O.update_forces(s, x)["f"]
    with pk.System(cfg) as g:
        g.set_option("cell_lists", 0)
        g.set_state(x, np.zeros_like(x))
        g.compute_forces()
        got = g.get_state()[2]
    assert rel_per_bead(got, want) < FP64_TOL


def test_step_io_graph_replay_equals_plain_launches():
    """On page-locked arrays a whole step_io call (state in, steps, deferred
    tail, state out, error word) is replayed as one CUDA graph, cached by
    step count, step state and arrays: bitwise the state of plain launches,
    with step counts and array sets changing between calls and ordinary
    calls in between."""
    torch = pytest.importorskip("torch")
    s, cfg = case(**TRAJ_CASES["nm_nmthermo_bosons_P64_aziz"])
    x = ring(s, seed=9, spread_ang=0.2)
    p = momenta(s, 9)
    bufs = [[torch.empty(x.shape, dtype=torch.float64, pin_memory=True) for _ in range(3)] for _ in range(2)]
    with pk.System(cfg) as a, pk.System(cfg) as b:
        a.set_option("cuda_graphs", 0)
        for g in (a, b):
            g.set_step(0)
            g.set_state(x, p)
            g.step(1)
        xa, pa, _ = a.get_state()
        for k, n in enumerate((1, 2, 1, 3, 1, 1)):
            hx, hp, hf = bufs[k % 2]
            hx.copy_(torch.from_numpy(xa))
            hp.copy_(torch.from_numpy(pa))
            xa, pa, fa = a.step_io(xa, pa, n)
            b.step_io_ptr(hx.data_ptr(), hp.data_ptr(), n, hx.data_ptr(), hp.data_ptr(), hf.data_ptr())
            for u, v in ((xa, hx), (pa, hp), (fa, hf)):
                assert np.array_equal(u, v.numpy()), (k, n)
            if k == 2:  # an ordinary call between graph replays
                a.step(1)
                b.step(1)
                xa, pa, _ = a.get_state()
                xb, pb, _ = b.get_state()
                assert np.array_equal(xa, xb) and np.array_equal(pa, pb)


def test_step_io_with_page_locked_buffers():
    """Page-locked host arrays are read and written by the state kernels
    directly: the same state, bitwise, as through copies of pageable arrays."""
    torch = pytest.importorskip("torch")
    s, cfg = case(**TRAJ_CASES["nm_nmthermo_bosons_P64_aziz"])
    x = ring(s, seed=6, spread_ang=0.2)
    p = momenta(s, 6)
    hx, hp, hf = (torch.empty(x.shape, dtype=torch.float64, pin_memory=True) for _ in range(3))
    hx.copy_(torch.from_numpy(x))
    hp.copy_(torch.from_numpy(p))
    with pk.System(cfg) as a, pk.System(cfg) as b:
        for g in (a, b):
            g.set_step(0)
        xa, pa = x.copy(), p.copy()
        for _ in range(3):
            xa, pa, fa = a.step_io(xa, pa, 1)
            b.step_io_ptr(hx.data_ptr(), hp.data_ptr(), 1, hx.data_ptr(), hp.data_ptr(), hf.data_ptr())
            for u, v in ((xa, hx), (pa, hp), (fa, hf)):
                assert np.array_equal(u, v.numpy())
        b.set_state_ptr(hx.data_ptr(), hp.data_ptr(), device=False)
        b.get_state_ptr(hx.data_ptr(), None, hf.data_ptr(), device=False)
        assert np.array_equal(hx.numpy(), xa)

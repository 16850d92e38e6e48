"""The factorial bosonic exchange (sum over all N! permutations,
src/bosonic_exchange/factorial_bosonic_exchange.cpp; the reference's
FACTORIAL_BOSONIC_ALGORITHM build) on the GPU against the oracle, whose
restatement is bit-identical to the compiled factorial reference
(test_oracle_vs_reference.py) and pinned on its golden dynamics frames
(test_oracle_golden.py).

Tolerances: FP64 within 1e-10 relative (forces per bead, V_B, primEstimator),
trajectories within 1e-9 relative per bead.  At 12 particles, too many
permutations for the oracle, the checks are size-independent: relabelling the
particles permutes the forces and leaves the scalars unchanged (a property of
the full permutation sum that the Feldman-Hirshberg recursion does not have),
and the exterior links' forces cancel between beads 1 and P."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_cases import MEV, case, momenta, pk, rel_per_bead, ring

FP64_TOL = 1e-10

CASES = {
    # name: case kwargs (exchange="factorial" added)
    "N1_P4": dict(natoms=1, nbeads=4, ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
    "N2_P2": dict(natoms=2, nbeads=2, ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
    "N3_P8_trap": dict(natoms=3, nbeads=8, T_K=5.802, ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
    "N4_P6_pairharm_cosine": dict(natoms=4, nbeads=6, inter="harmonic", int_p=(1.0 * MEV, 0, 0), ext="cosine",
                                  ext_p=(1.0 * MEV, 0.3, 0)),
    "N5_P4_aziz_pbc": dict(natoms=5, nbeads=4, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=8.0, inter="aziz",
                           cutoff_ang=4.0),
    "N6_P3_1d": dict(ndim=1, natoms=6, nbeads=3, ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
    "N7_P5_dipole_2d": dict(ndim=2, natoms=7, nbeads=5, T_K=2.0, inter="dipole", int_p=(2.4799673e-4, 0, 0),
                            ext="harmonic", ext_p=(1.0 * MEV, 0, 0), box_ang=20.0),
    "N8_P16_trap": dict(natoms=8, nbeads=16, ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
    "N9_P4_double_well_pbc": dict(natoms=9, nbeads=4, pbc=True, box_ang=9.0, ext="double_well",
                                  ext_p=(1.32684e-7 * MEV, 3.0 * 1.8897261, 0)),
}


def fcase(**kw):
    return case(exchange="factorial", **kw)


# ------------------------------------------------------------------------ CPU
def test_factorial_rejects_more_than_twelve_particles():
    _, cfg = fcase(natoms=13, nbeads=4)
    with pytest.raises(pk.ConfigError, match="at most 12 particles"):
        pk.System(cfg)


def test_batch_rejects_the_factorial_exchange():
    _, cfg = fcase(natoms=4, nbeads=4)
    with pytest.raises(pk.ConfigError, match="Feldman-Hirshberg"):
        pk.Batch([cfg])


def test_unknown_exchange_algorithm_is_rejected():
    _, cfg = case(natoms=4, nbeads=4)
    cfg.exchange = 7
    with pytest.raises(pk.ConfigError, match="exchange algorithm"):
        pk.System(cfg)


# ------------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_factorial_forces_and_scalars_match_oracle(name):
    s, cfg = fcase(**CASES[name])
    x = ring(s, seed=len(name), spread_ang=0.3)
    want = O.update_forces(s, x)["f"]
    ref = O.exchange(s, x)
    with pk.System(cfg) as g:
        g.set_state(x, np.zeros_like(x))
        g.compute_forces()
        _, _, f = g.get_state()
        got = g.exchange()
        with pytest.raises(pk.ConfigError):
            g.exchange_arrays()
    assert rel_per_bead(f, want) < FP64_TOL
    assert abs(got["VB"] - ref["VB"]) <= FP64_TOL * abs(ref["VB"])
    assert abs(got["prim"] - ref["prim"]) <= FP64_TOL * abs(ref["prim"])
    assert got["p_distinct"] == 0.0 and got["p_longest"] == 0.0
    for key in ("f1", "fP"):
        assert np.abs(got[key] - ref[key]).max() <= FP64_TOL * np.abs(ref[key]).max(), key


@pytest.mark.gpu
def test_factorial_ten_particles_matches_oracle():
    s, cfg = fcase(natoms=10, nbeads=4, ext="harmonic", ext_p=(3.0 * MEV, 0, 0))
    x = ring(s, seed=10, spread_ang=0.3)
    ref = O.exchange(s, x)
    with pk.System(cfg) as g:
        g.set_state(x, np.zeros_like(x))
        got = g.exchange()
    assert abs(got["VB"] - ref["VB"]) <= FP64_TOL * abs(ref["VB"])
    assert abs(got["prim"] - ref["prim"]) <= FP64_TOL * abs(ref["prim"])
    for key in ("f1", "fP"):
        assert np.abs(got[key] - ref[key]).max() <= FP64_TOL * np.abs(ref[key]).max(), key


@pytest.mark.gpu
@pytest.mark.parametrize("cells", [0, 1])
def test_factorial_trajectory_matches_oracle(cells):
    kw = dict(natoms=6, nbeads=8, T_K=2.0, ext="harmonic", ext_p=(3.0 * MEV, 0, 0), inter="harmonic",
              int_p=(1.0 * MEV, 0, 0))
    if cells:  # the cell-list force path adds fx in its finishing kernel
        kw = dict(natoms=8, nbeads=4, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=24.0, inter="aziz",
                  cutoff_ang=5.5)
    s, cfg = fcase(**kw)
    x = ring(s, seed=3, spread_ang=0.2)
    p = momenta(s, 3)
    tr = O.Trajectory(s, x, p)
    with pk.System(cfg) as g:
        if cells:
            g.set_option("cell_lists", 1)
        g.set_state(x, p)
        g.set_step(0)
        for st in range(10):
            xi = O.philox_noise_device(cfg.seed, cfg.replica, st, s.nbeads, s.natoms, s.ndim)
            assert tr.step(xi) == 0
            g.step(1)
            gx, gp, gf = g.get_state()
            for got, want, label in ((gx, tr.x, "x"), (gp, tr.p, "p"), (gf, tr.f, "f")):
                assert rel_per_bead(got, want) < 1e-9, (st, label, rel_per_bead(got, want))


@pytest.mark.gpu
def test_factorial_observables_match_oracle():
    s, cfg = fcase(natoms=5, nbeads=6, T_K=2.0, ext="harmonic", ext_p=(3.0 * MEV, 0, 0), inter="harmonic",
                   int_p=(1.0 * MEV, 0, 0))
    x = ring(s, seed=4, spread_ang=0.3)
    p = momenta(s, 4)
    want = O.observables(s, x, p)
    with pk.System(cfg) as g:
        g.set_state(x, p)
        got = g.observables()
        terms = g.potential_energy()
    for k, v in want.items():
        assert abs(got[k] - v) <= 1e-10 * abs(v) + 1e-300, (k, got[k], v)
    assert abs(terms[3] - O.exchange(s, x)["VB"]) <= FP64_TOL * abs(terms[3])


@pytest.mark.gpu
def test_factorial_twelve_particles_relabelling_and_link_balance():
    s, cfg = fcase(natoms=12, nbeads=3, ext="harmonic", ext_p=(3.0 * MEV, 0, 0), box_ang=6.0)
    x = ring(s, seed=12, spread_ang=0.3)
    perm = np.random.default_rng(1).permutation(12)
    with pk.System(cfg) as g:
        g.set_state(x, np.zeros_like(x))
        a = g.exchange()
        a2 = g.exchange()
        g.set_state(x[:, perm], np.zeros_like(x))
        b = g.exchange()
    for key in ("VB", "prim", "f1", "fP"):
        assert np.array_equal(np.asarray(a[key]), np.asarray(a2[key])), key  # deterministic
    assert abs(a["VB"] - b["VB"]) <= 1e-12 * abs(a["VB"])
    assert abs(a["prim"] - b["prim"]) <= 1e-12 * abs(a["prim"])
    for key in ("f1", "fP"):
        assert np.abs(a[key][perm] - b[key]).max() <= 1e-12 * np.abs(a[key]).max(), key
    # the exterior links' forces cancel: what remains is the interior springs
    k = s.spring_constant
    interior = k * ((x[1] - x[0]).sum(0) + (x[s.nbeads - 2] - x[s.nbeads - 1]).sum(0))
    total = a["f1"].sum(0) + a["fP"].sum(0)
    assert np.abs(total - interior).max() <= 1e-10 * np.abs(a["f1"]).max()


@pytest.mark.gpu
def test_factorial_graph_replay_equals_plain_launches():
    s, cfg = fcase(natoms=7, nbeads=4, ext="harmonic", ext_p=(3.0 * MEV, 0, 0))
    x = ring(s, seed=7, spread_ang=0.3)
    p = momenta(s, 7)
    out = []
    for graphs in (1, 0):
        with pk.System(cfg) as g:
            g.set_option("cuda_graphs", graphs)
            g.set_state(x, p)
            g.set_step(0)
            g.step(4)
            g.step(4)
            out.append(g.get_state())
    for u, v in zip(*out):
        assert np.array_equal(u, v)

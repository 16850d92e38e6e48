"""Batched replicas (pimdb_batch_*): many independent systems with their own
N, P, temperature and potentials advanced by one launch per step.

GPU parity: every replica of an FP64 batch matches the oracle run on that
replica alone (forces and exchange scalars within 1e-10, trajectories within
1e-9 relative per bead), and the one-system path within 1e-12.  Mixed
batches: FP32 pair forces with FP64 accumulation within 1e-6 norm-relative
force error of the FP64 oracle.  CPU: configuration checks that need no GPU.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_cases import MEV, case, momenta, pk, rel_per_bead, ring

REPLICAS_3D = [
    # case kwargs: uneven N, P, temperature and potentials
    dict(natoms=16, nbeads=32, ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
    dict(natoms=7, nbeads=5, T_K=2.5, ext="harmonic", ext_p=(3.0 * MEV, 0, 0), inter="harmonic",
         int_p=(1.0 * MEV, 0, 0)),
    dict(natoms=40, nbeads=8, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=12.0, inter="aziz", cutoff_ang=6.0),
    dict(natoms=33, nbeads=3, bosonic=False, ext="double_well", ext_p=(1.32684e-7 * MEV, 3.0 * 1.8897261, 0),
         inter="harmonic", int_p=(1.0 * MEV, 0, 0)),
    dict(natoms=1, nbeads=4, ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
    dict(natoms=9, nbeads=1, T_K=0.7, inter="harmonic", int_p=(1.0 * MEV, 0, 0), ext="cosine",
         ext_p=(1.0 * MEV, 0.3, 0)),
    dict(natoms=70, nbeads=16, T_K=3.0, ext="harmonic", ext_p=(3.0 * MEV, 0, 0), inter="harmonic",
         int_p=(1.0 * MEV, 0, 0), thermostat="none", fixcom=False),
    dict(natoms=6, nbeads=2, fixcom=False, ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
]

REPLICAS_2D = [
    dict(ndim=2, natoms=24, nbeads=5, T_K=2.0, inter="dipole", int_p=(2.4799673e-4, 0, 0), ext="harmonic",
         ext_p=(1.0 * MEV, 0, 0), box_ang=40.0),
    dict(ndim=2, natoms=11, nbeads=8, T_K=1.0, ext="harmonic", ext_p=(1.0 * MEV, 0, 0)),
]


def build(replicas, precision="fp64"):
    systems, cfgs, xs, ps = [], [], [], []
    for r, kw in enumerate(replicas):
        s, cfg = case(precision=precision, **kw)
        cfg.seed = 1000 + 17 * r
        cfg.replica = r
        systems.append(s)
        cfgs.append(cfg)
        xs.append(ring(s, seed=50 + r, spread_ang=0.2))
        ps.append(momenta(s, 50 + r))
    return systems, cfgs, xs, ps


def norm_rel(got, want):
    return float(np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300))


# ------------------------------------------------------------------------ CPU
def test_batch_rejects_mixed_dimensions():
    _, c3 = case(natoms=4, nbeads=2)
    _, c2 = case(ndim=2, natoms=4, nbeads=2)
    with pytest.raises(pk.ConfigError, match="same ndim"):
        pk.Batch([c3, c2])


def test_batch_rejects_nose_hoover():
    _, c = case(natoms=4, nbeads=4, bosonic=False, thermostat="nose_hoover")
    with pytest.raises(pk.ConfigError, match="Langevin thermostat"):
        pk.Batch([c])


def test_batch_accepts_normal_modes_and_rejects_too_many_beads():
    # normal modes pass the configuration checks (without a GPU the batch
    # then fails for want of a device, not of the configuration)
    _, c = case(natoms=4, nbeads=8, propagator="normal_modes", nmthermostat=True)
    try:
        pk.Batch([c]).close()
    except pk.ConfigError:
        pytest.fail("a normal-mode replica was rejected")
    except pk.PimdbError:
        pass
    _, big = case(natoms=2, nbeads=512, propagator="normal_modes")
    with pytest.raises(pk.ConfigError, match="256 beads"):
        pk.Batch([big])


def test_batch_rejects_mixed_precisions():
    _, a = case(natoms=4, nbeads=2)
    _, b = case(natoms=4, nbeads=2, precision="mixed")
    with pytest.raises(pk.ConfigError, match="same precision"):
        pk.Batch([a, b])


# ------------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("replicas", [REPLICAS_3D, REPLICAS_2D], ids=["3d", "2d"])
def test_batch_forces_match_oracle(replicas):
    systems, cfgs, xs, ps = build(replicas)
    with pk.Batch(cfgs) as b:
        b.set_states(xs, ps)
        b.compute_forces()
        _, _, fs = b.get_states()
    for r, s in enumerate(systems):
        want = O.update_forces(s, xs[r])["f"]
        assert rel_per_bead(fs[r], want) < 1e-10, r


@pytest.mark.gpu
def test_batch_large_replica_takes_smaller_blocks():
    """A 1000-particle replica beside a small one: every warp stages the
    largest replica's positions, which at 256 threads would need more
    shared memory than a block can have, so the batch is created with
    smaller blocks; its forces match the oracle (1e-10), and a block shape
    that cannot hold the replica is refused as a configuration error."""
    replicas = [dict(natoms=1000, nbeads=4, ext="harmonic", ext_p=(3.0 * MEV, 0, 0), box_ang=40.0),
                dict(natoms=12, nbeads=8, ext="harmonic", ext_p=(3.0 * MEV, 0, 0))]
    systems, cfgs, xs, ps = build(replicas)
    with pk.Batch(cfgs) as b:
        assert b.launch()["threads"] < 256
        with pytest.raises(pk.ConfigError):
            b.set_option("threads", 256)
        b.set_states(xs, ps)
        b.compute_forces()
        _, _, fs = b.get_states()
    for r, s in enumerate(systems):
        want = O.update_forces(s, xs[r])["f"]
        assert rel_per_bead(fs[r], want) < 1e-10, r


@pytest.mark.gpu
def test_batch_exchange_scalars_match_oracle():
    systems, cfgs, xs, ps = build(REPLICAS_3D)
    with pk.Batch(cfgs) as b:
        b.set_states(xs, ps)
        sc = b.exchange()
    for r, s in enumerate(systems):
        if not (s.bosonic and s.nbeads > 1):
            assert not sc[r].any()
            continue
        ex = O.exchange(s, xs[r])
        want = np.array([ex["VB"], ex["prim"], ex["p_distinct"], ex["p_longest"]])
        assert np.allclose(sc[r], want, rtol=1e-10, atol=0), (r, sc[r], want)


@pytest.mark.gpu
@pytest.mark.parametrize("replicas", [REPLICAS_3D, REPLICAS_2D], ids=["3d", "2d"])
def test_batch_trajectories_match_oracle(replicas):
    systems, cfgs, xs, ps = build(replicas)
    trs = [O.Trajectory(s, xs[r], ps[r]) for r, s in enumerate(systems)]
    with pk.Batch(cfgs) as b:
        b.set_states(xs, ps)
        b.set_step(0)
        for st in range(8):
            for r, (s, c) in enumerate(zip(systems, cfgs)):
                xi = O.philox_noise_device(c.seed, c.replica, st, s.nbeads, s.natoms, s.ndim)
                assert trs[r].step(xi) == 0
            b.step(1)
            gx, gp, gf = b.get_states()
            for r, tr in enumerate(trs):
                for got, want, label in ((gx[r], tr.x, "x"), (gp[r], tr.p, "p"), (gf[r], tr.f, "f")):
                    assert rel_per_bead(got, want) < 1e-9, (st, r, label, rel_per_bead(got, want))


@pytest.mark.gpu
def test_batch_replica_equals_one_system_path():
    systems, cfgs, xs, ps = build(REPLICAS_3D[:3])
    with pk.Batch(cfgs) as b:
        b.set_states(xs, ps)
        b.set_step(0)
        b.step(6)
        bx, bp, bf = b.get_states()
    for r, c in enumerate(cfgs):
        with pk.System(c) as g:
            g.set_state(xs[r], ps[r])
            g.set_step(0)
            g.step(6)
            x, p, f = g.get_state()
        for u, v in ((bx[r], x), (bp[r], p), (bf[r], f)):
            assert rel_per_bead(u, v) < 1e-12, r


REPLICAS_NM = [
    # the normal-mode propagator with each thermostat, and the normal-mode
    # thermostat under velocity Verlet; bosons and distinguishable, PBC, 2D
    dict(natoms=16, nbeads=32, propagator="normal_modes", nmthermostat=True, ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
    dict(natoms=20, nbeads=8, propagator="normal_modes", T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=11.0,
         inter="aziz", cutoff_ang=5.5, dt_fs=2.0),
    dict(natoms=13, nbeads=6, bosonic=False, propagator="normal_modes", nmthermostat=True, fixcom=False,
         ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
    dict(natoms=7, nbeads=5, bosonic=False, propagator="normal_modes", thermostat="none",
         ext="harmonic", ext_p=(3.0 * MEV, 0, 0), inter="harmonic", int_p=(1.0 * MEV, 0, 0)),
    dict(natoms=8, nbeads=8, nmthermostat=True, ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
    dict(ndim=2, natoms=11, nbeads=64, propagator="normal_modes", nmthermostat=True, ext="harmonic",
         ext_p=(1.0 * MEV, 0, 0)),
    dict(natoms=5, nbeads=1, propagator="normal_modes", ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
]


@pytest.mark.gpu
def test_batch_normal_modes_match_oracle():
    """Normal-mode replicas (normal_modes_propagator.cpp:19-71, the Langevin
    O-step in the normal-mode frame) against the oracle run on each alone:
    8 steps within 1e-9 relative per bead, as the Cartesian replicas."""
    for group in (REPLICAS_NM[:5], REPLICAS_NM[5:6], REPLICAS_NM[6:]):  # one batch per ndim (and P = 1 apart)
        systems, cfgs, xs, ps = build(group)
        trs = [O.Trajectory(s, xs[r], ps[r]) for r, s in enumerate(systems)]
        with pk.Batch(cfgs) as b:
            b.set_states(xs, ps)
            b.set_step(0)
            for st in range(8):
                for r, (s, c) in enumerate(zip(systems, cfgs)):
                    xi = O.philox_noise_device(c.seed, c.replica, st, s.nbeads, s.natoms, s.ndim)
                    assert trs[r].step(xi) == 0
                b.step(1)
                gx, gp, gf = b.get_states()
                for r, tr in enumerate(trs):
                    for got, want, label in ((gx[r], tr.x, "x"), (gp[r], tr.p, "p"), (gf[r], tr.f, "f")):
                        assert rel_per_bead(got, want) < 1e-9, (st, r, label, rel_per_bead(got, want))


@pytest.mark.gpu
def test_batch_normal_modes_equal_one_system_matrix_path():
    """The batch's transforms sum in the order of the one-system path's
    matrix kernels (fused_normal_modes 0): 6 steps within 1e-12."""
    systems, cfgs, xs, ps = build(REPLICAS_NM[:4])
    with pk.Batch(cfgs) as b:
        b.set_states(xs, ps)
        b.set_step(0)
        b.step(6)
        bx, bp, bf = b.get_states()
    for r, c in enumerate(cfgs):
        with pk.System(c) as g:
            g.set_option("fused_normal_modes", 0)
            g.set_state(xs[r], ps[r])
            g.set_step(0)
            g.step(6)
            x, p, f = g.get_state()
        for u, v in ((bx[r], x), (bp[r], p), (bf[r], f)):
            assert rel_per_bead(u, v) < 1e-12, r


@pytest.mark.gpu
def test_batch_normal_modes_mixed_tracks_fp64():
    _, c64, xs, ps = build(REPLICAS_NM[:5])
    _, c32, _, _ = build(REPLICAS_NM[:5], precision="mixed")
    out = []
    for cfgs in (c64, c32):
        with pk.Batch(cfgs) as b:
            b.set_states(xs, ps)
            b.step(5)
            out.append(b.get_states()[0])
    for r in range(len(c64)):
        assert norm_rel(out[1][r], out[0][r]) < 1e-6, r


@pytest.mark.gpu
@pytest.mark.parametrize("inter,int_p", [("harmonic", (1.0 * MEV, 0, 0)), ("dipole", (2.4799673e-4, 0, 0))])
def test_batch_fp64_double_float_pairs_at_edge_and_cutoff(inter, int_p):
    """The FP64 batch evaluates harmonic and dipole pairs in double-float; a
    pair within 1e-6 L of the half-box edge or within 1e-5 of the cutoff takes
    the FP64 image and in/out decision.  Six pairs with the cutoff at L/2,
    each with its separation along one axis 1e-9 .. 1e-5 L short of L/2 (or
    past it) and just inside the cutoff, match the oracle within 1e-10."""
    L_ang = 12.0
    eps_list = [1e-9, 1e-7, 5e-7, 2e-6, 1e-5, 3e-6]
    s, cfg = case(natoms=2 * len(eps_list), nbeads=2, T_K=2.0, pbc=True, box_ang=L_ang, inter=inter, int_p=int_p,
                  cutoff_ang=0.5 * L_ang)
    L = s.size
    pts = []
    for k, eps in enumerate(eps_list):
        axis = k % 3
        sign = 1.0 if (k // 3) % 2 == 0 else -1.0
        o1, o2 = (axis + 1) % 3, (axis + 2) % 3
        base = np.zeros(3)
        base[o1] = (k % 3 - 1) * 0.18 * L
        base[o2] = (k // 3 - 0.5) * 0.3 * L
        a, c = base.copy(), base.copy()
        a[axis] = -0.25 * L
        c[axis] = 0.25 * L - sign * eps * L
        c[o1] += 0.3 * np.sqrt(eps) * L
        pts += [a, c]
    x = np.repeat(np.array(pts)[None], s.nbeads, axis=0)
    x[1] += np.random.default_rng(19).normal(0.0, 1e-4, x[1].shape)
    want = O.update_forces(s, x)["f"]
    with pk.Batch([cfg]) as b:
        b.set_states([x], [np.zeros_like(x)])
        b.compute_forces()
        got = b.get_states()[2][0]
    assert rel_per_bead(got, want) < 1e-10


@pytest.mark.gpu
def test_batch_graph_replay_equals_plain_launches():
    _, cfgs, xs, ps = build(REPLICAS_3D)
    out = []
    for graph in (1, 0):
        with pk.Batch(cfgs) as b:
            b.set_option("graph", graph)
            b.set_states(xs, ps)
            b.step(5)
            b.step(5)  # the second call replays the cached graph
            assert b.get_step() == 10
            out.append(b.get_states(flat=True))
    for u, v in zip(*out):
        assert np.array_equal(u, v)


@pytest.mark.gpu
def test_batch_deterministic_and_block_shape_independent():
    _, cfgs, xs, ps = build(REPLICAS_3D)
    out = []
    for threads, ctas in ((256, 2), (256, 2), (128, 4), (512, 1)):
        with pk.Batch(cfgs) as b:
            b.set_option("threads", threads)
            b.set_option("ctas_per_sm", ctas)
            b.set_states(xs, ps)
            b.step(4)
            out.append(b.get_states(flat=True))
    for u, v in zip(out[0], out[1]):
        assert np.array_equal(u, v)
    for other in out[2:]:
        for u, v in zip(out[0], other):
            assert np.abs(u - v).max() <= 1e-12 * np.abs(v).max()


@pytest.mark.gpu
def test_batch_autotune_keeps_the_state():
    _, cfgs, xs, ps = build(REPLICAS_3D)
    with pk.Batch(cfgs) as a, pk.Batch(cfgs) as b:
        for g in (a, b):
            g.set_states(xs, ps)
            g.set_step(3)
        threads, ctas = a.autotune(steps=2)
        assert threads in (128, 256, 512) and ctas >= 1
        assert a.get_step() == 3
        a.step(3)
        b.step(3)
        for u, v in zip(a.get_states(flat=True), b.get_states(flat=True)):
            assert np.abs(u - v).max() <= 1e-12 * np.abs(v).max()


@pytest.mark.gpu
@pytest.mark.parametrize("replicas", [REPLICAS_3D, REPLICAS_2D], ids=["3d", "2d"])
def test_batch_mixed_force_error(replicas):
    systems, cfgs, xs, ps = build(replicas, precision="mixed")
    with pk.Batch(cfgs) as b:
        b.set_states(xs, ps)
        b.compute_forces()
        _, _, fs = b.get_states()
    for r, s in enumerate(systems):
        want = O.update_forces(s, xs[r])["f"]
        assert norm_rel(fs[r], want) <= 1e-6, (r, norm_rel(fs[r], want))


@pytest.mark.gpu
def test_batch_mixed_trajectory_tracks_fp64():
    _, c64, xs, ps = build(REPLICAS_3D)
    _, c32, _, _ = build(REPLICAS_3D, precision="mixed")
    out = []
    for cfgs in (c64, c32):
        with pk.Batch(cfgs) as b:
            b.set_states(xs, ps)
            b.step(5)
            out.append(b.get_states()[0])
    for r in range(len(c64)):
        assert norm_rel(out[1][r], out[0][r]) < 1e-6, r


@pytest.mark.gpu
def test_batch_nonfinite_exchange_names_the_replica():
    systems, cfgs, xs, ps = build(REPLICAS_3D[:3])
    xs[2] = xs[2].copy()
    xs[2][0, 0, 0] = np.nan
    with pk.Batch(cfgs) as b:
        b.set_states(xs, ps)
        with pytest.raises(pk.ExchangeOverflowError, match="replica 2"):
            b.compute_forces()


@pytest.mark.gpu
def test_batch_exchange_retry_after_large_jump():
    from tests.test_gpu_parity import _violent
    s, cfg, x, p = _violent()
    systems, cfgs, xs, ps = build(REPLICAS_3D[:2])
    systems.append(s)
    cfgs.append(cfg)
    xs.append(x)
    ps.append(p)
    trs = [O.Trajectory(q, xs[r], ps[r]) for r, q in enumerate(systems)]
    with pk.Batch(cfgs) as b:
        b.set_states(xs, ps)
        b.set_step(0)
        for st in range(4):
            for r, (q, c) in enumerate(zip(systems, cfgs)):
                xi = O.philox_noise_device(c.seed, c.replica, st, q.nbeads, q.natoms, q.ndim)
                assert trs[r].step(xi) == 0
            b.step(1)
            gx = b.get_states()[0]
            for r, tr in enumerate(trs):
                assert rel_per_bead(gx[r], tr.x) < 1e-9, (st, r)

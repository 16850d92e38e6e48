"""GPU parity at the full sizes of the benchmark systems, on the benchmark's
own initial states (bench.initial_state), against the oracle.

- N = 256, P = 64, Aziz with cutoff L/2 in a periodic box at 0.0218 A^-3,
  normal-mode propagator with the normal-mode Langevin thermostat (the
  headline workload);
- N = 4096, P = 128, Aziz with a 7 A cutoff (cell lists) plus the double
  well, normal-mode propagator with Cartesian Langevin, FP64 and mixed;
- N = 1024, P = 32 in 2D with the dipole interaction and a trap;
- N = 16, P = 32 in a trap;
- the 512-replica ensemble: every replica's forces, and trajectories of a
  stratified sample of replicas.

Tolerances as in the other parity tests: 1e-10 relative per bead for FP64
forces, V_B and the V / V_backwards arrays, 1e-9 per bead for trajectories,
1e-6 norm-relative force error for mixed precision.  The exterior spring
forces alone (the exchange part of beads 1 and P) are compared within 1e-10
of their largest component or within what the measured difference of V and
V_backwards implies through the formula's conditioning, whichever is
larger: at N = 1024 and 4096 a few units of rounding in V move them by 1e-10
to 1e-9 (exterior_force_conditioning).  Besides the initial states
(particles near the reference's grid placement), each large system is also
checked on a hot liquid: the state the GPU reaches after a run from random
placement, where ring polymers have spread, many pairs sit inside the Aziz
damping radius and the exchange is far from the distinguishable limit.
"""
import os

import numpy as np
import pytest

import bench
from oracle import oracle as O
from tests.gpu_cases import case, pk, rel_per_bead, ring

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
TRAJ_TOL = 1e-9
MIXED_TOL = 1e-6
NTH = os.cpu_count() or 1


def oracle_system(w):
    return O.make_system(ndim=w["ndim"], natoms=w["natoms"], nbeads=w["nbeads"], temperature=w["T_K"] * bench.KELVIN,
                         mass=w["mass_amu"] * bench.DALTON, bosonic=True, pbc=w["pbc"], size=w["box_ang"] * bench.ANG,
                         fixcom=True, propagator=w["propagator"], thermostat="langevin",
                         nmthermostat=w["nmthermostat"], dt=w["dt_fs"] * bench.FS, ext=w["ext"], ext_p=w["ext_p"],
                         interaction=w["inter"], int_p=w["int_p"], cutoff=w["cutoff_ang"] * bench.ANG)


def gpu_forces(cfg, x, options=None):
    with pk.System(cfg) as g:
        for k, v in (options or {}).items():
            g.set_option(k, v)
        g.set_state(x, np.zeros_like(x))
        g.compute_forces()
        f = g.get_state()[2]
        ex = g.exchange()
        arr = g.exchange_arrays()
    return f, ex, arr


def exterior_forces(s, x, E, V, Vb):
    """The reference's exterior spring forces on beads 1 and P
    (quadratic_bosonic_exchange.cpp:142-215) from given E, V, V_backwards,
    vectorised."""
    N, P, beta, k = s.natoms, s.nbeads, s.beta_ex, s.spring_constant
    x1, xP = x[0], x[P - 1]
    VN = V[N]

    def mi(d):
        return d - s.size * np.floor(d / s.size + 0.5) if s.pbc else d

    tri = lambda m: m * (m + 1) // 2
    f1, fP = mi(x[1 % P] - x1), mi(x[(P - 2 + P) % P] - xP)
    for l in range(N):
        q = np.arange(l, N)
        pr = np.exp(-beta * (V[l] + E[tri(q) + l] + Vb[q + 1] - VN)) / (q + 1)
        f1[l] += (pr[:, None] * mi(xP[q] - x1[l])).sum(0)
        n = np.arange(0, l + 1)
        pr = np.exp(-beta * (V[n] + E[tri(l) + n] + Vb[l + 1] - VN)) / (l + 1)
        fP[l] += (pr[:, None] * mi(x1[n] - xP[l])).sum(0)
        if l >= 1:  # the direct links l-1 -> l and l -> l+1
            f1[l] += (1.0 - np.exp(-beta * (V[l] + Vb[l] - VN))) * mi(xP[l - 1] - x1[l])
        if l + 1 < N:
            fP[l] += (1.0 - np.exp(-beta * (V[l + 1] + Vb[l + 1] - VN))) * mi(x1[l + 1] - xP[l])
    return k * f1, k * fP


def exterior_force_conditioning(s, x, ref, dv, seed=0):
    """How far the exterior spring forces move, relative to their largest
    component, when the oracle's own V and V_backwards are perturbed at
    random by `dv` (absolute): the agreement two FP64 evaluations of the
    recursion that differ by that much can reach.  The direct-link
    probabilities 1 - exp(-beta (V[l] + V_b[l] - V[N])) difference numbers
    of size V_B, so their rounding is scaled by beta_ex V_B (about 3e4 at
    N = 4096, T = 1 K)."""
    rng = np.random.default_rng(seed)
    f1, fP = exterior_forces(s, x, ref["E"], ref["V"], ref["Vb"])
    g1, gP = exterior_forces(s, x, ref["E"], ref["V"] + dv * rng.standard_normal(ref["V"].shape),
                             ref["Vb"] + dv * rng.standard_normal(ref["Vb"].shape))
    assert np.abs(f1 - ref["f1"]).max() <= 1e-12 * np.abs(ref["f1"]).max()  # the restatement itself
    return max(np.abs(g1 - f1).max() / np.abs(f1).max(), np.abs(gP - fP).max() / np.abs(fP).max())


def check_exchange(ex, arr, ref, s=None, x=None):
    """V_B, primEstimator and E, V, V_backwards within the FP64 tolerances;
    the exterior spring forces within 1e-10 of their largest component, or,
    where the recursion's conditioning allows less (s and x given), within
    twice the spread measured by exterior_force_conditioning."""
    assert abs(ex["VB"] - ref["VB"]) <= FP64_TOL * abs(ref["VB"])
    assert abs(ex["prim"] - ref["prim"]) <= 1e-9 * abs(ref["prim"]) + 1e-300
    np.testing.assert_allclose(arr["E"], ref["E"], rtol=1e-12, atol=1e-14 * np.abs(ref["E"]).max())
    np.testing.assert_allclose(arr["V"], ref["V"], rtol=FP64_TOL, atol=1e-14 * np.abs(ref["V"]).max())
    np.testing.assert_allclose(arr["Vb"][1:], ref["Vb"][1:], rtol=FP64_TOL, atol=1e-14 * np.abs(ref["Vb"]).max())
    tol = FP64_TOL
    if s is not None:
        # the GPU's V and V_backwards against the oracle's (at least 4 units
        # of rounding), carried to the forces through the formula's
        # conditioning, with a factor 3 for the random sampling of it
        n = s.natoms
        dv = max(float(np.max(np.abs(arr["V"][1:] - ref["V"][1:]))), float(np.max(np.abs(arr["Vb"][1:n] -
                                                                                          ref["Vb"][1:n]))),
                 2.0 * np.finfo(float).eps * abs(ref["VB"]))
        tol = max(tol, 3.0 * exterior_force_conditioning(s, x, ref, dv))
    for key in ("f1", "fP"):
        err = np.abs(ex[key] - ref[key]).max() / np.abs(ref[key]).max()
        assert err <= tol, (key, err, tol)


def hot_state(w, steps, placement="separated", min_sep_ang=2.2, seed=777):
    """A state the FP64 GPU path reaches from random placement after `steps`
    steps (the oracle then sees the same coordinates)."""
    wh = dict(w, placement=placement, min_sep_ang=min_sep_ang)
    x, p = bench.initial_state(wh, seed=seed)
    with pk.System(bench.workload_config(w, "fp64")) as g:
        g.set_state(x, p)
        g.step(steps)
        return g.get_state()[0]


def spread(x, w):
    """Mean distance of beads from their particle's centroid, angstrom."""
    c = x.mean(axis=0)
    return float(np.sqrt(((x - c[None]) ** 2).sum(-1)).mean() / bench.ANG)


# ---------------------------------------------------------------------------
# N = 256, P = 64 (the headline workload)

W2 = bench.WORKLOADS["cfg2"]


@pytest.fixture(scope="module")
def cfg2_hot():
    x = hot_state(W2, 400)
    assert spread(x, W2) > 0.3
    return x


@pytest.mark.parametrize("state", ["initial", "hot"])
def test_benchmark_system_forces_and_exchange(state, request):
    s = oracle_system(W2)
    x = bench.initial_state(W2)[0] if state == "initial" else request.getfixturevalue("cfg2_hot")
    want = O.update_forces(s, x, nthreads=NTH)
    ref = O.exchange(s, x)
    f, ex, arr = gpu_forces(bench.workload_config(W2, "fp64"), x)
    assert rel_per_bead(f, want["f"]) < FP64_TOL
    check_exchange(ex, arr, ref)
    fm, _, _ = gpu_forces(bench.workload_config(W2, "mixed"), x)
    assert np.linalg.norm(fm - want["f"]) / np.linalg.norm(want["f"]) <= MIXED_TOL


@pytest.mark.parametrize("options", [{}, {"cuda_graphs": 0}])
def test_benchmark_system_trajectory(options):
    """10 normal-mode steps with the normal-mode Langevin thermostat, step by
    step (each state read completes the deferred tail) and as one 10-step
    call (the fused launches take the stored normal modes)."""
    s = oracle_system(W2)
    cfg = bench.workload_config(W2, "fp64")
    x, p = bench.initial_state(W2)
    tr = O.Trajectory(s, x, p)
    with pk.System(cfg) as g, pk.System(cfg) as h:
        for k, v in options.items():
            g.set_option(k, v)
            h.set_option(k, v)
        g.set_state(x, p)
        g.set_step(0)
        h.set_state(x, p)
        h.set_step(0)
        h.step(10)
        for st in range(10):
            assert tr.step(O.philox_noise_device(cfg.seed, cfg.replica, st, s.nbeads, s.natoms, s.ndim),
                           nthreads=NTH) == 0
            g.step(1)
            gx, gp, gf = g.get_state()
            for got, want, label in ((gx, tr.x, "x"), (gp, tr.p, "p"), (gf, tr.f, "f")):
                assert rel_per_bead(got, want) < TRAJ_TOL, (st, label)
        hx, hp, hf = h.get_state()
        # smooth dynamics: the fast path (reused estimate, banded solve)
        # served every evaluation, none was redone from a fresh estimate
        assert g.exchange_retries() == 0 and h.exchange_retries() == 0
    for got, want, label in ((hx, tr.x, "x"), (hp, tr.p, "p"), (hf, tr.f, "f")):
        assert rel_per_bead(got, want) < TRAJ_TOL, label


# ---------------------------------------------------------------------------
# N = 4096, P = 128, cell lists, Aziz (7 A) + double well

W5 = bench.WORKLOADS["cfg5"]


@pytest.fixture(scope="module")
def cfg5_hot():
    x = hot_state(W5, 40)
    assert spread(x, W5) > 0.1
    return x


@pytest.mark.parametrize("state", ["initial", "hot"])
def test_large_system_forces_and_exchange(state, request):
    s = oracle_system(W5)
    x = bench.initial_state(W5)[0] if state == "initial" else request.getfixturevalue("cfg5_hot")
    want = O.update_forces(s, x, nthreads=NTH)
    ref = O.exchange(s, x)
    f, ex, arr = gpu_forces(bench.workload_config(W5, "fp64"), x)
    assert rel_per_bead(f, want["f"]) < FP64_TOL
    check_exchange(ex, arr, ref, s, x)
    fm, exm, _ = gpu_forces(bench.workload_config(W5, "mixed"), x)
    err = [np.linalg.norm(fm[b] - want["f"][b]) / np.linalg.norm(want["f"][b]) for b in range(s.nbeads)]
    assert max(err) <= MIXED_TOL, max(err)
    # the exchange stays FP64 in mixed precision
    assert abs(exm["VB"] - ref["VB"]) <= FP64_TOL * abs(ref["VB"])


def test_large_system_cell_lists_equal_tiles():
    """The two pair paths of the FP64 kernel agree on the hot liquid."""
    x = hot_state(W5, 40)
    cfg = bench.workload_config(W5, "fp64")
    fc, _, _ = gpu_forces(cfg, x, {"cell_lists": 1})
    ft, _, _ = gpu_forces(cfg, x, {"cell_lists": 0})
    assert rel_per_bead(fc, ft) < 1e-12


def test_large_system_trajectory():
    """5 steps from the benchmark's initial state: the exchange reuses and
    extrapolates its estimate from step to step."""
    s = oracle_system(W5)
    cfg = bench.workload_config(W5, "fp64")
    x, p = bench.initial_state(W5)
    tr = O.Trajectory(s, x, p)
    with pk.System(cfg) as g:
        g.set_state(x, p)
        g.set_step(0)
        for st in range(5):
            assert tr.step(O.philox_noise_device(cfg.seed, cfg.replica, st, s.nbeads, s.natoms, s.ndim),
                           nthreads=NTH) == 0
            g.step(1)
        gx, gp, gf = g.get_state()
        assert g.exchange_retries() == 0
    for got, want, label in ((gx, tr.x, "x"), (gp, tr.p, "p"), (gf, tr.f, "f")):
        assert rel_per_bead(got, want) < TRAJ_TOL, label


# ---------------------------------------------------------------------------
# N = 1024, P = 32, 2D dipole in a trap; N = 16, P = 32 in a trap


@pytest.mark.parametrize("name", ["cfg3", "cfg1"])
def test_other_benchmark_systems(name):
    w = bench.WORKLOADS[name]
    s = oracle_system(w)
    x, p = bench.initial_state(w)
    want = O.update_forces(s, x, nthreads=NTH)
    ref = O.exchange(s, x)
    f, ex, arr = gpu_forces(bench.workload_config(w, "fp64"), x)
    assert rel_per_bead(f, want["f"]) < FP64_TOL
    check_exchange(ex, arr, ref, s, x)
    fm, _, _ = gpu_forces(bench.workload_config(w, "mixed"), x)
    assert np.linalg.norm(fm - want["f"]) / np.linalg.norm(want["f"]) <= MIXED_TOL
    # 5 steps of the trajectory
    cfg = bench.workload_config(w, "fp64")
    tr = O.Trajectory(s, x, p)
    with pk.System(cfg) as g:
        g.set_state(x, p)
        g.set_step(0)
        for st in range(5):
            assert tr.step(O.philox_noise_device(cfg.seed, cfg.replica, st, s.nbeads, s.natoms, s.ndim),
                           nthreads=NTH) == 0
        g.step(5)
        gx, gp, _ = g.get_state()
        assert g.exchange_retries() == 0
    assert rel_per_bead(gx, tr.x) < TRAJ_TOL and rel_per_bead(gp, tr.p) < TRAJ_TOL


# ---------------------------------------------------------------------------
# The 512-replica ensemble


def ensemble_oracle(r, cfg):
    return O.make_system(ndim=3, natoms=cfg.natoms, nbeads=cfg.nbeads, temperature=cfg.temperature, mass=cfg.mass,
                         bosonic=True, pbc=False, size=cfg.size, fixcom=True, propagator="cartesian",
                         thermostat="langevin", dt=cfg.dt, ext="harmonic", ext_p=(3.0 * bench.MEV, 0, 0),
                         interaction="harmonic", int_p=(1.0 * bench.MEV, 0, 0), cutoff=-1.0)


def test_ensemble_forces_every_replica():
    c64, xs, ps = bench.batched_workload("fp64")
    cmx, _, _ = bench.batched_workload("mixed")
    with pk.Batch(c64) as b:
        b.set_states(xs, ps)
        b.compute_forces()
        f64 = b.get_states()[2]
    with pk.Batch(cmx) as b:
        b.set_states(xs, ps)
        b.compute_forces()
        fmx = b.get_states()[2]
    worst64, worstmx = 0.0, 0.0
    for r, cfg in enumerate(c64):
        want = O.update_forces(ensemble_oracle(r, cfg), xs[r])["f"]
        worst64 = max(worst64, rel_per_bead(f64[r], want))
        worstmx = max(worstmx, float(np.linalg.norm(fmx[r] - want) / np.linalg.norm(want)))
    assert worst64 < FP64_TOL, worst64
    assert worstmx <= MIXED_TOL, worstmx


def stratified_sample(cfgs, n=16):
    """n replicas spread over P and N: for each P in {16, 32, 64}, replicas
    at evenly spaced ranks of N."""
    out = []
    for P in (16, 32, 64):
        idx = sorted((c.natoms, r) for r, c in enumerate(cfgs) if c.nbeads == P)
        k = n // 3 + (1 if P == 64 else 0)
        out += [idx[int(round(j * (len(idx) - 1) / (k - 1)))][1] for j in range(k)]
    return sorted(set(out))


def test_ensemble_trajectories_of_a_stratified_sample():
    c64, xs, ps = bench.batched_workload("fp64")
    pick = stratified_sample(c64)
    assert len(pick) >= 16
    cfgs = [c64[r] for r in pick]
    with pk.Batch(cfgs) as b:
        b.set_states([xs[r] for r in pick], [ps[r] for r in pick])
        b.set_step(0)
        b.step(10)
        bx, bp, _ = b.get_states()
    for k, r in enumerate(pick):
        s = ensemble_oracle(r, c64[r])
        tr = O.Trajectory(s, xs[r], ps[r])
        for st in range(10):
            assert tr.step(O.philox_noise_device(c64[r].seed, c64[r].replica, st, s.nbeads, s.natoms, 3)) == 0
        assert rel_per_bead(bx[k], tr.x) < TRAJ_TOL and rel_per_bead(bp[k], tr.p) < TRAJ_TOL, r


@pytest.mark.parametrize("flat", [0, 1])
def test_exchange_energy_forms_at_2950_particles(flat):
    """Both cycle-energy forms at N = 2950: the link prefix sums (flat 1)
    and, with the flat form off, the warp-per-row kernel.  At this size the
    per-row kernel's scans would fit 48 KB of shared memory on their own but
    not beside its static tables, and the one-block solve's dynamic shared
    memory is within its static tables of 48 KB: both launches must count
    the static part.  Results as the full-size checks, with the exterior
    forces against the recursion's measured conditioning."""
    s, cfg = case(natoms=2950, nbeads=2, ext="harmonic", ext_p=(3.0 * 0.036749326e-3, 0, 0), box_ang=60.0)
    x = ring(s, seed=29, spread_ang=3.0)
    ref = O.exchange(s, x)
    with pk.System(cfg) as g:
        g.set_option("flat_energies", flat)
        g.set_state(x, np.zeros_like(x))
        ex = g.exchange()
        arr = g.exchange_arrays()
    check_exchange(ex, arr, ref, s, x)

"""Forward / adjoint consistency: the forces are the negative gradient of
the potential energy U (external + pair + non-exchange springs + V_B), and
the exported primEstimator is the beta-derivative of V_B at fixed cycle
energies, -d(beta_ex V_B)/d(beta_ex) / P (quadratic_bosonic_exchange.cpp:
250-279).  Checked by central finite differences, h = 1e-5 angstrom in the
coordinates and a relative 1e-5 in beta_ex (with the mass scaled so that the
spring constant m P^2 / beta^2, hence E, stays fixed).

CPU: the oracle against itself (pins its energy function).  GPU: the
library's energies against the oracle's (1e-10) and the library's forces
against finite differences of the library's energies, including the
differentiation benchmark system (N=1024 bosons, P=32, 2D dipole, harmonic
trap) through per-particle local energies.

The reference's double-well gradV uses |x|^2 of all axes while its V sums
per axis, so its force is not -dU/dx for ndim > 1; the double well is
checked in 1D only."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_cases import ANG, MEV, case, pk, ring

H = 1e-5 * ANG

SYSTEMS = {
    "bosons_harmonic_pair": dict(natoms=6, nbeads=4, ext="harmonic", ext_p=(3 * MEV, 0, 0), inter="harmonic",
                                 int_p=(1 * MEV, 0, 0)),
    "bosons_aziz_pbc": dict(natoms=12, nbeads=5, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=9.0, inter="aziz",
                            cutoff_ang=4.5),
    "bosons_dipole_2d_cosine": dict(ndim=2, natoms=10, nbeads=3, inter="dipole", int_p=(2.4799673e-4, 0, 0),
                                    ext="cosine", ext_p=(1 * MEV, 0.3, 0)),
    "distinguishable_trap": dict(natoms=7, nbeads=4, bosonic=False, ext="harmonic", ext_p=(3 * MEV, 0, 0)),
    "bosons_double_well_1d": dict(ndim=1, natoms=5, nbeads=6, ext="double_well",
                                  ext_p=(1.32684e-7 * MEV, 3.0 * ANG, 0)),
    "bosons_P2": dict(natoms=5, nbeads=2, ext="harmonic", ext_p=(3 * MEV, 0, 0)),
}


def coords(s, n, seed=0):
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(s.nbeads)), int(rng.integers(s.natoms)), int(rng.integers(s.ndim)))
            for _ in range(n)]


def fd_oracle(s, x, b, i, a):
    xp, xm = x.copy(), x.copy()
    xp[b, i, a] += H
    xm[b, i, a] -= H
    return -(O.potential_energy(s, xp).sum() - O.potential_energy(s, xm).sum()) / (2 * H)


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_oracle_forces_are_minus_energy_gradient(name):
    s, _ = case(**SYSTEMS[name])
    x = ring(s, seed=3, spread_ang=0.2)
    f = O.update_forces(s, x)["f"]
    for b, i, a in coords(s, 12):
        assert abs(fd_oracle(s, x, b, i, a) - f[b, i, a]) <= 1e-8 * np.abs(f[b]).max(), (b, i, a)


def vb_at(kw, x, fac, engine):
    """V_B with beta_ex scaled by fac at fixed E (mass scaled by fac^2)."""
    kw = dict(kw)
    kw["T_K"] = kw.get("T_K", 1.0) / fac
    kw["mass_amu"] = kw.get("mass_amu", 1.0) * fac * fac
    s, cfg = case(**kw)
    if engine == "oracle":
        return O.exchange(s, x)["VB"], s
    with pk.System(cfg) as g:
        g.set_state(x, np.zeros_like(x))
        return g.exchange()["VB"], s


def prim_fd(kw, x, engine, d=1e-5):
    vp, sp = vb_at(kw, x, 1 + d, engine)
    vm, sm = vb_at(kw, x, 1 - d, engine)
    assert sp.spring_constant == pytest.approx(sm.spring_constant, rel=1e-14)
    bp, bm = sp.beta_ex, sm.beta_ex
    return -(bp * vp - bm * vm) / (bp - bm) / sp.nbeads


@pytest.mark.parametrize("name", ["bosons_harmonic_pair", "bosons_aziz_pbc", "bosons_P2"])
def test_oracle_prim_estimator_is_beta_derivative(name):
    kw = SYSTEMS[name]
    s, _ = case(**kw)
    x = ring(s, seed=5, spread_ang=0.3)
    prim = O.exchange(s, x)["prim"]
    assert abs(prim_fd(kw, x, "oracle") - prim) <= 1e-7 * abs(prim)


# ------------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_gpu_energy_matches_oracle(name):
    s, cfg = case(**SYSTEMS[name])
    x = ring(s, seed=3, spread_ang=0.2)
    want = O.potential_energy(s, x)
    with pk.System(cfg) as g:
        g.set_state(x, np.zeros_like(x))
        got = g.potential_energy()
    for k in range(4):
        assert abs(got[k] - want[k]) <= 1e-10 * max(abs(want[k]), 1e-300), (k, got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_gpu_forces_are_minus_energy_gradient(name):
    s, cfg = case(**SYSTEMS[name])
    x = ring(s, seed=3, spread_ang=0.2)
    with pk.System(cfg) as g:
        g.set_state(x, np.zeros_like(x))
        g.compute_forces()
        f = g.get_state()[2]
        for b, i, a in coords(s, 12):
            xp, xm = x.copy(), x.copy()
            xp[b, i, a] += H
            xm[b, i, a] -= H
            g.set_state(xp, None)
            up = g.potential_energy().sum()
            g.set_state(xm, None)
            um = g.potential_energy().sum()
            fd = -(up - um) / (2 * H)
            assert abs(fd - f[b, i, a]) <= 1e-8 * np.abs(f[b]).max(), (b, i, a, fd, f[b, i, a])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["bosons_harmonic_pair", "bosons_aziz_pbc", "bosons_P2"])
def test_gpu_prim_estimator_is_beta_derivative(name):
    kw = SYSTEMS[name]
    s, cfg = case(**kw)
    x = ring(s, seed=5, spread_ang=0.3)
    with pk.System(cfg) as g:
        g.set_state(x, np.zeros_like(x))
        prim = g.exchange()["prim"]
    assert abs(prim_fd(kw, x, "gpu") - prim) <= 1e-7 * abs(prim)


def dipole_benchmark_system(natoms=1024, nbeads=32):
    """The differentiation benchmark: 2D bosons, dipole D = 1 meV A^3 (all
    pairs), harmonic trap 1 meV, T = 2 K; centres uniform in a 60 A square,
    beads jittered by 0.3 A (seed 12345)."""
    s, cfg = case(ndim=2, natoms=natoms, nbeads=nbeads, T_K=2.0, inter="dipole", int_p=(2.4799673e-4, 0, 0),
                  ext="harmonic", ext_p=(1 * MEV, 0, 0), box_ang=60.0)
    rng = np.random.default_rng(12345)
    c = rng.uniform(0.0, 60.0 * ANG, (natoms, 2))
    x = c[None] + rng.normal(0.0, 0.3 * ANG, (nbeads, natoms, 2))
    return s, cfg, x


@pytest.mark.gpu
def test_gpu_differentiation_benchmark_system_local_fd():
    """Forces of the N=1024, P=32 dipole system against central differences
    of the local energy (+ V_B on beads 1 and P) at 400 coordinates, and
    V_B and the forces against the oracle."""
    s, cfg, x = dipole_benchmark_system()
    rng = np.random.default_rng(7)
    picks = [(int(rng.integers(s.nbeads)), int(rng.integers(s.natoms)), int(rng.integers(2))) for _ in range(360)]
    picks += [(b, int(rng.integers(s.natoms)), int(rng.integers(2))) for b in (0, s.nbeads - 1) for _ in range(20)]
    with pk.System(cfg) as g:
        g.set_state(x, np.zeros_like(x))
        g.compute_forces()
        f = g.get_state()[2]
        VB = g.exchange()["VB"]
        worst = 0.0
        for b, i, a in picks:
            d = []
            for sign in (1, -1):
                xs = x.copy()
                xs[b, i, a] += sign * H
                g.set_state(xs, None)
                e = g.local_energy([(b, i)])[0]
                if b in (0, s.nbeads - 1):
                    e += g.potential_energy()[3]
                d.append(e)
            fd = -(d[0] - d[1]) / (2 * H)
            worst = max(worst, abs(fd - f[b, i, a]) / np.abs(f[b]).max())
        assert worst <= 1e-6, worst
    ref = O.exchange(s, x)
    assert abs(VB - ref["VB"]) <= 1e-10 * abs(ref["VB"])
    want = O.update_forces(s, x[:, :, :])["f"]
    for b in (0, 1, s.nbeads - 1):
        assert np.abs(f[b] - want[b]).max() <= 1e-10 * np.abs(want[b]).max()

"""The exchange as a forward function and its adjoint (pimdb_exchange_forward,
pimdb_exchange_adjoint, pimdb_exchange_dbeta), the split of
BosonicExchangeBase into prepare / effectivePotential / exteriorSpringForce
/ primEstimator (include/bosonic_exchange/bosonic_exchange_base.h:16-54).

Checked against the oracle (V_B, primEstimator and the exterior spring
forces of quadratic_bosonic_exchange.cpp:159-215 with their interior
neighbour spring removed), against central differences of the GPU's own
V_B (h = 1e-5 A), for linearity in the incoming cotangent, and against the
fused pimdb_exchange.  FP64 tolerance 1e-10 relative; the central
differences to 1e-6 of the largest gradient component.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_cases import ANG, MEV, case, pk, ring

pytestmark = pytest.mark.gpu

TOL = 1e-10

CASES = {
    "trap_N24_P8": (dict(natoms=24, nbeads=8, T_K=2.0, ext="harmonic", ext_p=(3.0 * MEV, 0, 0)), 0.5),
    "aziz_pbc_N64_P6": (dict(natoms=64, nbeads=6, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=13.0, inter="aziz",
                             cutoff_ang=6.5), 0.3),
    "dipole_2d_N40_P4": (dict(ndim=2, natoms=40, nbeads=4, T_K=2.0, inter="dipole", int_p=(2.4799673e-4, 0, 0),
                              box_ang=20.0), 0.4),
    "trap_N800_P3_grid_solve": (dict(natoms=800, nbeads=3, T_K=3.0, ext="harmonic", ext_p=(3.0 * MEV, 0, 0),
                                     box_ang=30.0), 1.0),
}


def interior(s, x, bead, nb):
    d = x[nb] - x[bead]
    if s.pbc:
        d -= s.size * np.floor(d / s.size + 0.5)
    return s.spring_constant * d


@pytest.mark.parametrize("name", sorted(CASES))
def test_forward_adjoint_dbeta_match_oracle(name):
    kw, spread = CASES[name]
    s, cfg = case(**kw)
    x = ring(s, seed=len(name), spread_ang=spread)
    ref = O.exchange(s, x)
    P = s.nbeads
    with pk.System(cfg) as g:
        g.set_state(x, np.zeros_like(x))
        vb = g.exchange_forward()
        x1b, xPb = g.exchange_adjoint(1.0)
        x1c, xPc = g.exchange_adjoint(-2.5)
        prim = g.exchange_dbeta()
        fused = g.exchange()
    assert abs(vb - ref["VB"]) <= TOL * abs(ref["VB"])
    assert abs(prim - ref["prim"]) <= 1e-9 * abs(ref["prim"]) + 1e-300
    # the exchange part of the exterior spring forces is minus the cotangent
    want1 = ref["f1"] - interior(s, x, 0, 1 % P)
    wantP = ref["fP"] - interior(s, x, P - 1, (P - 2 + P) % P)
    scale = max(np.abs(want1).max(), np.abs(wantP).max())
    assert np.abs(-x1b - want1).max() <= TOL * scale
    assert np.abs(-xPb - wantP).max() <= TOL * scale
    # linear in the cotangent
    assert np.abs(x1c + 2.5 * x1b).max() <= 1e-14 * scale
    assert np.abs(xPc + 2.5 * xPb).max() <= 1e-14 * scale
    # and the fused call is their composition
    assert abs(fused["VB"] - vb) <= 1e-13 * abs(vb) and abs(fused["prim"] - prim) <= 1e-12 * abs(prim)
    assert np.abs(fused["f1"] - (-x1b + interior(s, x, 0, 1 % P))).max() <= TOL * scale


@pytest.mark.parametrize("name", ["trap_N24_P8", "aziz_pbc_N64_P6", "dipole_2d_N40_P4"])
def test_adjoint_matches_central_differences(name):
    kw, spread = CASES[name]
    s, cfg = case(**kw)
    x = ring(s, seed=3 * len(name), spread_ang=spread)
    h = 1e-5 * ANG
    rng = np.random.default_rng(5)
    P = s.nbeads
    with pk.System(cfg) as g:
        g.set_state(x, np.zeros_like(x))
        g.exchange_forward()
        x1b, xPb = g.exchange_adjoint(1.0)
        scale = max(np.abs(x1b).max(), np.abs(xPb).max())
        for bead, grad in ((0, x1b), (P - 1, xPb)):
            for _ in range(8):
                i, a = int(rng.integers(s.natoms)), int(rng.integers(s.ndim))
                vals = []
                for sgn in (1.0, -1.0):
                    xx = x.copy()
                    xx[bead, i, a] += sgn * h
                    g.set_state(xx, np.zeros_like(xx))
                    vals.append(g.exchange_forward())
                fd = (vals[0] - vals[1]) / (2 * h)
                assert abs(fd - grad[i, a]) <= 1e-6 * scale, (bead, i, a, fd, grad[i, a])


def test_adjoint_needs_a_current_forward():
    kw, spread = CASES["trap_N24_P8"]
    s, cfg = case(**kw)
    x = ring(s, seed=1, spread_ang=spread)
    with pk.System(cfg) as g:
        g.set_state(x, np.zeros_like(x))
        with pytest.raises(pk.PimdbError):
            g.exchange_adjoint(1.0)
        g.exchange_forward()
        g.exchange_adjoint(1.0)
        g.set_state(x, np.zeros_like(x))
        with pytest.raises(pk.PimdbError):
            g.exchange_dbeta()
        g.exchange_forward()
        g.step(1)
        with pytest.raises(pk.PimdbError):
            g.exchange_adjoint(1.0)


def test_split_entry_points_reject_the_factorial_exchange():
    s, cfg = case(natoms=4, nbeads=4, ext="harmonic", ext_p=(3.0 * MEV, 0, 0), exchange="factorial")
    x = ring(s, seed=2, spread_ang=0.3)
    with pk.System(cfg) as g:
        g.set_state(x, np.zeros_like(x))
        with pytest.raises(pk.ConfigError):
            g.exchange_forward()

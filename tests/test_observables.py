"""The reference's observables (energy, classical, bosonic, gsf) on the GPU
(pimdb_compute_observables) against the oracle's restatement, which is itself
checked against the compiled reference's simulation.out rows in
test_oracle_vs_reference.py.  FP64: 1e-10 relative per observable."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_cases import ANG, MEV, case, momenta, pk, ring, ring_separated

pytestmark = pytest.mark.gpu

CASES = {
    "bosons_trap_pairharm": (dict(natoms=8, nbeads=6, T_K=3.0, ext="harmonic", ext_p=(3 * MEV, 0, 0),
                                  inter="harmonic", int_p=(1 * MEV, 0, 0)), None),
    "bosons_trap_free": (dict(natoms=16, nbeads=32, ext="harmonic", ext_p=(3 * MEV, 0, 0)), None),
    "dist_double_well": (dict(natoms=7, nbeads=5, bosonic=False, ext="double_well",
                              ext_p=(1.32684e-7 * MEV, 3.0 * ANG, 0)), None),
    "bosons_aziz_pbc": (dict(natoms=64, nbeads=8, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=14.0, inter="aziz",
                             cutoff_ang=7.0), 2.2),
    "bosons_dipole_2d_cosine": (dict(ndim=2, natoms=24, nbeads=5, T_K=2.0, inter="dipole",
                                     int_p=(2.4799673e-4, 0, 0), ext="cosine", ext_p=(1 * MEV, 0.3, 0),
                                     box_ang=40.0), 1.0),
    "dist_P1": (dict(natoms=9, nbeads=1, inter="harmonic", int_p=(1 * MEV, 0, 0), ext="harmonic",
                     ext_p=(3 * MEV, 0, 0)), None),
    "bosons_P2": (dict(natoms=5, nbeads=2, ext="harmonic", ext_p=(3 * MEV, 0, 0)), None),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_observables_match_oracle(name):
    kw, dmin = CASES[name]
    s, cfg = case(**kw)
    x = ring_separated(s, seed=4, dmin_ang=dmin) if dmin else ring(s, seed=4, spread_ang=0.3)
    p = momenta(s, 4)
    want = O.observables(s, x, p)
    with pk.System(cfg) as g:
        g.set_state(x, p)
        got = g.observables()
    for k, v in want.items():
        assert abs(got[k] - v) <= 1e-10 * abs(v) + 1e-300, (k, got[k], v)


def test_observables_after_steps_see_the_completed_step():
    """After pimdb_step the observables are those of the state at the end
    of the step (the deferred tail is completed first)."""
    kw = dict(natoms=16, nbeads=8, propagator="normal_modes", nmthermostat=True, T_K=1.5, mass_amu=4.0026,
              pbc=True, box_ang=11.0, inter="aziz", cutoff_ang=5.5, dt_fs=2.0)
    s, cfg = case(**kw)
    x = ring_separated(s, seed=5, dmin_ang=2.2)
    p = momenta(s, 5)
    with pk.System(cfg) as g:
        g.set_state(x, p)
        g.set_step(0)
        g.step(3)
        got = g.observables()
        gx, gp, _ = g.get_state()
    want = O.observables(s, gx, gp)
    for k, v in want.items():
        assert abs(got[k] - v) <= 1e-10 * abs(v) + 1e-300, (k, got[k], v)

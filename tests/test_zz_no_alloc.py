"""The allocation-free exchange entry point against the oracle and against the
handle-based one.

pimdb_exchange_noalloc exists for callers that must not call cudaMalloc while
they evaluate the exchange: device memory owned by another allocator or held
to a fixed budget, or a loop that cannot take cudaMalloc's implicit device
synchronisation.  It keeps its work arrays in a fixed device array shared by
every call, so each case runs two calls in a row with different rings: the
second must not see anything the first left behind.  The file is collected
last on purpose, so that a run stopping at its first failure has run every
other test already.

Shapes: the 96-particle periodic Aziz ring, the 256-particle limit (the
packed triangle arrays fill the fixed array to its end), P = 2 and P = 3
(beads 1, 2, P-1 and P overlap) in 1D and 2D, and a call with both force
outputs NULL.  Tolerance 1e-10 relative, as every FP64 exchange test.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_cases import case, pk, ring

pytestmark = pytest.mark.gpu

TOL = 1e-10
MEV = 0.036749326e-3

CASES = {
    "aziz_pbc_N96_P8_3d": dict(natoms=96, nbeads=8, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=16.0,
                               inter="aziz", cutoff_ang=8.0),
    "trap_N256_P4_3d": dict(natoms=256, nbeads=4, ext="harmonic", ext_p=(3.0 * MEV, 0, 0), box_ang=20.0),
    "trap_N17_P2_1d": dict(ndim=1, natoms=17, nbeads=2, ext="harmonic", ext_p=(3.0 * MEV, 0, 0)),
    "pbc_N33_P3_2d": dict(ndim=2, natoms=33, nbeads=3, pbc=True, box_ang=12.0),
}


def _noalloc(x_dev, s, scal, f1, fP, torch):
    L = pk.lib()
    fn = L.pimdb_exchange_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double,
                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int]
    fn.restype = C.c_int
    err = C.create_string_buffer(256)
    ptr = lambda t: None if t is None else t.data_ptr()
    st = fn(x_dev.data_ptr(), s.nbeads, s.natoms, s.ndim, s.spring_constant, s.beta_ex, s.pbc, s.size,
            scal.data_ptr(), ptr(f1), ptr(fP), C.c_void_p(torch.cuda.current_stream().cuda_stream), err, len(err))
    return st, err.value.decode()


def _close(got, want, what):
    assert abs(got - want) <= TOL * abs(want) + 1e-300, (what, got, want)


@pytest.mark.parametrize("name", sorted(CASES))
def test_noalloc_exchange_matches_oracle_and_handle_twice(name):
    torch = pytest.importorskip("torch")
    s, cfg = case(**CASES[name])
    for call, seed in enumerate((11, 12)):
        x = ring(s, seed=seed, spread_ang=0.3 + 0.4 * call)
        ref = O.exchange(s, x)
        with pk.System(cfg) as g:
            g.set_state(x, np.zeros_like(x))
            want = g.exchange()
        x_dev = torch.tensor(x, dtype=torch.float64, device="cuda")
        scal = torch.zeros(4, dtype=torch.float64, device="cuda")
        f1 = torch.zeros((s.natoms, s.ndim), dtype=torch.float64, device="cuda")
        fP = torch.zeros_like(f1)
        st, msg = _noalloc(x_dev, s, scal, f1, fP, torch)
        assert st == pk.OK, msg
        got = scal.cpu().numpy()
        for k, key in enumerate(("VB", "prim", "p_distinct", "p_longest")):
            _close(got[k], ref[key], (call, key, "oracle"))
            _close(got[k], want[key], (call, key, "handle"))
        for dev, key in ((f1, "f1"), (fP, "fP")):
            g_f = dev.cpu().numpy()
            assert np.abs(g_f - ref[key]).max() <= TOL * np.abs(ref[key]).max(), (call, key, "oracle")
            assert np.abs(g_f - want[key]).max() <= TOL * np.abs(want[key]).max(), (call, key, "handle")


def test_noalloc_without_force_outputs():
    torch = pytest.importorskip("torch")
    s, _ = case(**CASES["aziz_pbc_N96_P8_3d"])
    x = ring(s, seed=21, spread_ang=0.4)
    ref = O.exchange(s, x)
    x_dev = torch.tensor(x, dtype=torch.float64, device="cuda")
    scal = torch.zeros(4, dtype=torch.float64, device="cuda")
    st, msg = _noalloc(x_dev, s, scal, None, None, torch)
    assert st == pk.OK, msg
    got = scal.cpu().numpy()
    for k, key in enumerate(("VB", "prim", "p_distinct", "p_longest")):
        _close(got[k], ref[key], key)


def test_noalloc_rejects_more_particles_than_its_array_holds():
    torch = pytest.importorskip("torch")
    s, _ = case(natoms=257, nbeads=4)
    x_dev = torch.zeros((4, 257, 3), dtype=torch.float64, device="cuda")
    scal = torch.zeros(4, dtype=torch.float64, device="cuda")
    f = torch.zeros((257, 3), dtype=torch.float64, device="cuda")
    st, msg = _noalloc(x_dev, s, scal, f, f, torch)
    assert st == pk.ERR_ARG and "256" in msg

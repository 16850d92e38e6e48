"""The allocation-free exchange entry point against the handle-based one.

pimdb_exchange_noalloc exists for callers that must not call cudaMalloc while
they evaluate the exchange (an open stream capture, memory owned by another
allocator, no tolerance for cudaMalloc's device synchronisation).  It keeps
its work arrays in a fixed device array shared by every call, so this checks
two calls in a row with different rings: the second must not see anything the
first left behind.  The file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from tests.gpu_cases import case, pk, ring

pytestmark = pytest.mark.gpu


def _noalloc(x_dev, s, scal, f1, fP, torch):
    L = pk.lib()
    fn = L.pimdb_exchange_noalloc
    fn.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double,
                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int]
    fn.restype = C.c_int
    err = C.create_string_buffer(256)
    st = fn(x_dev.data_ptr(), s.nbeads, s.natoms, s.ndim, s.spring_constant, s.beta_ex, s.pbc, s.size,
            scal.data_ptr(), f1.data_ptr(), fP.data_ptr(), C.c_void_p(torch.cuda.current_stream().cuda_stream), err,
            len(err))
    return st, err.value.decode()


def test_noalloc_exchange_matches_handle_exchange_twice():
    torch = pytest.importorskip("torch")
    s, cfg = case(natoms=96, nbeads=8, T_K=1.5, mass_amu=4.0026, pbc=True, box_ang=16.0, inter="aziz",
                  cutoff_ang=8.0)
    for call, seed in enumerate((11, 12)):
        x = ring(s, seed=seed, spread_ang=0.3 + 0.4 * call)
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
            assert abs(got[k] - want[key]) <= 1e-10 * abs(want[key]) + 1e-300, (call, key)
        for dev, key in ((f1, "f1"), (fP, "fP")):
            ref = want[key]
            assert np.abs(dev.cpu().numpy() - ref).max() <= 1e-10 * np.abs(ref).max(), (call, key)


def test_noalloc_rejects_more_particles_than_its_array_holds():
    torch = pytest.importorskip("torch")
    s, _ = case(natoms=257, nbeads=4)
    x_dev = torch.zeros((4, 257, 3), dtype=torch.float64, device="cuda")
    scal = torch.zeros(4, dtype=torch.float64, device="cuda")
    f = torch.zeros((257, 3), dtype=torch.float64, device="cuda")
    st, msg = _noalloc(x_dev, s, scal, f, f, torch)
    assert st == pk.ERR_ARG and "256" in msg

"""Python access to the CPU oracle (``oracle/pimdb_oracle.c``).

TEST INFRASTRUCTURE ONLY: the tests, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use this module
as the checker.  The GPU product never imports it.

Also holds the oracle harness's own reading of the reference's config.ini
schema (src/params.cpp:8-260) and unit table (include/units.h:18-220), kept
independent of the product's C++ parser so that the two can be cross-checked.
"""
from __future__ import annotations

import configparser
import ctypes as C
import math
import os
import re
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "build"
LIB = BUILD / "libpimdb_oracle.so"

EXT = {"free": 0, "harmonic": 1, "double_well": 2, "cosine": 3}
INT = {"free": 0, "harmonic": 1, "aziz": 2, "dipole": 3}


def build(force: bool = False) -> Path:
    """Compile the oracle with gcc (-ffp-contract=off keeps the reference's
    rounding on aarch64 too)."""
    src = HERE / "pimdb_oracle.c"
    hdr = HERE / "pimdb_oracle.h"
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(src.stat().st_mtime, hdr.stat().st_mtime):
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11", "-o", str(tmp), str(src),
                    "-lm", "-lpthread"], check=True)
    os.replace(tmp, LIB)
    return LIB


class System(C.Structure):
    _fields_ = [
        ("ndim", C.c_int), ("natoms", C.c_int), ("nbeads", C.c_int), ("bosonic", C.c_int), ("pbc", C.c_int),
        ("fixcom", C.c_int), ("propagator", C.c_int), ("thermostat", C.c_int), ("nmthermostat", C.c_int),
        ("size", C.c_double), ("mass", C.c_double), ("dt", C.c_double), ("gamma", C.c_double),
        ("beta", C.c_double), ("thermo_beta", C.c_double), ("omega_p", C.c_double),
        ("spring_constant", C.c_double), ("beta_ex", C.c_double),
        ("ext_kind", C.c_int), ("ext_p", C.c_double * 3),
        ("int_kind", C.c_int), ("int_p", C.c_double * 3), ("cutoff", C.c_double), ("nchains", C.c_int),
        ("factorial", C.c_int),
    ]


class State(C.Structure):
    _fields_ = [("x", C.c_void_p), ("p", C.c_void_p), ("f", C.c_void_p), ("ext_f", C.c_void_p),
                ("spring_f", C.c_void_p), ("nh", C.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        dp = C.POINTER(C.c_double)
        S = C.POINTER(System)
        L.orc_system_init.argtypes = [S, C.c_double, C.c_double]
        L.orc_exchange.argtypes = [S, dp, dp, dp, dp, dp, dp, dp, dp]
        L.orc_exchange.restype = C.c_int
        L.orc_nh_chains.argtypes = [S]
        L.orc_nh_chains.restype = C.c_long
        L.orc_nh_energy.argtypes = [S, dp]
        L.orc_nh_energy.restype = C.c_double
        L.orc_observables.argtypes = [S, dp, dp, dp]
        L.orc_observables.restype = C.c_int
        L.orc_potential_energy.argtypes = [S, dp, dp]
        L.orc_potential_energy.restype = C.c_int
        L.orc_update_forces.argtypes = [S, dp, dp, dp, dp, C.c_int]
        L.orc_update_forces.restype = C.c_int
        L.orc_md_step.argtypes = [S, C.POINTER(State), dp, C.c_int]
        L.orc_md_step.restype = C.c_int
        L.orc_sample_run.argtypes = [S, C.POINTER(State), C.c_int, C.c_long, C.c_long, dp]
        L.orc_sample_run.restype = C.c_int
        L.orc_philox_normals.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_int, C.c_int64, dp]
        L.orc_ranmars_new.argtypes = [C.c_int]
        L.orc_ranmars_new.restype = C.c_void_p
        L.orc_ranmars_free.argtypes = [C.c_void_p]
        L.orc_ranmars_gaussians.argtypes = [C.c_void_p, C.c_int64, dp]
        L.orc_nm_matrices.argtypes = [S, dp, dp]
        L.orc_ext_value.argtypes = [S, dp, C.c_int]
        L.orc_ext_value.restype = C.c_double
        L.orc_pair_grad.argtypes = [S, dp, dp]
        L.orc_pair_value.argtypes = [S, dp]
        L.orc_pair_value.restype = C.c_double
        L.orc_min_image.argtypes = [C.c_double, C.c_double]
        L.orc_min_image.restype = C.c_double
        _lib = L
    return _lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


THERMOSTATS = {"none": 0, "langevin": 1, "nose_hoover": 2, "nose_hoover_np": 3, "nose_hoover_np_dim": 4}


def make_system(*, ndim, natoms, nbeads, temperature, mass, bosonic=False, pbc=False, size=1.0, fixcom=True,
                propagator="cartesian", thermostat="langevin", nmthermostat=False, dt=1.0, gamma=-1.0,
                ext="free", ext_p=(0.0, 0.0, 0.0), interaction="free", int_p=(0.0, 0.0, 0.0), cutoff=-1.0,
                nchains=4, factorial=False):
    """Builds the oracle's system record; all quantities in atomic units.
    factorial=True selects the permutation-sum exchange of
    factorial_bosonic_exchange.cpp (the reference's compile-time
    FACTORIAL_BOSONIC_ALGORITHM)."""
    s = System()
    s.ndim, s.natoms, s.nbeads = ndim, natoms, nbeads
    s.bosonic, s.pbc, s.fixcom = int(bosonic), int(pbc), int(fixcom)
    s.propagator = 1 if propagator == "normal_modes" else 0
    s.thermostat = THERMOSTATS[thermostat]
    s.nchains = nchains
    s.factorial = int(factorial)
    s.nmthermostat = int(nmthermostat)
    s.size, s.mass, s.dt = size, mass, dt
    s.gamma = gamma if gamma >= 0 else 1 / (100.0 * dt)  # params.cpp:17-20
    s.ext_kind = EXT[ext]
    s.int_kind = INT[interaction]
    for i in range(3):
        s.ext_p[i] = ext_p[i]
        s.int_p[i] = int_p[i]
    lib().orc_system_init(C.byref(s), temperature, cutoff)
    return s


def exchange(s: System, x: np.ndarray):
    """Whole FH exchange on the ring polymer x[P][N][D]."""
    N, D, P = s.natoms, s.ndim, s.nbeads
    x = np.ascontiguousarray(x, dtype=np.float64)
    assert x.shape == (P, N, D)
    f1 = np.zeros((N, D))
    fP = np.zeros((N, D))
    sc = np.zeros(4)
    E = np.zeros(N * (N + 1) // 2)
    V = np.zeros(N + 1)
    Vb = np.zeros(N + 1)
    prob = np.zeros((N, N))
    st = lib().orc_exchange(C.byref(s), _dp(x), _dp(f1), _dp(fP), _dp(sc), _dp(E), _dp(V), _dp(Vb), _dp(prob))
    return dict(status=st, f1=f1, fP=fP, VB=sc[0], prim=sc[1], p_distinct=sc[2], p_longest=sc[3], E=E, V=V, Vb=Vb,
                prob=prob)


OBSERVABLES = ["kinetic", "potential", "ext_pot", "int_pot", "virial", "temperature", "cl_kinetic", "cl_spring",
               "prob_dist", "prob_all", "w_gsf", "pot_gsf"]


def observables(s: System, x: np.ndarray, p: np.ndarray) -> dict:
    """The reference's observables of one state, summed over beads (atomic
    units; temperature in kelvin): orc_observables."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    out = np.zeros(12)
    lib().orc_observables(C.byref(s), _dp(x), _dp(p), _dp(out))
    return dict(zip(OBSERVABLES, out))


def potential_energy(s: System, x: np.ndarray) -> np.ndarray:
    """[external, pair, non-exchange springs, V_B] (orc_potential_energy)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    t = np.zeros(4)
    lib().orc_potential_energy(C.byref(s), _dp(x), _dp(t))
    return t


def update_forces(s: System, x: np.ndarray, nthreads: int = 1):
    P, N, D = s.nbeads, s.natoms, s.ndim
    x = np.ascontiguousarray(x, dtype=np.float64)
    f = np.zeros((P, N, D))
    sp = np.zeros((P, N, D))
    ph = np.zeros((P, N, D))
    st = lib().orc_update_forces(C.byref(s), _dp(x), _dp(f), _dp(sp), _dp(ph), nthreads)
    return dict(status=st, f=f, spring=sp, phys=ph)


class Trajectory:
    """Whole-ring-polymer state stepped by orc_md_step (simulation.cpp:236-260).
    Forces start at zero, as in the reference (the constructor never computes
    them, simulation.cpp:16-101)."""

    def __init__(self, s: System, x: np.ndarray, p: np.ndarray):
        self.s = s
        shp = (s.nbeads, s.natoms, s.ndim)
        self.x = np.ascontiguousarray(x, dtype=np.float64).reshape(shp).copy()
        self.p = np.ascontiguousarray(p, dtype=np.float64).reshape(shp).copy()
        self.f = np.zeros(shp)
        self.ext_f = np.zeros(shp)
        self.spring_f = np.zeros(shp)
        self.nh = np.zeros(max(1, 3 * lib().orc_nh_chains(C.byref(s)) * s.nchains))
        self._st = State(self.x.ctypes.data, self.p.ctypes.data, self.f.ctypes.data, self.ext_f.ctypes.data,
                         self.spring_f.ctypes.data, self.nh.ctypes.data)

    def nh_energy(self) -> float:
        """Sum over beads of the Nose-Hoover chains' getAdditionToH."""
        return lib().orc_nh_energy(C.byref(self.s), _dp(self.nh))

    def sample_run(self, seed: int, nsteps: int, every: int) -> np.ndarray:
        """nsteps MD steps with RanMars noise (streams seed+bead); the
        observables after every `every`-th step, rows of OBSERVABLES."""
        rows = nsteps // every if every > 0 else 0
        out = np.zeros((max(rows, 1), len(OBSERVABLES)))
        st = lib().orc_sample_run(C.byref(self.s), C.byref(self._st), seed, nsteps, every, _dp(out))
        if st != 0:
            raise RuntimeError(f"orc_sample_run status {st}")
        return out[:rows]

    def step(self, xi: np.ndarray, nthreads: int = 1) -> int:
        xi = np.ascontiguousarray(xi, dtype=np.float64)
        assert xi.size == 2 * self.x.size
        return lib().orc_md_step(C.byref(self.s), C.byref(self._st), _dp(xi), nthreads)


def philox_normals(seed: int, replica: int, step: int, substep: int, ndof: int) -> np.ndarray:
    out = np.zeros(ndof)
    lib().orc_philox_normals(seed, replica, step, substep, ndof, _dp(out))
    return out


class RanMars:
    """RANMAR stream with the polar Gaussian (one per bead, seed + bead)."""

    def __init__(self, seed: int):
        self._h = lib().orc_ranmars_new(seed)
        if not self._h:
            raise ValueError("Invalid seed for Marsaglia random # generator")

    def gaussians(self, n: int) -> np.ndarray:
        out = np.zeros(n)
        lib().orc_ranmars_gaussians(self._h, n, _dp(out))
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_ranmars_free(self._h)
            self._h = None


def ranmars_noise(streams, natoms: int, ndim: int) -> np.ndarray:
    """Noise for both O-steps of one MD step, drawn per bead in the reference's
    order (langevin.cpp:18-25): xi[2][P][N][D]."""
    P = len(streams)
    xi = np.zeros((2, P, natoms, ndim))
    for o in range(2):
        for b, r in enumerate(streams):
            xi[o, b] = r.gaussians(natoms * ndim).reshape(natoms, ndim)
    return xi


def philox_noise(seed: int, replica: int, step: int, nbeads: int, natoms: int, ndim: int) -> np.ndarray:
    """The project's Langevin noise for both O-steps of MD step `step`,
    indexed [substep][bead][particle][axis] (dof = (bead*N + i)*D + axis)."""
    n = nbeads * natoms * ndim
    return np.stack([philox_normals(seed, replica, step, o, n).reshape(nbeads, natoms, ndim) for o in range(2)])


# --------------------------------------------------------------------------
# The oracle harness's own reading of config.ini (params.cpp) and units.h.

_PREFIX = {"yotta": 1e24, "zetta": 1e21, "exa": 1e18, "peta": 1e15, "tera": 1e12, "giga": 1e9, "mega": 1e6,
           "kilo": 1e3, "hecto": 1e2, "deci": 1e-1, "centi": 1e-2, "milli": 1e-3, "micro": 1e-6, "nano": 1e-9,
           "pico": 1e-12, "femto": 1e-15, "atto": 1e-18, "zepto": 1e-21, "yocto": 1e-24}
_UNITS = {
    "energy": {"electronvolt": 0.036749326, "j/mol": 0.00000038087989, "cal/mol": 0.0000015946679,
               "kelvin": 3.1668152e-06},
    "temperature": {"kelvin": 3.1668152e-06},
    "time": {"second": 4.1341373e16},
    "length": {"angstrom": 1.8897261, "meter": 1.8897261e10, "radian": 1.00, "degree": 0.017453292519943295},
    "velocity": {"angstrom/ps": 4.5710289e-5, "m/s": 4.5710289e-7},
    "mass": {"dalton": 1822.8885, "amu": 1822.8885, "electronmass": 1.00},
    "force": {"newton": 12137805, "ev/ang": 0.019446904},
}


def to_internal(family: str, unit: str, value: float) -> float:
    """units.cpp:16-60: optional metric prefixes, then the base unit."""
    prefix = ""
    rest = unit
    while True:
        for p in _PREFIX:
            if rest.startswith(p):
                prefix, rest = p, rest[len(p):]
                break
        else:
            break
    table = dict(_UNITS.get(family, {}))
    table.update({"": 1.0, "automatic": 1.0, "atomic_unit": 1.0})
    if rest not in table:
        raise ValueError(f"{rest} is an undefined unit for kind {family}.")
    return value * table[rest] * (_PREFIX[prefix] if prefix else 1.0)


def _quantity(family, text):
    m = re.match(r"\s*([-+0-9.eE]+)\s*(\S+)\s*$", text)
    if not m:
        raise ValueError("Invalid input format")
    return to_internal(family, m.group(2), float(m.group(1)))


def system_from_ini(path, **overrides):
    """Oracle system record from a reference config.ini (subset used by the
    hot path).  Returns (System, extras)."""
    cp = configparser.ConfigParser(inline_comment_prefixes=(";", "#"))
    cp.read(path)

    def get(sec, key, default):
        if not cp.has_section(sec) or not cp.has_option(sec, key):
            return default
        return cp.get(sec, key).strip()

    def getb(sec, key, default):
        v = get(sec, key, None)
        return default if v is None else v.lower() in ("true", "yes", "on", "1")

    dt = _quantity("time", get("simulation", "dt", "1.0 femtosecond"))
    gamma = float(get("simulation", "gamma", "-1.0"))
    nbeads = int(float(get("simulation", "nbeads", "4")))
    T = _quantity("temperature", get("system", "temperature", "1.0 kelvin"))
    natoms = int(float(get("system", "natoms", "1")))
    mass = _quantity("mass", get("system", "mass", "1.0 dalton"))
    size = _quantity("length", get("system", "size", "1.0 picometer"))
    iname = get("interaction_potential", "name", "free")
    ename = get("external_potential", "name", "free")
    cutoff = _quantity("length", get("interaction_potential", "cutoff", "-1.0 angstrom"))
    int_p = [0.0, 0.0, 0.0]
    ext_p = [0.0, 0.0, 0.0]
    if iname == "harmonic":
        int_p[0] = _quantity("energy", get("interaction_potential", "omega", "1.0 millielectronvolt"))
    elif iname == "dipole":
        int_p[0] = float(get("interaction_potential", "strength", "1.0"))
    if ename == "harmonic":
        ext_p[0] = _quantity("energy", get("external_potential", "omega", "1.0 millielectronvolt"))
    elif ename == "double_well":
        ext_p[0] = _quantity("energy", get("external_potential", "strength", "1.0 millielectronvolt"))
        ext_p[1] = _quantity("length", get("external_potential", "location", "1.0 angstrom"))
    elif ename == "cosine":
        ext_p[0] = _quantity("energy", get("external_potential", "amplitude", "1.0 millielectronvolt"))
        ext_p[1] = float(get("external_potential", "phase", "1.0"))
    kw = dict(ndim=3, natoms=natoms, nbeads=nbeads, temperature=T, mass=mass,
              bosonic=getb("simulation", "bosonic", False), pbc=getb("simulation", "pbc", False), size=size,
              fixcom=getb("simulation", "fixcom", True), propagator=get("simulation", "propagator", "cartesian"),
              thermostat=get("simulation", "thermostat", "none"),
              nmthermostat=getb("simulation", "nmthermostat", False), dt=dt, gamma=gamma, ext=ename, ext_p=ext_p,
              nchains=int(float(get("simulation", "nchains", "4"))),
              interaction=iname, int_p=int_p, cutoff=cutoff)
    kw.update(overrides)
    extras = dict(steps=int(float(get("simulation", "steps", "1e5"))), sfreq=int(get("simulation", "sfreq", "1000")),
                  seed=int(float(get("simulation", "seed", "1234"))), temperature=T)
    return make_system(**kw), extras


def philox_noise_device(seed: int, replica: int, step: int, nbeads: int, natoms: int, ndim: int) -> np.ndarray:
    """The project's Langevin noise for both O-steps of MD step `step`, as the
    GPU kernels draw it: the normal number of (bead-or-mode b, axis a,
    particle i) is element i%2 of the Box-Muller pair number
    (b*ndim + a)*ceil(natoms/2) + i//2.  Returned as [substep][b][i][a]."""
    half = (natoms + 1) // 2
    n = nbeads * ndim * half * 2
    out = np.empty((2, nbeads, natoms, ndim))
    for o in range(2):
        z = philox_normals(seed, replica, step, o, n).reshape(nbeads, ndim, 2 * half)[:, :, :natoms]
        out[o] = z.transpose(0, 2, 1)
    return out

"""Shared set-up for the GPU parity tests: one parameter dict builds both the
oracle's system record and the library's pimdb_config, and seeded
ring-polymer configurations with the shapes of the benchmark systems."""
import importlib

import numpy as np

from oracle import oracle as O

pk = importlib.import_module("pimd-b_gb300")

ANG = 1.8897261           # include/units.h:95
KELVIN = 3.1668152e-06    # include/units.h:64
MEV = 0.036749326e-3      # include/units.h:61 with the milli prefix
DALTON = 1822.8885        # include/units.h:122
FS = 4.1341373e16 * 1e-15  # include/units.h:76 with the femto prefix


def case(ndim=3, natoms=8, nbeads=4, T_K=1.0, mass_amu=1.0, bosonic=True, pbc=False, box_ang=10.0,
         ext="free", ext_p=(0.0, 0.0, 0.0), inter="free", int_p=(0.0, 0.0, 0.0), cutoff_ang=-1.0,
         propagator="cartesian", thermostat="langevin", nmthermostat=False, fixcom=True, dt_fs=1.0, gamma=-1.0,
         precision="fp64", seed=12345, exchange="feldman_hirshberg"):
    p = dict(ndim=ndim, natoms=natoms, nbeads=nbeads, temperature=T_K * KELVIN, mass=mass_amu * DALTON,
             bosonic=bosonic, pbc=pbc, size=box_ang * ANG, ext=ext, ext_p=tuple(ext_p), interaction=inter,
             int_p=tuple(int_p), cutoff=cutoff_ang * ANG, propagator=propagator, thermostat=thermostat,
             nmthermostat=nmthermostat, fixcom=fixcom, dt=dt_fs * FS, gamma=gamma)
    s = O.make_system(**p, factorial=exchange == "factorial")
    cfg = pk.make_config(ndim=ndim, natoms=natoms, nbeads=nbeads, bosonic=int(bosonic), pbc=int(pbc),
                         fixcom=int(fixcom), propagator=propagator, thermostat=thermostat,
                         nmthermostat=int(nmthermostat), precision=precision, temperature=p["temperature"],
                         mass=p["mass"], size=p["size"], dt=p["dt"], gamma=gamma, ext_kind=ext, ext_params=ext_p,
                         int_kind=inter, int_params=int_p, cutoff=p["cutoff"], seed=seed, replica=0,
                         exchange=exchange)
    return s, cfg


def ring(s, seed, spread_ang=0.3, box_ang=None):
    """Particles at uniform centres in the box, each bead displaced by a
    Gaussian jitter (the configuration family of the benchmark systems)."""
    rng = np.random.default_rng(seed)
    L = (box_ang * ANG) if box_ang else s.size
    centres = rng.uniform(-0.5 * L, 0.5 * L, (s.natoms, s.ndim))
    return centres[None] + rng.normal(0.0, spread_ang * ANG, (s.nbeads, s.natoms, s.ndim))


def ring_separated(s, seed, dmin_ang=2.2, spread_ang=0.05):
    """Centres placed by random sequential addition at least dmin apart
    (minimum image under PBC), each bead displaced by a Gaussian jitter: a
    liquid-like configuration without overlapping cores."""
    rng = np.random.default_rng(seed)
    L, dmin = s.size, dmin_ang * ANG
    pts = []
    while len(pts) < s.natoms:
        c = rng.uniform(-0.5 * L, 0.5 * L, s.ndim)
        if pts:
            d = np.asarray(pts) - c
            if s.pbc:
                d -= L * np.floor(d / L + 0.5)
            if np.min(np.einsum("ij,ij->i", d, d)) < dmin * dmin:
                continue
        pts.append(c)
    return np.asarray(pts)[None] + rng.normal(0.0, spread_ang * ANG, (s.nbeads, s.natoms, s.ndim))


def momenta(s, seed):
    rng = np.random.default_rng(seed + 1)
    return rng.normal(0.0, np.sqrt(s.mass / s.thermo_beta), (s.nbeads, s.natoms, s.ndim))


def rel_per_bead(got, want):
    """max over beads of max|got-want| / max|want| within that bead."""
    worst = 0.0
    for b in range(want.shape[0]):
        scale = np.abs(want[b]).max()
        if scale == 0:
            worst = max(worst, float(np.abs(got[b]).max()))
            continue
        worst = max(worst, float(np.abs(got[b] - want[b]).max() / scale))
    return worst

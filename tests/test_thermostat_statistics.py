"""Thermostatted estimator means against an exact answer, within statistical
error.

Trajectory parity with a shared noise stream cannot see a wrong Langevin
amplitude c2 = sqrt((1 - c1^2) m / beta_P), a biased Gaussian generator or its
truncated tail: both sides would share the mistake.  The mean of an estimator
over a long thermostatted run can.  The reference's primitive kinetic and
potential estimators (src/observables/energy.cpp:30-110, with the bosonic
term of primEstimator, src/bosonic_exchange/quadratic_bosonic_exchange.cpp:
250-279) average to the thermodynamic energy of the discretised (P-bead)
system, E = -d ln Z_P / d beta, for any P.

For N bosons in an isotropic d-dimensional harmonic trap that energy is
exact.  A k-particle exchange cycle is one ring polymer of kP beads at the
same imaginary-time step tau = beta/P; its partition function per dimension,
after the Gaussian integral over the beads, is
    z_k = prod_{j=0}^{kP-1} (4 sin^2(pi j / kP) + u^2)^(-1/2),   u = beta hbar omega / P,
and the bosonic one follows from the permutation-cycle recursion
    Z_N = (1/N) sum_{k=1}^{N} z_k^d Z_{N-k},   Z_0 = 1,
the same recursion the Feldman-Hirshberg V_B evaluates configuration by
configuration.  Then E = -(hbar omega / P) d ln Z_N / du, and the
potential estimator averages to E/2 (d ln Z/d omega at fixed beta).

The runs: N = 3, P = 8 or 16, beta hbar omega = 2, where exchange lowers E
by 11-12% (P = 16: 5.255 against 5.899 hbar omega for distinguishable
particles).  fixcom is
off: removing the centre-of-mass momentum in a trap would freeze the centroid
and bias the means.  Each mean is a 20-block average; a run must agree with
the exact E within 4 standard errors, and that band must be narrow enough to
tell bosons from distinguishable particles.  The velocity-Verlet runs carry
an O(dt^2) bias of about 0.03 hbar omega at dt = 1 fs (measured with the
oracle: 0.5 fs removes it), well inside the band.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_cases import KELVIN, MEV, case, pk

HW = 3.0 * MEV            # trap hbar omega, hartree
BHW = 2.0                 # beta hbar omega
T_K = HW / (BHW * KELVIN)
NSIG = 4.0


def exact_energy(natoms, nbeads, bhw, ndim=3, bosons=True):
    """E / (hbar omega) of N particles in a d-dimensional harmonic trap,
    discretised with P beads (see the module docstring)."""
    u = bhw / nbeads
    lz, dlz = [0.0], [0.0]
    for k in range(1, natoms + 1):
        n = k * nbeads
        s2 = 4.0 * np.sin(np.pi * np.arange(n) / n) ** 2
        lz.append(-0.5 * ndim * float(np.sum(np.log(s2 + u * u))))
        dlz.append(-ndim * float(np.sum(u / (s2 + u * u))))
    if not bosons:
        return -natoms * dlz[1] / nbeads
    Z, dZ = [1.0], [0.0]
    for m in range(1, natoms + 1):
        Z.append(sum(np.exp(lz[k]) * Z[m - k] for k in range(1, m + 1)) / m)
        dZ.append(sum(np.exp(lz[k]) * (dlz[k] * Z[m - k] + dZ[m - k]) for k in range(1, m + 1)) / m)
    return -(dZ[natoms] / Z[natoms]) / nbeads


def block_mean(v, nblocks=20):
    v = np.asarray(v, dtype=np.float64)
    b = v[: len(v) // nblocks * nblocks].reshape(nblocks, -1).mean(axis=1)
    return float(b.mean()), float(b.std(ddof=1) / np.sqrt(nblocks))


def trap_case(nbeads=16, **kw):
    return case(natoms=3, nbeads=nbeads, T_K=T_K, mass_amu=1.0, ext="harmonic", ext_p=(HW, 0, 0), fixcom=False,
                **kw)


def start(s, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(0.0, 0.3 * 1.8897261, (s.nbeads, s.natoms, s.ndim))
    p = rng.normal(0.0, np.sqrt(s.mass / s.thermo_beta), (s.nbeads, s.natoms, s.ndim))
    return x, p


def check_means(kin, pot, nbeads, label):
    """kin, pot: samples in hartree.  Returns the energy mean and its error."""
    e_exact = exact_energy(3, nbeads, BHW)
    e_dist = exact_energy(3, nbeads, BHW, bosons=False)
    E, sE = block_mean((np.asarray(kin) + np.asarray(pot)) / HW)
    K, sK = block_mean(np.asarray(kin) / HW)
    V, sV = block_mean(np.asarray(pot) / HW)
    msg = f"{label}: E {E:.4f}+-{sE:.4f} (exact {e_exact:.4f}), K {K:.4f}+-{sK:.4f}, V {V:.4f}+-{sV:.4f}"
    # the band resolves exchange: bosons and distinguishable particles differ
    assert NSIG * sE < 0.5 * (e_dist - e_exact), msg
    assert abs(E - e_exact) < NSIG * sE, msg
    assert abs(K - 0.5 * e_exact) < NSIG * sK, msg
    assert abs(V - 0.5 * e_exact) < NSIG * sV, msg
    return E, sE


def test_exact_energy_limits():
    # one bead: the classical oscillator, d/beta per particle
    assert exact_energy(3, 1, 2.0, bosons=False) == pytest.approx(3 * 3 / 2.0, rel=1e-12)
    # many beads: the quantum oscillator, (d/2) coth(beta hbar omega / 2) per particle
    assert exact_energy(1, 4096, 2.0) == pytest.approx(1.5 / np.tanh(1.0), rel=1e-6)
    # one particle: bosons and distinguishable agree
    assert exact_energy(1, 16, 2.0) == pytest.approx(exact_energy(1, 16, 2.0, bosons=False), rel=1e-14)
    # low temperature: three bosons in the ground state, 3 * d/2
    assert exact_energy(3, 4096, 40.0) == pytest.approx(4.5, rel=1e-4)


def test_oracle_langevin_means_match_exact_energy():
    """The oracle, RanMars noise as the reference draws it, P = 4."""
    s, _ = trap_case(nbeads=4)
    x, p = start(s, 3)
    tr = O.Trajectory(s, x, p)
    tr.sample_run(101, 20000, 0)
    obs = tr.sample_run(202, 800000, 20)
    check_means(obs[:, 0], obs[:, 1], 4, "oracle VV Langevin P=4")


def _gpu_run(kw, nbeads, nsteps, every, seed=7):
    s, cfg = trap_case(nbeads=nbeads, **kw)
    x, p = start(s, seed)
    kin, pot = [], []
    with pk.System(cfg) as g:
        g.set_state(x, p)
        g.step(20000)
        for _ in range(nsteps // every):
            g.step(every)
            o = g.observables()
            kin.append(o["kinetic"])
            pot.append(o["potential"])
    return s, np.asarray(kin), np.asarray(pot)


@pytest.mark.gpu
@pytest.mark.parametrize("kw", [dict(), dict(propagator="normal_modes", nmthermostat=True)],
                         ids=["vv_langevin", "nm_nm_langevin"])
def test_gpu_thermostatted_means_match_exact_energy_and_oracle(kw):
    # P = 8 halves the variance of the primitive kinetic estimator against
    # P = 16; 800000 steps then give a standard error near 0.04 hbar omega
    s, kin, pot = _gpu_run(kw, nbeads=8, nsteps=800000, every=40)
    E, sE = check_means(kin, pot, 8, f"GPU {kw}")
    # and an independent oracle run of the same system (RanMars streams)
    x, p = start(s, 8)
    tr = O.Trajectory(s, x, p)
    tr.sample_run(303, 20000, 0)
    obs = tr.sample_run(404, 800000, 40)
    Eo, sEo = block_mean((obs[:, 0] + obs[:, 1]) / HW)
    assert abs(E - Eo) < NSIG * np.hypot(sE, sEo), (E, sE, Eo, sEo)


@pytest.mark.gpu
def test_gpu_batched_replicas_means_match_exact_energy():
    """64 replicas of the same trap in the batched engine (Philox noise per
    replica): their pooled estimator means."""
    nrep, nsteps, every = 64, 100000, 100
    s, _ = trap_case()
    cfgs, xs, ps = [], [], []
    for r in range(nrep):
        _, c = trap_case()
        c.seed, c.replica = 500 + r, r
        cfgs.append(c)
        x, p = start(s, 1000 + r)
        xs.append(x)
        ps.append(p)
    kin, pot = [], []
    with pk.Batch(cfgs) as b:
        b.set_states(xs, ps)
        b.step(20000)
        for _ in range(nsteps // every):
            b.step(every)
            bx, bp, _ = b.get_states()
            k_row, v_row = [], []
            for r in range(nrep):
                o = O.observables(s, bx[r], bp[r])
                k_row.append(o["kinetic"])
                v_row.append(o["potential"])
            kin.append(np.mean(k_row))
            pot.append(np.mean(v_row))
    check_means(kin, pot, 16, "GPU batch x64")

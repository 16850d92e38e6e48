"""Python access to ``libpimdb_gb300.so`` — the GB300-native PIMD-B++ hot
path behind its C ABI (``include/pimdb_gb300.h``).

The package directory name contains a hyphen, so import it with
``importlib.import_module("pimd-b_gb300")``.  There is no CPU fallback: every
entry point runs the CUDA kernels, and loading fails loudly when the shared
library has not been built (``build.build()``).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libpimdb_gb300.so"

# status codes (pimdb_status)
OK, ERR_CONFIG, ERR_NONFINITE_VB, ERR_CUDA, ERR_TIMEOUT, ERR_BOUNDS, ERR_ARG, ERR_NO_DEVICE, ERR_PARSE = range(9)
POT = {"free": 0, "harmonic": 1, "double_well": 2, "cosine": 3, "aziz": 4, "dipole": 5}
PROP = {"cartesian": 0, "normal_modes": 1}
THERMO = {"none": 0, "langevin": 1, "nose_hoover": 2, "nose_hoover_np": 3, "nose_hoover_np_dim": 4}
PRECISION = {"fp64": 0, "mixed": 1}
EXCHANGE = {"feldman_hirshberg": 0, "factorial": 1}
RNG = {"philox": 0, "ranmars": 1}

EXPORTS = [
    "pimdb_config_default", "pimdb_config_from_ini", "pimdb_create", "pimdb_destroy", "pimdb_set_state",
    "pimdb_set_state_device", "pimdb_get_state", "pimdb_get_state_device", "pimdb_set_step", "pimdb_get_step",
    "pimdb_step_io",
    "pimdb_compute_forces", "pimdb_step", "pimdb_step_async", "pimdb_synchronize", "pimdb_exchange",
    "pimdb_exchange_arrays", "pimdb_exchange_forward", "pimdb_exchange_adjoint", "pimdb_exchange_dbeta",
    "pimdb_exchange_retries",
    "pimdb_exchange_fresh_estimates",
    "pimdb_last_error", "pimdb_status_string", "pimdb_profile",
    "pimdb_measure_fp64_peak", "pimdb_measure_fp32_peak", "pimdb_math_check", "pimdb_set_option", "pimdb_thermostat_step", "pimdb_zero_momentum",
    "pimdb_propagate", "pimdb_compute_observables", "pimdb_potential_energy", "pimdb_local_energy", "pimdb_batch_create", "pimdb_batch_destroy", "pimdb_batch_size", "pimdb_batch_set_states",
    "pimdb_batch_get_states", "pimdb_batch_set_step", "pimdb_batch_get_step", "pimdb_batch_compute_forces",
    "pimdb_batch_step", "pimdb_batch_step_async", "pimdb_batch_synchronize", "pimdb_batch_exchange",
    "pimdb_batch_set_option", "pimdb_batch_get_launch", "pimdb_batch_autotune", "pimdb_batch_last_error",
]
OBSERVABLES = ["kinetic", "potential", "ext_pot", "int_pot", "virial", "temperature", "cl_kinetic", "cl_spring",
               "prob_dist", "prob_all", "w_gsf", "pot_gsf", "nh_energy"]
KERNEL_CLASSES = ["bead_forces", "exch_energies", "exch_recursions", "exch_forces", "exch_estimators",
                  "cart_update", "nm_propagate", "nm_thermo"]


class Config(C.Structure):
    """Mirror of ``pimdb_config``."""
    _fields_ = [
        ("ndim", C.c_int), ("natoms", C.c_int), ("nbeads", C.c_int), ("bosonic", C.c_int), ("pbc", C.c_int),
        ("fixcom", C.c_int), ("propagator", C.c_int), ("thermostat", C.c_int), ("nmthermostat", C.c_int),
        ("precision", C.c_int), ("temperature", C.c_double), ("mass", C.c_double), ("size", C.c_double),
        ("dt", C.c_double), ("gamma", C.c_double), ("ext_kind", C.c_int), ("ext_params", C.c_double * 3),
        ("int_kind", C.c_int), ("int_params", C.c_double * 3), ("cutoff", C.c_double),
        ("seed", C.c_ulonglong), ("replica", C.c_uint), ("nchains", C.c_int), ("exchange", C.c_int),
        ("rng", C.c_int),
    ]


class PimdbError(RuntimeError):
    pass


class ConfigError(PimdbError, ValueError):
    """The reference's std::invalid_argument."""


class ExchangeOverflowError(PimdbError, OverflowError):
    """The reference's std::overflow_error (non-finite V_B)."""


_lib = None


def lib():
    """Loads the shared library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: run build.build() (nvcc, sm_103a) first")
        L = C.CDLL(str(LIB_PATH))
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
        cfgp = C.POINTER(Config)
        sig = {
            "pimdb_config_default": ([cfgp], C.c_int),
            "pimdb_config_from_ini": ([C.c_char_p, C.c_int, cfgp, C.c_char_p, C.c_int], C.c_int),
            "pimdb_create": ([cfgp, vp, C.POINTER(vp)], C.c_int),
            "pimdb_destroy": ([vp], C.c_int),
            "pimdb_set_state": ([vp, vp, vp], C.c_int),
            "pimdb_set_state_device": ([vp, vp, vp], C.c_int),
            "pimdb_get_state": ([vp, vp, vp, vp], C.c_int),
            "pimdb_get_state_device": ([vp, vp, vp, vp], C.c_int),
            "pimdb_set_step": ([vp, C.c_longlong], C.c_int),
            "pimdb_get_step": ([vp, C.POINTER(C.c_longlong)], C.c_int),
            "pimdb_compute_forces": ([vp], C.c_int),
            "pimdb_step": ([vp, C.c_int], C.c_int),
            "pimdb_step_io": ([vp, vp, vp, C.c_int, vp, vp, vp], C.c_int),
            "pimdb_step_async": ([vp, C.c_int], C.c_int),
            "pimdb_synchronize": ([vp], C.c_int),
            "pimdb_exchange": ([vp, vp, vp, vp], C.c_int),
            "pimdb_exchange_arrays": ([vp, vp, vp, vp], C.c_int),
            "pimdb_exchange_forward": ([vp, vp], C.c_int),
            "pimdb_exchange_adjoint": ([vp, C.c_double, vp, vp], C.c_int),
            "pimdb_exchange_dbeta": ([vp, vp], C.c_int),
            "pimdb_exchange_retries": ([vp, C.POINTER(C.c_longlong)], C.c_int),
            "pimdb_exchange_fresh_estimates": ([vp, C.POINTER(C.c_longlong)], C.c_int),
            "pimdb_last_error": ([vp, C.c_char_p, C.c_int], C.c_int),
            "pimdb_status_string": ([C.c_int], C.c_char_p),
            "pimdb_profile": ([vp, C.c_int, vp, vp, vp], C.c_int),
            "pimdb_measure_fp64_peak": ([vp], C.c_int),
            "pimdb_measure_fp32_peak": ([vp], C.c_int),
            "pimdb_math_check": ([vp, C.c_int, vp], C.c_int),
            "pimdb_set_option": ([vp, C.c_char_p, C.c_int], C.c_int),
            "pimdb_thermostat_step": ([vp, C.c_int], C.c_int),
            "pimdb_zero_momentum": ([vp], C.c_int),
            "pimdb_propagate": ([vp], C.c_int),
            "pimdb_compute_observables": ([vp, vp], C.c_int),
            "pimdb_potential_energy": ([vp, vp], C.c_int),
            "pimdb_local_energy": ([vp, C.c_int, vp, vp], C.c_int),
            "pimdb_batch_create": ([cfgp, C.c_int, vp, C.POINTER(vp)], C.c_int),
            "pimdb_batch_destroy": ([vp], C.c_int),
            "pimdb_batch_size": ([vp, ip, C.POINTER(C.c_longlong)], C.c_int),
            "pimdb_batch_set_states": ([vp, vp, vp], C.c_int),
            "pimdb_batch_get_states": ([vp, vp, vp, vp], C.c_int),
            "pimdb_batch_set_step": ([vp, C.c_longlong], C.c_int),
            "pimdb_batch_get_step": ([vp, C.POINTER(C.c_longlong)], C.c_int),
            "pimdb_batch_compute_forces": ([vp], C.c_int),
            "pimdb_batch_step": ([vp, C.c_int], C.c_int),
            "pimdb_batch_step_async": ([vp, C.c_int], C.c_int),
            "pimdb_batch_synchronize": ([vp], C.c_int),
            "pimdb_batch_exchange": ([vp, vp], C.c_int),
            "pimdb_batch_set_option": ([vp, C.c_char_p, C.c_int], C.c_int),
            "pimdb_batch_get_launch": ([vp, ip, ip, ip, C.POINTER(C.c_longlong)], C.c_int),
            "pimdb_batch_autotune": ([vp, C.c_int, ip, ip], C.c_int),
            "pimdb_batch_last_error": ([vp, C.c_char_p, C.c_int], C.c_int),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _last_error(h=None) -> str:
    buf = C.create_string_buffer(1024)
    lib().pimdb_last_error(h, buf, len(buf))
    return buf.value.decode()


def _batch_last_error(b=None) -> str:
    buf = C.create_string_buffer(1024)
    lib().pimdb_batch_last_error(b, buf, len(buf))
    return buf.value.decode()


def _check(st: int, h=None, batch=False):
    if st == OK:
        return
    detail = _batch_last_error(h) if batch else _last_error(h)
    msg = f"{lib().pimdb_status_string(st).decode()}: {detail}"
    if st in (ERR_CONFIG, ERR_PARSE):
        raise ConfigError(msg)
    if st == ERR_NONFINITE_VB:
        raise ExchangeOverflowError(msg)
    raise PimdbError(msg)


def measure_fp32_peak() -> float:
    """FP32 FMA throughput of the current device, TFLOP/s."""
    v = C.c_double()
    _check(lib().pimdb_measure_fp32_peak(C.byref(v)))
    return v.value


def measure_fp64_peak() -> float:
    """Measured FP64 FMA throughput of the current device, TFLOP/s."""
    v = C.c_double()
    _check(lib().pimdb_measure_fp64_peak(C.byref(v)))
    return v.value


def math_check(x):
    """CUDA's exp and rsqrt beside the library's exp_tang, exp_tang256 and
    rsqrt_newton, and the bit-pattern conversions: array (n, 8) of exp(x),
    exp_tang(x), exp_tang256(x), rsqrt(r), rsqrt_newton(r) with
    r = |x| + 1e-3, hi and lo of split_f32(x), f32_to_f64(float(x))."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros((x.size, 8))
    _check(lib().pimdb_math_check(_ptr(x), x.size, _ptr(out)))
    return out


def default_config() -> Config:
    c = Config()
    _check(lib().pimdb_config_default(C.byref(c)))
    return c


def config_from_ini(path, ndim: int = 3) -> Config:
    """Reads a reference config.ini through the library's C++ reader."""
    c = Config()
    err = C.create_string_buffer(512)
    st = lib().pimdb_config_from_ini(str(path).encode(), ndim, C.byref(c), err, len(err))
    if st != OK:
        raise ConfigError(err.value.decode())
    return c


def make_config(**kw) -> Config:
    """Builds a config from keyword arguments (atomic units); potential,
    propagator, thermostat, precision, exchange algorithm and noise generator
    may be given by name."""
    c = default_config()
    for k, v in kw.items():
        if k in ("ext_kind", "int_kind") and isinstance(v, str):
            v = POT[v]
        elif k == "propagator" and isinstance(v, str):
            v = PROP[v]
        elif k == "thermostat" and isinstance(v, str):
            v = THERMO[v]
        elif k == "precision" and isinstance(v, str):
            v = PRECISION[v]
        elif k == "exchange" and isinstance(v, str):
            v = EXCHANGE[v]
        elif k == "rng" and isinstance(v, str):
            v = RNG[v]
        if k in ("ext_params", "int_params"):
            arr = getattr(c, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(c, k, v)
    return c


class System:
    """One ring-polymer system on the GPU (all beads), driven through the C ABI.

    Arrays use the reference's per-bead order, stacked: [bead][particle][axis].
    """

    def __init__(self, cfg: Config, stream: int | None = None):
        self.cfg = cfg
        self.shape = (cfg.nbeads, cfg.natoms, cfg.ndim)
        h = C.c_void_p()
        _check(lib().pimdb_create(C.byref(cfg), C.c_void_p(stream) if stream else None, C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().pimdb_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def _arr(self, a):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float64)
        if a.size != np.prod(self.shape):
            raise ValueError(f"expected {self.shape} elements, got {a.shape}")
        return a

    def set_state(self, x=None, p=None):
        x, p = self._arr(x), self._arr(p)
        _check(lib().pimdb_set_state(self._h, _ptr(x), _ptr(p)), self._h)

    def get_state(self):
        x, p, f = (np.empty(self.shape) for _ in range(3))
        _check(lib().pimdb_get_state(self._h, _ptr(x), _ptr(p), _ptr(f)), self._h)
        return x, p, f

    def set_state_ptr(self, x_ptr, p_ptr, device: bool):
        fn = lib().pimdb_set_state_device if device else lib().pimdb_set_state
        _check(fn(self._h, C.c_void_p(x_ptr) if x_ptr else None, C.c_void_p(p_ptr) if p_ptr else None), self._h)

    def get_state_ptr(self, x_ptr, p_ptr, f_ptr, device: bool):
        fn = lib().pimdb_get_state_device if device else lib().pimdb_get_state
        args = [C.c_void_p(v) if v else None for v in (x_ptr, p_ptr, f_ptr)]
        _check(fn(self._h, *args), self._h)

    def step_io_ptr(self, x_in, p_in, nsteps, x_out, p_out, f_out):
        """pimdb_step_io on host pointers (0 / None for an absent array)."""
        a = [C.c_void_p(v) if v else None for v in (x_in, p_in)]
        b = [C.c_void_p(v) if v else None for v in (x_out, p_out, f_out)]
        _check(lib().pimdb_step_io(self._h, *a, int(nsteps), *b), self._h)

    def step_io(self, x=None, p=None, nsteps: int = 1):
        """Sets x and p (None keeps them), runs nsteps and returns (x, p, f)."""
        x, p = self._arr(x), self._arr(p)
        out = [np.empty(self.shape) for _ in range(3)]
        _check(lib().pimdb_step_io(self._h, _ptr(x), _ptr(p), int(nsteps), *(_ptr(o) for o in out)), self._h)
        return tuple(out)

    def set_option(self, name: str, value: int):
        _check(lib().pimdb_set_option(self._h, name.encode(), int(value)), self._h)

    def set_step(self, step: int):
        _check(lib().pimdb_set_step(self._h, step), self._h)

    def get_step(self) -> int:
        v = C.c_longlong()
        _check(lib().pimdb_get_step(self._h, C.byref(v)), self._h)
        return v.value

    def compute_forces(self):
        _check(lib().pimdb_compute_forces(self._h), self._h)

    def step(self, nsteps: int = 1):
        _check(lib().pimdb_step(self._h, nsteps), self._h)

    def step_async(self, nsteps: int = 1):
        _check(lib().pimdb_step_async(self._h, nsteps), self._h)

    def thermostat_step(self, substep: int):
        _check(lib().pimdb_thermostat_step(self._h, substep), self._h)

    def zero_momentum(self):
        _check(lib().pimdb_zero_momentum(self._h), self._h)

    def propagate(self):
        _check(lib().pimdb_propagate(self._h), self._h)

    def synchronize(self):
        _check(lib().pimdb_synchronize(self._h), self._h)

    def exchange(self):
        N, D = self.cfg.natoms, self.cfg.ndim
        sc = np.zeros(4)
        f1 = np.zeros((N, D))
        fP = np.zeros((N, D))
        _check(lib().pimdb_exchange(self._h, _ptr(sc), _ptr(f1), _ptr(fP)), self._h)
        return dict(VB=sc[0], prim=sc[1], p_distinct=sc[2], p_longest=sc[3], f1=f1, fP=fP)

    def profile(self, enable: int = -1):
        """Per-kernel-class device ms and launch counts, and total launches."""
        ms = np.zeros(len(KERNEL_CLASSES))
        n = np.zeros(len(KERNEL_CLASSES), dtype=np.int64)
        tot = C.c_longlong()
        _check(lib().pimdb_profile(self._h, enable, _ptr(ms), _ptr(n), C.byref(tot)), self._h)
        return dict(ms=dict(zip(KERNEL_CLASSES, ms.tolist())), counts=dict(zip(KERNEL_CLASSES, n.tolist())),
                    launches=tot.value)

    def observables(self) -> dict:
        """The reference's observables of the current state, summed over
        beads (atomic units; temperature in kelvin)."""
        out = (C.c_double * len(OBSERVABLES))()
        _check(lib().pimdb_compute_observables(self._h, C.byref(out)), self._h)
        return dict(zip(OBSERVABLES, list(out)))

    def potential_energy(self):
        """Terms of U: external, pair, non-exchange springs, V_B."""
        t = np.zeros(4)
        _check(lib().pimdb_potential_energy(self._h, _ptr(t)), self._h)
        return t

    def local_energy(self, items):
        """Energy of every term involving (bead, particle) for each item."""
        it = np.ascontiguousarray(np.asarray(items, dtype=np.int32).reshape(-1, 2))
        out = np.zeros(len(it))
        _check(lib().pimdb_local_energy(self._h, len(it), _ptr(it), _ptr(out)), self._h)
        return out

    def exchange_forward(self) -> float:
        """V_B of the current coordinates (the forward half of the exchange)."""
        v = C.c_double()
        _check(lib().pimdb_exchange_forward(self._h, C.byref(v)), self._h)
        return v.value

    def exchange_adjoint(self, vb_bar: float = 1.0):
        """(vb_bar dV_B/dx_1, vb_bar dV_B/dx_P), each [particle][axis], from
        the last exchange_forward."""
        N, D = self.cfg.natoms, self.cfg.ndim
        x1, xP = np.zeros((N, D)), np.zeros((N, D))
        _check(lib().pimdb_exchange_adjoint(self._h, float(vb_bar), _ptr(x1), _ptr(xP)), self._h)
        return x1, xP

    def exchange_dbeta(self) -> float:
        """primEstimator of the last exchange_forward."""
        v = C.c_double()
        _check(lib().pimdb_exchange_dbeta(self._h, C.byref(v)), self._h)
        return v.value

    def exchange_retries(self) -> int:
        """Exchange evaluations redone from a fresh estimate since creation."""
        v = C.c_longlong()
        _check(lib().pimdb_exchange_retries(self._h, C.byref(v)), self._h)
        return v.value

    def exchange_fresh_estimates(self) -> int:
        """Exchange evaluations that began with a fresh FP32 estimate."""
        v = C.c_longlong()
        _check(lib().pimdb_exchange_fresh_estimates(self._h, C.byref(v)), self._h)
        return v.value

    def exchange_arrays(self):
        N = self.cfg.natoms
        E = np.zeros(N * (N + 1) // 2)
        V = np.zeros(N + 1)
        Vb = np.zeros(N + 1)
        _check(lib().pimdb_exchange_arrays(self._h, _ptr(E), _ptr(V), _ptr(Vb)), self._h)
        return dict(E=E, V=V, Vb=Vb)


class Batch:
    """Independent replicas (each its own Config) advanced together by the
    batched engine: one launch per MD step, runs of steps replayed as one
    CUDA graph.  Per-replica arrays are [bead][particle][axis]; the batch's
    host layout is their concatenation in replica order."""

    def __init__(self, cfgs, stream: int | None = None):
        cfgs = list(cfgs)
        arr = (Config * len(cfgs))(*cfgs)
        self.cfgs = cfgs
        self.shapes = [(c.nbeads, c.natoms, c.ndim) for c in cfgs]
        self.offsets = np.cumsum([0] + [int(np.prod(s)) for s in self.shapes])
        b = C.c_void_p()
        _check(lib().pimdb_batch_create(arr, len(cfgs), C.c_void_p(stream) if stream else None, C.byref(b)),
               None, batch=True)
        self._b = b

    def close(self):
        if getattr(self, "_b", None):
            lib().pimdb_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _c(self, st):
        _check(st, self._b, batch=True)

    def flatten(self, arrays):
        """Concatenates per-replica arrays into the batch's host layout."""
        return np.ascontiguousarray(np.concatenate([np.asarray(a, dtype=np.float64).ravel() for a in arrays]))

    def split(self, flat):
        return [flat[self.offsets[r]:self.offsets[r + 1]].reshape(self.shapes[r]) for r in range(len(self.shapes))]

    def set_states(self, xs=None, ps=None):
        x = None if xs is None else (xs if isinstance(xs, np.ndarray) and xs.ndim == 1 else self.flatten(xs))
        p = None if ps is None else (ps if isinstance(ps, np.ndarray) and ps.ndim == 1 else self.flatten(ps))
        self._c(lib().pimdb_batch_set_states(self._b, _ptr(x), _ptr(p)))

    def get_states(self, flat=False):
        n = int(self.offsets[-1])
        x, p, f = np.zeros(n), np.zeros(n), np.zeros(n)
        self._c(lib().pimdb_batch_get_states(self._b, _ptr(x), _ptr(p), _ptr(f)))
        if flat:
            return x, p, f
        return self.split(x), self.split(p), self.split(f)

    def set_step(self, step: int):
        self._c(lib().pimdb_batch_set_step(self._b, step))

    def get_step(self) -> int:
        v = C.c_longlong()
        self._c(lib().pimdb_batch_get_step(self._b, C.byref(v)))
        return v.value

    def compute_forces(self):
        self._c(lib().pimdb_batch_compute_forces(self._b))

    def step(self, nsteps: int = 1):
        self._c(lib().pimdb_batch_step(self._b, nsteps))

    def step_async(self, nsteps: int = 1):
        self._c(lib().pimdb_batch_step_async(self._b, nsteps))

    def synchronize(self):
        self._c(lib().pimdb_batch_synchronize(self._b))

    def exchange(self) -> np.ndarray:
        sc = np.zeros((len(self.cfgs), 4))
        self._c(lib().pimdb_batch_exchange(self._b, _ptr(sc)))
        return sc

    def set_option(self, name: str, value: int):
        self._c(lib().pimdb_batch_set_option(self._b, name.encode(), int(value)))

    def launch(self):
        t, c, g = C.c_int(), C.c_int(), C.c_int()
        n = C.c_longlong()
        self._c(lib().pimdb_batch_get_launch(self._b, C.byref(t), C.byref(c), C.byref(g), C.byref(n)))
        return dict(threads=t.value, ctas_per_sm=c.value, grid=g.value, launches=n.value)

    def autotune(self, steps: int = 3):
        t, c = C.c_int(), C.c_int()
        self._c(lib().pimdb_batch_autotune(self._b, steps, C.byref(t), C.byref(c)))
        return t.value, c.value

"""CPU checks of the C ABI library: it loads, exports every entry point the
header declares, and its config.ini reader agrees with the oracle harness's
independent reading of the reference schema (src/params.cpp:8-260)."""
import importlib
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G

ROOT = Path(__file__).resolve().parents[1]
pk = importlib.import_module("pimd-b_gb300")


def header_symbols():
    syms = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        syms |= set(re.findall(r"^\s*(?:int|const char\*|void)\s+\**(pimdb_\w+)\s*\(", text, re.M))
    return sorted(syms)


def test_library_exports_every_declared_symbol():
    L = pk.lib()
    syms = header_symbols()
    assert len(syms) >= 18
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing
    assert set(pk.EXPORTS) <= set(syms)


def test_status_strings():
    L = pk.lib()
    assert L.pimdb_status_string(0) == b"ok"
    assert b"exchange" in L.pimdb_status_string(2)


@pytest.mark.parametrize("case", sorted(G.load()[1]))
def test_ini_reader_matches_oracle_reading(case, tmp_path):
    path = G.write_ini(case, tmp_path)
    c = pk.config_from_ini(path)
    s, extra = O.system_from_ini(path)
    assert (c.natoms, c.nbeads, c.ndim) == (s.natoms, s.nbeads, s.ndim)
    assert bool(c.bosonic) == bool(s.bosonic) or s.nbeads == 1
    assert bool(c.fixcom) == bool(s.fixcom) and bool(c.pbc) == bool(s.pbc)
    assert c.propagator == s.propagator and bool(c.nmthermostat) == bool(s.nmthermostat)
    assert c.thermostat == s.thermostat and c.nchains == s.nchains
    for a, b in ((c.temperature, extra["temperature"]), (c.mass, s.mass), (c.dt, s.dt), (c.gamma, s.gamma),
                 (c.ext_params[0], s.ext_p[0])):
        assert a == b
    assert c.seed == extra["seed"]


INVALID = [
    ("[simulation]\nnbeads = 4\n", "Thermostat must be specified!"),
    ("[simulation]\nthermostat = none\nnmthermostat = true\n", "nmthermostat cannot be used in nve ensemble!"),
    ("[simulation]\nthermostat = langevin\nbosonic = true\npropagator = normal_modes\n",
     "Normal modes propogation is currently not available for bosons!"),
    ("[simulation]\nthermostat = langevin\nnchains = 3\n", "nchains can only be used with Nose-Hoover thermostats!"),
    ("[simulation]\nthermostat = langevin\nnbeads = 0\n", "The specified number of beads (0) is less than one!"),
    ("[simulation]\nthermostat = langevin\n[system]\ntemperature = -1 kelvin\n", "is unphysical!"),
    ("[simulation]\nthermostat = langevin\n[interaction_potential]\nname = lennard_jones\n",
     "The specified interaction potential (lennard_jones) is not supported!"),
    ("[simulation]\nthermostat = langevin\n[external_potential]\nname = aziz\n",
     "The specified external potential (aziz) is not supported!"),
    ("[simulation]\nthermostat = langevin\ndt = 1.0 fortnight\n", "fortnight is an undefined unit for kind time."),
    ("[simulation]\nthermostat = langevin\ndt = femtosecond\n", "Invalid input format"),
    ("[simulation]\nthermostat = langevin\ninitial_position = lattice\n",
     "The specified coordinate initialization method (lattice) is not supported!"),
]


@pytest.mark.parametrize("text,msg", INVALID)
def test_ini_reader_rejects_like_the_reference(text, msg, tmp_path):
    p = tmp_path / "bad.ini"
    p.write_text(text)
    with pytest.raises(pk.ConfigError) as ei:
        pk.config_from_ini(p)
    assert msg in str(ei.value)


def test_ini_reader_units_and_defaults(tmp_path):
    p = tmp_path / "u.ini"
    p.write_text("[simulation]\nthermostat = langevin ; inline comment\nnbeads = 8.0\ndt = 2 femtosecond\n"
                 "[system]\nmass = 4.0026 dalton\nsize = 22.7297 angstrom\nnatoms = 256\n"
                 "[interaction_potential]\nname = aziz\ncutoff = 11.3649 angstrom\n"
                 "[external_potential]\nname = double_well\nstrength = 1.32684e-7 millielectronvolt\n"
                 "location = 3 angstrom\n")
    c = pk.config_from_ini(p)
    assert c.nbeads == 8 and c.natoms == 256
    assert c.dt == 2 * 4.1341373e16 * 1e-15
    assert c.mass == 4.0026 * 1822.8885
    assert c.size == 22.7297 * 1.8897261
    assert c.cutoff == 11.3649 * 1.8897261
    assert c.ext_params[0] == 1.32684e-7 * 0.036749326 * 1e-3
    assert c.fixcom == 1 and c.pbc == 0 and c.gamma == 1 / (100.0 * c.dt)
    assert c.seed == 1234


def test_missing_file_is_a_parse_error(tmp_path):
    with pytest.raises(pk.ConfigError, match="Unable to read the configuration file"):
        pk.config_from_ini(tmp_path / "nope.ini")


def test_create_validates_before_touching_the_gpu():
    c = pk.make_config(natoms=0)
    with pytest.raises(pk.ConfigError):
        pk.System(c)


def test_bosonic_system_size_limit():
    """A bosonic ring polymer is limited to 14000 particles, where the
    one-block solve's shared memory (2 (N + 1) + 32 doubles beside its
    static tables) still fits a block; larger ones are rejected as a
    configuration error before any GPU work, distinguishable ones are not
    limited by it."""
    c = pk.make_config(natoms=14001, nbeads=4, bosonic=1)
    with pytest.raises(pk.ConfigError, match="at most 14000 particles"):
        pk.System(c)
    c = pk.make_config(natoms=14001, nbeads=1, bosonic=1)   # one bead: no exchange
    try:
        pk.System(c).close()
    except pk.ConfigError:
        pytest.fail("a one-bead system has no exchange to limit it")
    except pk.PimdbError:
        pass  # no GPU here


def test_normal_mode_bead_limit():
    """The normal-mode propagator and thermostat take at most 1536 beads,
    where the matrix-transform step's shared memory still fits a block;
    more are a configuration error before any GPU work."""
    for kw in (dict(propagator="normal_modes"), dict(nmthermostat=1)):
        c = pk.make_config(natoms=2, nbeads=1537, bosonic=0, **kw)
        with pytest.raises(pk.ConfigError, match="at most 1536 beads"):
            pk.System(c)


def test_integration_snippets_compile_against_the_header(tmp_path):
    """Every C++ snippet of INTEGRATION.md that uses only the C ABI compiles
    against include/pimdb_gb300.h (g++ -fsyntax-only), so the documented calls
    keep the header's names, argument counts and types.  The caller's own
    variables are declared by the stub below; `= ...;` placeholders become
    value-initialisation.  The BosonicExchange snippet needs the reference's
    own headers and is left out."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    text = (ROOT / "INTEGRATION.md").read_text()
    blocks = re.findall(r"```cpp\n(.*?)```", text, re.S)
    abi = [b for b in blocks if "pimdb_" in b and "BosonicExchangeBase" not in b]
    assert len(abi) >= 4
    stub = """#include <stdexcept>
#include <vector>
#include "pimdb_gb300.h"
static double x_all_beads[1], p_all_beads[1], x[1], p[1], f[1], g_first[1], g_last[1];
static double x_all[1], p_all[1], f_all[1];
static const long steps = 1, sfreq = 1;
static const int NDIM = 3;
static double dLoss_dVB(double v) { return v; }
static pimdb_handle* h = nullptr;
"""
    fixed = [re.sub(r"= \.\.\.;", "{};", blk) for blk in abi]
    body = "".join(f"void snippet_{k}() {{\n{blk}}}\n" for k, blk in enumerate(fixed))
    src = tmp_path / "snippets.cpp"
    src.write_text(stub + body)
    r = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wno-unused", "-I", str(ROOT / "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_integration_bosonic_exchange_snippet_compiles_against_the_reference(tmp_path):
    """The guide's GpuBosonicExchange overrides the reference's own
    BosonicExchangeBase (include/bosonic_exchange/bosonic_exchange_base.h):
    compiled with g++ -fsyntax-only against the reference's headers (and
    the oracle's MPI declarations), every `override` must match.  Skipped
    where the reference checkout is absent."""
    import shutil
    import subprocess
    from oracle import build_ref
    ref = build_ref.DEFAULT_REF
    gxx = shutil.which("g++")
    if gxx is None or not (ref / "include" / "bosonic_exchange" / "bosonic_exchange_base.h").exists():
        pytest.skip("reference checkout or g++ not available")
    text = (ROOT / "INTEGRATION.md").read_text()
    blk = [b for b in re.findall(r"```cpp\n(.*?)```", text, re.S) if "BosonicExchangeBase" in b]
    assert len(blk) == 1
    src = tmp_path / "gpu_bosonic_exchange.cpp"
    src.write_text("#include <algorithm>\n#include <stdexcept>\n#include <vector>\n" + blk[0])
    r = subprocess.run([gxx, "-std=c++20", "-fsyntax-only", "-I", str(ref / "include"), "-I",
                        str(ROOT / "oracle" / "ref"), "-I", str(ROOT / "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]

"""Build recipe for ``oracle/_ref``: the unmodified PIMD-B++ reference compiled
from its own sources (where they lie in the reference checkout) against the
project's process-based MPI shim (``oracle/ref/mpi_shim.c``).

Test infrastructure only: the GPU product never links or calls these binaries.

Variants (the reference fixes NDIM and the exchange algorithm at compile time,
CMakeLists.txt:44-54, include/common.h:10-28):
  d3       NDIM=3, Feldman-Hirshberg exchange
  d3_fact  NDIM=3, factorial exchange (FACTORIAL_BOSONIC_ALGORITHM)
  d2       NDIM=2, Feldman-Hirshberg exchange
Each variant produces ``pimdb_<v>`` (the reference's own main, run with
PIMDB_SHIM_NP ranks) and ``ref_probe_<v>`` (single-process force/exchange
probe, ``oracle/ref/ref_probe.cpp``).

Flags: -O2 -DNDEBUG -ffp-contract=off, so the x86-64 and aarch64 builds round
identically (no fused multiply-add contraction).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
# The reference checkout: $PIMDB_REFERENCE_DIR, else a directory named
# "reference" beside this repository (where the build container keeps it).
# The GPU host has neither, and nothing there needs it.
DEFAULT_REF = Path(os.environ["PIMDB_REFERENCE_DIR"]) if os.environ.get("PIMDB_REFERENCE_DIR") else \
    HERE.parent.parent / "reference"

VARIANTS = {
    "d3": ["-DNDIM=3"],
    "d3_fact": ["-DNDIM=3", "-DFACTORIAL_BOSONIC_ALGORITHM=1"],
    "d2": ["-DNDIM=2"],
}
CXXFLAGS = ["-std=c++20", "-O2", "-DNDEBUG", "-ffp-contract=off", "-w"]


def _sources(ref: Path):
    srcs = sorted(p for p in (ref / "src").rglob("*.cpp") if p.name != "pimdb.cpp")
    srcs += [ref / "libs" / "inireader.cpp", ref / "libs" / "random_mars.cpp"]
    return srcs


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(map(str, cmd))}\n{r.stderr[-4000:]}")


def _newer(target: Path, deps) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(Path(d).stat().st_mtime <= t for d in deps)


def build(ref: Path = DEFAULT_REF, variants=None, jobs: int | None = None, quiet: bool = True) -> bool:
    """Compile the reference variants.  Returns False when the reference
    sources are not available (e.g. on a machine without the checkout)."""
    if not (ref / "src" / "simulation.cpp").exists():
        return False
    variants = variants or list(VARIANTS)
    OUT.mkdir(parents=True, exist_ok=True)
    inc = ["-I", str(HERE / "ref"), "-I", str(ref / "include"), "-I", str(ref / "libs")]
    jobs = jobs or max(1, os.cpu_count() or 1)
    shim_o = OUT / "mpi_shim.o"
    ini_o = OUT / "ini.o"
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = []
        if not _newer(shim_o, [HERE / "ref" / "mpi_shim.c", HERE / "ref" / "mpi.h"]):
            futs.append(ex.submit(_run, ["gcc", "-O2", "-c", "-I", str(HERE / "ref"), str(HERE / "ref" / "mpi_shim.c"),
                                         "-o", str(shim_o)]))
        if not _newer(ini_o, [ref / "libs" / "ini.c"]):
            futs.append(ex.submit(_run, ["gcc", "-O2", "-c", str(ref / "libs" / "ini.c"), "-o", str(ini_o)]))
        objs = {}
        for v in variants:
            odir = OUT / f"obj_{v}"
            odir.mkdir(exist_ok=True)
            objs[v] = []
            for src in _sources(ref) + [HERE / "ref" / "ref_probe.cpp", ref / "src" / "pimdb.cpp"]:
                rel = src.name if src.parent == HERE / "ref" else str(src.relative_to(ref)).replace("/", "_")
                o = odir / (rel + ".o")
                objs[v].append(o)
                if not _newer(o, [src]):
                    futs.append(ex.submit(_run, ["g++", *CXXFLAGS, *VARIANTS[v], *inc, "-c", str(src), "-o", str(o)]))
        for f in futs:
            f.result()
        links = []
        for v in variants:
            common = [o for o in objs[v] if not o.name.endswith(("ref_probe.cpp.o", "src_pimdb.cpp.o"))]
            main_o = [o for o in objs[v] if o.name == "src_pimdb.cpp.o"]
            probe_o = [o for o in objs[v] if o.name == "ref_probe.cpp.o"]
            for exe, extra in ((OUT / f"pimdb_{v}", main_o), (OUT / f"ref_probe_{v}", probe_o)):
                links.append(ex.submit(_run, ["g++", "-o", str(exe), *map(str, common + extra), str(shim_o), str(ini_o),
                                              "-lpthread"]))
        for f in links:
            f.result()
    if not quiet:
        print(f"built reference variants {variants} into {OUT}")
    return True


if __name__ == "__main__":
    ok = build(Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_REF, quiet=False)
    sys.exit(0 if ok else 1)

"""Builds the in-tree shared library ``libpimdb_gb300.so`` (CUDA kernels for
sm_103a + C ABI + the C++20 host reader of config.ini) and the
``pimdb_gb300`` command-line driver.

nvcc compiles every .cu for ``-gencode arch=compute_103a,code=sm_103a`` only;
g++ compiles the host C++20 sources.  Objects go to ``_build/`` next to this
file; translation units are compiled in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
BUILD = HERE / "_build"
LIB = HERE / "libpimdb_gb300.so"
CLI = HERE / "pimdb_gb300"

CU_SOURCES = ["csrc/forces.cu", "csrc/exchange.cu", "csrc/factorial.cu", "csrc/integrator.cu", "csrc/api.cu",
              "csrc/noalloc.cu", "csrc/batch.cu"]
CPP_SOURCES = ["host/params.cpp"]
CLI_SOURCES = ["host/pimdb_main.cpp"]
HEADERS = ["csrc/common.cuh", "csrc/kernels.h", "csrc/config.h", "csrc/exchange_dev.cuh", "csrc/forces_dev.cuh",
           "csrc/dfloat.cuh", "csrc/aziz_df.cuh",
           "host/units.hpp", "host/pimdb_host.hpp"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=HERE)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout[-3000:]}\n{r.stderr[-6000:]}")
    return r


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    include = ["-I", str(ROOT / "include")]
    hdrs = [HERE / h for h in HEADERS if (HERE / h).exists()] + [ROOT / "include" / "pimdb_gb300.h"]
    objs, jobs_list = [], []
    for src in CU_SOURCES:
        o = BUILD / (Path(src).stem + ".o")
        objs.append(o)
        if _stale(o, [HERE / src, *hdrs]):
            jobs_list.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *include,
                              "-c", src, "-o", str(o)])
    for src in CPP_SOURCES:
        o = BUILD / (Path(src).stem + ".o")
        objs.append(o)
        if _stale(o, [HERE / src, *hdrs]):
            jobs_list.append(["g++", "-std=c++20", "-O2", "-fPIC", *include, "-c", src, "-o", str(o)])
    with cf.ThreadPoolExecutor(jobs or min(8, os.cpu_count() or 1)) as ex:
        for f in [ex.submit(_run, j) for j in jobs_list]:
            f.result()
    if jobs_list or not LIB.exists():
        tmp = LIB.with_suffix(f".so.{os.getpid()}")
        _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lstdc++"])
        os.replace(tmp, LIB)
    cli_srcs = [HERE / s for s in CLI_SOURCES if (HERE / s).exists()]
    if cli_srcs and _stale(CLI, [*cli_srcs, LIB, *hdrs]):
        _run(["g++", "-std=c++20", "-O2", *include, "-I", str(HERE / "host"), *map(str, cli_srcs), "-o", str(CLI),
              "-L", str(HERE), "-lpimdb_gb300", f"-Wl,-rpath,$ORIGIN"])
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)

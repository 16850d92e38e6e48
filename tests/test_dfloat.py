"""The double-float arithmetic of the pair kernels' far path
(pimd-b_gb300/csrc/dfloat.cuh, aziz_df.cuh), compiled for the host and
checked against long double (tests/dfloat_check.cpp).

Bounds, with u = 2^-24: the sum and product primitives within the published
error bounds (AccurateDWPlusDW 3u^2, DWTimesDW 5u^2), the exponential within
a few u^2 over [-69, 80], the logarithm within a few u^2 of max(|log y|, 1)
over [1e-20, 1e20], 1/sqrt within a few u^2 (and within 1e-12 from a
seed eight float ulps off), and the Aziz far-field gradient scale within
1e-12 relative (inside the damping radius, where the force crosses zero
at r_m, within 1e-12 of the size of its terms): the GPU's FP64 parity bar (1e-10 per bead) is two orders of
magnitude above what a sum of such pair terms can lose.
"""
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent
U2 = 2.0 ** -48


@pytest.fixture(scope="module")
def errors(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("dfloat") / "dfloat_check"
    subprocess.run([gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-o", str(exe), str(HERE / "dfloat_check.cpp")],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: float(v) for k, v in (ln.split() for ln in out.strip().splitlines())}


def test_sum_and_product_bounds(errors):
    assert errors["add"] <= 3 * U2
    assert errors["add_sloppy_abs"] <= 4 * U2
    assert errors["mul"] <= 5 * U2
    assert errors["sqr"] <= 5 * U2


def test_exp_and_rsqrt(errors):
    assert errors["exp"] <= 8 * U2
    # log (the exchange solve's log y): within a few u^2 of max(|log y|, 1)
    assert errors["log"] <= 8 * U2
    assert errors["rsqrt"] <= 8 * U2
    assert errors["rsqrt_seed8ulp"] <= 1e-12


def test_aziz_far_scale(errors):
    assert errors["aziz_far"] <= 1e-12


def test_aziz_near_scale(errors):
    # inside the damping radius, against the size of the cancelling terms
    assert errors["aziz_near"] <= 1e-12

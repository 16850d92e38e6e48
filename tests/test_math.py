"""The library's hand-written FP64 functions against CUDA's own, on the GPU
(pimdb_math_check):
- exp_tang: Tang's table-driven exp (ACM TOMS 15(2), 1989) with a 32-entry
  table and a degree-6 Taylor polynomial (exchange weights, factorial
  exchange);
- exp_tang256: the same method with a 256-entry table and a degree-4
  polynomial (pair forces);
- rsqrt_newton: rsqrtf on the float image of the bit pattern, then one
  Newton step with its second-order term (far-field pair gradient);
- split_f32 and f32_to_f64: float <-> double conversions by bit patterns
  (mixed-precision paths), which keep conversions off the FP64 pipe.

Bounds: each within 2 ulp (4.5e-16 relative) of CUDA's exp and rsqrt, and of
numpy's exp, over the whole argument range they serve ([-700, 5]; the pair
forces use [-48, -12]) and for 1/sqrt over [1e-3, 700].  split_f32: hi is x
truncated to a float (same sign, |x - hi| < 2^-23 |x|) and hi + lo
reproduces x within 2^-47 on its bit-pattern range 2^-60 <= |x| < 2^100
(elsewhere hi is the hardware conversion); f32_to_f64 equals the hardware
conversion exactly."""
import numpy as np
import pytest

from tests.gpu_cases import pk

TWO_ULP = 4.5e-16


def _args():
    rng = np.random.default_rng(7)
    return np.concatenate([rng.uniform(-700.0, 5.0, 200000), rng.uniform(-48.0, -12.0, 200000),
                           np.linspace(-700.0, 5.0, 4097)])


@pytest.mark.gpu
def test_table_exps_match_cuda_exp():
    x = _args()
    out = pk.math_check(x)
    ref = out[:, 0]
    for col, name in ((1, "exp_tang"), (2, "exp_tang256")):
        rel = np.abs(out[:, col] - ref) / ref
        assert rel.max() <= TWO_ULP, (name, rel.max(), x[np.argmax(rel)])
        rel_np = np.abs(out[:, col] - np.exp(x)) / np.exp(x)
        assert rel_np.max() <= TWO_ULP, (name, rel_np.max())


@pytest.mark.gpu
def test_newton_rsqrt_matches_cuda_rsqrt():
    x = _args()
    out = pk.math_check(x)
    r = np.abs(x) + 1e-3
    rel = np.abs(out[:, 4] - out[:, 3]) / out[:, 3]
    assert rel.max() <= TWO_ULP, (rel.max(), r[np.argmax(rel)])
    rel_np = np.abs(out[:, 4] - 1.0 / np.sqrt(r)) * np.sqrt(r)
    assert rel_np.max() <= TWO_ULP, rel_np.max()


@pytest.mark.gpu
def test_bit_pattern_conversions():
    rng = np.random.default_rng(3)
    x = rng.choice([-1.0, 1.0], 100000) * 10.0 ** rng.uniform(-15.0, 25.0, 100000)
    x = np.concatenate([x, [0.0, -0.0, 1.0, -1.0, 2.0 ** -60, 3.0e-38, 1.0e-40, 1e38]])
    out = pk.math_check(x)
    hi, lo, back = out[:, 5], out[:, 6], out[:, 7]
    # bit-pattern path for 2^-60 <= |x| < 2^100; the conversions elsewhere
    fast = (np.abs(x) >= 2.0 ** -60) & (np.abs(x) < 2.0 ** 100)
    assert np.all(np.abs(hi[fast] + lo[fast] - x[fast]) <= 2.0 ** -47 * np.abs(x[fast]))
    assert np.array_equal(hi[~fast], x[~fast].astype(np.float32).astype(np.float64))
    assert np.all(np.sign(hi[fast]) == np.sign(x[fast]))
    assert np.all(np.abs(hi[fast]) <= np.abs(x[fast]))
    assert np.all(np.abs(x[fast] - hi[fast]) < 2.0 ** -23 * np.abs(x[fast]))
    assert np.all(hi == hi.astype(np.float32)) and np.all(lo == lo.astype(np.float32))
    f = x.astype(np.float32).astype(np.float64)
    assert np.array_equal(back, f)

"""bench.py's reference arm on CPU: one JSON line with the benchmark
contract's keys (the same metric, unit and config as the GPU arm, an
`impl` of "reference", the CPU baseline it times and an `e2e` with no host
copies), printed by rank 0 only; other ranks of a torchrun launch exit 0
without work."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1"],
                          cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)


def test_reference_arm_prints_one_contract_line():
    r = _run({"RANK": "0", "WORLD_SIZE": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference"
    assert d["unit"] == "bead-steps/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["steps"] == 1 and d["warmup"] == 1
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_do_no_work():
    r = _run({"RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [l for l in r.stdout.splitlines() if l.strip().startswith("{")]


def test_exchange_latency_accounting():
    """The exchange chain's report: ns per recursion level from the
    recursions class, and its FP64 rate from 19 N^2 FLOPs over the chain's
    classes; nothing for a step without exchange."""
    sys.path.insert(0, str(ROOT))
    import bench
    per_class = {"bead_forces": 0.070, "exch_energies": 0.019, "exch_recursions": 0.0432, "exch_forces": 0.0104,
                 "nm_propagate": 0.028}
    x = bench.exchange_latency(per_class, 256, 1.25)
    assert x["levels_per_direction"] == 257
    assert abs(x["ns_per_level"] - 0.0432e6 / 257) < 1e-9
    assert abs(x["chain_ms_per_step"] - (0.019 + 0.0432 + 0.0104)) < 1e-12
    assert set(x["classes"]) == {"exch_energies", "exch_recursions", "exch_forces"}
    assert abs(x["fp64_tflops"] - 19.0 * 256 ** 2 / (x["chain_ms_per_step"] * 1e-3) / 1e12) < 1e-12
    assert abs(x["vs_fp64_peak"] - x["fp64_tflops"] / 1.25) < 1e-12
    assert x["exp_per_step"] == 1.5 * 256 ** 2
    assert bench.exchange_latency({"bead_forces": 0.07, "cart_update": 0.03}, 256, 1.25) is None

"""CPU tests of the measurement helpers in bench.py (no GPU): the CPU
baseline's sampling contract and the JSON line of the reference arm."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_cpu_baseline_takes_the_median_of_at_least_five_timed_steps():
    """Even with a zero time budget the sample holds min_steps timed steps
    after the warm-up, and the rate is that of the median step time."""
    import bench
    rate, done, cores, s_per_step = bench.cpu_step_rate(32, 100, 1, budget_s=0.0, cores=1)
    assert done == 5 and cores == 1
    assert rate > 0 and s_per_step > 0
    assert abs(rate - 32 * 32 / s_per_step / 1e6) <= 1e-9 * rate
    # a step cap below min_steps is honoured
    _, done2, _, _ = bench.cpu_step_rate(32, 3, 0, budget_s=0.0, cores=1)
    assert done2 == 3


def test_reference_arm_prints_one_json_line_with_its_contract_keys():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "64",
                          "--steps", "3", "--warmup", "1"],
                         capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["unit"] == "Mpt*steps/s" and line["higher_is_better"]
    assert line["steps"] == 3 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "Mpt*steps/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}

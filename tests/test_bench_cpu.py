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


def _dry(*extra):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--dry-cpu",
                          "--steps", "3", "--warmup", "3", *extra],
                         capture_output=True, text=True, timeout=300, cwd=ROOT,
                         env={k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")})
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]   # rank 0 alone prints
    return json.loads(lines[0])


def test_gpus_2_shards_the_ensemble_by_cost_over_two_gloo_ranks():
    """bench.py --gpus 2 without a launcher starts two ranks; the 96-run
    ensemble is split by cost, every run exactly once, and value is all
    runs' points x steps over the slowest rank's time."""
    import bench
    from spectral2d_gb300.replicas import run_cost
    line = _dry("--workload", "ensemble")
    assert line["n_gpus"] == 2 and line["dry_cpu"] and line["scaling"] == "strong"
    shards = line["shards"]
    assert len(shards) == 2 and sorted(shards[0] + shards[1]) == list(range(96))
    nxs, _ = bench.ensemble_runs()
    loads = [sum(run_cost(nxs[i]) for i in s) for s in shards]
    assert abs(loads[0] - loads[1]) <= max(run_cost(n) for n in nxs)
    ms = line["ms_per_rank"]
    pts = sum(n * n for n in nxs)
    assert abs(line["value"] - pts * 3 / (max(ms) * 1e-3) / 1e6) <= 1e-9 * line["value"]
    assert line["runs_per_rank"] == [len(s) for s in shards]


def test_gpus_2_splits_the_les_batch_evenly():
    line = _dry("--workload", "les-batch", "--les-runs", "10")
    assert line["n_gpus"] == 2 and line["runs_per_rank"] == [5, 5]
    assert sorted(line["shards"][0] + line["shards"][1]) == list(range(10))


def test_gpus_2_replicas_sum_their_rates():
    """The headline DNS workload: one replica per rank; value is the sum of
    the per-rank rates taken at the slowest rank's time."""
    line = _dry("--n", "64")
    assert line["n_gpus"] == 2 and line["scaling"] == "weak"
    ms = line["ms_per_rank"]
    assert len(ms) == 2
    per_rank = 64 * 64 * 3 / (max(ms) * 1e-3) / 1e6
    assert abs(line["value"] - 2 * per_rank) <= 1e-9 * line["value"]

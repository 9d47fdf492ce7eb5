"""bench.py's JSON line on the CPU: the reference arm (the oracle port in reference semantics on
the host cores) prints one line with the contract's keys, and a rank other than 0 prints nothing."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"}


def _run(args, env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return [l for l in r.stdout.splitlines() if l.startswith("{")]


@pytest.mark.parametrize("workload", ["c5", "at"])
def test_reference_arm_prints_the_contract_line(workload):
    lines = _run(["--impl", "reference", "--steps", "1", "--warmup", "3", "--workload", workload, "--no-tta"])
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert KEYS <= set(d)
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "flips/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1 and d["vs_baseline"] is None
    assert d["config"]["workload"].startswith({"c5": "ising2d_L64_64win_x8", "at": "ashkin_teller2d_L32"}[workload])
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "flips/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_print_nothing():
    assert _run(["--impl", "reference", "--steps", "1", "--warmup", "3"], {"RANK": "1", "WORLD_SIZE": "2"}) == []


def test_default_workload_is_the_headline_configuration():
    """The default line is quoted on Ising L = 64, 64 windows x 8 walkers (the configuration the
    metric names), with the 1/t schedule and walkers started from all +1 as the reference's."""
    sys.path.insert(0, str(ROOT))
    import bench
    w = bench.WORKLOADS["c5"]
    assert bench.WORKLOAD is w
    assert (w["L"], w["num_windows"], w["replicas_per_window"]) == (64, 64, 8)
    assert (w["sweeps_per_exchange"], w["sweeps_per_check"], w["one_over_t"], w["init_mode"]) == (500, 1000, 1, 1)
    assert bench.flips_per_sweep(w) * w["sweeps_per_check"] == 2_097_152_000


def test_warmup_below_three_is_refused():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--warmup", "2"], cwd=ROOT, capture_output=True,
                       text=True, timeout=120)
    assert r.returncode != 0 and "--warmup must be >= 3" in r.stderr


@pytest.mark.parametrize("workload", ["at", "mixed"])
def test_bench_batches_give_every_walker_its_own_key(workload):
    """Walker keys are (key_lo XOR walker, key_hi) with key the instance seed's SplitMix64 mix: the
    bench's consecutive instance seeds give every walker of a batch its own key."""
    sys.path.insert(0, str(ROOT))
    import bench
    import rewl_simulator_gb300 as rg
    old = bench.WORKLOAD
    try:
        bench.select_workload(workload)
        batch = bench.make_batch(rg, bench.rank_seed(0), device=0)
    finally:
        bench.WORKLOAD = old
    keys = set()
    for ins in batch.instances:
        k = rg.instance_key(ins.seed)
        for u in range(ins.num_windows * ins.replicas_per_window):
            keys.add(((k & 0xFFFFFFFF) ^ u, k >> 32))
    assert len(keys) == sum(i.num_windows * i.replicas_per_window for i in batch.instances)

#!/usr/bin/env python3
"""Benchmark of the REWL hot path on GB300.

Default workload (the configuration the headline metric is quoted on): 2D Ising,
L = 64 periodic, J = 1, energy levels -8192..8192 step 4 (bins of width 4 over
[-8192, 8196)), 64 equal windows at 75 % overlap x 8 walkers = 512 walkers, int8
spins, replica exchange every 500 sweeps, flatness (min >= 0.8 mean over the valid
levels) checked every 1000 sweeps, ln f from 1 with the reference's default 1/t
schedule (ONE_OVER_T_ALGORITHM), walkers started from all spins +1 as the
reference's are, int64 logDoS in 2^-36 units.  Inputs are synthetic.

A step is one check interval: 2 x (500 sweeps of all 512 walkers + one replica
exchange round) + the flatness / averaging / ln f kernel, i.e. 2,097,152,000
attempted single-spin flips.  `value` is attempted flips per second over the whole
job (device time, CUDA events on the engine's stream, L2 flushed between steps by a
256 MiB write).  `e2e` runs the same steps through the public API with the walker
state host-resident in pinned memory: restore (H2D) + step + snapshot (D2H) per
step, wall clock.

The default line also carries `time_to_accuracy`: for the same L = 64 system, the
simulation time until the concatenated, normalised ln g is within each of a ladder
of tolerances (1 .. 1e-2) of the exact density of states (Beale), for the MLP warm
start (trained here on plain GPU runs at L <= 32) and for plain WL from ln f0 = 1,
each capped at --tta-seconds; and the same criterion for 2D Ising L = 16 (16 windows x
64 walkers) run to 1e-2 on the GPU, whose CPU counterpart is the reference arm's
`time_to_accuracy`.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl {gb300,reference}]
                    [--workload {c5,c2,at,mixed}] [--observables {0,1,2}] [--no-tta]
                    [--at-spread CYCLES]

Other workloads: c2 (Ising L = 32, 16 windows x 8 walkers), at (Ashkin-Teller L = 32,
K = 0.5, Baxter fields sigma 0.5, bins of 0.05, 64 realisations x 8 windows x 4
walkers), mixed (Ising L = 16..48 and Ashkin-Teller L = 24 at three K in one batch).

--impl reference times the CPU restatement of the reference's hot path (the oracle
port, reference semantics: mt19937_64 streams, draw-on-demand, FP64 logDoS) on all
host cores for the same workload, and runs Ising L = 16 (16 windows x 64 walkers) to
max |d ln g| <= 1e-2 on those cores; under torchrun only rank 0 runs.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "time to ln g within 1e-2 of exact, MLP warm-start vs plain WL, 1 GB300; flips/s"
# Cycles per attempted flip of one walker's accept chain at the speed of light of the
# bin-tracking kernel's design, from probe kernels on a GB300: a dependent shared-memory load
# (29 cycles) plus a 64-bit compare and select (11 cycles).
CHAIN_FLOOR_CYCLES = 40.0


def _ising_workload(name, L, nwin, R, se, sc, lnf_final, one_over_t, init_mode, profile):
    N = L * L
    return dict(name=name, model="ising2d", L=L, energy_min=-2.0 * N, energy_max=2.0 * N + 4, bin_width=4.0,
                num_windows=nwin, replicas_per_window=R, window_overlap=0.75, sweeps_per_exchange=se,
                sweeps_per_check=sc, lnf_initial=1.0, lnf_final=lnf_final, one_over_t=one_over_t,
                init_mode=init_mode, flatness="min >= 0.8 mean over valid levels", realizations=1,
                bytes_per_flip=46, kernel="k_sweep_ising_bins", bound="latency", profile=profile, graphs=1)


WORKLOADS = {
    # the headline configuration (default): 2D Ising L = 64, 64 windows x 8 walkers
    "c5": _ising_workload("ising2d_L64_64win_x8walkers_rewl", 64, 64, 8, 500, 1000, 1e-8, 1, 1,
                          "sweep_ising_L64_64x8_rewl.md"),
    # batched Ising L = 32, 16 windows x 8 walkers, halving ln f 1 -> 1e-8, random initial spins
    "c2": _ising_workload("ising2d_L32_16win_x8walkers_rewl", 32, 16, 8, 500, 1000, 1e-8, 0, 0,
                          "sweep_ising_L32_rewl.md"),
    # 2D Ashkin-Teller, K = 0.5, Gaussian Baxter fields (sigma 0.5), 64 realisations x 8 windows x 4 walkers
    "at": dict(name="ashkin_teller2d_L32_K0.5_h0.5_64real_8win_x4walkers_rewl", model="ashkin_teller2d", L=32, K=0.5,
               sigma_h=0.5, energy_min=-5120.0, energy_max=0.0, bin_width=0.05, num_windows=8, replicas_per_window=4,
               window_overlap=0.75, sweeps_per_exchange=100, sweeps_per_check=200, lnf_initial=1.0, lnf_final=1e-7,
               flatness="min >= 0.8 mean over visited bins", realizations=64, one_over_t=0, init_mode=0,
               bytes_per_flip=51, kernel="k_sweep_tables<AshkinTeller2dModel>", bound="latency",
               profile="sweep_at_L32_64real_rewl.md", graphs=0),
}


def _mixed_components():
    """The uneven batch: 2D Ising at L = 16, 24, 32, 48 (16 windows x 4 walkers each) and 2D
    Ashkin-Teller at L = 24 with K = 0.25, 0.5, 0.75, Baxter fields h ~ N(0, 0.3^2), 32
    realisations each (8 windows x 4 walkers, bins of 0.05)."""
    comps = []
    for L in (16, 24, 32, 48):
        N = L * L
        comps.append(dict(model="ising2d", L=L, energy_min=-2.0 * N, energy_max=2.0 * N + 4, bin_width=4.0,
                          num_windows=16, replicas_per_window=4, window_overlap=0.75, realizations=1))
    for K in (0.25, 0.5, 0.75):
        N = 24 * 24
        comps.append(dict(model="ashkin_teller2d", L=24, K=K, sigma_h=0.3, energy_min=-(2.0 + K) * 2 * N,
                          energy_max=0.0, bin_width=0.05, num_windows=8, replicas_per_window=4, window_overlap=0.75,
                          realizations=32))
    return comps


WORKLOADS["mixed"] = dict(
    name="mixed_ising_L16_24_32_48_x16win_x4_at_L24_K0.25_0.5_0.75_x32real_x8win_x4_rewl", model="mixed",
    components=_mixed_components(), sweeps_per_exchange=100, sweeps_per_check=200, lnf_initial=1.0,
    lnf_final=1e-8, flatness="min >= 0.8 mean over visited bins", realizations=1, one_over_t=0, init_mode=0,
    kernel="k_sweep_tables<AshkinTeller2dModel> + k_sweep_ising_bins (launch groups on concurrent streams)",
    bound="latency", profile="", graphs=1, autotune=1)
for _c in WORKLOADS["mixed"]["components"]:
    _c["bytes_per_flip"] = 46 if _c["model"] == "ising2d" else 51
WORKLOAD = WORKLOADS["c5"]


def select_workload(name: str) -> None:
    global WORKLOAD
    WORKLOAD = WORKLOADS[name]


def step_text() -> str:
    w = WORKLOAD
    k = w["sweeps_per_check"] // w["sweeps_per_exchange"]
    return f"one check interval: {k} x ({w['sweeps_per_exchange']} sweeps + exchange) + flatness/averaging/ln f"


def ndof(w) -> int:
    return w["L"] ** 2 * (2 if w["model"] == "ashkin_teller2d" else 1)


def flips_per_sweep(w) -> int:
    if w["model"] == "mixed":
        return sum(flips_per_sweep(c) for c in w["components"])
    return w["realizations"] * w["num_windows"] * w["replicas_per_window"] * ndof(w)


def bytes_per_flip(w) -> float:
    """Algorithmic bytes per attempted flip (46 Ising, 51 Ashkin-Teller), flip-weighted for a mix."""
    if w["model"] == "mixed":
        return sum(c["bytes_per_flip"] * flips_per_sweep(c) for c in w["components"]) / flips_per_sweep(w)
    return w["bytes_per_flip"]


def at_fields(w, k: int) -> np.ndarray:
    """Gaussian Baxter fields of realisation k, rounded to multiples of 2^-20."""
    h = np.random.default_rng(100 + k).normal(0.0, w["sigma_h"], w["L"] ** 2)
    return np.round(h * 2**20) / 2**20


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def rank_seed(rank: int) -> int:
    """Each rank runs its own copy of the workload (weak scaling) with its own seed: the ranks'
    instances are independent and exchange nothing."""
    return 1000 + rank


def reduce_over_ranks(times, counts, device: str = "cpu"):
    """Job-wide figures from per-rank ones: the maximum over ranks of each time (the slowest rank
    ends the job) and the sum of each count.  One all-reduce each over the default group (NCCL
    tensors on the GPU, gloo on CPU)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x) for x in times], dtype=torch.float64, device=device)
    c = torch.tensor([float(x) for x in counts], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return t.tolist(), c.tolist()


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), float(d.get("sm_max_mhz", 2070.0)), "measured"
    return 6800.0, 2070.0, "fallback"


def profile_figures():
    """Figures of the committed ncu summary of the workload's sweep kernel, if any: lines
    `key: value ...` (traffic per launch, shared-memory and issue throughput)."""
    if not WORKLOAD["profile"]:
        return {}
    p = ROOT / "profiles" / WORKLOAD["profile"]
    if not p.exists():
        return {}
    out = {}
    for line in p.read_text().splitlines():
        for key in ("traffic_bytes_per_launch", "shared_throughput_pct", "l1_throughput_pct",
                    "issue_slots_busy_pct", "dram_throughput_pct", "warps_active_pct", "ncu_workload"):
            if line.startswith(key + ":"):
                val = line.split(":", 1)[1].strip()
                try:
                    out[key] = float(val.split()[0])
                except ValueError:
                    out[key] = val
    return out


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def instance_seed(seed: int, k: int) -> int:
    """Seed of the k-th instance of a batch (the engine mixes it into the walkers' Philox keys)."""
    return seed * 100000 + k


def make_batch(rg, seed: int, device: int, observables: int | None = None):
    w = WORKLOAD
    obs = w.get("observables", 0) if observables is None else observables
    if w["model"] == "mixed":
        inss = []
        for ci, c in enumerate(w["components"]):
            for k in range(c["realizations"]):
                at = c["model"] != "ising2d"
                inss.append(rg.Instance(model=rg.MODEL_ASHKIN_TELLER2D if at else rg.MODEL_ISING2D, L=c["L"],
                                        K=c.get("K", 0.0), fields=at_fields(c, 1000 * ci + k) if at else None,
                                        energy_min=c["energy_min"], energy_max=c["energy_max"],
                                        bin_width=c["bin_width"], num_windows=c["num_windows"],
                                        replicas_per_window=c["replicas_per_window"],
                                        window_overlap=c["window_overlap"], seed=instance_seed(seed, 100 * ci + k)))
        return rg.Batch(instances=inss, sweeps_per_exchange=w["sweeps_per_exchange"],
                        sweeps_per_check=w["sweeps_per_check"], flatness_param=0.8, lnf_initial=w["lnf_initial"],
                        lnf_final=w["lnf_final"], device=device, mask_mode=rg.MASK_VISITED,
                        graphs=w["graphs"], autotune=w["autotune"], observables=obs,
                        persistent=w.get("persistent", 0))
    if w["model"] == "ising2d":
        inss = [rg.Instance(model=rg.MODEL_ISING2D, L=w["L"], energy_min=w["energy_min"], energy_max=w["energy_max"],
                            bin_width=w["bin_width"], num_windows=w["num_windows"],
                            replicas_per_window=w["replicas_per_window"], window_overlap=w["window_overlap"],
                            init_mode=w["init_mode"], seed=seed)]
        mask = rg.MASK_STATIC
    else:
        inss = [rg.Instance(model=rg.MODEL_ASHKIN_TELLER2D, L=w["L"], K=w["K"], fields=at_fields(w, k),
                            energy_min=w["energy_min"], energy_max=w["energy_max"], bin_width=w["bin_width"],
                            num_windows=w["num_windows"], replicas_per_window=w["replicas_per_window"],
                            window_overlap=w["window_overlap"], seed=instance_seed(seed, k))
                for k in range(w["realizations"])]
        mask = rg.MASK_VISITED
    return rg.Batch(instances=inss, sweeps_per_exchange=w["sweeps_per_exchange"],
                    sweeps_per_check=w["sweeps_per_check"], flatness_param=0.8, lnf_initial=w["lnf_initial"],
                    lnf_final=w["lnf_final"], device=device, mask_mode=mask, observables=obs,
                    one_over_t=w["one_over_t"], graphs=w["graphs"], persistent=w.get("persistent", 0))


# --------------------------------------------------------------------------- CPU leg
def _port_config(po, w, threads, observables=0, seed=2024):
    at = w["model"] != "ising2d"
    return po.Config(model=po.MODEL_AT if at else po.MODEL_ISING, L=w["L"], K=w.get("K", 0.0),
                     escale_bits=20 if at else 0, nwin=w["num_windows"], R=w["replicas_per_window"],
                     sweeps_per_exchange=w["sweeps_per_exchange"], sweeps_per_check=w["sweeps_per_check"],
                     emin=w["energy_min"], emax=w["energy_max"], bw=w["bin_width"], overlap=w["window_overlap"],
                     lnf0=w["lnf_initial"], lnf_final=w["lnf_final"], semantics=po.SEM_REFERENCE, nthreads=threads,
                     mask_mode=po.MASK_VISITED if at else po.MASK_STATIC, one_over_t=w.get("one_over_t", 0),
                     init_mode=w.get("init_mode", 0), observables=observables, seed=seed)


def sample_sweeps(w) -> int:
    """Sweeps per timed CPU sample: about 2e8 attempted flips of the instance (one exchange
    interval at most), so that a sample takes about a second on the host cores."""
    per = w["num_windows"] * w["replicas_per_window"] * ndof(w)
    return int(max(1, min(w["sweeps_per_exchange"], 200_000_000 // per)))


def cpu_port_rate(target_seconds: float, threads: int, steps: int | None = None, warmup: int = 0,
                  observables: int = 0):
    """Flips/s of the oracle port (reference semantics) on `threads` host threads (one instance:
    the port drives one instance at a time, so for a batch of realisations it times one of them).
    A sample is sample_sweeps() sweeps of every walker followed by one replica-exchange round.
    For the uneven batch, one instance of every component is timed and the rate is the batch's
    flips over the time the CPU needs for all of them."""
    if WORKLOAD["model"] == "mixed":
        return _cpu_port_rate_mixed(target_seconds, threads, steps, warmup)
    return _cpu_port_rate_one(WORKLOAD, target_seconds, threads, steps, warmup, observables)


def _cpu_port_rate_mixed(target_seconds, threads, steps, warmup):
    comps = WORKLOAD["components"]
    cpu_s, n_total, t_total, times = 0.0, 0, 0.0, []
    for c in comps:
        w = dict(c, sweeps_per_exchange=WORKLOAD["sweeps_per_exchange"], sweeps_per_check=WORKLOAD["sweeps_per_check"],
                 lnf_initial=WORKLOAD["lnf_initial"], lnf_final=WORKLOAD["lnf_final"])
        rate, n, total, ts = _cpu_port_rate_one(w, target_seconds / len(comps), threads,
                                                None if steps is None else max(1, steps // len(comps)), 0)
        cpu_s += flips_per_sweep(c) / rate     # one sweep of component c
        n_total += n
        t_total += total
        times += ts
    return flips_per_sweep(WORKLOAD) / cpu_s, n_total, t_total, times


def _cpu_port_rate_one(w, target_seconds, threads, steps, warmup, observables=0):
    from oracle import pyoracle as po
    at = w["model"] != "ising2d"
    orc = po.Oracle(_port_config(po, w, threads, observables), fields=at_fields(w, 0) if at else None)
    sweeps = sample_sweeps(w)
    fps = w["num_windows"] * w["replicas_per_window"] * ndof(w)
    for _ in range(warmup):
        orc.run_sweeps(max(1, sweeps // 10))
    times = []
    done_steps = 0
    t_start = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        orc.run_sweeps(sweeps)
        orc.exchange()
        times.append(time.perf_counter() - t0)
        done_steps += 1
        if steps is not None:
            if done_steps >= steps:
                break
        elif time.perf_counter() - t_start >= target_seconds:
            break
    orc.close()
    total = sum(times)
    rate = done_steps * sweeps * fps / total
    return rate, done_steps, total, times


def _sample_text(n, total):
    w = WORKLOAD
    if w["model"] == "mixed":
        return (f"{n} samples of one instance of each of the {len(w['components'])} components "
                f"({sample_sweeps(w['components'][0])} sweeps + exchange each, {total:.1f} s)")
    return (f"{n} samples of one instance of the workload ({w['num_windows'] * w['replicas_per_window']} walkers; "
            f"each sample {sample_sweeps(w)} sweeps of every walker + one exchange round, {total:.1f} s)")


# Time to accuracy: Ising L = 16, 16 windows x 64 walkers, to 1e-2 (both arms run it).  Measured
# on a GB300 and its 16 Grace cores: 16 x 64 GPU 1.5 s; 4 x 64 GPU 4.3 s, CPU 32.5 s; 4 x 8 GPU
# 20.5 s, CPU 17.7 s -- the GPU's advantage is the number of walkers it runs at once.
SMALL_TTA = dict(L=16, num_windows=16, replicas_per_window=64, sweeps_per_exchange=500, sweeps_per_check=1000,
                 tolerance=1e-2, cap_seconds=150.0, seed=5)
TTA_TOLERANCES = [1.0, 0.5, 0.3, 0.2, 0.15, 0.1, 0.08, 0.05, 0.03, 0.02, 0.01]


def exact_lng(L: int):
    z = np.load(ROOT / "tests" / "golden" / f"exact_ising_L{L}.npz")
    return dict(zip(z["E"].astype(np.int64).tolist(), z["lng"]))


def _max_error(E, g, exact) -> float:
    return float(np.max(np.abs([g[i] - exact[int(round(E[i]))] for i in range(len(E))])))


def cpu_small_tta(threads: int):
    """The reference's algorithm (oracle port, reference semantics) on the host cores: Ising
    L = 16 in SMALL_TTA's layout, 1/t, walkers from all +1, until max |d ln g| <= 1e-2 against the
    exact density of states or the cap.  The clock stops while the accuracy is evaluated."""
    from oracle import pyoracle as po
    import rewl_simulator_gb300 as rg
    s = SMALL_TTA
    L, N = s["L"], s["L"] ** 2
    w = dict(model="ising2d", L=L, energy_min=-2.0 * N, energy_max=2.0 * N + 4, bin_width=4.0,
             num_windows=s["num_windows"], replicas_per_window=s["replicas_per_window"], window_overlap=0.75,
             sweeps_per_exchange=s["sweeps_per_exchange"], sweeps_per_check=s["sweeps_per_check"], lnf_initial=1.0,
             lnf_final=1e-12, one_over_t=1, init_mode=1)
    orc = po.Oracle(_port_config(po, w, threads, seed=s["seed"]))
    exact = exact_lng(L)
    hit, t_sim, cycles, best, flips = {}, 0.0, 0, float("inf"), 0
    per_cycle = s["sweeps_per_check"] * s["num_windows"] * s["replicas_per_window"] * N
    while t_sim < s["cap_seconds"]:
        t0 = time.perf_counter()
        orc.cycle()
        t_sim += time.perf_counter() - t0
        cycles += 1
        flips += per_cycle
        wins = []
        for k in range(s["num_windows"]):
            lo, _, _, nb = orc.windows[k]
            m = orc.window_mask(k)
            wins.append(((lo + 4.0 * np.arange(nb))[m], orc.window_logdos(k)[m]))
        E, g = rg.concatenate_windows(wins, 2.0, N)
        err = _max_error(E, g, exact)
        best = min(best, err)
        for tol in TTA_TOLERANCES:
            if err <= tol and str(tol) not in hit:
                hit[str(tol)] = round(t_sim, 2)
        if err <= s["tolerance"]:
            break
    orc.close()
    return {"workload": f"ising2d_L{L}_{s['num_windows']}win_x{s['replicas_per_window']}walkers",
            "schedule": "1/t (ONE_OVER_T_ALGORITHM), min >= 0.8 mean, walkers from all +1, exchange every 500 sweeps, "
                        "check every 1000", "seconds_to": hit, "best_max_abs_dlng": best, "cycles": cycles,
            "flips": flips, "seconds": round(t_sim, 2), "cap_seconds": s["cap_seconds"], "threads": threads,
            "clock": "simulation only (stopped while the accuracy is evaluated)"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    w = WORKLOAD
    rate, n, total, times = cpu_port_rate(0, threads, steps=args.steps, warmup=args.warmup)
    line = {
        "metric": METRIC, "value": rate, "unit": "flips/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / n, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": w["name"], **{k: v for k, v in w.items() if k != "name"},
                   "step": "a bounded sample: " + _sample_text(n, total)},
        "cpu_baseline": {"value": rate, "unit": "flips/s", "cores": threads, "kind": "port",
                         "sample": _sample_text(n, total)},
        "e2e": {"value": rate, "unit": "flips/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not args.no_tta and w["model"] == "ising2d":
        line["time_to_accuracy"] = cpu_small_tta(threads)
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------- GPU leg
TTA_SEED = 3


def ising_batch(rg, L: int, nwin: int, R: int, lnf0: float, lnf_final: float, seed: int, device: int,
                one_over_t: int = 1, sweeps_per_exchange: int = 500, sweeps_per_check: int = 1000):
    """Ising on the full spectrum; walkers start from all spins +1 and walk up into their windows,
    as the reference's do (a quench from random spins into the lowest windows can end in a
    stripe state that never reaches the window's lowest levels)."""
    N = L * L
    ins = rg.Instance(model=rg.MODEL_ISING2D, L=L, energy_min=-2.0 * N, energy_max=2.0 * N + 4, bin_width=4.0,
                      num_windows=nwin, replicas_per_window=R, window_overlap=0.75, seed=seed, init_mode=1)
    return rg.Batch(instances=[ins], sweeps_per_exchange=sweeps_per_exchange, sweeps_per_check=sweeps_per_check,
                    flatness_param=0.8, lnf_initial=lnf0, lnf_final=lnf_final, one_over_t=one_over_t, device=device,
                    graphs=1)


def track_accuracy(ws, eng, exact, max_seconds: float, burn_in: int = 0, stall_checks: int = 0, t_setup: float = 0.0,
                   stop_at: float | None = None):
    """Run check intervals, recording the simulation time (setup + the intervals, the clock stopped
    while the accuracy is evaluated) at which the max error first falls to each tolerance."""
    hit, flips_at, best, t_sim, last = {}, {}, [float("inf")], [t_setup], [None]
    stop_at = TTA_TOLERANCES[-1] if stop_at is None else stop_at
    t_mark = [time.perf_counter()]

    def on_cycle(e, st):
        t_sim[0] += time.perf_counter() - t_mark[0]
        E, g = e.global_logdos(0)
        err = _max_error(E, g, exact)
        best[0] = min(best[0], err)
        last[0] = err
        for tol in TTA_TOLERANCES:
            if err <= tol and str(tol) not in hit:
                hit[str(tol)] = round(t_sim[0], 2)
                flips_at[str(tol)] = st.attempted_flips
                # progress on stderr, so that a long run cut short still leaves its record
                print(json.dumps({"tolerance": tol, "seconds": hit[str(tol)], "flips": st.attempted_flips}),
                      file=sys.stderr, flush=True)
        t_mark[0] = time.perf_counter()
        return t_sim[0] > max_seconds or err <= stop_at

    stopped = None
    try:
        st, fallbacks = ws.run(eng, 1 << 30, stall_checks=stall_checks, on_cycle=on_cycle, burn_in=burn_in)
        flips = st.attempted_flips
    except Exception as exc:                # e.g. a window that never went flat (REWL_ESTATE)
        stopped, fallbacks, flips = str(exc), None, None
    out = {"seconds_to": hit, "flips_to": flips_at, "best_max_abs_dlng": best[0], "last_max_abs_dlng": last[0],
           "flips": flips, "seconds": round(t_sim[0], 2), "fallbacks": fallbacks}
    if stopped:
        out["stopped"] = stopped
    return out


def gpu_small_tta(rg, device: int):
    """SMALL_TTA on the GPU: the same system and criterion as the reference arm's CPU run."""
    from rewl_simulator_gb300 import warmstart as ws
    s = SMALL_TTA
    t0 = time.perf_counter()
    eng = rg.Engine(ising_batch(rg, s["L"], s["num_windows"], s["replicas_per_window"], 1.0, 1e-12, s["seed"], device,
                                sweeps_per_exchange=s["sweeps_per_exchange"], sweeps_per_check=s["sweeps_per_check"]))
    out = track_accuracy(ws, eng, exact_lng(s["L"]), s["cap_seconds"], t_setup=time.perf_counter() - t0,
                         stop_at=s["tolerance"])
    eng.close()
    out["workload"] = f"ising2d_L{s['L']}_{s['num_windows']}win_x{s['replicas_per_window']}walkers"
    return out


def warm_start_tta(rg, device: int, max_seconds: float, cpu_rate: float | None, data_seconds: float,
                   train_steps: int, replicas: int = 8):
    """Time to accuracy of 2D Ising L=64 (64 windows x `replicas` walkers): MLP warm start at
    ln f0 = 1e-4 against plain WL from ln f0 = 1, both from engine creation, each capped at
    max_seconds.  The network is trained on the ln g that plain GPU runs at L = 16, 24, 32 (one
    batched engine, data_seconds of GPU time) reach; that time and the training time are
    reported separately."""
    from rewl_simulator_gb300 import warmstart as ws
    from rewl_simulator_gb300.mlp import MLP

    t0 = time.perf_counter()
    sizes = ((32, 16, 8), (24, 16, 4), (16, 4, 8))
    inss = [ising_batch(rg, L, nw, R, 1.0, 1e-12, TTA_SEED + k, device).instances[0]
            for k, (L, nw, R) in enumerate(sizes)]
    train_batch = rg.Batch(instances=inss, sweeps_per_exchange=500, sweeps_per_check=1000, flatness_param=0.8,
                           lnf_initial=1.0, lnf_final=1e-12, one_over_t=1, device=device, graphs=1)
    with rg.Engine(train_batch) as eng:
        t_end = time.perf_counter() + data_seconds
        while time.perf_counter() < t_end:
            eng.run_cycles(1)
        base = ws.Baseline.from_engine(eng, 0)
        rows = [ws.training_rows(eng, i, base=base) for i in range(len(sizes))]
        data_err = {}
        for i, (L, _, _) in enumerate(sizes):
            E, g = eng.global_logdos(i)
            data_err[f"L{L}"] = _max_error(E, g, exact_lng(L))
    X = np.concatenate([r[0] for r in rows])
    y = np.concatenate([r[1] for r in rows])
    data_s = time.perf_counter() - t0
    mlp = MLP(hidden=256, layers=4, seed=7, device=device)
    mlp.set_data(X, y)
    t0 = time.perf_counter()
    losses = mlp.train(train_steps, batch=4096, lr=1e-3)
    train_s = time.perf_counter() - t0

    exact = exact_lng(64)
    t0 = time.perf_counter()
    eng = rg.Engine(ising_batch(rg, 64, 64, replicas, 1e-4, 1e-12, TTA_SEED, device))
    ws.warm_start(eng, mlp, 0, lnf0=1e-4, base=base)
    setup = time.perf_counter() - t0
    E, g = eng.global_logdos(0)
    warm0 = _max_error(E, g, exact)
    warm = track_accuracy(ws, eng, exact, max_seconds, burn_in=8, stall_checks=40, t_setup=setup)
    warm["setup_seconds"] = round(setup, 3)
    warm["max_abs_dlng_at_injection"] = warm0
    eng.close()
    mlp.close()
    t0 = time.perf_counter()
    eng = rg.Engine(ising_batch(rg, 64, 64, replicas, 1.0, 1e-12, TTA_SEED, device))
    plain = track_accuracy(ws, eng, exact, max_seconds, t_setup=time.perf_counter() - t0)
    eng.close()
    speedup = {k: round(plain["seconds_to"][k] / v, 2) for k, v in warm["seconds_to"].items()
               if k in plain["seconds_to"] and v > 0}
    out = {"workload": f"ising2d_L64_64win_x{replicas}walkers", "seed": TTA_SEED, "cap_seconds": max_seconds,
           "criterion": "max |ln g - exact| over all levels, windows concatenated and normalised to sum g = 2^N, "
                        "checked every 1000 sweeps",
           "clock": "simulation only: engine creation, warm-start inference and upload, check intervals "
                    "(stopped while the accuracy is evaluated)",
           "schedule": "1/t (the reference's ONE_OVER_T_ALGORITHM default), min >= 0.8 mean, walkers from all +1",
           "warm": warm, "plain": plain, "speedup_warm_over_plain": speedup,
           "mlp": {"training_rows": int(len(y)), "training_data_seconds": round(data_s, 1),
                   "training_data_max_abs_dlng": data_err, "adam_steps": train_steps,
                   "train_seconds": round(train_s, 2), "final_loss": float(np.mean(losses[-50:])),
                   "target": "ln g/N minus the L=32 ln g/N interpolated in E/N",
                   "warm_start": "ln f0 = 1e-4, histograms cleared after each of the first 8 check intervals, "
                                 "plain-WL fallback for windows without a flat event in 40 intervals"}}
    if cpu_rate:
        # not a run: what the CPU port would need for the same number of flips
        out["cpu_port_estimate"] = {
            "basis": "flips the plain GPU arm needed to each tolerance / the CPU port's measured flips/s on this "
                     "workload (an estimate, not a CPU run; the reference arm times a CPU run at L = 16)",
            "seconds_to": {k: round(v / cpu_rate, 1) for k, v in plain["flips_to"].items()}}
    return out


def at_spread(rg, device: int, cycles: int, runs: int):
    """Ashkin-Teller ln g on the GPU against the run-to-run spread of the reference's algorithm on
    the host cores, at the benchmark's size: one realisation of L = 32, K = 0.5, Baxter fields
    sigma 0.5, bins of 0.05, 8 windows x 4 walkers, halving ln f from 1, `cycles` check intervals
    of 200 sweeps.  `runs` reference-semantics runs (the oracle port: mt19937_64 streams,
    draw-on-demand, FP64 logDoS) with different seeds give the spread; `runs` GPU instances with
    other seeds run in one engine.  Windows are compared one by one, each run's window ln g
    (replicas averaged by their visits) on the bins every run visited, shifted to zero mean there
    (early in a run the visited parts of neighbouring windows need not overlap yet, so the windows
    are not concatenated).  Reported: every run's RMS distance from the mean of the reference
    runs, over all compared bins (a reference run held out of that mean)."""
    from oracle import pyoracle as po
    w = dict(WORKLOADS["at"], realizations=1)
    threads = os.cpu_count() or 1
    fields = at_fields(w, 0)
    nw = w["num_windows"]
    cpu = []
    t0 = time.perf_counter()
    for k in range(runs):
        orc = po.Oracle(_port_config(po, w, threads, seed=1 + k), fields=fields)
        for _ in range(cycles):
            orc.cycle()
        cpu.append(([(orc.window_logdos(j), orc.window_mask(j)) for j in range(nw)],
                    [orc.lnf(j * w["replicas_per_window"]) for j in range(nw)]))
        orc.close()
    cpu_s = time.perf_counter() - t0
    inss = [rg.Instance(model=rg.MODEL_ASHKIN_TELLER2D, L=w["L"], K=w["K"], fields=fields, energy_min=w["energy_min"],
                        energy_max=w["energy_max"], bin_width=w["bin_width"], num_windows=nw,
                        replicas_per_window=w["replicas_per_window"], window_overlap=w["window_overlap"],
                        seed=101 + k) for k in range(runs)]
    b = rg.Batch(instances=inss, sweeps_per_exchange=w["sweeps_per_exchange"], sweeps_per_check=w["sweeps_per_check"],
                 flatness_param=0.8, lnf_initial=1.0, lnf_final=w["lnf_final"], mask_mode=rg.MASK_VISITED,
                 device=device)
    t0 = time.perf_counter()
    gpu = []
    with rg.Engine(b) as eng:
        eng.run_cycles(cycles)
        for k in range(runs):
            gpu.append(([(eng.window_logdos(k, j), eng.window_mask(k, j).astype(bool)) for j in range(nw)],
                        [eng.window_state(k, j)[0] for j in range(nw)]))
    gpu_s = time.perf_counter() - t0
    C_parts, G_parts, per_window = [], [], []
    for j in range(nw):
        common = np.logical_and.reduce([t[j][1] for t, _ in cpu + gpu])
        if common.sum() < 2:
            continue
        Cw = np.array([t[j][0][common] - t[j][0][common].mean() for t, _ in cpu])
        Gw = np.array([t[j][0][common] - t[j][0][common].mean() for t, _ in gpu])
        C_parts.append(Cw)
        G_parts.append(Gw)
        per_window.append({"window": j, "bins": int(common.sum()),
                           "reference_rms_spread": float(np.sqrt(np.mean(Cw.var(0, ddof=1)))),
                           "gpu_mean_minus_reference_mean_rms": float(np.sqrt(np.mean((Gw.mean(0) - Cw.mean(0)) ** 2)))})
    C = np.concatenate(C_parts, axis=1)
    G = np.concatenate(G_parts, axis=1)
    mu = C.mean(0)
    d_ref = [float(np.sqrt(np.mean((C[k] - np.delete(C, k, 0).mean(0)) ** 2))) for k in range(runs)]
    d_gpu = [float(np.sqrt(np.mean((G[k] - mu) ** 2))) for k in range(runs)]
    # a GPU run against the mean of runs-1 reference runs, like the held-out reference runs
    d_gpu_loo = [float(np.sqrt(np.mean((G[k] - np.delete(C, k, 0).mean(0)) ** 2))) for k in range(runs)]
    return {"workload": "ashkin_teller2d_L32_K0.5_h0.5_bw0.05_8win_x4walkers (one realisation)",
            "check_intervals": cycles, "sweeps": cycles * w["sweeps_per_check"], "runs_per_side": runs,
            "bins_compared": int(C.shape[1]), "per_window": per_window,
            "rms_from_reference_mean": {"reference_held_out": d_ref, "gpu": d_gpu, "gpu_vs_held_out_mean": d_gpu_loo},
            "rms_gpu_mean_minus_reference_mean": float(np.sqrt(np.mean((G.mean(0) - mu) ** 2))),
            "lnf_by_window": {"reference": [l for _, l in cpu], "gpu": [l for _, l in gpu]},
            "seconds": {"reference_runs": round(cpu_s, 1), "gpu_engine": round(gpu_s, 1)}, "threads": threads}


AT_WARM_TOLERANCES = [100.0, 50.0, 20.0, 10.0, 5.0, 2.0, 1.0, 0.5, 0.3, 0.2, 0.1, 0.05]


def warm_start_at(rg, device: int, cap: float, ref_seconds: float, data_seconds: float, train_steps: int,
                  realizations: int = 32):
    """The Ashkin-Teller arm of the warm-start measurement: L = 48, K = 0.5, Baxter fields sigma 0.5,
    `realizations` realisations x 8 windows x 4 walkers in one engine, bins of width 1 over the half
    spectrum [-(2J + K) 2N, 0), halving ln f (the Ashkin-Teller benchmark's schedule), walkers from
    random spins.  There is no exact density of states: each window is judged against a long
    plain-WL run of the same realisation (ref_seconds, other seeds), and only windows whose judge
    reached ln f <= 1e-3 are judged (a window still at ln f = 1 grows its logDoS by a nat per visit
    and judges nothing).  Error of a window: the largest |d - mean(d)|, d = its replica-averaged
    ln g - the judge's, over the bins both visited (ln g is defined up to a constant); a snapshot's
    error is the median over the judged windows.  The network is trained on plain runs at L = 8,
    12, 16 (4 realisations each, data_seconds of GPU time).  Arms: plain WL from ln f0 = 1, and warm
    starts at ln f0 = 1e-4 and 1e-2 (8 burn-in intervals, 40-interval stall fallback), each capped at
    `cap` seconds of simulation (clock stopped while the error is measured)."""
    from rewl_simulator_gb300 import warmstart as ws
    from rewl_simulator_gb300.mlp import MLP
    K, sh, bw, nw = 0.5, 0.5, 1.0, 8

    def fields(L, k):
        return np.round(np.random.default_rng(7000 + 100 * L + k).normal(0.0, sh, L * L) * 2**20) / 2**20

    def batch(L, nreal, R, lnf0, seed0):
        N = L * L
        inss = [rg.Instance(model=rg.MODEL_ASHKIN_TELLER2D, L=L, K=K, fields=fields(L, k),
                            energy_min=-(2.0 + K) * 2 * N, energy_max=0.0, bin_width=bw, num_windows=nw if L >= 32 else 4,
                            replicas_per_window=R, window_overlap=0.75, seed=seed0 + k) for k in range(nreal)]
        return rg.Batch(instances=inss, sweeps_per_exchange=100, sweeps_per_check=200, flatness_param=0.8,
                        lnf_initial=lnf0, lnf_final=1e-7, mask_mode=rg.MASK_VISITED, device=device, graphs=1)

    def windows(eng, keys):
        return {(i, w): (eng.window_logdos(i, w), eng.window_mask(i, w).astype(bool)) for i, w in keys}

    def shape_error(g, m, jg, jm):
        both = m & jm
        if both.sum() < 2:
            return float("inf")
        d = g[both] - jg[both]
        return float(np.max(np.abs(d - d.mean())))

    n = realizations
    every = [(i, w) for i in range(n) for w in range(nw)]
    t0 = time.perf_counter()
    with rg.Engine(batch(48, n, 4, 1.0, 90000)) as eng:
        t_end = time.perf_counter() + ref_seconds
        while time.perf_counter() < t_end:
            eng.run_cycles(10)
        judged = [(i, w) for i, w in every if eng.window_state(i, w)[0] <= 1e-3]
        judge = windows(eng, judged)
        wins48 = [list(eng.windows[i]) for i in range(n)]
    ref_s = time.perf_counter() - t0
    by_window = [sum(1 for i, w in judged if w == k) for k in range(nw)]
    t0 = time.perf_counter()
    sizes = (16, 12, 8)
    inss = []
    for L in sizes:
        inss += batch(L, 4, 4, 1.0, 500 + L).instances
    tb = rg.Batch(instances=inss, sweeps_per_exchange=100, sweeps_per_check=200, flatness_param=0.8, lnf_initial=1.0,
                  lnf_final=1e-7, mask_mode=rg.MASK_VISITED, device=device, graphs=1)
    with rg.Engine(tb) as eng:
        t_end = time.perf_counter() + data_seconds
        while time.perf_counter() < t_end:
            eng.run_cycles(5)
        base = ws.Baseline.from_engine(eng, 0)
        rows = [ws.training_rows(eng, i, sigma_h=sh, base=base) for i in range(len(inss))]
    X = np.concatenate([r[0] for r in rows])
    y = np.concatenate([r[1] for r in rows])
    data_s = time.perf_counter() - t0
    mlp = MLP(hidden=256, layers=4, seed=9, device=device)
    mlp.set_data(X, y)
    t0 = time.perf_counter()
    losses = mlp.train(train_steps, batch=4096, lr=1e-3)
    train_s = time.perf_counter() - t0
    # the prediction's own error in the judged windows (all of a window's bins predicted)
    pred_err = []
    for i, w in judged:
        lo, hi, nb = wins48[i][w]
        p = ws.predict_lng(mlp, lo + bw * np.arange(nb), 48, 1.0, K, sh, lo, hi, base=base)
        jg, jm = judge[(i, w)]
        pred_err.append(shape_error(p, np.ones(nb, bool), jg, jm))

    def arm(lnf0):
        warm = lnf0 < 1.0
        t0 = time.perf_counter()
        eng = rg.Engine(batch(48, n, 4, lnf0, 1000))
        if warm:
            for i in range(n):
                ws.warm_start(eng, mlp, i, sigma_h=sh, lnf0=lnf0, base=base)
        hit, t_sim, t_mark, best, count = {}, [time.perf_counter() - t0], [time.perf_counter()], [float("inf")], [0]

        def on_cycle(e, st):
            count[0] += 1
            if count[0] % 5:
                return False
            t_sim[0] += time.perf_counter() - t_mark[0]
            cur = windows(e, judged)
            med = float(np.median([shape_error(*cur[k], *judge[k]) for k in judged]))
            best[0] = min(best[0], med)
            for tol in AT_WARM_TOLERANCES:
                if med <= tol and str(tol) not in hit:
                    hit[str(tol)] = round(t_sim[0], 2)
            t_mark[0] = time.perf_counter()
            return t_sim[0] > cap

        try:
            st, fb = ws.run(eng, 1 << 30, stall_checks=40 if warm else 0, burn_in=8 if warm else 0, on_cycle=on_cycle)
            stopped = None
        except Exception as exc:
            st, fb, stopped = None, None, str(exc)
        eng.close()
        out = {"lnf0": lnf0, "seconds_to": hit, "best_median": best[0], "seconds": round(t_sim[0], 2), "fallbacks": fb}
        if stopped:
            out["stopped"] = stopped
        return out

    arms = [arm(1e-4), arm(1e-2)] if judged else []
    mlp.close()
    plain = arm(1.0) if judged else {}
    speed = {str(w["lnf0"]): {k: round(plain["seconds_to"][k] / v, 2) for k, v in w["seconds_to"].items()
                              if k in plain["seconds_to"] and v > 0} for w in arms}
    return {"workload": f"ashkin_teller2d_L48_K0.5_h0.5_bw1_{n}real_8win_x4walkers", "cap_seconds": cap,
            "criterion": "median over the judged windows of max |d - mean d|, d = window ln g - judge's over the bins "
                         "both visited; judge = a long plain run of each realisation; judged = windows whose judge "
                         "reached ln f <= 1e-3",
            "judge": {"seconds": round(ref_s, 1), "windows_judged": len(judged), "windows_total": len(every),
                      "judged_by_window_index": by_window},
            "prediction_error_in_judged_windows": {"median": float(np.median(pred_err)) if pred_err else None,
                                                   "max": float(np.max(pred_err)) if pred_err else None},
            "warm": arms, "plain": plain, "speedup_warm_over_plain": speed,
            "mlp": {"training_rows": int(len(y)), "training_data_seconds": round(data_s, 1), "adam_steps": train_steps,
                    "train_seconds": round(train_s, 2), "final_loss": float(np.mean(losses[-50:])),
                    "training_sizes": list(sizes), "target": "ln g/N minus the first L=16 realisation's ln g/N"}}


def time_steps(eng, stream, flush, steps):
    import torch
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for k in range(steps):
        flush.zero_()
        evs[k][0].record(stream)
        eng.run_cycles(1)
        evs[k][1].record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in evs]


def run_gpu(args):
    import torch
    import rewl_simulator_gb300 as rg

    rank, world, local = dist_env()
    device = local
    torch.cuda.set_device(device)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", device))
    rg.build()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    batch = make_batch(rg, seed=rank_seed(rank), device=device)
    eng = rg.Engine(batch)
    stream = torch.cuda.ExternalStream(eng.stream_handle(), device=torch.device("cuda", device))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{device}")
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            eng.run_cycles(1)
        eng.sweep_kernel_time()
        st0 = eng.status()
        barrier()
        torch.cuda.synchronize()
        sampler = ClockSampler(device)
        with sampler:
            step_ms = time_steps(eng, stream, flush, args.steps)
        barrier()
        st1 = eng.status()
        kern_ms, kern_launches = eng.sweep_kernel_time()
        shapes = np.asarray(eng.launch_shapes()).tolist()
        groups = 1 if WORKLOAD.get("persistent") else max(1, len(shapes))    # launches per sweep phase
    total_ms = sum(step_ms)
    flips = st1.attempted_flips - st0.attempted_flips
    launches = st1.kernel_launches - st0.kernel_launches

    # end to end through the public API with host-resident walker state (pinned)
    nbytes = eng.snapshot_size()
    host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    eng.snapshot_into(host.data_ptr(), nbytes)
    e2e_steps = max(3, args.steps // 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        eng.restore_from(host.data_ptr(), nbytes)
        eng.run_cycles(1)
        eng.snapshot_into(host.data_ptr(), nbytes)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    flips_per_step = WORKLOAD["sweeps_per_check"] * flips_per_sweep(WORKLOAD)
    e2e_rate = e2e_steps * flips_per_step / e2e_s
    eng.close()

    if world > 1:
        (total_ms, e2e_s), (flips, e2e_flips) = reduce_over_ranks([total_ms, e2e_s], [flips, e2e_steps * flips_per_step],
                                                                  device=f"cuda:{device}")
        e2e_rate = e2e_flips / e2e_s
    value = flips / (total_ms * 1e-3)
    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return 0

    hbm_peak, sm_max_mhz, peak_kind = peaks()
    clocks = sampler.summary()
    # one sweep phase = one launch per launch group, concurrent; its span is what the events time
    avg_launch_ms = kern_ms / max(kern_launches / groups, 1)
    flips_per_launch = WORKLOAD["sweeps_per_exchange"] * flips_per_sweep(WORKLOAD)
    achieved_gbs = bytes_per_flip(WORKLOAD) * flips_per_launch / (avg_launch_ms * 1e-3) / 1e9
    prof = profile_figures()
    sm_mhz = clocks.get("sm_mhz") or sm_max_mhz
    roofline = {"bound": WORKLOAD["bound"], "kernel": WORKLOAD["kernel"], "avg_launch_ms": avg_launch_ms,
                "flips_per_launch": flips_per_launch, "launch_shapes": shapes}
    if WORKLOAD["model"] != "mixed":
        # the serial accept chain of one walker: cycles per attempted flip against the design's floor
        walker_flips = WORKLOAD["sweeps_per_exchange"] * ndof(WORKLOAD)
        cycles = avg_launch_ms * 1e-3 * sm_mhz * 1e6 / walker_flips
        kind = "chain floor: dependent shared load (29) + 64-bit compare/select (11), measured on a GB300"
        if WORKLOAD["model"] != "ising2d":
            kind += "; this kernel's dependent loads come from L1/L2 (tables of tens of thousands of bins)"
        roofline.update({"unit": "cycles/flip", "achieved": cycles, "peak": CHAIN_FLOOR_CYCLES,
                         "frac": CHAIN_FLOOR_CYCLES / cycles, "walkers_per_warp": int(shapes[0][2]) if shapes else 1,
                         "peak_kind": kind,
                         "note": "per walker: launch time x median SM clock / flips of one walker; frac = floor / "
                                 "achieved"})
    else:
        roofline.update({"unit": "GB/s", "achieved": achieved_gbs, "peak": hbm_peak, "frac": achieved_gbs / hbm_peak,
                         "peak_kind": peak_kind + " HBM copy bandwidth"})
    roofline["hbm"] = {"algorithmic_gbs": achieved_gbs, "peak_gbs": hbm_peak, "frac": achieved_gbs / hbm_peak,
                       "bytes_per_flip": bytes_per_flip(WORKLOAD),
                       "traffic_bytes_per_launch": prof.get("traffic_bytes_per_launch")}
    roofline["traffic"] = prof.get("traffic_bytes_per_launch")
    if prof:
        roofline["ncu"] = prof
    line = {
        "metric": METRIC, "value": value, "unit": "flips/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int64", "data": "synthetic",
        "config": {"workload": WORKLOAD["name"], **{k: v for k, v in WORKLOAD.items() if k != "name"},
                   "step": step_text(),
                   "l2": "flushed between timed steps (256 MiB write)", "parallelism": f"instances x{world}"},
        "roofline": roofline,
        "e2e": {"value": e2e_rate, "unit": "flips/s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": e2e_steps},
        "clocks": clocks,
        "gpu_launches": int(launches),
    }
    if world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, n, total, _ = cpu_port_rate(args.cpu_seconds, threads)
        line["cpu_baseline"] = {"value": rate, "unit": "flips/s", "cores": threads, "kind": "port",
                                "sample": _sample_text(n, total)}
        if WORKLOAD["model"] != "mixed" and not args.observables:
            # the reference's default build keeps per-bin observables and the G(q_min) correlators
            obs_rate, on, ot, _ = cpu_port_rate(args.cpu_seconds / 2, threads, observables=2)
            oeng = rg.Engine(make_batch(rg, seed=rank_seed(rank), device=device, observables=2))
            ostream = torch.cuda.ExternalStream(oeng.stream_handle(), device=torch.device("cuda", device))
            with torch.cuda.stream(ostream):
                for _ in range(3):
                    oeng.run_cycles(1)
                ost0 = oeng.status()
                oms = time_steps(oeng, ostream, flush, max(3, args.steps // 4))
                ost1 = oeng.status()
            oeng.close()
            gpu_obs = (ost1.attempted_flips - ost0.attempted_flips) / (sum(oms) * 1e-3)
            line["observables_on"] = {
                "observables": "per-bin moments and G(q_min) correlators (the reference's default build)",
                "value": gpu_obs, "unit": "flips/s", "steps": len(oms),
                "cpu_baseline": {"value": obs_rate, "unit": "flips/s", "cores": threads, "kind": "port",
                                 "sample": _sample_text(on, ot)},
                "gpu_over_cpu": gpu_obs / obs_rate, "gpu_over_cpu_observables_off": value / rate}
    if world == 1 and not args.no_tta and WORKLOAD["model"] == "ising2d" and WORKLOAD["L"] == 64:
        line["time_to_accuracy"] = warm_start_tta(rg, device, args.tta_seconds,
                                                  line.get("cpu_baseline", {}).get("value"), args.tta_data_seconds,
                                                  args.tta_train_steps, args.tta_replicas)
        line["time_to_accuracy"]["small"] = gpu_small_tta(rg, device)
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--no-tta", action="store_true", help="skip the time-to-accuracy runs")
    ap.add_argument("--tta-seconds", type=float, default=60.0, help="cap of each L=64 time-to-accuracy arm")
    ap.add_argument("--tta-replicas", type=int, default=8, help="walkers per window of the L=64 time-to-accuracy arms")
    ap.add_argument("--tta-data-seconds", type=float, default=30.0,
                    help="GPU time of the plain L <= 32 runs that make the network's training data")
    ap.add_argument("--tta-train-steps", type=int, default=20000, help="Adam steps of the warm-start network")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU-baseline sample length")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--observables", type=int, choices=[0, 1, 2], default=0,
                    help="1: keep the per-bin observables during the sweeps; 2: also the G(q_min) correlators "
                         "(the reference's default build)")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="c5",
                    help="c5: Ising L=64, 64 windows x 8 walkers (default, the headline configuration); c2: Ising "
                         "L=32, 16 x 8; at: Ashkin-Teller L=32, 64 realisations; mixed: the uneven batch")
    ap.add_argument("--persistent", action="store_true",
                    help="every launch group in one persistent work-stealing launch per sweep phase")
    ap.add_argument("--replicas", type=int, default=0,
                    help="walkers per window (default: the workload's; Ising workloads only)")
    ap.add_argument("--at-spread", type=int, default=0, metavar="CYCLES",
                    help="only measure Ashkin-Teller L=32 ln g on the GPU against the spread of reference runs on "
                         "the host cores after CYCLES check intervals")
    ap.add_argument("--at-spread-runs", type=int, default=4)
    ap.add_argument("--at-warm", type=float, default=0.0, metavar="CAP",
                    help="only measure the Ashkin-Teller L=48 warm-start arm (each arm capped at CAP seconds)")
    ap.add_argument("--tta-seed", type=int, default=5, help="instance seed of the --tta-pair runs")
    ap.add_argument("--tta-pair", default="", metavar="L,WINDOWS,WALKERS[,CAP[,gpu]]",
                    help="only measure Ising time to max |d ln g| <= 1e-2 in this layout on the GPU and on all host "
                         "cores (reference semantics), each capped at CAP seconds (default 150); 'gpu': the GPU only")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.tta_pair:
        import rewl_simulator_gb300 as rg
        rg.build()
        fields = args.tta_pair.split(",")
        gpu_only = fields[-1] == "gpu"
        v = [float(x) for x in (fields[:-1] if gpu_only else fields)]
        SMALL_TTA.update(L=int(v[0]), num_windows=int(v[1]), replicas_per_window=int(v[2]),
                         cap_seconds=v[3] if len(v) > 3 else 150.0, seed=args.tta_seed)
        gpu = gpu_small_tta(rg, 0)
        cpu = None if gpu_only else cpu_small_tta(os.cpu_count() or 1)
        print(json.dumps({"tta_pair": {"gpu": gpu, "cpu": cpu,
                                       "cpu_over_gpu": cpu["seconds"] / gpu["seconds"]
                                       if cpu and "0.01" in gpu["seconds_to"] and "0.01" in cpu["seconds_to"] else None}}),
              flush=True)
        return 0
    if args.at_warm:
        import rewl_simulator_gb300 as rg
        rg.build()
        print(json.dumps({"at_warm_start": warm_start_at(rg, 0, args.at_warm, 2.0 * args.at_warm, 40.0,
                                                         args.tta_train_steps)}), flush=True)
        return 0
    if args.at_spread:
        import rewl_simulator_gb300 as rg
        rg.build()
        print(json.dumps({"at_spread": at_spread(rg, 0, args.at_spread, args.at_spread_runs)}), flush=True)
        return 0
    select_workload(args.workload)
    if args.observables:
        WORKLOADS[args.workload]["observables"] = args.observables
        select_workload(args.workload)
    if args.persistent:
        WORKLOADS[args.workload]["persistent"] = 1
        WORKLOADS[args.workload]["name"] += "_persistent"
    if args.replicas:
        if WORKLOAD["model"] != "ising2d":
            ap.error("--replicas applies to the Ising workloads")
        w = WORKLOADS[args.workload]
        w["replicas_per_window"] = args.replicas
        w["name"] = w["name"].replace("x8walkers", f"x{args.replicas}walkers")
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())

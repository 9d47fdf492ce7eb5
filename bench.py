#!/usr/bin/env python3
"""Benchmark of the REWL hot path on GB300.

Workload (the batched configuration the headline metric is quoted on): 2D Ising,
L = 32 periodic, J = 1, energy levels -2048..2048 step 4 (bins of width 4 over
[-2048, 2052)), 16 equal windows at 75 % overlap x 8 walkers = 128 walkers in one
launch, int8 spins, replica exchange every 500 sweeps, flatness (min >= 0.8 mean)
checked every 1000 sweeps, ln f halved from 1 towards 1e-8, int64 logDoS in 2^-40
units.  Inputs are synthetic (spins drawn from the seed).

A step is one check interval: 2 x (500 sweeps of all 128 walkers + one replica
exchange round) + the flatness / averaging / ln f kernel, i.e. 131,072,000
attempted single-spin flips.  `value` is attempted flips per second over the
whole job (device time, CUDA events on the engine's stream, L2 flushed between
steps by a 256 MiB write).  `e2e` runs the same steps through the public API with
the walker state host-resident in pinned memory: restore (H2D) + step +
snapshot (D2H) per step, wall clock.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl {gb300,reference}] [--tta]

--impl reference times the CPU restatement of the reference's hot path (the
oracle port, reference semantics: mt19937_64 streams, draw-on-demand, FP64
logDoS) on all host cores for the same workload; under torchrun only rank 0 runs.
--tta additionally measures, for 2D Ising L=64 (64 windows x 8 walkers), the wall
time until the concatenated, normalised ln g is within each of a ladder of
tolerances (1 .. 1e-2) of the exact density of states, for the MLP warm start
(trained here on plain GPU runs at L <= 32) and for plain WL from ln f0 = 1, both
with the reference's default build: the 1/t schedule (ONE_OVER_T_ALGORITHM) and
every walker started from all spins +1.
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
WORKLOADS = {
    # the headline configuration (default)
    "ising": dict(name="ising2d_L32_16win_x8walkers_rewl", model="ising2d", L=32, energy_min=-2048.0,
                  energy_max=2052.0, bin_width=4.0, num_windows=16, replicas_per_window=8, window_overlap=0.75,
                  sweeps_per_exchange=500, sweeps_per_check=1000, lnf_initial=1.0, lnf_final=1e-8,
                  flatness="min >= 0.8 mean over valid bins", realizations=1,
                  bytes_per_flip=46, kernel="k_sweep_ising_bins", profile="sweep_ising_L32_rewl.md"),
    # 2D Ashkin-Teller, K = 0.5, Gaussian Baxter fields (sigma 0.5), 64 realisations x 8 windows x 4 walkers
    "at": dict(name="ashkin_teller2d_L32_K0.5_h0.5_64real_8win_x4walkers_rewl", model="ashkin_teller2d", L=32, K=0.5,
               sigma_h=0.5, energy_min=-5120.0, energy_max=0.0, bin_width=0.05, num_windows=8, replicas_per_window=4,
               window_overlap=0.75, sweeps_per_exchange=100, sweeps_per_check=200, lnf_initial=1.0, lnf_final=1e-7,
               flatness="min >= 0.8 mean over visited bins", realizations=64,
               bytes_per_flip=51, kernel="k_sweep_tables<AshkinTeller2dModel>", profile="sweep_at_L32_64real_rewl.md"),
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
    lnf_final=1e-8, flatness="min >= 0.8 mean over visited bins", realizations=1,
    kernel="k_sweep_tables<AshkinTeller2dModel> + k_sweep_ising_bins (launch groups on concurrent streams)", profile="",
    graphs=1, autotune=1)
for _c in WORKLOADS["mixed"]["components"]:
    _c["bytes_per_flip"] = 46 if _c["model"] == "ising2d" else 51
WORKLOAD = WORKLOADS["ising"]


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
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_launch():
    """dram bytes per sweep-kernel launch from the committed ncu summary, if any."""
    if not WORKLOAD["profile"]:
        return None
    p = ROOT / "profiles" / WORKLOAD["profile"]
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


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
    """Seed of the k-th instance of a batch: a multiple of 2^20, so that no two walkers of the
    batch (fewer than 2^20 per instance) share a Philox key (walker keys are seed XOR walker)."""
    return (seed * 100000 + k) << 20


def make_batch(rg, seed: int, device: int):
    w = WORKLOAD
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
                        graphs=w["graphs"], autotune=w["autotune"])
    if w["model"] == "ising2d":
        inss = [rg.Instance(model=rg.MODEL_ISING2D, L=w["L"], energy_min=w["energy_min"], energy_max=w["energy_max"],
                            bin_width=w["bin_width"], num_windows=w["num_windows"],
                            replicas_per_window=w["replicas_per_window"], window_overlap=w["window_overlap"],
                            seed=seed)]
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
                    lnf_final=w["lnf_final"], device=device, mask_mode=mask, observables=w.get("observables", 0))


# --------------------------------------------------------------------------- CPU leg
def cpu_port_rate(target_seconds: float, threads: int, steps: int | None = None, warmup: int = 0):
    """Flips/s of the oracle port (reference semantics) on `threads` host threads (one instance:
    the port drives one instance at a time, so for a batch of realisations it times one of them).
    For the uneven batch, one instance of every component is timed and the rate is the batch's
    flips over the time the CPU needs for all of them."""
    if WORKLOAD["model"] == "mixed":
        return _cpu_port_rate_mixed(target_seconds, threads, steps, warmup)
    return _cpu_port_rate_one(WORKLOAD, target_seconds, threads, steps, warmup)


def _cpu_port_rate_mixed(target_seconds, threads, steps, warmup):
    comps = WORKLOAD["components"]
    cpu_s, n_total, t_total, times = 0.0, 0, 0.0, []
    for c in comps:
        w = dict(c, sweeps_per_exchange=WORKLOAD["sweeps_per_exchange"], sweeps_per_check=WORKLOAD["sweeps_per_check"],
                 lnf_initial=WORKLOAD["lnf_initial"], lnf_final=WORKLOAD["lnf_final"])
        rate, n, total, ts = _cpu_port_rate_one(w, target_seconds / len(comps), threads,
                                                None if steps is None else max(1, steps // len(comps)), 0)
        cpu_s += flips_per_sweep(c) * WORKLOAD["sweeps_per_check"] / rate     # one check interval of component c
        n_total += n
        t_total += total
        times += ts
    return flips_per_sweep(WORKLOAD) * WORKLOAD["sweeps_per_check"] / cpu_s, n_total, t_total, times


def _cpu_port_rate_one(w, target_seconds, threads, steps, warmup):
    from oracle import pyoracle as po
    at = w["model"] != "ising2d"
    cfg = po.Config(model=po.MODEL_AT if at else po.MODEL_ISING, L=w["L"], K=w.get("K", 0.0),
                    escale_bits=20 if at else 0, nwin=w["num_windows"], R=w["replicas_per_window"],
                    sweeps_per_exchange=w["sweeps_per_exchange"], sweeps_per_check=w["sweeps_per_check"],
                    emin=w["energy_min"], emax=w["energy_max"], bw=w["bin_width"], overlap=w["window_overlap"],
                    lnf0=w["lnf_initial"], lnf_final=w["lnf_final"], semantics=po.SEM_REFERENCE, nthreads=threads,
                    mask_mode=po.MASK_VISITED if at else po.MASK_STATIC, seed=2024)
    orc = po.Oracle(cfg, fields=at_fields(w, 0) if at else None)
    w = dict(w, realizations=1)
    fps = w["num_windows"] * w["replicas_per_window"] * ndof(w)
    for _ in range(warmup):
        orc.run_sweeps(w["sweeps_per_exchange"])
    times = []
    done_steps = 0
    t_start = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        orc.cycle()
        times.append(time.perf_counter() - t0)
        done_steps += 1
        if steps is not None:
            if done_steps >= steps:
                break
        elif time.perf_counter() - t_start >= target_seconds:
            break
    orc.close()
    total = sum(times)
    rate = done_steps * w["sweeps_per_check"] * fps / total
    return rate, done_steps, total, times


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
        "config": {"workload": WORKLOAD["name"], **{k: v for k, v in WORKLOAD.items() if k != "name"},
                   "step": step_text()},
        "cpu_baseline": {"value": rate, "unit": "flips/s", "cores": threads, "kind": "port",
                         "sample": (f"{n} check intervals of one instance of each of the {len(w['components'])} components"
                                    if w["model"] == "mixed" else
                                    f"{n} check intervals of one instance of the workload "
                                    f"({w['num_windows'] * w['replicas_per_window']} walkers, {w['sweeps_per_check']} sweeps each)")},
        "e2e": {"value": rate, "unit": "flips/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------- GPU leg
TTA_TOLERANCES = [1.0, 0.5, 0.3, 0.2, 0.15, 0.1, 0.08, 0.05, 0.03, 0.02, 0.01]
TTA_SEEDS = (3, 5)


def ising_batch(rg, L: int, nwin: int, R: int, lnf0: float, lnf_final: float, seed: int, device: int,
                one_over_t: int = 0):
    """Ising on the full spectrum; walkers start from all spins +1 and walk up into their windows,
    as the reference's do (a quench from random spins into the lowest windows can end in a
    stripe state that never reaches the window's lowest levels)."""
    N = L * L
    ins = rg.Instance(model=rg.MODEL_ISING2D, L=L, energy_min=-2.0 * N, energy_max=2.0 * N + 4, bin_width=4.0,
                      num_windows=nwin, replicas_per_window=R, window_overlap=0.75, seed=seed, init_mode=1)
    return rg.Batch(instances=[ins], sweeps_per_exchange=500, sweeps_per_check=1000, flatness_param=0.8,
                    lnf_initial=lnf0, lnf_final=lnf_final, one_over_t=one_over_t, device=device)


def exact_lng(L: int):
    z = np.load(ROOT / "tests" / "golden" / f"exact_ising_L{L}.npz")
    return dict(zip(z["E"].astype(np.int64).tolist(), z["lng"]))


def max_error(eng, exact) -> float:
    E, g = eng.global_logdos(0)
    return float(np.max(np.abs([g[i] - exact[int(round(E[i]))] for i in range(len(E))])))


def track_accuracy(ws, eng, exact, t_start: float, max_seconds: float, burn_in: int = 0, stall_checks: int = 0):
    """Run check intervals, recording the first wall time (from t_start) at or below each tolerance."""
    hit, flips_at, best = {}, {}, [float("inf")]

    def on_cycle(e, st):
        el = time.perf_counter() - t_start
        err = max_error(e, exact)
        best[0] = min(best[0], err)
        for tol in TTA_TOLERANCES:
            if err <= tol and tol not in hit:
                hit[tol] = round(el, 2)
                flips_at[tol] = st.attempted_flips
        return el > max_seconds or TTA_TOLERANCES[-1] in hit

    stopped = None
    try:
        st, fallbacks = ws.run(eng, 1 << 30, stall_checks=stall_checks, on_cycle=on_cycle, burn_in=burn_in)
        flips = st.attempted_flips
    except Exception as exc:                # e.g. a window that never went flat (REWL_ESTATE)
        stopped, fallbacks, flips = str(exc), None, None
    out = {"seconds_to": {str(k): v for k, v in sorted(hit.items(), reverse=True)},
           "flips_to": {str(k): v for k, v in sorted(flips_at.items(), reverse=True)}, "best_max_abs_dlng": best[0],
           "flips": flips, "seconds": round(time.perf_counter() - t_start, 2), "fallbacks": fallbacks}
    if stopped:
        out["stopped"] = stopped
    return out


def warm_start_tta(rg, device: int, max_seconds: float, cpu_rate: float | None):
    """Time to accuracy of 2D Ising L=64 (64 windows x 8 walkers): MLP warm start at ln f0 = 1e-4
    against plain WL from ln f0 = 1, both timed from engine creation, for each seed in TTA_SEEDS.
    The network is trained on the ln g that plain GPU runs at L = 16, 24, 32 converge to (that
    time is reported separately)."""
    from rewl_simulator_gb300 import warmstart as ws
    from rewl_simulator_gb300.mlp import MLP

    t0 = time.perf_counter()
    engines = [rg.Engine(ising_batch(rg, L, nw, R, 1.0, fin, 3, device))
               for L, nw, R, fin in ((32, 16, 8, 1e-8), (24, 16, 4, 1e-8), (16, 4, 8, 1e-6))]
    for e in engines:
        e.simulate(max_cycles=4000)
    base = ws.Baseline.from_engine(engines[0], 0)
    rows = [ws.training_rows(e, 0, base=base) for e in engines]
    for e in engines:
        e.close()
    X = np.concatenate([r[0] for r in rows])
    y = np.concatenate([r[1] for r in rows])
    data_s = time.perf_counter() - t0
    steps = 20000
    mlp = MLP(hidden=256, layers=4, seed=7, device=device)
    mlp.set_data(X, y)
    t0 = time.perf_counter()
    losses = mlp.train(steps, batch=4096, lr=1e-3)
    train_s = time.perf_counter() - t0

    exact = exact_lng(64)
    arms, infer_s = {}, None
    for seed in TTA_SEEDS:
        t0 = time.perf_counter()
        eng = rg.Engine(ising_batch(rg, 64, 64, 8, 1e-4, 1e-12, seed, device, one_over_t=1))
        t1 = time.perf_counter()
        ws.warm_start(eng, mlp, 0, lnf0=1e-4, base=base)
        infer_s = time.perf_counter() - t1
        warm = track_accuracy(ws, eng, exact, t0, max_seconds, burn_in=8, stall_checks=40)
        warm["engine_create_seconds"] = round(t1 - t0, 2)
        eng.close()
        t0 = time.perf_counter()
        eng = rg.Engine(ising_batch(rg, 64, 64, 8, 1.0, 1e-12, seed, device, one_over_t=1))
        plain = track_accuracy(ws, eng, exact, t0, max_seconds)
        eng.close()
        speedup = {k: round(plain["seconds_to"][k] / v, 2) for k, v in warm["seconds_to"].items()
                   if k in plain["seconds_to"]}
        arms[f"seed{seed}"] = {"warm": warm, "plain": plain, "speedup_warm_over_plain": speedup}
    mlp.close()
    out = {"workload": "ising2d_L64_64win_x8walkers", "criterion": "max |ln g - exact| over all levels, "
           "windows concatenated and normalised to sum g = 2^N, checked every 1000 sweeps",
           "schedule": "1/t (the reference's ONE_OVER_T_ALGORITHM default), walkers started from all +1",
           "runs": arms,
           "mlp": {"training_rows": int(len(y)), "training_data_seconds": round(data_s, 1),
                   "adam_steps": steps, "train_seconds": round(train_s, 2), "final_loss": float(np.mean(losses[-50:])),
                   "target": "ln g/N minus the L=32 ln g/N interpolated in E/N",
                   "inference_and_upload_seconds": round(infer_s, 3),
                   "warm_start": "ln f0 = 1e-4, histograms cleared after each of the first 8 check intervals, "
                                 "plain-WL fallback for windows without a flat event in 40 intervals"}}
    if cpu_rate:
        # not a run: what the CPU port would need for the same number of flips
        out["cpu_port_estimate"] = {
            "basis": "flips the plain GPU arm needed to each tolerance / the CPU port's measured flips/s "
                     "(estimate; the CPU run itself was not made)",
            "seconds_to": {name: {k: round(v / cpu_rate, 1) for k, v in run["plain"]["flips_to"].items()}
                           for name, run in arms.items()}}
    return out


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
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        sampler = ClockSampler(device)
        with sampler:
            for k in range(args.steps):
                flush.zero_()
                evs[k][0].record(stream)
                eng.run_cycles(1)
                evs[k][1].record(stream)
            torch.cuda.synchronize()
        barrier()
        step_ms = [a.elapsed_time(b) for a, b in evs]
        st1 = eng.status()
        kern_ms, kern_launches = eng.sweep_kernel_time()
        groups = max(1, len(eng.launch_shapes()))
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

    peak, peak_kind = peaks()
    # one sweep phase = one launch per launch group, concurrent; its span is what the events time
    avg_launch_ms = kern_ms / max(kern_launches / groups, 1)
    flips_per_launch = WORKLOAD["sweeps_per_exchange"] * flips_per_sweep(WORKLOAD)
    achieved = bytes_per_flip(WORKLOAD) * flips_per_launch / (avg_launch_ms * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "flips/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int64", "data": "synthetic",
        "config": {"workload": WORKLOAD["name"], **{k: v for k, v in WORKLOAD.items() if k != "name"},
                   "step": step_text(),
                   "l2": "flushed between timed steps (256 MiB write)", "parallelism": f"instances x{world}"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": traffic_per_launch(),
                     "kernel": WORKLOAD["kernel"], "bytes_per_flip": bytes_per_flip(WORKLOAD),
                     "avg_launch_ms": avg_launch_ms, "flips_per_launch": flips_per_launch},
        "e2e": {"value": e2e_rate, "unit": "flips/s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": e2e_steps},
        "clocks": sampler.summary(),
        "gpu_launches": int(launches),
    }
    if world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, n, total, _ = cpu_port_rate(args.cpu_seconds, threads)
        sample = (f"{n} check intervals of one instance of each of the {len(WORKLOAD['components'])} components "
                  f"({total:.1f} s)" if WORKLOAD["model"] == "mixed"
                  else f"{n} check intervals of the same workload ({total:.1f} s)")
        line["cpu_baseline"] = {"value": rate, "unit": "flips/s", "cores": threads, "kind": "port", "sample": sample}
    if args.tta and world == 1:
        line["time_to_accuracy"] = warm_start_tta(rg, device, args.tta_seconds,
                                                  line.get("cpu_baseline", {}).get("value"))
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
    ap.add_argument("--tta", action="store_true",
                    help="also measure time to accuracy at L=64: MLP warm start against plain WL")
    ap.add_argument("--tta-seconds", type=float, default=90.0, help="wall-time limit of each time-to-accuracy arm")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU-baseline sample length")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--observables", type=int, choices=[0, 1, 2], default=0,
                    help="1: keep the per-bin observables during the sweeps; 2: also the G(q_min) correlators "
                         "(the reference's default build)")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="ising",
                    help="ising: the headline configuration (default); at: 2D Ashkin-Teller, 64 realisations; "
                         "mixed: the uneven batch (Ising L = 16..48 and Ashkin-Teller L = 24, K = 0.25..0.75)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    select_workload(args.workload)
    if args.observables:
        WORKLOADS[args.workload]["observables"] = args.observables
        select_workload(args.workload)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())

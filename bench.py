"""Benchmark: batched-walker bead updates per second on one GB300.

Workload (the batched-walker configuration of the reference benchmark):
1024 independent canonical He-4 chains, Aziz HFD-HE2, density 0.02186 A^-3,
N ~ U{8..128}, T ~ U[1, 4] K, tau = 0.004 1/K, M = even round(1/(T tau)) (the
reference forces M even), Philox streams per walker.  One *step* is one
Monte Carlo sweep of every walker: numUpdates = max(100, ceil(N M / Mbar))
staging / centre-of-mass moves per walker followed by one thermodynamic
energy sample (the reference's PathIntegralMonteCarlo::step with the energy
estimator).  A bead update is one bead proposed and Metropolis-tested.

Reported on one JSON line:
  value     bead-updates/s with the worldlines resident in HBM (CUDA events on
            the library's stream, L2 flushed between timed steps)
  e2e       the same through the C ABI with host buffers: every step uploads the
            whole worldline state from pinned host memory, runs the sweep and
            reads the per-walker estimator accumulators back
  roofline  the walker kernel against the FP32 pipe (pair sums are FP32 FMA +
            SFU work; HBM and tensor cores do not bind)
  cpu_baseline / plain_fp64  the FP64 CPU oracle walkers on the host cores and
            the plain FP64 GPU form (host-driven moves) on a sample walker

`--impl reference` times the reference's CPU path for the same workload (the
oracle restatement: the reference itself cannot be built here).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PAIR_FLOP = 40          # nominal FP32 FLOP per Aziz pair evaluation (plus 3-4 SFU ops)
L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--walkers", type=int, default=1024)
    ap.add_argument("--no-baseline", action="store_true")
    return ap.parse_args()


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    return rank, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self):
        self.f = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9 and parts[0] == os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]:
                rows.append(parts)
            elif len(parts) >= 9 and not rows:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, n in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(rows)}


def workload(num, seed=0):
    from pimc_gb300 import worldlines
    return worldlines.workload_walkers(num=num, seed=seed)


def pair_evals_per_sweep(w):
    """Algorithmic pair evaluations of one sweep of every walker: staging moves
    evaluate old and new positions of (len-1) beads against N-1 partners,
    len ~ 2 + U{0..Mbar-2}; COM moves M (N-1) pairs, twice; the energy sample
    N(N-1)/2 pairs per slice."""
    n, m, mb = w["n"].astype(float), w["m"].astype(float), w["mbar"].astype(float)
    nu = np.maximum(100, np.ceil(n * m / mb))
    mean_moved = mb / 2.0                      # E[len - 1] with len = 2 + U{0..Mbar-2}
    p_com = 0.05
    per_move = (1 - p_com) * 2 * mean_moved * (n - 1) + p_com * 2 * m * (n - 1)
    beads = (1 - p_com) * mean_moved + p_com * m
    return float((nu * per_move + m * n * (n - 1) / 2).sum()), float((nu * beads).sum())


def measured_fp32_peak():
    """cuBLAS SGEMM (CUDA cores, no TF32) on this GPU as the FP32 denominator."""
    import torch
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device="cuda", dtype=torch.float32)
    b = torch.randn(n, n, device="cuda", dtype=torch.float32)
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ b
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    return 2.0 * n ** 3 / best / 1e12


def cpu_baseline(w, threads, budget_s=15.0):
    """Oracle walkers (FP64, MT19937, reference staging with winding sampling)
    on a stratified sample of the workload's walkers, all host threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    order = np.argsort(w["n"].astype(float) ** 2 * w["m"])
    idx = order[np.linspace(0, len(order) - 1, num=min(len(order), max(threads, 16))).astype(int)]
    sel = {k: (v[idx] if isinstance(v, np.ndarray) else v) for k, v in w.items()}
    seeds = np.arange(len(idx), dtype=np.uint32) + 139853
    # one sweep per walker; repeat while within the budget
    total_bu, total_s, reps = 0, 0.0, 0
    while total_s < budget_s and reps < 4:
        sec, en, bu = pyoracle.walkers_cpu(sel["n"], sel["m"], sel["temperature"], sel["side"], seeds,
                                           w["tau"], w["lam"], 1, threads)
        total_bu += int(bu.sum())
        total_s += sec
        reps += 1
    # per-bead-update cost of the sample scaled to the whole workload's mix
    rate = total_bu / total_s
    return dict(value=rate, unit="bead-updates/s", cores=threads, kind="port",
                sample="%d walkers stratified by N^2 M (N %d..%d), %d sweep(s) each from fresh "
                       "seeded worldlines, FP64 oracle with MT19937, %d threads"
                       % (len(idx), int(sel["n"].min()), int(sel["n"].max()), reps, threads))


def plain_form_rate(pgb, n=64, t=2.0, tau=0.004, steps=1):
    """The plain FP64 GPU form: the reference's move loop on the host (MT19937,
    staging + centre of mass) with one FP64 device action call per Metropolis
    decision, on one walker of the workload's mean size."""
    from pimc_gb300 import worldlines as wl
    m = wl.even_slices(t, tau)
    L = wl.box_side(n)
    mbar = wl.default_mbar(n, L ** 3, wl.LAMBDA_HE4, tau, m)
    a = pgb.Action(L, m, n, tau, wl.LAMBDA_HE4, precision=pgb.PGB_FP64)
    a.load(wl.seeded_worldlines(n, m, L, wl.LAMBDA_HE4, tau, 5))
    a.plain_seed(139853)
    a.plain_run(1, mbar=mbar, temperature=1.0 / (m * tau), num_updates=50)   # warm-up
    t0 = time.perf_counter()
    r = a.plain_run(steps, mbar=mbar, temperature=1.0 / (m * tau))
    dt = time.perf_counter() - t0
    return dict(value=r["bead_updates"] / dt, unit="bead-updates/s",
                walker="N=%d M=%d T=%.3f Mbar=%d, %d step(s), energy sampled per step" % (n, m, 1.0 / (m * tau), mbar, steps),
                accepted=r["accepted"], attempted=r["attempted"])


def run_reference(args):
    rank, ws = dist_init()
    if rank != 0:
        return
    w = workload(args.walkers)
    threads = os.cpu_count() or 1
    base = cpu_baseline(w, threads, budget_s=max(5.0, 2.0 * args.steps))
    line = {"metric": "bead-updates/s", "value": base["value"], "unit": "bead-updates/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": "batched walkers: 1024 canonical He-4 chains, "
                                             "N~U{8..128}, T~U[1,4] K, tau=0.004, Aziz, rho=0.02186",
                                             "sample": base["sample"]},
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": "bead-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    rank, ws = dist_init()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    import pimc_gb300 as pgb

    w = workload(args.walkers, seed=rank)
    W = pgb.Walkers(w["n"], w["m"], w["temperature"], w["side"], w["mbar"], w["tau"], w["lam"],
                    seed=1000 + rank)
    W.init()                                   # autotunes threads per walker
    stream = torch.cuda.ExternalStream(W.stream())
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    pair_per_step, bu_nominal = pair_evals_per_sweep(w)

    # warm-up
    W.run(args.warmup, measure=1)
    W.reset_stats()
    # device-resident timed steps
    barrier(ws)
    torch.cuda.synchronize()
    clk = Clocks()
    evs = []
    l0 = W.launch_count()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            W.run(1, measure=1, sync=False)
            e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    barrier(ws)
    clocks = clk.stop()
    launches = W.launch_count() - l0
    step_ms = [a.elapsed_time(b) for a, b in evs]
    t_dev = sum(step_ms) / 1e3
    st = W.stats()
    bu = sum(s["bead_updates"] for s in st)
    t_max = max_over_ranks(t_dev, ws)
    bu_all = sum_over_ranks(float(bu), ws)
    value = bu_all / t_max

    # e2e: host worldline buffer uploaded every step, stats read back every step
    state_bytes = int(W.lib.pgb_walkers_state_bytes(W.h))
    host = torch.empty(state_bytes // 8, dtype=torch.float64, pin_memory=True)
    host_np = host.numpy()
    off = 0
    for i in range(W.W):
        p = W.positions(i).ravel()
        host_np[off:off + len(p)] = p
        off += len(p)
    W.reset_stats()
    stats_bytes = 64 * W.W
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    for k in range(args.steps):
        W._chk(W.lib.pgb_walkers_set_all_positions(W.h, host_np.ctypes.data_as(
            pgb._lib._DP)))
        W.run(1, measure=1, sync=False)
        st = W.stats()                          # synchronous D2H of the accumulators
    t_e2e = time.perf_counter() - t0
    bu_e2e = sum(s["bead_updates"] for s in st)
    t_e2e = max_over_ranks(t_e2e, ws)
    e2e_val = sum_over_ranks(float(bu_e2e), ws) / t_e2e

    # roofline of the walker kernel: pair evaluations x nominal FLOP
    peak_fp32 = measured_fp32_peak()
    pairs = pair_per_step * args.steps
    achieved = pairs * PAIR_FLOP / t_dev / 1e12

    out = {"metric": "bead-updates/s", "value": value, "unit": "bead-updates/s", "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32+f64",
           "data": "synthetic",
           "config": {"workload": "batched walkers: %d canonical He-4 chains, N~U{8..128}, "
                                  "T~U[1,4] K, tau=0.004, M even, Aziz HFDHE2, rho=0.02186, "
                                  "staging (Mbar 32) + COM moves, energy sampled every sweep"
                                  % W.W,
                      "schedule": W.threads(), "autotune_ms": W.tuning(),
                      "l2": "flushed between timed steps",
                      "parallelism": "replicas" if ws > 1 else "single"},
           "e2e": {"value": e2e_val, "unit": "bead-updates/s", "h2d_bytes_per_step": state_bytes,
                   "d2h_bytes_per_step": stats_bytes},
           "gpu_launches": int(launches),
           "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak_fp32,
                        "unit": "TFLOP/s", "frac": achieved / peak_fp32, "traffic": None,
                        "kernel": "k_walkers_run",
                        "note": "pair evaluations x %d FLOP; peak = measured cuBLAS SGEMM "
                                "(no TF32) on this GPU" % PAIR_FLOP},
           "clocks": clocks}
    if rank == 0 and not args.no_baseline:
        out["cpu_baseline"] = cpu_baseline(w, os.cpu_count() or 1)
        out["plain_fp64"] = plain_form_rate(pgb)
        out["plain_fp64"]["batched_over_plain"] = value / out["plain_fp64"]["value"]
    if rank == 0:
        print(json.dumps(out))


if __name__ == "__main__":
    main()

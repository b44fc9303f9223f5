"""Benchmark: batched bosonic walkers, bead updates per second on one GB300.

Workload (the batched-walker configuration of the reference benchmark):
1024 independent He-4 paths, Aziz HFD-HE2, density 0.02186 A^-3,
N ~ U{8..128}, T ~ U[1, 4] K, tau = 0.004 1/K, M = even round(1/(T tau)) (the
reference forces M even), Philox streams per walker, each run by the worm
algorithm with the reference's default PIMC move list (centre of mass,
bisection, open, close, insert, remove, advance/recede head and tail, swap
head and tail; setup.cpp:467-471) and a canonical window of one particle, so
exchange cycles are sampled.  One *step* is one PathIntegralMonteCarlo::step
of every walker: numUpdates = max(100, ceil(N M / Mbar)) moves followed by the
energy sample when the configuration is closed.  A bead update is one bead
proposed and Metropolis-tested.

Reported on one JSON line:
  value     bead-updates/s with the worldlines resident in HBM (CUDA events on
            the walkers' stream, L2 flushed between timed steps)
  e2e       the same through the C ABI with host buffers: every step uploads the
            whole device state image from pinned host memory, runs the step and
            reads the per-walker estimator accumulators back
  roofline  the walker kernel against the FP32 and special-function pipes (pair
            sums are FP32 FMA + SFU work; HBM and tensor cores do not bind)
  cpu_baseline / plain_fp64  the FP64 oracle's worm engine on the same 1024
            walkers on the host cores (set-up untimed), and the plain FP64 GPU
            form (host-driven moves) on one walker
  matched_energy  E/N of the batched walkers beside the FP64 oracle's, with
            error bars

`--workload canonical` runs the canonical staging + centre-of-mass walkers
(no exchange moves) on the same 1024 paths.  `--impl reference` times the
reference's CPU path for the default workload (the oracle restatement: the
reference itself cannot be built on the benchmark host).
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

# Algorithmic cost of one pair evaluation (minimum image, r^2, Aziz V):
# 40 FP32 FLOP and 4 special-function ops; V and gradV together: 52 FLOP and
# 4 special-function ops.  The kernels issue 3 special-function ops for V
# (rsqrt and two ex2), so the SFU fractions below overstate their use by 4/3.
PAIR_FLOP = 40
PAIR_SFU = 4
PAIR_FLOP_VG = 52
SFU_PER_SM_CLK = 16     # nominal special-function results per SM per clock
# DRAM bytes (read + write) per launch from one ncu capture of each kernel on
# the workload its bench leg runs (profiles/ holds the summaries)
NCU_TRAFFIC = {"k_walkers_pipe": 160.4e6, "k_walkers_group": 158.9e6}
# DRAM bytes of one k_worm_walkers step on the 1024-walker workload, L2 flushed
# before it (profiles/k_worm_walkers_walkers1024.md): 344.5 MB read + 47.3 MB
# written, about the walkers' resident state (396 MB) once
NCU_TRAFFIC_WORM = 391.9e6
L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--walkers", type=int, default=1024)
    ap.add_argument("--serve-canonical", action="store_true",
                    help="serve canonical staging + COM chains instead of grand-canonical worm jobs")
    ap.add_argument("--schedule", type=int, default=0,
                    help="walker schedule code (0: autotune)")
    ap.add_argument("--no-baseline", action="store_true")
    ap.add_argument("--workload", default="walkers",
                    choices=["walkers", "canonical", "serving", "isf", "pair", "plain", "gp"])
    ap.add_argument("--diagonal", default="bisection", choices=["bisection", "staging"],
                    help="diagonal move of the worm walkers (the reference's default is bisection)")
    ap.add_argument("--serve-seconds", type=float, default=12.0)
    return ap.parse_args()


def dist_init():
    """One process per GPU over NCCL; without a GPU (the reference arm and
    the host-logic tests) the ranks meet over gloo."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        import torch
        if torch.cuda.is_available():
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
    return rank, ws


def _reduce_device():
    import torch.distributed as dist
    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=_reduce_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=_reduce_device())
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


def err_stats(got, want, floor=1.0):
    """Error of a result against the FP64 oracle: max and median of the
    absolute error and of the relative error |got - want| / max(|want|, floor)."""
    got, want = np.asarray(got, dtype=float).ravel(), np.asarray(want, dtype=float).ravel()
    a = np.abs(got - want)
    r = a / np.maximum(np.abs(want), floor)
    return {"max_abs": float(a.max()), "median_abs": float(np.median(a)), "max_rel": float(r.max()),
            "median_rel": float(np.median(r)), "count": int(a.size), "rel_floor": floor}


def walker_kernel(sched):
    """Kernel that runs a walker schedule code."""
    if sched >= 7000:
        return "k_walkers_group"
    if sched >= 5000:
        return "k_walkers_pipe"
    if sched >= 4000:
        return "k_walkers_tma"
    if sched >= 3000:
        return "k_walkers_windows"
    if sched >= 1000:
        return "k_walkers_team"
    return "k_walkers_run"


def sfu_peak(sm_mhz):
    """Nominal special-function throughput at the sampled SM clock (ops/s)."""
    import pimc_gb300 as pgb
    sms = pgb.device_info()["sm_count"]
    mhz = sm_mhz or 2070.0
    return SFU_PER_SM_CLK * sms * mhz * 1e6


def pair_roofline(pairs, pairs_vg, seconds, kernel, peak_fp32, sm_mhz, traffic=None):
    """FP32 and SFU fractions of a pair-sum kernel; frac is the larger, as the
    binding pipe."""
    flops = (pairs * PAIR_FLOP + pairs_vg * PAIR_FLOP_VG) / seconds / 1e12
    sfu = (pairs + pairs_vg) * PAIR_SFU / seconds
    sfu_pk = sfu_peak(sm_mhz)
    f_fp32, f_sfu = flops / peak_fp32, sfu / sfu_pk
    return {"bound": "fp32" if f_fp32 >= f_sfu else "sfu", "achieved": flops, "peak": peak_fp32,
            "unit": "TFLOP/s", "frac": max(f_fp32, f_sfu), "fp32_frac": f_fp32,
            "sfu": {"achieved_gops": sfu / 1e9, "peak_gops": sfu_pk / 1e9, "frac": f_sfu},
            "traffic": traffic, "kernel": kernel,
            "note": "achieved = pair evaluations x %d FLOP (%d for V+gradV) / kernel time; FP32 "
                    "peak = measured cuBLAS SGEMM (no TF32) on this GPU; SFU peak = nominal %d/clk/SM "
                    "x SMs x median SM clock, %d SFU ops per pair; frac = the larger fraction"
                    % (PAIR_FLOP, PAIR_FLOP_VG, SFU_PER_SM_CLK, PAIR_SFU)}


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


def cpu_baseline(w, threads, nequil=1, nsteps=5, every=4):
    """Oracle walkers (FP64, MT19937, the reference's staging with winding
    sampling and centre-of-mass moves) on a stratified quarter of the
    workload's walkers (every 4th by N^2 M), all host threads: set-up and
    nequil steps untimed, nsteps steps of every sampled walker timed."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    order = np.argsort(w["n"].astype(float) ** 2 * w["m"], kind="stable")
    idx = np.sort(order[::every])
    sel = {k: (v[idx] if isinstance(v, np.ndarray) else v) for k, v in w.items()}
    seeds = np.arange(len(idx), dtype=np.uint32) + 139853
    sec, en, bu, setup = pyoracle.walkers_cpu(sel["n"], sel["m"], sel["temperature"], sel["side"], seeds,
                                              w["tau"], w["lam"], nsteps, threads, nequil=nequil,
                                              with_setup=True)
    return dict(value=float(bu.sum()) / sec, unit="bead-updates/s", cores=threads, kind="port",
                timed="sweeps only",
                sample="%d of the %d walkers (every %d-th by N^2 M), %d timed sweep(s) each after %d "
                       "untimed (set-up %.1f s untimed), FP64 oracle with MT19937, %d threads, %.1f s timed"
                       % (len(idx), len(w["n"]), every, nsteps, nequil, setup, threads, sec))


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


def matched_energy(pgb, threads, n=64, t=2.0, tau=0.004, replicas=256, equil=100, sweeps=200,
                   oracle_replicas=16, oracle_equil=100, oracle_sweeps=100):
    """Energy per particle of the batched mixed-precision walkers beside the
    FP64 oracle's walkers on the same configuration (the plain leg's walker):
    each the mean over independent replicas with its standard error, and
    their difference in combined standard errors.  One long chain of the
    plain FP64 form would need thousands of steps for an honest error bar
    (its 50-step block means scatter by about 1.7 K here), so the FP64 side is
    the oracle's replicas on the host cores, which the plain form matches
    draw for draw."""
    from pimc_gb300 import worldlines as wl
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    m = wl.even_slices(t, tau)
    L = wl.box_side(n)
    mbar = wl.default_mbar(n, L ** 3, wl.LAMBDA_HE4, tau, m)
    T = 1.0 / (m * tau)
    W = pgb.Walkers(np.full(replicas, n), np.full(replicas, m), np.full(replicas, T), np.full(replicas, L),
                    np.full(replicas, mbar), tau, wl.LAMBDA_HE4, seed=4242)
    W.init()
    W.run(equil, measure=0)
    W.reset_stats()
    W.run(sweeps, measure=1)
    st = W.stats_array()
    e_rep = st["energy_sum"] / np.maximum(st["samples"], 1)
    eb, sb = float(e_rep.mean()), float(e_rep.std(ddof=1) / np.sqrt(replicas))
    W.close()
    sec, en, _ = pyoracle.walkers_cpu(np.full(oracle_replicas, n), np.full(oracle_replicas, m),
                                      np.full(oracle_replicas, T), np.full(oracle_replicas, L),
                                      np.arange(oracle_replicas, dtype=np.uint32) + 99, tau, wl.LAMBDA_HE4,
                                      oracle_sweeps, threads, nequil=oracle_equil)
    eo, so = float(en.mean()), float(en.std(ddof=1) / np.sqrt(oracle_replicas))
    return dict(config="N=%d M=%d T=%.3f Mbar=%d" % (n, m, T, mbar),
                batched=[eb, sb], oracle_fp64=[eo, so],
                diff_sigma=abs(eb - eo) / math.hypot(sb, so),
                sample="batched: %d replicas, %d + %d sweeps; FP64 oracle walkers: %d replicas, %d + %d "
                       "sweeps on %d host threads (%.0f s)"
                       % (replicas, equil, sweeps, oracle_replicas, oracle_equil, oracle_sweeps, threads, sec))


# ---------------------------------------------------------------------------
# Serving leg: Poisson job stream (50 jobs/s, seeded), each job N0 log-uniform
# in [8, 512], T uniform in [0.5, 4] K, mu uniform in [-10, 0] K, sweeps
# log-uniform in [1e3, 1e5], admitted under a 150 GB HBM budget.  Offered
# load far exceeds capacity, so the window is bounded and the report states
# how many jobs reached a first bin / completed (the rest are censored).
# ---------------------------------------------------------------------------
def km_quantiles(durations, observed, qs=(50, 99), with_risk=False):
    """Kaplan-Meier estimate of the event-time distribution from right-censored
    durations (observed False: the event had not happened when the window
    closed, the duration is the time the job was watched).  Returns, per
    quantile, the smallest duration t with 1 - S(t) >= q/100, or None when
    the estimate never reaches q (the quantile lies beyond the window).
    With with_risk, also the number of jobs at risk where each quantile was
    reached: a quantile reached with few jobs at risk rests on few jobs."""
    d = np.asarray(durations, dtype=float)
    o = np.asarray(observed, dtype=bool)
    order = np.lexsort((~o, d))                 # events before censorings at equal times
    d, o = d[order], o[order]
    at_risk = len(d)
    surv = 1.0
    out = {q: None for q in qs}
    risk = {q: None for q in qs}
    for t, ev in zip(d, o):
        if ev:
            surv *= 1.0 - 1.0 / at_risk
            for q in qs:
                if out[q] is None and 1.0 - surv >= q / 100.0 - 1e-12:
                    out[q] = float(t)
                    risk[q] = at_risk
        at_risk -= 1
    if with_risk:
        return out, risk
    return out


def serving_run(pgb, seconds=12.0, rate=50.0, seed=0, round_seconds=0.02, grand_canonical=True,
                arrival_seconds=None):
    """Poisson arrivals at `rate` for arrival_seconds (0.6 of the window by
    default), the server stepped until `seconds` have passed.  Time to first
    bin and to completion are reported over every arrived job with the jobs
    still waiting at the window's end treated as right-censored
    (Kaplan-Meier), beside the plain percentiles over the jobs that reached
    the event."""
    rng = np.random.Generator(np.random.Philox(seed))
    arrive_for = 0.6 * seconds if arrival_seconds is None else arrival_seconds
    arrivals = []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > arrive_for:
            break
        arrivals.append(t)
    srv = pgb.Server(150e9, max_active=1024, bin_sweeps=100, round_seconds=round_seconds,
                     grand_canonical=grand_canonical)
    ids = []
    for k, ta in enumerate(arrivals):
        n = int(round(math.exp(rng.uniform(math.log(8), math.log(512)))))
        T = float(rng.uniform(0.5, 4.0))
        mu = float(rng.uniform(-10.0, 0.0))
        sweeps = int(round(math.exp(rng.uniform(math.log(1e3), math.log(1e5)))))
        ids.append(srv.submit(n=n, temperature=T, sweeps=sweeps, seed=seed * 100000 + k,
                              arrival=srv.clock() + ta, mu=mu))
    t0 = time.perf_counter()
    rounds = 0
    nbins = 0
    peak_active = 0
    while time.perf_counter() - t0 < seconds:
        a, q = srv.step()
        rounds += 1
        peak_active = max(peak_active, a)
        nbins += len(srv.bins())
    elapsed = time.perf_counter() - t0
    t_end = srv.clock()
    bu = srv.bead_updates()
    infos = [srv.job(j) for j in ids]
    arrived = [i for i in infos if i["state"] >= 1]
    ttfb = [i["first_bin"] - i["arrival"] for i in arrived if i["first_bin"] >= 0]
    done = [i["completed"] - i["arrival"] for i in arrived if i["completed"] >= 0]
    pct = lambda v, p: float(np.percentile(v, p)) if v else None
    km_first, risk_first = km_quantiles(
        [(i["first_bin"] if i["first_bin"] >= 0 else t_end) - i["arrival"] for i in arrived],
        [i["first_bin"] >= 0 for i in arrived], with_risk=True)
    km_done, risk_done = km_quantiles(
        [(i["completed"] if i["completed"] >= 0 else t_end) - i["arrival"] for i in arrived],
        [i["completed"] >= 0 for i in arrived], with_risk=True)
    srv.close()
    n_arr = max(len(arrived), 1)
    return {"bead_updates_per_s": bu / elapsed, "window_s": round(elapsed, 2),
            "arrival_window_s": round(arrive_for, 2), "rounds": rounds,
            "jobs_arrived": len(arrived), "jobs_admitted": sum(1 for i in arrived if i["admitted"] >= 0),
            "jobs_with_first_bin": len(ttfb), "jobs_completed": len(done),
            "censored_first_bin_frac": 1.0 - len(ttfb) / n_arr,
            "censored_completion_frac": 1.0 - len(done) / n_arr,
            "jobs_failed": sum(1 for i in arrived if i["state"] == 4), "bins": nbins,
            "peak_active": peak_active,
            "ttfb_p50_s": km_first[50], "ttfb_p99_s": km_first[99],
            "completion_p50_s": km_done[50], "completion_p99_s": km_done[99],
            "at_risk": {"ttfb_p50": risk_first[50], "ttfb_p99": risk_first[99],
                        "completion_p50": risk_done[50], "completion_p99": risk_done[99]},
            "uncensored": {"ttfb_p50_s": pct(ttfb, 50), "ttfb_p99_s": pct(ttfb, 99),
                           "completion_p50_s": pct(done, 50), "completion_p99_s": pct(done, 99)},
            "note": "Poisson %g jobs/s for %.1f s of a %.1f s window; p50/p99 are Kaplan-Meier "
                    "estimates over every arrived job, a job still waiting when the window closed "
                    "counted as right-censored at its time in the system (null: the quantile lies "
                    "beyond the window); 'uncensored' gives the percentiles over the jobs that "
                    "reached the event; %s, bins of 100 sweeps, rounds of %g s of device time"
                    % (rate, arrive_for, seconds,
                       "grand-canonical worm walkers at each job's mu (the full move list, bisection)"
                       if grand_canonical else "canonical chains (staging + COM)", round_seconds)}


def run_serving(args, pgb):
    arrive = args.serve_seconds if args.serve_seconds >= 120 else None
    r = serving_run(pgb, seconds=args.serve_seconds, grand_canonical=not args.serve_canonical,
                    arrival_seconds=arrive)
    out = {"metric": "serving p99 time-to-first-bin", "value": r["ttfb_p99_s"], "unit": "s",
           "n_gpus": 1, "steps": r["rounds"], "warmup": 0, "higher_is_better": False,
           "scaling": "weak", "vs_baseline": None, "dtype": "fp32+f64", "data": "synthetic",
           "config": {"workload": "serving: Poisson 50 jobs/s, N0 log-U[8,512], T U[0.5,4], "
                                  "mu U[-10,0], sweeps log-U[1e3,1e5], 150 GB HBM budget",
                      "censoring": "Kaplan-Meier over all arrived jobs"},
           "serving": r}
    print(json.dumps(out))


# ---------------------------------------------------------------------------
# F(q,tau) leg: N=512, M=512 (T = 1/(M tau)), 2048 lattice q with |q| <= 4/A.
# ---------------------------------------------------------------------------
def run_isf(args, pgb):
    import torch
    from pimc_gb300 import worldlines as wl
    w = wl.workload_isf()
    n, m = w["n"], w["m"]
    L = w["side"]
    q, _ = wl.isf_qvectors(L, count=2048, seed=0)
    nq = len(q)
    cfg = wl.seeded_worldlines(n, m, L, w["lam"], w["tau"], 0)
    a = pgb.Action(L, m, n, w["tau"], w["lam"], precision=pgb.PGB_MIXED)
    a.load(cfg)
    stream = torch.cuda.ExternalStream(pgb._lib.load().pgb_stream(a.h))
    d_q = torch.from_numpy(q).cuda()
    d_out = torch.empty((nq, m // 2 + 1), dtype=torch.float64, device="cuda")
    d_s = torch.empty(nq, dtype=torch.float64, device="cuda")
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    res = {}
    clk = Clocks()
    calls = {0: lambda: a.lib.pgb_isf_device_async(a.h, d_q.data_ptr(), nq, 0, d_out.data_ptr()),
             1: lambda: a.lib.pgb_isf_device_async(a.h, d_q.data_ptr(), nq, 1, d_out.data_ptr()),
             "ssf": lambda: a.lib.pgb_ssf_device_async(a.h, d_q.data_ptr(), nq, d_s.data_ptr())}
    for mode, call in calls.items():
        for _ in range(args.warmup):
            a._chk(call())
        torch.cuda.synchronize()
        ms = []
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(k))
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                a._chk(call())
                e1.record(stream)
            ms.append((e0, e1))
        torch.cuda.synchronize()
        res[mode] = sum(x.elapsed_time(y) for x, y in ms) / len(ms)
    clocks = clk.stop()
    # e2e through the C ABI with host buffers: positions uploaded each step
    # (the reference copies its bead array to the device every sample)
    a.update_positions(cfg["pos"])          # untimed: grows the pinned and scratch buffers
    a.isf(q, mode=1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        a.update_positions(cfg["pos"])      # the bead array, as the reference copies it per sample
        a.isf(q, mode=1)
    t_e2e = (time.perf_counter() - t0) / args.steps
    # the adjacent path-wide estimators on the same path (host calls,
    # synchronous): g(r) over all slices, winding sums, permutation cycles
    adj = {}
    for name, fn in (("pair_correlation", lambda: a.pair_correlation(-1)),
                     ("superfluid", a.superfluid), ("permutation_cycles", a.permutation_cycles)):
        fn()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            fn()
        adj[name + "_ms"] = 1e3 * (time.perf_counter() - t0) / args.steps
    # rho_q (the dominant kernel): Q M N phase evaluations, 2 special-function
    # ops (sin, cos) each; S(q) = rho_q plus an O(Q M) reduction, so its time
    # stands for the rho_q kernel.  Correlation (the GEMM part): the
    # algorithmic 2 M^2 2Q FLOP of the slice-correlation contraction, over the
    # F(q,tau) time less the S(q) time.
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"bf16_tflops": 1900.0}
    t_rho = res["ssf"] / 1e3
    sfu = 2.0 * nq * m * n / t_rho
    sfu_pk = sfu_peak(clocks.get("sm_mhz"))
    t_corr = max(res[1] - res["ssf"], 1e-6) / 1e3
    corr_flops = 2.0 * m * m * 2 * nq
    bf16 = peaks.get("bf16_tflops", 1900.0)
    out = {"metric": "F(q,tau) configurations/s", "value": 1e3 / res[1], "unit": "configurations/s",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": res[1],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32+bf16x3",
           "data": "synthetic",
           "config": {"workload": "F(q,tau): N=512, M=512, 2048 lattice q |q|<=4/A, tau in [0,M/2]",
                      "l2": "flushed between timed steps",
                      "ms_cuda_core_correlation": res[0], "ms_tensor_core_correlation": res[1],
                      "ms_ssf": res["ssf"], "adjacent_estimators": adj,
                      "phase_evaluations_per_s": nq * m * n / t_rho},
           "e2e": {"value": 1.0 / t_e2e, "unit": "configurations/s",
                   "h2d_bytes_per_step": int(cfg["pos"].nbytes + q.nbytes),
                   "d2h_bytes_per_step": int(nq * (m // 2 + 1) * 8)},
           "roofline": {"bound": "sfu", "kernel": "k_rhoq32", "achieved": sfu / 1e9,
                        "peak": sfu_pk / 1e9, "unit": "Gop/s", "frac": sfu / sfu_pk, "traffic": None,
                        "note": "2 special-function ops (sin, cos) per phase evaluation, Q M N of "
                                "them, over the S(q) call time (rho_q + an O(Q M) reduction); peak "
                                "= nominal %d/clk/SM x SMs x median SM clock" % SFU_PER_SM_CLK},
           "roofline_correlation": {"bound": "tensor", "kernel": "k_gemm_split_bf16 + split/prep kernels",
                                    "achieved": corr_flops / t_corr / 1e12, "peak": bf16,
                                    "unit": "TFLOP/s", "frac": corr_flops / t_corr / 1e12 / bf16,
                                    "note": "algorithmic 2 M^2 2Q FLOP of the correlation over "
                                            "(F(q,tau) time - S(q) time); the split-BF16 DFT form "
                                            "executes more (3 products, DFT then cosine GEMM); peak "
                                            "= MEASURED_PEAKS bf16 burst"},
           "clocks": clocks}
    # error against the FP64 oracle's rho_q form on 64 of the q-vectors
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    o = pyoracle.Oracle(L, m, n, w["tau"], w["lam"])
    o.load(cfg)
    sub_q = np.arange(0, nq, max(1, nq // 64))
    want = o.isf_rhoq(q[sub_q], threads=os.cpu_count() or 1)
    out["err_vs_oracle"] = {"tensor_core": err_stats(a.isf(q[sub_q], mode=1), want),
                            "cuda_core": err_stats(a.isf(q[sub_q], mode=0), want),
                            "note": "F(q,tau) for %d of the %d q-vectors against the FP64 oracle's "
                                    "rho_q form; values of order one" % (len(sub_q), nq)}
    if not args.no_baseline:
        thr = os.cpu_count() or 1
        sub = q[:max(thr * 4, 32)]
        t0 = time.perf_counter()
        o.isf_rhoq(sub, threads=thr)
        dt = time.perf_counter() - t0
        per_cfg = dt * nq / len(sub)
        out["cpu_baseline"] = {"value": 1.0 / per_cfg, "unit": "configurations/s", "cores": thr,
                               "kind": "port", "sample": "FP64 rho_q form for %d of the %d q-vectors, "
                               "scaled to all of them" % (len(sub), nq)}
        cpu_adj = {}
        for name, fn in (("pair_correlation", lambda: o.pair_correlation(-1)),
                         ("superfluid", o.superfluid), ("permutation_cycles", o.permutation_cycles)):
            t0 = time.perf_counter()
            fn()
            cpu_adj[name + "_ms"] = 1e3 * (time.perf_counter() - t0)
        out["cpu_baseline"]["adjacent_estimators_1_thread"] = cpu_adj
    print(json.dumps(out))


# ---------------------------------------------------------------------------
# Pair-action leg: N=256, M=250, GSF, rc = L: full-path potential action and
# virial energy per configuration (host call, synchronous) and 10^6
# single-bead trial displacements, FP64 and mixed.
# ---------------------------------------------------------------------------
def run_pair(args, pgb):
    import torch
    from pimc_gb300 import worldlines as wl
    w = wl.workload_pair_action()
    n, m, L = w["n"], w["m"], w["side"]
    cfg = wl.seeded_worldlines(n, m, L, w["lam"], w["tau"], 0)
    v_pairs = m * n * (n - 1) / 2.0
    g_pairs = (m / 2) * n * (n - 1.0)
    res = {}
    ntrial = 1000000
    rng = np.random.default_rng(0)
    lam_db = 2 * math.sqrt(math.pi * w["lam"] / w["temperature"])
    beads = np.stack([rng.integers(0, m, ntrial), rng.integers(0, n, ntrial)], 1).astype(np.int32)
    disp = rng.uniform(-0.04 * lam_db, 0.04 * lam_db, (ntrial, 3))
    clk = Clocks()
    for prec in (pgb.PGB_FP64, pgb.PGB_MIXED):
        a = pgb.Action(L, m, n, w["tau"], w["lam"], action="gsf", precision=prec)
        a.load(cfg)
        for _ in range(2):
            a.full_action()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            a.full_action()
        t_full = (time.perf_counter() - t0) / args.steps
        a.virial()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            a.virial()
        t_vir = (time.perf_counter() - t0) / args.steps
        pos = cfg["pos"][beads[:, 0], beads[:, 1]] + disp
        pos -= L * np.floor(pos / L + 0.5)
        d_b = torch.from_numpy(beads).cuda()
        d_p = torch.from_numpy(np.ascontiguousarray(pos)).cuda()
        d_o = torch.empty(ntrial, dtype=torch.float64, device="cuda")
        d_w = torch.empty(2 * ntrial, dtype=torch.float64, device="cuda")
        stream = torch.cuda.ExternalStream(a.lib.pgb_stream(a.h))
        k = ntrial if prec == pgb.PGB_MIXED else 20000
        a._chk(a.lib.pgb_trial_actions_device_async(a.h, d_b.data_ptr(), d_p.data_ptr(), 1000, 1, 0,
                                                    d_o.data_ptr(), d_w.data_ptr()))
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            a._chk(a.lib.pgb_trial_actions_device_async(a.h, d_b.data_ptr(), d_p.data_ptr(), k, 1, 0,
                                                        d_o.data_ptr(), d_w.data_ptr()))
            e1.record(stream)
        torch.cuda.synchronize()
        t_trial = e0.elapsed_time(e1) / 1e3
        # pair evaluations of a trial as the reference's per-bead action makes
        # them, old and new: 2 (n-1) V pairs, and on odd (gradV) slices
        # 2 (n-1)^2 gradV pairs (gradVnnSquared over the bead's list).  With
        # rc covering the box the mixed form gets the inner gradient sums from
        # cached slice forces and evaluates 2 (n-1) gradV pairs instead (trial
        # and current position, one fused launch); the roofline counts the
        # pairs it evaluates.
        odd = (beads[:k, 0] % 2 == 1).mean()
        tp_v = k * 2.0 * (n - 1)
        tp_vg_ref = k * odd * 2.0 * (n - 1) ** 2
        tp_vg = tp_vg_ref if prec == pgb.PGB_FP64 else k * odd * 2.0 * (n - 1)
        trial_pairs = tp_v + tp_vg_ref
        res["fp64" if prec == pgb.PGB_FP64 else "mixed"] = {
            "full_action_ms": 1e3 * t_full, "full_action_pairs_per_s": (v_pairs + g_pairs) / t_full,
            "virial_ms": 1e3 * t_vir,
            "trials": k, "trial_ms": 1e3 * t_trial,
            "reference_equivalent_pairs_per_s": trial_pairs / t_trial,
            "trial_moves_per_s": k / t_trial, "_pv": tp_v, "_pvg": tp_vg, "_t": t_trial}
    clocks = clk.stop()
    # error of the trial-move action differences against the FP64 oracle on
    # 256 of the trials (FP64 and mixed device forms, through the C ABI)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    o = pyoracle.Oracle(L, m, n, w["tau"], w["lam"], action="gsf")
    o.load(cfg)
    ks = np.arange(0, ntrial, ntrial // 256)[:256]
    tb = beads[ks]
    tp = cfg["pos"][tb[:, 0], tb[:, 1]] + disp[ks]
    tp -= L * np.floor(tp / L + 0.5)
    want = np.empty(len(ks))
    for i, (s_, p_) in enumerate(tb):
        u0 = o.bead_action(int(s_), int(p_))
        old = cfg["pos"][s_, p_].copy()
        o.update_bead(int(s_), int(p_), tp[i])
        want[i] = o.bead_action(int(s_), int(p_)) - u0
        o.update_bead(int(s_), int(p_), old)
    err = {}
    for prec, tag in ((pgb.PGB_FP64, "fp64"), (pgb.PGB_MIXED, "mixed")):
        a = pgb.Action(L, m, n, w["tau"], w["lam"], action="gsf", precision=prec)
        a.load(cfg)
        err[tag] = err_stats(a.trial_actions(tb, tp), want)
        err[tag + "_full_action"] = err_stats([a.full_action()], [o.full_action()])
        a.close()
    err["note"] = ("trial-move action differences dU of 256 of the trials and the full-path action "
                   "against the FP64 oracle")
    mx = res["mixed"]
    roof = pair_roofline(mx.pop("_pv"), mx.pop("_pvg"), mx.pop("_t"), "k_bead_actions32_full",
                         measured_fp32_peak(), clocks.get("sm_mhz"))
    for r in res.values():
        for key in ("_pv", "_pvg", "_t"):
            r.pop(key, None)
    out = {"metric": "single-bead trial moves/s (potential-action differences, mixed)",
           "value": mx["trial_moves_per_s"], "unit": "trial-moves/s", "n_gpus": 1,
           "steps": args.steps, "warmup": 2, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "fp32+f64", "data": "synthetic",
           "config": {"workload": "pair action: N=256, M=250, GSF, rc=L, 10^6 trial displacements "
                                  "uniform in [-0.04 lambda_dB, 0.04 lambda_dB]^3", "results": res},
           "roofline": roof, "clocks": clocks, "err_vs_oracle": err}
    if not args.no_baseline:
        t0 = time.perf_counter()
        cnt = 0
        while time.perf_counter() - t0 < 5.0:
            s_, p_ = int(beads[cnt, 0]), int(beads[cnt, 1])
            o.bead_action(s_, p_)
            cnt += 1
        dt = time.perf_counter() - t0
        odd = (beads[:cnt, 0] % 2 == 1).mean()
        pairs = cnt * ((n - 1) + odd * (n - 1) ** 2)
        # a trial move is two per-bead actions (before and after)
        out["cpu_baseline"] = {"value": cnt / 2.0 / dt, "unit": "trial-moves/s", "cores": 1,
                               "kind": "port", "sample": "%d per-bead GSF actions (FP64 oracle, 1 "
                               "thread, rc=L) in %.1f s, %.3g pair evaluations/s"
                               % (cnt, dt, pairs / dt)}
    print(json.dumps(out))


# ---------------------------------------------------------------------------
# Plain worm-PIMC leg (N=16, T=2 K -> M=124, tau=1/248): the plain FP64 GPU
# form running the worm algorithm (the reference's default move list, host
# moves, FP64 device actions, MT19937) against the oracle on one host thread,
# with the energy and S(q) (|q| <= 4/A) estimators sampled every diagonal step.
# ---------------------------------------------------------------------------
WORM_MOVES = ["center of mass", "diagonal", "open", "close", "insert", "remove", "advance head",
              "recede head", "advance tail", "recede tail", "swap head", "swap tail"]


def run_plain(args, pgb):
    from pimc_gb300 import worldlines as wl
    w = wl.workload_plain_small()
    n, m, L = w["n"], w["m"], w["side"]
    ne = 2 * n
    cfg = wl.seeded_worldlines(n, m, L, w["lam"], w["tau"], 0, extent=ne)
    mbar = wl.default_mbar(n, L ** 3, w["lam"], 0.004, m)
    q = pgb.qvectors("max_float", "4 0 0", [L, L, L])
    kw = dict(mbar=mbar, temperature=w["temperature"], initial_num_particles=n, window=1, mu=0.0)
    a = pgb.Action(L, m, ne, w["tau"], w["lam"])
    a.load(cfg)
    a.plain_seed(139853)
    a.plain_worm_run(1, **kw)
    t0 = time.perf_counter()
    bu, att, acc = 0, np.zeros(12, dtype=np.int64), np.zeros(12, dtype=np.int64)
    nssf = 0
    for _ in range(args.steps):
        r = a.plain_worm_run(1, **kw)
        bu += r["bead_updates"]
        att += r["attempted"]; acc += r["accepted"]
        if r["diagonal"]:
            a.ssf(q)
            nssf += 1
    dt = time.perf_counter() - t0
    out = {"metric": "bead-updates/s (plain FP64 GPU form, worm algorithm)", "value": bu / dt,
           "unit": "bead-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": 1,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic",
           "config": {"workload": "plain worm PIMC N=16, T=2 K, M=124 (tau=1/248), Mbar=%d, the "
                                  "reference's default move list, canonical window 1, energy + "
                                  "S(q) (%d q) every diagonal step" % (mbar, len(q)),
                      "ssf_samples": nssf,
                      "acceptance": {WORM_MOVES[i]: [int(acc[i]), int(att[i])] for i in range(12)}}}
    if not args.no_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle
        o = pyoracle.Oracle(L, m, ne, w["tau"], w["lam"])
        o.load(cfg)
        mt = pyoracle.MT(139853)
        o.run_worm_steps(mt, 1, **kw)
        t0 = time.perf_counter()
        bu_o = 0
        for _ in range(args.steps):
            r = o.run_worm_steps(mt, 1, **kw)
            bu_o += r["bead_updates"]
            if r["diagonal"]:
                o.ssf_pairwise(q)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": bu_o / dt, "unit": "bead-updates/s", "cores": 1,
                               "kind": "port", "sample": "%d worm-algorithm steps of the oracle on "
                               "one thread, same seed" % args.steps}
    print(json.dumps(out))


# ---------------------------------------------------------------------------
# Gaussian-process external potential leg: one call evaluates the potential
# at every bead of a path (64 particles x 64 slices) against 16384 training
# points, the largest case of the reference's GP action sweep.
# ---------------------------------------------------------------------------
GP_FLOP = 38     # FP32 pipe instructions per kernel evaluation of k_gp32 (nu = 5/2)
GP_SFU = 2       # exp2 and rsqrt per evaluation


def run_gp(args, pgb):
    import torch
    from pimc_gb300 import worldlines as wl
    from pimc_gb300.gp import GaussianProcess
    npts, nptcl, nsl = 16384, 64, 64
    w = wl.workload_gp(points=npts, num_ptcl=nptcl, num_slices=nsl, seed=0)
    pos = np.ascontiguousarray(w["pos"])
    count = len(pos)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    clk = Clocks()
    res = {}
    for prec, tag in ((pgb.PGB_FP64, "fp64"), (pgb.PGB_MIXED, "mixed")):
        g = GaussianProcess(w["training"], precision=prec, **w["params"])
        d_pos = torch.from_numpy(pos).cuda()
        d_out = torch.empty(count, dtype=torch.float64, device="cuda")
        stream = torch.cuda.ExternalStream(g.stream())
        for _ in range(max(3, args.warmup)):
            g._chk(g.lib.pgb_gp_eval_device_async(g.h, d_pos.data_ptr(), d_out.data_ptr(), count))
        torch.cuda.synchronize()
        ts = []
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            with torch.cuda.stream(stream):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                g._chk(g.lib.pgb_gp_eval_device_async(g.h, d_pos.data_ptr(), d_out.data_ptr(), count))
                e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        t_dev = sum(ts) / len(ts)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            g(pos)
        t_e2e = (time.perf_counter() - t0) / args.steps
        res[tag] = {"call_ms": 1e3 * t_dev, "evaluations_per_s": count * npts / t_dev,
                    "points_per_s": count / t_dev, "e2e_points_per_s": count / t_e2e,
                    "e2e_call_ms": 1e3 * t_e2e, "_t": t_dev}
        g.close()
    clocks = clk.stop()
    mx = res["mixed"]
    t = mx.pop("_t")
    res["fp64"].pop("_t")
    peak = measured_fp32_peak()
    ev = count * npts
    flops = ev * GP_FLOP / t / 1e12
    sfu = ev * GP_SFU / t
    sfu_pk = sfu_peak(clocks.get("sm_mhz"))
    f32, fs = flops / peak, sfu / sfu_pk
    roof = {"bound": "fp32" if f32 >= fs else "sfu", "achieved": flops, "peak": peak,
            "unit": "TFLOP/s", "frac": max(f32, fs), "fp32_frac": f32,
            "sfu": {"achieved_gops": sfu / 1e9, "peak_gops": sfu_pk / 1e9, "frac": fs},
            "traffic": None, "kernel": "k_gp32",
            "note": "achieved = kernel evaluations x %d FP32 instructions / kernel time; FP32 peak "
                    "= measured cuBLAS SGEMM (no TF32); SFU = %d ops per evaluation against "
                    "nominal %d/clk/SM x SMs x median SM clock" % (GP_FLOP, GP_SFU, SFU_PER_SM_CLK)}
    out = {"metric": "GP potential points/s (mixed, 16384 training points)",
           "value": mx["points_per_s"], "unit": "points/s", "n_gpus": 1, "steps": args.steps,
           "warmup": max(3, args.warmup), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "fp32+f64", "data": "synthetic",
           "config": {"workload": "Gaussian-process external potential, Matern nu=5/2, 16384 "
                                  "training points, %d positions per call (%d particles x %d "
                                  "slices), periodic separations" % (count, nptcl, nsl),
                      "l2": "flushed between timed calls", "results": res},
           "e2e": {"value": mx["e2e_points_per_s"], "unit": "points/s",
                   "h2d_bytes_per_step": count * 24, "d2h_bytes_per_step": count * 8},
           "gpu_launches": args.steps, "roofline": roof, "clocks": clocks}
    if not args.no_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle
        from concurrent.futures import ThreadPoolExecutor
        threads = os.cpu_count() or 1
        sample = pos
        chunks = np.array_split(sample, threads)
        t0 = time.perf_counter()
        with ThreadPoolExecutor(threads) as ex:
            want = np.concatenate(list(ex.map(
                lambda c: pyoracle.gp_eval(w["training"], c, **w["params"]), chunks)))
        dt = time.perf_counter() - t0
        g = GaussianProcess(w["training"], precision=pgb.PGB_MIXED, **w["params"])
        got = g(pos)
        g.close()
        out["config"]["mixed_max_abs_err_vs_fp64_oracle"] = float(np.max(np.abs(got - want)))
        out["err_vs_oracle"] = {"mixed": err_stats(got, want), "note": "GP potential at every position "
                                "of the call against the FP64 oracle"}
        out["cpu_baseline"] = {"value": len(sample) / dt, "unit": "points/s", "cores": threads,
                               "kind": "port", "sample": "%d positions against 16384 training "
                               "points, FP64 oracle, %d threads, %.1f s" % (len(sample), threads, dt)}
    print(json.dumps(out))


# ---------------------------------------------------------------------------
# The default line: the batched-walker workload (1024 He-4 paths,
# N ~ U{8..128}, T ~ U[1,4] K, tau = 0.004, M even) run by the device worm
# walkers with the reference's default move list and a canonical window of
# one particle.
# ---------------------------------------------------------------------------
DIAGONAL = {"bisection": 0, "staging": 1}


def worm_pair_evals(w, st):
    """Algorithmic pair evaluations of the walkers' steps: every bead update
    compares the bead's action before and after the proposal against its N-1
    partners (2 (N-1) pairs; the single-bead worm moves evaluate one action per
    bead and are counted the same way), and each energy sample sums
    M N (N-1)/2 pairs.  N is the walker's target particle number."""
    n, m = w["n"].astype(float), w["m"].astype(float)
    return float((2.0 * (n - 1) * st["bead_updates"] + st["samples"] * m * n * (n - 1) / 2.0).sum())


PRE_SWEEPS = 20       # diagonal pre-equilibration steps before the warm-up (both arms)


def worm_sample(w, every=4):
    """Every `every`-th walker of the workload in order of cost N^2 M: a
    stratified sample with the workload's mix of sizes."""
    order = np.argsort(w["n"].astype(float) ** 2 * w["m"], kind="stable")
    idx = np.sort(order[::every])
    return {k: (v[idx] if isinstance(v, np.ndarray) else v) for k, v in w.items()}


def cpu_baseline_worm(w, threads, nequil=3, nsteps=5, diagonal_move=0, seed=7, every=4):
    """The oracle's FP64 worm engine (MT19937, the same move list, window and
    worm constant) on a stratified quarter of the workload's walkers, all host
    threads: set-up, PRE_SWEEPS diagonal pre-equilibration steps and nequil
    steps untimed, nsteps steps of every sampled walker timed (the walkers
    outnumber the threads 16 to 1, taken largest first, so none idles)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    s = worm_sample(w, every)
    r = pyoracle.worm_walkers_cpu(s["n"], s["m"], s["side"], s["mbar"],
                                  np.arange(len(s["n"]), dtype=np.uint32) + seed, w["tau"], w["lam"],
                                  nsteps, threads, nequil=nequil, window=1, diagonal_move=diagonal_move,
                                  npre=PRE_SWEEPS)
    bu = int(r["bead_updates"].sum())
    return dict(value=bu / r["seconds"], unit="bead-updates/s", cores=threads, kind="port",
                timed="sweeps only",
                sample="%d of the %d walkers (every %d-th by N^2 M), %d timed step(s) each after %d "
                       "pre-equilibration and %d untimed steps (set-up %.1f s untimed), FP64 oracle "
                       "worm engine with MT19937, %s, window 1, C0 1, %d threads, %.1f s timed"
                       % (len(s["n"]), len(w["n"]), every, nsteps, PRE_SWEEPS, nequil,
                          r["setup_seconds"], ["bisection", "staging"][diagonal_move], threads,
                          r["seconds"]),
                failed_walkers=r["failed"])


def plain_worm_rate(pgb, n=64, t=2.0, tau=0.004, steps=2, diagonal_move=0):
    """The plain FP64 GPU form of the same algorithm: the reference's move
    loop on the host (MT19937, worm moves, window 1) with one FP64 device
    action call per Metropolis decision, on one walker of the workload's mean
    size."""
    from pimc_gb300 import worldlines as wl
    m = wl.even_slices(t, tau)
    L = wl.box_side(n)
    mbar = wl.default_mbar(n, L ** 3, wl.LAMBDA_HE4, tau, m)
    ne = 2 * n + 8
    a = pgb.Action(L, m, ne, tau, wl.LAMBDA_HE4, precision=pgb.PGB_FP64)
    a.load(wl.seeded_worldlines(n, m, L, wl.LAMBDA_HE4, tau, 5, extent=ne))
    a.plain_seed(139853)
    kw = dict(mbar=mbar, temperature=1.0 / (m * tau), initial_num_particles=n, window=1,
              diagonal_move=diagonal_move)
    a.plain_worm_run(1, **kw)                                  # warm-up
    t0 = time.perf_counter()
    r = a.plain_worm_run(steps, **kw)
    dt = time.perf_counter() - t0
    a.close()
    return dict(value=r["bead_updates"] / dt, unit="bead-updates/s",
                walker="N=%d M=%d T=%.3f Mbar=%d, %d step(s) of the worm algorithm, window 1"
                       % (n, m, 1.0 / (m * tau), mbar, steps))


def matched_energy_worm(pgb, diagonal_move=0, path=None):
    """Energy per particle of the batched walkers (FP32 pair sums, Philox)
    beside the FP64 oracle's worm engine (MT19937) at the points of
    tests/golden/matched_energy.json, which holds the oracle side (hours of
    host time, made once by tests/golden/make_matched_energy.py).  The GPU
    side runs the same replicas, pre-equilibration, equilibration and
    sampled steps; each side's value is the mean over replicas of the
    replica's mean E/N over its closed steps, with the standard error over
    replicas, and diff_sigma the difference in combined standard errors."""
    path = path or os.path.join(ROOT, "tests", "golden", "matched_energy.json")
    if not os.path.exists(path):
        return {"note": "no oracle fixture (tests/golden/matched_energy.json)"}
    fx = json.load(open(path))
    out = []
    for pt in fx["points"]:
        if pt.get("diagonal_move", 0) != diagonal_move:
            continue
        R = pt["replicas"]
        n, m, L, mbar = pt["n"], pt["m"], pt["side"], pt["mbar"]
        W = pgb.WormWalkers(np.full(R, n), m, L, mbar, fx["tau"], fx["lambda"], window=fx["window"],
                            seed=777 + n, diagonal_move=diagonal_move, worm_constant=pt["worm_constant"])
        W.seed_device(777 + n)
        t0 = time.perf_counter()
        W.equilibrate(pt["pre"])
        W.run(pt["equil"])
        W.reset_stats()
        W.run(pt["sweeps"])
        dt = time.perf_counter() - t0
        st = W.stats()
        W.close()
        has = st["samples"] > 0
        e = st["energy_sum"][has] / st["samples"][has]
        eb, sb = float(e.mean()), float(e.std(ddof=1) / math.sqrt(max(len(e), 1)))
        eo, so = pt["mean"], pt["stderr"]
        out.append({"config": "N=%d M=%d T=%.3f Mbar=%d C0=%.4g" % (n, m, pt["temperature"], mbar,
                                                                     pt["worm_constant"]),
                    "batched": [eb, sb], "oracle_fp64": [eo, so],
                    "diff_sigma": abs(eb - eo) / math.hypot(sb, so),
                    "closed_replicas": [int(has.sum()), pt["closed_replicas"]],
                    "sample": "%d replicas each side, %d pre-equilibration + %d + %d sampled steps; "
                              "GPU side %.1f s" % (R, pt["pre"], pt["equil"], pt["sweeps"], dt)})
    return out


def walker_pair_sum_errors(W, w, walkers=8, beads=48, seed=3):
    """The walkers' FP32 pair sums against the FP64 oracle on the walkers'
    own current paths: the bare potential action of `beads` active beads of
    `walkers` walkers spread over N (worm open or closed as the steps left
    them), through pgb_worm_walkers_bead_actions."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    rng = np.random.default_rng(seed)
    order = np.argsort(w["n"], kind="stable")
    picks = order[np.linspace(0, len(order) - 1, walkers).astype(int)]
    got, want = [], []
    for i in picks:
        p = W.path(int(i))
        o = pyoracle.Oracle(float(w["side"][i]), int(w["m"][i]), int(W.capacity[i]), w["tau"], w["lam"])
        o.load(p)
        act = np.argwhere(p["on"])
        b = act[rng.choice(len(act), size=min(beads, len(act)), replace=False)].astype(np.int32)
        got.append(W.bead_actions(int(i), b))
        want.append([o.bead_action(int(t), int(q), mode=1) for t, q in b])
    return dict(err_stats(np.concatenate(got), np.concatenate(want)),
                note="bare potential action of %d active beads in each of %d walkers (N %d..%d) by "
                     "the walkers' FP32 pair sums against the FP64 oracle on the same paths"
                     % (beads, walkers, int(w["n"][picks].min()), int(w["n"][picks].max())))


def run_walkers(args, pgb, rank, ws):
    import torch
    dm = DIAGONAL[args.diagonal]
    w = workload(args.walkers, seed=rank)
    W = pgb.WormWalkers(w["n"], w["m"], w["side"], w["mbar"], w["tau"], w["lam"], window=1,
                        seed=1000 + rank, diagonal_move=dm)
    W.seed_device(1000 + rank)
    stream = torch.cuda.ExternalStream(W.stream())
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    warm = max(3, args.warmup)
    W.equilibrate(PRE_SWEEPS)
    W.run(warm)
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
            W.run(1, sync=False)
            e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    barrier(ws)
    clocks = clk.stop()
    launches = W.launch_count() - l0
    step_ms = [a.elapsed_time(b) for a, b in evs]
    t_dev = sum(step_ms) / 1e3
    st = W.stats()
    bu = float(st["bead_updates"].sum())
    pairs = worm_pair_evals(w, st)
    errors = int((st["error"] != 0).sum())
    att, acc = st["attempted"].sum(axis=0), st["accepted"].sum(axis=0)
    closed = int(st["samples"].sum())
    t_max = max_over_ranks(t_dev, ws)
    value = sum_over_ranks(bu, ws) / t_max

    # e2e through the C ABI with host buffers: every step uploads the whole
    # device state image from pinned memory, runs one step and reads the
    # per-walker accumulators back
    nbytes = W.state_bytes()
    host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    image = host.numpy()
    W.get_state(image)
    stats_host = torch.empty(W.W * W.STATS_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
    st_view = stats_host.numpy().view(W.STATS_DTYPE)
    W.reset_stats()
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        W.set_state_async(image)
        W.run(1, sync=False)
        W.stats_async(st_view)
        W.synchronize()
    t_e2e = time.perf_counter() - t0
    bu_e2e = float(st_view["bead_updates"].sum())
    t_e2e = max_over_ranks(t_e2e, ws)
    e2e_val = sum_over_ranks(bu_e2e, ws) / t_e2e

    roof = pair_roofline(pairs, 0.0, t_dev, "k_worm_walkers", measured_fp32_peak(),
                         clocks.get("sm_mhz"), NCU_TRAFFIC_WORM)
    roof["note"] += ("; pair evaluations = 2 (N-1) per bead update + M N (N-1)/2 per energy "
                     "sample, N the walker's target particle number")
    out = {"metric": "bead-updates/s", "value": value, "unit": "bead-updates/s", "n_gpus": ws,
           "steps": args.steps, "warmup": warm, "ms_per_step": 1e3 * t_max / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32+f64",
           "data": "synthetic",
           "config": {"workload": "batched bosonic walkers: %d He-4 paths, N~U{8..128}, T~U[1,4] K, "
                                  "tau=0.004, M even, Aziz HFDHE2, rho=0.02186, primitive action, "
                                  "the reference's default PIMC move list (centre of mass, %s, open, "
                                  "close, insert, remove, advance/recede head and tail, swap head and "
                                  "tail), canonical window 1, C0 1, energy sampled at every closed "
                                  "step; %d staging + COM pre-equilibration steps from the seeded "
                                  "worldlines, then the warm-up" % (W.W, args.diagonal, PRE_SWEEPS),
                      "l2": "flushed between timed steps",
                      "parallelism": "replicas" if ws > 1 else "single",
                      "walker_errors": errors, "closed_samples": closed,
                      "step_ms": [round(x, 3) for x in step_ms],
                      "pair_evaluations_per_step": pairs / args.steps,
                      "acceptance": {WORM_MOVES[i]: [int(acc[i]), int(att[i])] for i in range(12)}},
           "e2e": {"value": e2e_val, "unit": "bead-updates/s", "h2d_bytes_per_step": nbytes,
                   "d2h_bytes_per_step": W.W * W.STATS_DTYPE.itemsize},
           "gpu_launches": int(launches),
           "roofline": roof,
           "clocks": clocks}
    if rank == 0:
        out["err_vs_oracle"] = {"pair_sums": walker_pair_sum_errors(W, w)}
    W.close()
    if rank == 0 and not args.no_baseline:
        threads = os.cpu_count() or 1
        out["cpu_baseline"] = cpu_baseline_worm(w, threads, diagonal_move=dm)
        out["plain_fp64"] = plain_worm_rate(pgb, diagonal_move=dm)
        out["plain_fp64"]["batched_over_plain"] = value / out["plain_fp64"]["value"]
        out["matched_energy"] = matched_energy_worm(pgb, diagonal_move=dm)
        out["serving"] = serving_run(pgb, seconds=args.serve_seconds, grand_canonical=not args.serve_canonical)
    if rank == 0:
        print(json.dumps(out))


def run_reference(args):
    rank, ws = dist_init()
    if rank != 0:
        return
    w = workload(args.walkers)
    threads = os.cpu_count() or 1
    dm = DIAGONAL[args.diagonal]
    base = cpu_baseline_worm(w, threads, nequil=max(3, args.warmup), nsteps=args.steps, diagonal_move=dm)
    line = {"metric": "bead-updates/s", "value": base["value"], "unit": "bead-updates/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": "batched bosonic walkers: %d He-4 paths, N~U{8..128}, T~U[1,4] K, "
                                   "tau=0.004, Aziz, rho=0.02186, the reference's default PIMC move "
                                   "list (%s), canonical window 1, C0 1" % (len(w["n"]), args.diagonal),
                       "sample": base["sample"], "timed": "sweeps only"},
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": "bead-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_canonical(args, pgb, rank, ws):
    """The canonical staging + centre-of-mass walkers (no exchange moves) on
    the same 1024 paths: the persistent packed-team kernel with its
    autotuned schedule."""
    import torch
    w = workload(args.walkers, seed=rank)
    W = pgb.Walkers(w["n"], w["m"], w["temperature"], w["side"], w["mbar"], w["tau"], w["lam"],
                    seed=1000 + rank, threads_per_walker=args.schedule)
    W.init()                                   # autotunes the schedule when 0
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
    st = W.stats_array()
    upload = lambda: W._chk(W.lib.pgb_walkers_set_all_positions(W.h, host_np.ctypes.data_as(
        pgb._lib._DP)))
    t0 = time.perf_counter()
    upload()                                    # step 0's state
    for k in range(args.steps):
        W.run(1, measure=1, sync=False)
        if k + 1 < args.steps:
            upload()                            # step k+1's state: its copy overlaps sweep k
        W.stats_array(st)                       # synchronous D2H of the accumulators
    t_e2e = time.perf_counter() - t0
    bu_e2e = int(st["bead_updates"].sum())
    t_e2e = max_over_ranks(t_e2e, ws)
    e2e_val = sum_over_ranks(float(bu_e2e), ws) / t_e2e

    # roofline of the walker kernel: pair evaluations x nominal FLOP / SFU ops
    peak_fp32 = measured_fp32_peak()
    pairs = pair_per_step * args.steps
    kname = walker_kernel(W.threads())
    roof = pair_roofline(pairs, 0.0, t_dev, kname, peak_fp32, clocks.get("sm_mhz"),
                         NCU_TRAFFIC.get(kname))

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
           "roofline": roof,
           "clocks": clocks}
    if rank == 0 and not args.no_baseline:
        out["cpu_baseline"] = cpu_baseline(w, os.cpu_count() or 1)
        out["plain_fp64"] = plain_form_rate(pgb)
        out["plain_fp64"]["batched_over_plain"] = value / out["plain_fp64"]["value"]
        out["matched_energy"] = matched_energy(pgb, os.cpu_count() or 1)
    if rank == 0:
        print(json.dumps(out))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    rank, ws = dist_init()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    import pimc_gb300 as pgb
    if args.workload == "walkers":
        run_walkers(args, pgb, rank, ws)
    elif args.workload == "canonical":
        run_canonical(args, pgb, rank, ws)
    elif rank == 0:
        {"serving": run_serving, "isf": run_isf, "pair": run_pair,
         "plain": run_plain, "gp": run_gp}[args.workload](args, pgb)


if __name__ == "__main__":
    main()

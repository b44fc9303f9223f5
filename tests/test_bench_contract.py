"""bench.py's host side on CPU: the reference arm's JSON line, one line from
rank 0 under torchrun with two ranks over gloo, and the rank reductions the
GPU arm times with (max of the step times, sum of the bead updates)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _json_lines(text):
    return [json.loads(l) for l in text.splitlines() if l.startswith("{")]


def _cpu_env():
    env = dict(os.environ)
    env["CUDA_VISIBLE_DEVICES"] = ""
    return env


def test_reference_arm_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1",
                        "--walkers", "64"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600, env=_cpu_env())
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["metric"] == "bead-updates/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["unit"] == "bead-updates/s"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference")
    assert cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_under_torchrun_prints_once():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port),
           "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1",
           "--walkers", "64"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=_cpu_env())
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2


def _reduce_worker(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    r, ws = bench.dist_init()
    bench.barrier(ws)
    q.put((r, bench.max_over_ranks(1.5 + r, ws), bench.sum_over_ranks(10.0 * (r + 1), ws)))
    dist.destroy_process_group()


def test_rank_reductions_over_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_reduce_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2.5, 30.0), (1, 2.5, 30.0)]


def _bench_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_kaplan_meier_quantiles():
    """The serving line's time-to-first-bin and completion percentiles:
    the Kaplan-Meier estimate over right-censored durations, worked by hand.
    Without censoring it is the empirical quantile; a job censored at t
    leaves the risk set after the events at t; a quantile the estimate never
    reaches is None; the jobs at risk where each quantile is reached."""
    km = _bench_module().km_quantiles
    # no censoring: S = 3/4, 1/2, 1/4, 0 after 1, 2, 3, 4
    assert km([1, 2, 3, 4], [True] * 4) == {50: 2.0, 99: 4.0}
    # one censored job at 2: S = 3/4 after 1, then 3/4 (1 - 1/3) = 1/2 at 3,
    # then 0 at 4 (one job at risk)
    out, risk = km([4, 2, 1, 3], [True, False, True, True], with_risk=True)
    assert out == {50: 3.0, 99: 4.0}
    assert risk == {50: 2, 99: 1}
    # the event and a censoring at the same time: the event first (4 at risk)
    assert km([2, 2, 5, 6], [False, True, False, False], qs=(25,)) == {25: 2.0}
    # most jobs still waiting when the window closes: the median lies beyond
    out = km([1, 9, 9, 9, 9], [True, False, False, False, False])
    assert out == {50: None, 99: None}
    assert km([], [], qs=(50,)) == {50: None}

"""Batched walkers: schedules, determinism and matched energy against the
FP64 oracle's walkers (the reference CPU move loop restated).

The batched engine uses Philox streams and FP32 pair sums while the oracle
uses MT19937 and the FP64 table, so the two agree statistically, not bead for
bead: the test compares the mean energy per particle of many independent
chains, within 3 combined standard errors.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _walkers(pgb, num, seed, sched, n=8, t=4.0, tau=0.004):
    from pimc_gb300 import worldlines as wl
    m = 2 * int(round(1.0 / (2.0 * t * tau)))
    L = wl.box_side(n)
    mbar = wl.default_mbar(n, L ** 3, wl.LAMBDA_HE4, tau, m)
    W = pgb.Walkers(np.full(num, n), np.full(num, m), np.full(num, 1.0 / (m * tau)),
                    np.full(num, L), np.full(num, mbar), tau, wl.LAMBDA_HE4, seed=seed,
                    threads_per_walker=sched)
    return W, dict(n=n, m=m, L=L, mbar=mbar, t=1.0 / (m * tau), tau=tau)


@pytest.mark.parametrize("sched", [128, 1004, 1008, 1016, 2008, 3002, 3003, 4004, 4008, 4016,
                                   5000, 5008, 5016, 6000, 6008, 6016, 7000, 7008, 7016,
                                   8000, 8008, 8016])
def test_schedule_runs_and_is_deterministic(pgb, sched):
    # N <= 90 keeps two Mbar-row buffers of every walker within the 100 KB
    # budget of the 256-thread pipelined schedules (5008/5016)
    w = pgb.worldlines.workload_walkers(num=40, seed=2, nmax=90)
    runs = []
    for _ in range(2):
        W = pgb.Walkers(w["n"], w["m"], w["temperature"], w["side"], w["mbar"], w["tau"], w["lam"],
                        seed=5, threads_per_walker=sched)
        W.init()
        W.run(2, measure=1)
        runs.append((W.stats(), W.positions(7)))
    st = runs[0][0]
    assert all(s["samples"] == 2 for s in st)
    assert all(s["attempted"][1] > 0 for s in st)
    assert [s["accepted"] for s in st] == [s["accepted"] for s in runs[1][0]]
    assert np.array_equal(runs[0][1], runs[1][1])
    L = w["side"][7]
    assert np.all(np.abs(runs[0][1]) <= L / 2 + 1e-5)


@pytest.mark.parametrize("sched", [128, 3002, 5008, 6000, 7016, 8016])
def test_matched_energy_vs_oracle_walkers(pgb, oracle_lib, sched):
    num, equil, prod = 256, 60, 200
    W, p = _walkers(pgb, num, 11, sched)
    W.init()
    W.run(equil, measure=0)
    W.reset_stats()
    W.run(prod, measure=1)
    st = W.stats()
    per = np.array([s["energy_sum"] / s["samples"] for s in st])
    g_mean, g_err = per.mean(), per.std(ddof=1) / math.sqrt(num)
    # oracle: independent MT19937 chains, same workload, on the host cores
    nw = 64
    sec, en, bu = oracle_lib.walkers_cpu(np.full(nw, p["n"]), np.full(nw, p["m"]),
                                         np.full(nw, p["t"]), np.full(nw, p["L"]),
                                         np.arange(nw) + 7, p["tau"], pgb.worldlines.LAMBDA_HE4,
                                         prod, 16, nequil=equil)
    o_mean, o_err = en.mean(), en.std(ddof=1) / math.sqrt(nw)
    diff = abs(g_mean - o_mean)
    assert diff <= 3.0 * math.hypot(g_err, o_err), (g_mean, g_err, o_mean, o_err)


def test_prefetch_pipeline_matches_unpipelined(pgb):
    """The pipelined schedule (next move's rows prefetched and patched after an
    accepted move) must leave exactly the configuration the unpipelined TMA
    schedule leaves: same teams, same draws, same arithmetic."""
    w = pgb.worldlines.workload_walkers(num=48, seed=9, nmax=90)
    out = []
    for sched in (4008, 5008):
        W = pgb.Walkers(w["n"], w["m"], w["temperature"], w["side"], w["mbar"], w["tau"], w["lam"],
                        seed=21, threads_per_walker=sched)
        W.init()
        W.run(3, measure=1)
        out.append((W.stats(), [W.positions(k) for k in (0, 5, 17, 40)]))
    (s1, p1), (s2, p2) = out
    assert [x["accepted"] for x in s1] == [x["accepted"] for x in s2]
    assert [x["energy_sum"] for x in s1] == [x["energy_sum"] for x in s2]
    for a, b in zip(p1, p2):
        assert np.array_equal(a, b)


def test_infeasible_schedule_is_an_error(pgb):
    """A schedule whose shared-memory buffers cannot hold a walker fails with a
    message instead of running something else."""
    w = pgb.worldlines.workload_walkers(num=4, seed=1, nmin=128, nmax=128)
    W = pgb.Walkers(w["n"], w["m"], w["temperature"], w["side"], w["mbar"], w["tau"], w["lam"],
                    seed=1, threads_per_walker=5008)
    W.init()
    with pytest.raises(pgb.PgbError):
        W.run(1)


def test_stats_array_matches_stats(pgb):
    w = pgb.worldlines.workload_walkers(num=20, seed=4, nmax=40)
    W = pgb.Walkers(w["n"], w["m"], w["temperature"], w["side"], w["mbar"], w["tau"], w["lam"],
                    seed=2, threads_per_walker=6016)
    W.init()
    W.run(2, measure=1)
    st, arr = W.stats(), W.stats_array()
    assert list(arr["bead_updates"]) == [s["bead_updates"] for s in st]
    assert list(arr["energy_sum"]) == [s["energy_sum"] for s in st]
    assert [list(a) for a in arr["accepted"]] == [s["accepted"] for s in st]


def test_set_all_positions_double_buffered(pgb):
    """Back-to-back uploads go through two staging buffers on a copy stream;
    each one takes effect in stream order and the last one wins."""
    import ctypes as C
    w = pgb.worldlines.workload_walkers(num=6, seed=8, nmax=24)
    W = pgb.Walkers(w["n"], w["m"], w["temperature"], w["side"], w["mbar"], w["tau"], w["lam"],
                    seed=1, threads_per_walker=6016)
    W.init()
    nbytes = int(W.lib.pgb_walkers_state_bytes(W.h))
    rng = np.random.default_rng(0)
    states = [rng.uniform(-0.4, 0.4, nbytes // 8) for _ in range(3)]
    for k in range(3):
        sides = np.repeat(w["side"], w["n"] * w["m"] * 3)
        states[k] *= sides
        W._chk(W.lib.pgb_walkers_set_all_positions(W.h, states[k].ctypes.data_as(C.POINTER(C.c_double))))
    W.sync()
    off = 0
    for i in range(6):
        n = int(w["n"][i] * w["m"][i] * 3)
        want = states[2][off:off + n].reshape(w["m"][i], w["n"][i], 3)
        assert np.allclose(W.positions(i), want, rtol=0, atol=1e-5 * w["side"][i])
        off += n

"""Continuous-batching server: admission by HBM footprint, overlapping jobs in
shared launches, bins streamed back, and each job's results identical alone
and in a mix (its streams are keyed by its own seed and its team size depends
only on its own N and Mbar, so the comparison is exact)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(server, ids, timeout=120.0):
    t0 = time.time()
    bins = []
    while time.time() - t0 < timeout:
        server.step()
        bins += server.bins()
        if all(server.job(j)["state"] == 3 for j in ids):
            return bins
    raise AssertionError("jobs did not finish")


def test_job_same_alone_and_in_mix(pgb):
    X = dict(n=24, temperature=2.0, sweeps=60, seed=5)
    alone = pgb.Server(2e9, sweeps_per_round=10, bin_sweeps=20)
    jx = alone.submit(**X)
    b_alone = [b for b in _run(alone, [jx]) if b["job"] == jx]
    assert len(b_alone) == 3

    mix = pgb.Server(2e9, sweeps_per_round=10, bin_sweeps=20)
    rng = np.random.default_rng(0)
    others = []
    for k in range(6):
        others.append(mix.submit(n=int(rng.integers(8, 64)), temperature=float(rng.uniform(1, 4)),
                                 sweeps=int(rng.integers(20, 90)), seed=100 + k))
    jm = mix.submit(**X)
    for k in range(6):   # late arrivals join while the others run
        others.append(mix.submit(n=int(rng.integers(8, 96)), temperature=float(rng.uniform(1, 4)),
                                 sweeps=40, seed=200 + k, arrival=0.02 * (k + 1)))
    bins = _run(mix, others + [jm])
    b_mix = [b for b in bins if b["job"] == jm]
    assert [b["energy"] for b in b_mix] == [b["energy"] for b in b_alone]
    assert all(np.isfinite(b["energy"]) for b in bins)


@pytest.mark.parametrize("round_seconds", [0.0, 0.0004, 0.003])
def test_bins_do_not_depend_on_round_length(pgb, round_seconds):
    """Timed rounds stop a job between two moves and resume it there; its
    draws are indexed by (sweep, move) and its samples summed in order, so
    the bins equal those of whole-sweep rounds bit for bit."""
    X = dict(n=40, temperature=1.5, sweeps=45, seed=9)
    ref = pgb.Server(2e9, sweeps_per_round=7, bin_sweeps=20)
    jr = ref.submit(**X)
    want = [b["energy"] for b in _run(ref, [jr])]
    assert len(want) == 3                       # 20 + 20 + the remaining 5
    s = pgb.Server(2e9, sweeps_per_round=7, bin_sweeps=20, round_seconds=round_seconds)
    j = s.submit(**X)
    others = [s.submit(n=96, temperature=1.0, sweeps=30, seed=77)]
    bins = _run(s, [j] + others)
    assert [b["energy"] for b in bins if b["job"] == j] == want
    assert s.job(j)["sweeps_done"] == 45


def test_admission_by_memory_budget(pgb):
    # each job: N=128, T=1 -> M=250 -> 128*250*16 B = 512 KB; the budget holds two
    s = pgb.Server(1.2e6, max_active=16, sweeps_per_round=5, bin_sweeps=10)
    ids = [s.submit(n=128, temperature=1.0, sweeps=10, seed=k) for k in range(5)]
    peak = 0
    t0 = time.time()
    while time.time() - t0 < 120:
        active, queued = s.step()
        peak = max(peak, active)
        if all(s.job(j)["state"] == 3 for j in ids):
            break
    assert peak == 2
    for j in ids:
        info = s.job(j)
        assert info["state"] == 3 and info["sweeps_done"] == 10
        assert info["arrival"] <= info["admitted"] <= info["first_bin"] <= info["completed"]
    assert s.bead_updates() > 0


def test_oversized_job_rejected(pgb):
    s = pgb.Server(1e6, sweeps_per_round=5, bin_sweeps=10)
    with pytest.raises(pgb.PgbError):
        s.submit(n=512, temperature=0.5, sweeps=10, seed=1)


# ---------------------------------------------------------------------------
# grand-canonical jobs: every job a device worm walker at its own mu
# ---------------------------------------------------------------------------
def test_grand_canonical_job_same_alone_and_in_mix(pgb):
    X = dict(n=12, temperature=2.5, sweeps=30, seed=7, mu=-4.0)
    alone = pgb.Server(2e9, sweeps_per_round=4, bin_sweeps=10, grand_canonical=True)
    jx = alone.submit(**X)
    b_alone = [b for b in _run(alone, [jx]) if b["job"] == jx]
    assert [b["bin"] for b in b_alone] == [0, 1, 2]

    mix = pgb.Server(2e9, sweeps_per_round=4, bin_sweeps=10, grand_canonical=True, round_seconds=0.005)
    rng = np.random.default_rng(1)
    others = [mix.submit(n=int(rng.integers(6, 24)), temperature=float(rng.uniform(1.5, 4)),
                         mu=float(rng.uniform(-10, 0)), sweeps=int(rng.integers(10, 40)), seed=300 + k,
                         arrival=0.01 * k) for k in range(6)]
    jm = mix.submit(**X)
    bins = _run(mix, others + [jm])
    b_mix = [b for b in bins if b["job"] == jm]
    # the same sweeps in every bin, whatever the rounds: identical bins
    assert [(b["bin"], b["samples"]) for b in b_mix] == [(b["bin"], b["samples"]) for b in b_alone]
    ea = np.array([b["energy"] for b in b_alone])
    em = np.array([b["energy"] for b in b_mix])
    assert np.array_equal(np.isnan(ea), np.isnan(em))
    ok = ~np.isnan(ea)
    assert np.array_equal(ea[ok], em[ok])
    for j in others + [jm]:
        info = mix.job(j)
        assert info["state"] == 3 and info["sweeps_done"] > 0 and info["first_bin"] >= info["admitted"]
    assert mix.bead_updates() > 0
    # rounds of 0.2 ms stop most sweeps part-way: the resumed sweeps draw the
    # same numbers
    tiny = pgb.Server(2e9, sweeps_per_round=4, bin_sweeps=10, grand_canonical=True, round_seconds=0.0002)
    jt = tiny.submit(**X)
    b_tiny = [b for b in _run(tiny, [jt]) if b["job"] == jt]
    assert [(b["bin"], b["samples"]) for b in b_tiny] == [(b["bin"], b["samples"]) for b in b_alone]
    et = np.array([b["energy"] for b in b_tiny])
    assert np.array_equal(np.isnan(ea), np.isnan(et)) and np.array_equal(ea[ok], et[ok])


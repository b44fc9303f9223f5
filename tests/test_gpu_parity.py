"""GPU parity of the C ABI against the FP64 oracle.

Tolerances (stated per the workload's precision rules):
  * plain FP64 form: |gpu - oracle| <= 1e-12 * max(|oracle|, 1); both sides
    evaluate each pair term with the same IEEE operations (the kernels are
    built with -fmad=false, the oracle with -ffp-contract=off), so differences
    come only from summation order;
  * mixed form (FP32 analytic Aziz pairs, FP64 accumulation): per-bead
    actions within 2e-4 relative of the FP64 oracle (the oracle's piecewise-
    constant table alone differs from the analytic potential by |V'| dr),
    estimator totals within 1e-4 relative.
"""
import math

import numpy as np
import pytest

from helpers import benchmark_samples, make_pair, random_beads, rel_err

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


@pytest.fixture(scope="module")
def small(pgb, oracle_lib):
    n, m, L, lam, tau = 24, 16, 9.5, 6.0596, 0.004
    cfg = pgb.worldlines.seeded_worldlines(n, m, L, lam, tau, 21)
    return dict(n=n, m=m, L=L, lam=lam, tau=tau, cfg=cfg)


def test_tables_match_oracle(pgb, oracle_lib):
    L = 9.0107
    a = pgb.Action(L, 4, 2, 0.004, 6.0596)
    o = oracle_lib.Oracle(L, 4, 2, 0.004, 6.0596)
    n, dr, tail = a.table_info()
    assert n == o.table_length()
    assert tail == o.tailV()
    V, dV, d2V = a.tables()
    oV, odV, od2V = o.tables()
    # device exp may differ from libm's by an ulp
    for x, y in ((V, oV), (dV, odV), (d2V, od2V)):
        assert rel_err(x, y, floor=1.0) < 1e-13


def test_potential_batch_benchmark_samples(pgb, oracle_lib):
    """potential_benchmark batch check (1e-9) on its own samples, GPU vs oracle."""
    L = 22.709
    a = pgb.Action(L, 4, 2, 0.004, 6.0596)
    o = oracle_lib.Oracle(L, 4, 2, 0.004, 6.0596)
    s = benchmark_samples()
    want = np.array([o.V(x) for x in s])
    for bs in (1, 7, 257, len(s)):
        got = np.concatenate([a.V_batch(s[b:b + bs]) for b in range(0, len(s), bs)])
        assert rel_err(got, want) <= 1e-14
    g = a.gradV_batch(s)
    assert rel_err(g, np.array([o.gradV(x) for x in s])) <= 1e-14
    assert rel_err(a.grad2V_batch(s), np.array([o.grad2V(x) for x in s])) <= 1e-14


@pytest.mark.parametrize("action", ["primitive", "gsf", "li_broughton"])
@pytest.mark.parametrize("rc", [None, 4.5])
def test_bead_actions_fp64(pgb, oracle_lib, small, action, rc):
    d = small
    a, o = make_pair(pgb, oracle_lib, d["cfg"], d["L"], d["m"], d["n"], d["tau"], d["lam"],
                     rc=rc, action=action)
    rng = np.random.default_rng(5)
    beads = random_beads(rng, d["m"], d["n"], 40)
    for mode in (0, 1, 2):
        for shift in (1, 2):
            o.set_shift(shift)
            want = np.array([o.bead_action(int(s), int(p), mode) for s, p in beads])
            got, tot = a.bead_actions(beads, shift=shift, mode=mode)
            assert rel_err(got, want) <= TOL64, (mode, shift)
            assert abs(tot - want.sum()) <= TOL64 * max(1.0, np.abs(want).sum())
    o.set_shift(1)


def test_range_list_full_kinetic_fp64(pgb, oracle_lib, small):
    d = small
    a, o = make_pair(pgb, oracle_lib, d["cfg"], d["L"], d["m"], d["n"], d["tau"], d["lam"],
                     action="gsf")
    assert abs(a.range_action((3, 5), (10, 5)) - o.range_action((3, 5), (10, 5))) <= TOL64 * 100
    assert abs(a.range_action((12, 2), (1, 2)) - o.range_action((12, 2), (1, 2))) <= TOL64 * 100
    fu, ofu = a.full_action(), o.full_action()
    assert abs(fu - ofu) <= TOL64 * max(1, abs(ofu))
    k, ok = a.kinetic_action(), o.kinetic_action()
    assert abs(k - ok) <= TOL64 * max(1, abs(ok))


def test_slice_terms_fp64(pgb, oracle_lib, small):
    d = small
    a, o = make_pair(pgb, oracle_lib, d["cfg"], d["L"], d["m"], d["n"], d["tau"], d["lam"],
                     action="gsf")
    t = a.slice_terms()
    tau, lam = d["tau"], d["lam"]
    vf, gf = (2 / 3, 4 / 3), (0.0, 2 / 9)
    for s in range(d["m"]):
        eo = s % 2
        assert abs(t["vint"][s] - o.V_slice(s)[1]) <= TOL64 * max(1, abs(t["vint"][s]))
        assert abs(t["g2"][s] - o.slice_fn("gradVSquared_slice", s)) <= TOL64 * max(1, t["g2"][s])
        assert abs(vf[eo] * tau * t["r1"][s] - o.slice_fn("rdotgradU1", s)) <= TOL64 * max(1, abs(t["r1"][s]))
        assert abs(vf[eo] * tau * t["d1"][s] - o.slice_fn("deltadotgradU1", s)) <= TOL64 * max(1, abs(t["d1"][s]))
        c = 2.0 * gf[eo] * tau ** 3 * lam
        assert abs(c * t["r2"][s] - o.slice_fn("rdotgradU2", s)) <= TOL64 * max(1, abs(c * t["r2"][s]))
        assert abs(c * t["d2"][s] - o.slice_fn("deltadotgradU2", s)) <= TOL64 * max(1, abs(c * t["d2"][s]))


@pytest.mark.parametrize("action", ["primitive", "gsf"])
def test_energy_virial_fp64(pgb, oracle_lib, small, action):
    d = small
    a, o = make_pair(pgb, oracle_lib, d["cfg"], d["L"], d["m"], d["n"], d["tau"], d["lam"],
                     action=action, mu=-7.2)
    assert rel_err(a.energy(), o.energy()) <= TOL64
    for quirk in (True, False):
        assert rel_err(a.virial(quirk), o.virial(quirk)) <= 1e-11


def test_worm_factors_fp64(pgb, oracle_lib, small):
    d = small
    cfg = pgb.worldlines.open_worm(d["cfg"], head=(5, 3), tail=(9, 3))
    cfg["worm"][4:8] = [2, 7, 11, 0]      # special beads
    a, o = make_pair(pgb, oracle_lib, cfg, d["L"], d["m"], d["n"], d["tau"], d["lam"], action="gsf")
    beads = np.array([[5, 3], [9, 3], [5, 4], [9, 7], [2, 7], [11, 0], [6, 3], [2, 1]], np.int32)
    want = np.array([o.bead_action(int(s), int(p)) for s, p in beads])
    got, _ = a.bead_actions(beads)
    assert rel_err(got, want) <= TOL64
    assert got[6] == 0.0          # switched-off bead


def test_checkmove_identity_on_gpu(pgb, oracle_lib, small):
    """Full-path action change equals the per-bead change (move.cpp:184-246)."""
    d = small
    a, _ = make_pair(pgb, oracle_lib, d["cfg"], d["L"], d["m"], d["n"], d["tau"], d["lam"],
                     action="gsf")
    rng = np.random.default_rng(1)
    for _ in range(5):
        s, p = int(rng.integers(d["m"])), int(rng.integers(d["n"]))
        u0, (b0,) = a.full_action(), a.bead_actions([[s, p]])[0]
        r = a.positions()[s, p] + rng.normal(0, 0.2, 3)
        r -= d["L"] * np.floor(r / d["L"] + 0.5)
        a.update_beads([[s, p]], [r])
        u1, (b1,) = a.full_action(), a.bead_actions([[s, p]])[0]
        assert abs((u1 - u0) - (b1 - b0)) <= 1e-9 * max(1.0, abs(u0))


def test_pair_action_full_size(pgb, oracle_lib):
    """Pair-action workload at full size: N=256, M=250, GSF, rc = L and rc = 7."""
    w = pgb.worldlines.workload_pair_action()
    cfg = pgb.worldlines.seeded_worldlines(w["n"], w["m"], w["side"], w["lam"], w["tau"], 0)
    for rc in (None, 7.0):
        a, o = make_pair(pgb, oracle_lib, cfg, w["side"], w["m"], w["n"], w["tau"], w["lam"],
                         rc=rc, action="gsf")
        rng = np.random.default_rng(3)
        beads = random_beads(rng, w["m"], w["n"], 24)
        want = np.array([o.bead_action(int(s), int(p)) for s, p in beads])
        got, _ = a.bead_actions(beads)
        assert rel_err(got, want) <= TOL64
        assert abs(a.full_action() - o.full_action()) <= TOL64 * abs(o.full_action())
        m = pgb.Action(w["side"], w["m"], w["n"], w["tau"], w["lam"], rc=rc, action="gsf",
                       precision=pgb.PGB_MIXED)
        m.load(cfg)
        g32, _ = m.bead_actions(beads)
        assert rel_err(g32, want) <= 2e-4


def test_ssf_isf_fp64(pgb, oracle_lib, small):
    d = small
    a, o = make_pair(pgb, oracle_lib, d["cfg"], d["L"], d["m"], d["n"], d["tau"], d["lam"])
    L = d["L"]
    q = oracle_lib.qvectors("max_float", "2 0 0", [L, L, L])
    assert rel_err(a.ssf(q), o.ssf_pairwise(q)) <= 1e-12
    qi = q[:12]
    assert rel_err(a.isf(qi), o.isf_gpu_form(qi)) <= 1e-12
    assert rel_err(a.rhoq(qi), o.rhoq(qi), floor=1.0) <= 1e-12


def test_ssf_isf_mixed(pgb, oracle_lib):
    w = pgb.worldlines.workload_isf()
    n, m = 128, 64
    L = pgb.worldlines.box_side(n)
    cfg = pgb.worldlines.seeded_worldlines(n, m, L, w["lam"], w["tau"], 4)
    a, o = make_pair(pgb, oracle_lib, cfg, L, m, n, w["tau"], w["lam"], precision=pgb.PGB_MIXED)
    q, _ = pgb.worldlines.isf_qvectors(L, count=256)
    want = o.isf_rhoq(q, threads=4)
    got = a.isf(q, mode=0)
    # FP32 phases and products: absolute error against F ~ O(1) values
    assert np.max(np.abs(got - want)) <= 2e-4
    s = a.ssf(q)
    assert np.max(np.abs(s - want[:, 0])) <= 2e-4


def test_mixed_estimators(pgb, oracle_lib, small):
    d = small
    a, o = make_pair(pgb, oracle_lib, d["cfg"], d["L"], d["m"], d["n"], d["tau"], d["lam"],
                     action="gsf", precision=pgb.PGB_MIXED)
    e, oe = a.energy(), o.energy()
    assert rel_err(e, oe, floor=10.0) <= 1e-4
    v, ov = a.virial(), o.virial()
    assert rel_err(v[[1, 2, 4, 7, 8, 10, 17]], ov[[1, 2, 4, 7, 8, 10, 17]], floor=10.0) <= 1e-3


def test_plain_form_reproduces_oracle_sequence(pgb, oracle_lib):
    """Same MT19937 seed -> same accept/reject sequence and worldlines."""
    n, m, L, lam, tau = 8, 32, 7.5, 6.0596, 0.01
    cfg = pgb.worldlines.seeded_worldlines(n, m, L, lam, tau, 4)
    T = 1 / (m * tau)
    for move in (1, 0):
        a, o = make_pair(pgb, oracle_lib, cfg, L, m, n, tau, lam)
        a.plain_seed(17)
        mt = oracle_lib.MT(17)
        ra = a.plain_run(2, mbar=8, temperature=T, diagonal_move=move, num_updates=60, trace_cap=500)
        ro = o.run_steps(mt, 2, mbar=8, temperature=T, diagonal_move=move, num_updates=60, trace_cap=500)
        assert np.array_equal(ra["trace"], ro["trace"])
        assert ra["attempted"] == ro["attempted"] and ra["accepted"] == ro["accepted"]
        assert np.max(np.abs(a.positions() - o.positions())) <= 1e-12
        assert rel_err(ra["energies"], ro["energies"]) <= 1e-11


def test_walkers_run_and_energy(pgb):
    w = pgb.worldlines.workload_walkers(num=16, seed=1)
    W = pgb.Walkers(w["n"], w["m"], w["temperature"], w["side"], w["mbar"], w["tau"], w["lam"],
                    seed=3, threads_per_walker=128)
    W.init()
    W.run(2, measure=1)
    st = W.stats()
    assert all(s["samples"] == 2 for s in st)
    assert all(s["attempted"][1] > 0 and 0 < s["accepted"][1] <= s["attempted"][1] for s in st)
    e32 = W.energy(pgb.PGB_MIXED)
    e64 = W.energy(pgb.PGB_FP64)
    assert np.all(np.isfinite(e32))
    assert rel_err(e32, e64, floor=10.0) <= 1e-4
    # determinism: same seed, same trajectory
    W2 = pgb.Walkers(w["n"], w["m"], w["temperature"], w["side"], w["mbar"], w["tau"], w["lam"],
                     seed=3, threads_per_walker=128)
    W2.init()
    W2.run(2, measure=1)
    assert [s["accepted"] for s in W2.stats()] == [s["accepted"] for s in st]
    assert np.array_equal(W2.positions(0), W.positions(0))


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 2e-4)])
def test_trial_displacements(pgb, oracle_lib, small, precision, tol):
    """Independent single-bead trial moves: delta U against the oracle's
    before/after potentialAction(bead)."""
    d = small
    a, o = make_pair(pgb, oracle_lib, d["cfg"], d["L"], d["m"], d["n"], d["tau"], d["lam"],
                     action="gsf", precision=precision)
    rng = np.random.default_rng(11)
    beads = random_beads(rng, d["m"], d["n"], 30)
    pos = d["cfg"]["pos"][beads[:, 0], beads[:, 1]] + rng.uniform(-0.3, 0.3, (30, 3))
    pos -= d["L"] * np.floor(pos / d["L"] + 0.5)
    got = a.trial_actions(beads, pos)
    want, scale = [], []
    for (s_, p_), r in zip(beads, pos):
        u0 = o.bead_action(int(s_), int(p_))
        old = d["cfg"]["pos"][s_, p_].copy()
        o.update_bead(int(s_), int(p_), r)
        u1 = o.bead_action(int(s_), int(p_))
        want.append(u1 - u0)
        o.update_bead(int(s_), int(p_), old)
        # the error of a difference is relative to the larger of its terms
        scale.append(max(abs(u0), abs(u1), 1.0))
    want = np.array(want)
    assert np.max(np.abs(got - want) / np.array(scale)) <= tol


def test_mixed_correction_follows_updates(pgb, oracle_lib, small):
    """Mixed GSF actions with rc covering the box take the O(n) correction
    through cached slice forces; the cache must follow every bead update and
    the on/off state of an open worm."""
    d = small
    for worm in (False, True):
        cfg = pgb.worldlines.open_worm(d["cfg"], head=(3, 2), tail=(9, 2)) if worm else d["cfg"]
        o = oracle_lib.Oracle(d["L"], d["m"], d["n"], d["tau"], d["lam"], action="gsf")
        o.load(cfg)
        a = pgb.Action(d["L"], d["m"], d["n"], d["tau"], d["lam"], action="gsf",
                       precision=pgb.PGB_MIXED)
        a.load(cfg)
        rng = np.random.default_rng(21)
        beads = random_beads(rng, d["m"], d["n"], 30)
        for step in range(3):
            want = np.array([o.bead_action(int(s), int(p)) for s, p in beads])
            got, _ = a.bead_actions(beads)
            scale = np.maximum(np.abs(want), 1.0)
            assert np.max(np.abs(got - want) / scale) <= 2e-4, (worm, step)
            # move a bead on an odd (gradient) slice that the next check reads
            s, p = int(beads[step, 0]) | 1, int(beads[step, 1])
            r = a.positions()[s, p] + rng.normal(0, 0.15, 3)
            r -= d["L"] * np.floor(r / d["L"] + 0.5)
            a.update_beads([[s, p]], [r])
            o.update_bead(s, p, r)


@pytest.mark.parametrize("precision", [0, 1])
def test_update_positions(pgb, oracle_lib, small, precision):
    """All positions replaced through the on-device transpose: positions,
    actions and S(q) follow, with links and worm kept."""
    d = small
    a, o = make_pair(pgb, oracle_lib, d["cfg"], d["L"], d["m"], d["n"], d["tau"], d["lam"],
                     action="gsf", precision=precision)
    cfg2 = pgb.worldlines.seeded_worldlines(d["n"], d["m"], d["L"], d["lam"], d["tau"], 99)
    a.bead_actions([[1, 1]])                 # builds any cached slice forces first
    a.update_positions(cfg2["pos"])
    o.load(dict(d["cfg"], pos=cfg2["pos"]))
    assert np.array_equal(a.positions(), cfg2["pos"])
    rng = np.random.default_rng(2)
    beads = random_beads(rng, d["m"], d["n"], 20)
    want = np.array([o.bead_action(int(s), int(p)) for s, p in beads])
    got, _ = a.bead_actions(beads)
    tol = TOL64 if precision == 0 else 2e-4
    assert np.max(np.abs(got - want) / np.maximum(np.abs(want), 1.0)) <= tol


def test_path_estimators_match_oracle(pgb, oracle_lib, small):
    """g(r) (exact histograms), winding sums and permutation cycles against the
    oracle, on the identity permutation and on one with exchange cycles."""
    d = small
    for cycles in ([], [(0, 1), (2, 3, 4), (5, 6, 7, 8)]):
        cfg = pgb.worldlines.permute(d["cfg"], cycles)
        a, o = make_pair(pgb, oracle_lib, cfg, d["L"], d["m"], d["n"], d["tau"], d["lam"])
        for s in (-1, 0, d["m"] - 1):
            assert np.array_equal(a.pair_correlation(s), o.pair_correlation(s)), s
        assert np.array_equal(a.permutation_cycles(), o.permutation_cycles())
        got, want = a.superfluid(), o.superfluid()
        # W^2 columns: sums of O(N M) minimum-image steps that cancel around
        # closed worldlines, compared with an absolute tolerance on that scale
        scale = d["n"] * d["m"] * d["L"]
        assert np.all(np.abs(got[:4] - want[:4]) <= (1e-12 * scale) ** 2 + 1e-12 * np.abs(want[:4]))
        assert np.array_equal(got[4:25], want[4:25])
        assert abs(got[25] - want[25]) <= 1e-12 * max(1.0, abs(want[25]))


def test_pair_correlation_large_and_mixed(pgb, oracle_lib):
    """The FP32-screened histogram at a size where many pairs sit near bin
    edges (N = 256, M = 32), on FP64 and mixed contexts: every count exact."""
    n, m, lam, tau = 256, 32, 6.0596, 0.004
    L = pgb.worldlines.box_side(n)
    cfg = pgb.worldlines.seeded_worldlines(n, m, L, lam, tau, 13)
    for prec in (pgb.PGB_FP64, pgb.PGB_MIXED):
        a, o = make_pair(pgb, oracle_lib, cfg, L, m, n, tau, lam, precision=prec)
        want = o.pair_correlation(-1)
        assert np.all(want[:40] > 0.0)
        assert np.array_equal(a.pair_correlation(-1), want)
        assert np.array_equal(a.pair_correlation(7), o.pair_correlation(7))


def test_permutation_cycles_open_worm_is_an_error(pgb, small):
    d = small
    cfg = pgb.worldlines.open_worm(d["cfg"], head=(3, 2), tail=(9, 2))
    a = pgb.Action(d["L"], d["m"], d["n"], d["tau"], d["lam"])
    a.load(cfg)
    with pytest.raises(pgb.PgbError):
        a.permutation_cycles()

"""Device-resident worm walkers (one warp per walker): path invariants after
many steps, determinism, and statistical agreement with the oracle's worm
engine, which the plain GPU form matches bit for bit, with either diagonal
move (bisection, the reference's default, or staging).

The walkers draw from Philox streams and evaluate FP32 pair sums, so the
comparison is of ensemble averages: the energy per particle and the particle
number over closed configurations, within four combined standard errors.
"""
import numpy as np
import pytest

from pimc_gb300 import worldlines as wl
from test_worm import check_path

pytestmark = pytest.mark.gpu

N, M, TAU, LAM = 8, 32, 0.01, 6.0596


def _walkers(pgb, num, seed, window=1, mu=0.0, diagonal_move=0):
    L = wl.box_side(N)
    W = pgb.WormWalkers(np.full(num, N), M, L, 8, TAU, LAM, mu=mu, window=window, seed=seed,
                        diagonal_move=diagonal_move)
    W.load_seeded(seed)
    return W, L


@pytest.mark.parametrize("diagonal_move", [0, 1], ids=["bisection", "staging"])
def test_worm_walkers_invariants_and_moves(pgb, diagonal_move):
    W, L = _walkers(pgb, 16, seed=3, window=-1, diagonal_move=diagonal_move)
    for _ in range(4):
        W.run(25)
        st = W.stats()
        assert np.all(st["error"] == 0), st["error"]
        for w in (0, 5, 15):
            check_path(W.path(w), M)
    st = W.stats()
    att, acc = st["attempted"].sum(axis=0), st["accepted"].sum(axis=0)
    # every move of the list was attempted and accepted somewhere
    assert np.all(att > 0) and np.all(acc > 0), (att, acc)
    assert np.all(st["samples"] > 0)
    # positions stay in the box
    p = W.path(0)
    assert np.all(np.abs(p["pos"][p["on"].astype(bool)]) <= L / 2 + 1e-5)


def test_worm_walkers_deterministic(pgb):
    runs = []
    for _ in range(2):
        W, _ = _walkers(pgb, 8, seed=9)
        W.run(30)
        runs.append((W.stats(), W.path(3)))
    (s0, p0), (s1, p1) = runs
    assert np.array_equal(s0["attempted"], s1["attempted"])
    assert np.array_equal(s0["energy_sum"], s1["energy_sum"])
    assert np.array_equal(p0["next"], p1["next"]) and np.array_equal(p0["pos"], p1["pos"])


@pytest.mark.parametrize("diagonal_move", [0, 1], ids=["bisection", "staging"])
def test_worm_walkers_match_oracle_statistically(pgb, oracle_lib, diagonal_move):
    # oracle: one long chain, binned, with the same diagonal move
    L = wl.box_side(N)
    cfg = wl.seeded_worldlines(N, M, L, LAM, TAU, 1, extent=3 * N)
    o = oracle_lib.Oracle(L, M, 3 * N, TAU, LAM)
    o.load(cfg)
    # at this small N with a window of one particle some chains keep the worm
    # open for thousands of steps (the walkers' statistics below skip such
    # walkers too): these MT seeds give chains that close
    mt = oracle_lib.MT({0: 7, 1: 5}[diagonal_move])
    kw = dict(mbar=8, temperature=1.0 / (M * TAU), initial_num_particles=N, window=1, mu=0.0,
              diagonal_move=diagonal_move)
    o.run_worm_steps(mt, 200, **kw)
    r = o.run_worm_steps(mt, 2400, **kw)
    e = r["energies"]
    n = r["num_particles"].astype(float)
    ok = ~np.isnan(e)
    assert ok.sum() > 500
    eb = [e[i:i + 200][ok[i:i + 200]].mean() for i in range(0, 2400, 200)]
    nb = [n[i:i + 200][ok[i:i + 200]].mean() for i in range(0, 2400, 200)]
    eo, se_o = np.mean(eb), np.std(eb, ddof=1) / np.sqrt(len(eb))
    no, sn_o = np.mean(nb), np.std(nb, ddof=1) / np.sqrt(len(nb))

    W, _ = _walkers(pgb, 256, seed=11, diagonal_move=diagonal_move)
    W.run(150)
    W.reset_stats()
    W.run(250)
    st = W.stats()
    assert np.all(st["error"] == 0)
    has = st["samples"] > 0
    ew = st["energy_sum"][has] / st["samples"][has]
    nw = st["n_sum"][has] / st["samples"][has]
    e_w, se_w = ew.mean(), ew.std(ddof=1) / np.sqrt(len(ew))
    n_w, sn_w = nw.mean(), nw.std(ddof=1) / np.sqrt(len(nw))
    assert abs(e_w - eo) <= 4.0 * np.hypot(se_w, se_o), (e_w, se_w, eo, se_o)
    assert abs(n_w - no) <= 4.0 * np.hypot(sn_w, sn_o) + 1e-9, (n_w, sn_w, no, sn_o)


@pytest.mark.parametrize("skip", [0, 1, 3, 6])
def test_parallel_normals_equal_serial_draws(pgb, skip):
    """A staging move's deviates made by the lanes together are the serial
    draws bit for bit, and leave the stream at the same position."""
    import ctypes as C
    from pimc_gb300 import _lib
    lib = _lib.load()
    for count in (1, 7, 45, 189):
        a = np.zeros(count, dtype=np.float32)
        b = np.zeros(count, dtype=np.float32)
        st = np.zeros(6, dtype=np.int32)
        rc = lib.pgb_worm_normals_check(12345 + skip, skip, count,
                                        a.ctypes.data_as(_lib._FP), b.ctypes.data_as(_lib._FP),
                                        st.ctypes.data_as(_lib._IP))
        assert rc == 0
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (count, a[:4], b[:4])
        assert np.array_equal(st[:3], st[3:]), st
        assert np.all(np.isfinite(a)) and abs(a.std() - 1.0) < 0.6 if count > 40 else True


def test_worm_walker_with_full_slices_stops_alone(pgb):
    """A walker whose slices are full (capacity = N) stops with error 1 on its
    first bead insertion, its arrays untouched beyond their capacity; the
    other walkers run on."""
    L = wl.box_side(N)
    W = pgb.WormWalkers(np.full(4, N), M, L, 8, TAU, LAM, mu=0.0, window=-1, seed=5,
                        capacity=np.array([N, 2 * N + 8, 2 * N + 8, 2 * N + 8]))
    W.load_seeded(5)
    W.run(40)
    st = W.stats()
    assert st["error"][0] == 1, st["error"]
    assert np.all(st["error"][1:] == 0), st["error"]
    assert np.all(st["sweeps"][1:] == 40) and st["sweeps"][0] < 40
    p = W.path(0)
    assert np.all(p["nbs"] <= N)
    check_path(W.path(1), M)


@pytest.mark.parametrize("diagonal_move", [0, 1], ids=["bisection", "staging"])
def test_worm_walkers_grand_canonical_match_oracle_statistically(pgb, oracle_lib, diagonal_move):
    """Grand canonical (no window) at mu = -2 K, as the serving jobs run:
    <N> and <E/N> over closed configurations agree with the oracle's worm
    engine within four combined standard errors."""
    mu = -2.0
    L = wl.box_side(N)
    cfg = wl.seeded_worldlines(N, M, L, LAM, TAU, 1, extent=3 * N)
    o = oracle_lib.Oracle(L, M, 3 * N, TAU, LAM, mu=mu)
    o.load(cfg)
    mt = oracle_lib.MT(17)
    kw = dict(mbar=8, temperature=1.0 / (M * TAU), initial_num_particles=N, window=-1, mu=mu,
              diagonal_move=diagonal_move)
    o.run_worm_steps(mt, 500, **kw)
    r = o.run_worm_steps(mt, 8000, **kw)
    e = r["energies"]
    n = r["num_particles"].astype(float)
    ok = ~np.isnan(e)
    assert ok.sum() > 1000
    eb = [e[i:i + 500][ok[i:i + 500]].mean() for i in range(0, 8000, 500)]
    nb = [n[i:i + 500][ok[i:i + 500]].mean() for i in range(0, 8000, 500)]
    eo, se_o = np.mean(eb), np.std(eb, ddof=1) / np.sqrt(len(eb))
    no, sn_o = np.mean(nb), np.std(nb, ddof=1) / np.sqrt(len(nb))

    W, _ = _walkers(pgb, 256, seed=21, window=-1, mu=mu, diagonal_move=diagonal_move)
    W.run(200)
    W.reset_stats()
    W.run(300)
    st = W.stats()
    assert np.all(st["error"] == 0)
    has = st["samples"] > 0
    ew = st["energy_sum"][has] / st["samples"][has]
    nw = st["n_sum"][has] / st["samples"][has]
    e_w, se_w = ew.mean(), ew.std(ddof=1) / np.sqrt(len(ew))
    n_w, sn_w = nw.mean(), nw.std(ddof=1) / np.sqrt(len(nw))
    assert abs(n_w - no) <= 4.0 * np.hypot(sn_w, sn_o), (n_w, sn_w, no, sn_o)
    assert abs(e_w - eo) <= 4.0 * np.hypot(se_w, se_o), (e_w, se_w, eo, se_o)


@pytest.mark.parametrize("n", [8, 48, 112], ids=["one_warp", "pair_team", "quad_team"])
def test_walker_pair_sums_match_fp64_oracle(pgb, oracle_lib, n):
    """The walkers' FP32 pair sums (Kahan lanes, double-float warp reduction)
    against the FP64 oracle's barePotentialAction on the walkers' own paths
    after some steps (worm open or closed, special beads set): within 2e-4
    relative, most of it the oracle's piecewise-constant table (|V'| dr).
    N = 48 walkers run as two-warp teams, N = 112 as four-warp teams."""
    L = wl.box_side(n)
    W = pgb.WormWalkers(np.full(8, n), M, L, 8, TAU, LAM, mu=-1.0, window=-1, seed=13)
    W.seed_device(13)
    W.equilibrate(10)
    W.run(30)
    assert np.all(W.stats()["error"] == 0)
    rng = np.random.default_rng(2)
    for w in range(8):
        p = W.path(w)
        check_path(p, M)
        o = oracle_lib.Oracle(L, M, int(W.capacity[w]), TAU, LAM, mu=-1.0)
        o.load(p)
        act = np.argwhere(p["on"])
        beads = act[rng.choice(len(act), size=min(40, len(act)), replace=False)].astype(np.int32)
        got = W.bead_actions(w, beads)
        want = np.array([o.bead_action(int(t), int(q), mode=1) for t, q in beads])
        assert np.max(np.abs(got - want) / np.maximum(np.abs(want), 1.0)) <= 2e-4, w


@pytest.mark.parametrize("n", [48, 100], ids=["pair_team", "quad_team"])
def test_team_walkers_match_oracle_statistically(pgb, oracle_lib, n):
    """Walkers of 32 <= N0 < 64 run as two-warp teams, N0 >= 64 as four-warp
    teams (pair sums and energy samples split over the warps): grand canonical
    at mu = -1 K, M = 16, <E/N> and <N> over closed configurations within
    four combined standard errors of the oracle's worm engine; a team walker
    and the same walker run twice give the same chain."""
    m, tau, mu = 16, 0.01, -1.0
    L = wl.box_side(n)
    cfg = wl.seeded_worldlines(n, m, L, LAM, tau, 1, extent=3 * n)
    kw = dict(mbar=8, temperature=1.0 / (m * tau), initial_num_particles=n, window=-1, mu=mu,
              diagonal_move=0)
    es, ns = [], []
    for seed in range(6):
        o = oracle_lib.Oracle(L, m, 3 * n, tau, LAM, mu=mu)
        o.load(cfg)
        mt = oracle_lib.MT(31 + seed)
        o.run_steps(mt, 60, mbar=8, temperature=kw["temperature"], diagonal_move=1, p_com=0.05)
        o.run_worm_steps(mt, 100, **kw)
        r = o.run_worm_steps(mt, 500, **kw)
        ok = ~np.isnan(r["energies"])
        if ok.sum() > 20:
            es.append(r["energies"][ok].mean())
            ns.append(r["num_particles"][ok].mean())
    assert len(es) >= 4
    eo, se_o = np.mean(es), np.std(es, ddof=1) / np.sqrt(len(es))
    no, sn_o = np.mean(ns), np.std(ns, ddof=1) / np.sqrt(len(ns))

    runs = []
    for _ in range(2):
        W = pgb.WormWalkers(np.full(64, n), m, L, 8, tau, LAM, mu=mu, window=-1, seed=7)
        W.seed_device(7)
        W.equilibrate(60)
        W.run(100)
        W.reset_stats()
        W.run(500)                  # the oracle's window: N still drifts up from N0 after 160 steps
        runs.append((W.stats(), W.path(5)))
    (st, p0), (st1, p1) = runs
    assert np.array_equal(st["energy_sum"], st1["energy_sum"])
    assert np.array_equal(p0["pos"], p1["pos"]) and np.array_equal(p0["next"], p1["next"])
    assert np.all(st["error"] == 0)
    check_path(p0, m)
    has = st["samples"] > 20
    ew = st["energy_sum"][has] / st["samples"][has]
    nw = st["n_sum"][has] / st["samples"][has]
    e_w, se_w = ew.mean(), ew.std(ddof=1) / np.sqrt(len(ew))
    n_w, sn_w = nw.mean(), nw.std(ddof=1) / np.sqrt(len(nw))
    assert abs(e_w - eo) <= 4.0 * np.hypot(se_w, se_o), (e_w, se_w, eo, se_o)
    assert abs(n_w - no) <= 4.0 * np.hypot(sn_w, sn_o), (n_w, sn_w, no, sn_o)


def test_walker_chain_independent_of_the_mix(pgb):
    """A walker's chain depends only on its own parameters and stream, not on
    the walkers beside it.  Walker 0 (N0 = 48, a two-warp team) and walker 1
    (N0 = 80, a four-warp team) give the same statistics and paths in two
    mixes that place walker 0 first and then second of its CTA's two-warp
    teams, one mix with an odd number of two-warp walkers (a CTA with an
    empty second place) and small walkers beside them."""
    m, tau, mu = 16, 0.01, -1.0
    out = []
    for ns in ([48, 80, 48, 10, 20], [48, 80, 50, 33, 100, 8]):
        ns = np.array(ns)
        W = pgb.WormWalkers(ns, m, wl.box_side(ns), 8, tau, LAM, mu=mu, window=-1, seed=21)
        W.seed_device(21)
        W.equilibrate(20)
        W.run(40)
        st = W.stats()
        assert np.all(st["error"] == 0)
        out.append((st, W.path(0), W.path(1)))
        for w in range(len(ns)):
            check_path(W.path(w), m)
        W.close()
    (sa, a0, a1), (sb, b0, b1) = out
    for key in ("energy_sum", "n_sum", "samples", "attempted", "accepted", "bead_updates"):
        assert np.array_equal(sa[key][:2], sb[key][:2]), key
    for pa, pb in ((a0, b0), (a1, b1)):
        assert np.array_equal(pa["next"], pb["next"]) and np.array_equal(pa["pos"], pb["pos"])

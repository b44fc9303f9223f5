"""The oracle pinned to the reference itself.

tests/golden/reference_golden.json holds outputs of the reference's own
sources (compiled unchanged into oracle/_ref, see oracle/ref_harness.cpp and
tests/golden/make_ref_golden.py) on seeded inputs that pimc_gb300.worldlines
regenerates.  These tests hold the oracle's restatement to them:

* Aziz table lookups and the tail correction: equal bit for bit;
* per-bead, full-path and kinetic actions and one energy, virial, S(q) and
  F(q,tau) sample, primitive and GSF, the cutoff at the box side and below it
  (the reference's cell-grid neighbour lists): within 1e-12 relative, the
  difference being summation order only;
* PathIntegralMonteCarlo::step() with the default move list from the same
  worldlines and MTRand seed: the same per-move attempted and accepted
  counts, the same links, active flags, worm locators and generator state,
  positions within 1e-12.

With the reference tree present, a second set of configurations is run on
the reference live (skipped elsewhere).  No GPU is needed.
"""
import json
import math
import os

import numpy as np
import pytest

from pimc_gb300 import worldlines as wl

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = json.load(open(os.path.join(HERE, "golden", "reference_golden.json")))
LAM = FIX["lambda"]
REL = 1e-12


def _rel(a, b, floor=1.0):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if a.size else 0.0


def _qvectors(oracle_lib, side):
    return oracle_lib.qvectors("int", FIX["q_int"], [side, side, side])


def test_potential_matches_reference(oracle_lib):
    from helpers import benchmark_samples
    p = FIX["potential"]
    n, L = p["n"], p["side"]
    o = oracle_lib.Oracle(L, 16, n, 1.0 / 32.0, LAM)
    assert o.table_length() == p["table_length"]
    assert o.tailV() == p["tailV"]
    sep = benchmark_samples(count=512)
    V = np.array([o.V(s) for s in sep])
    g = np.array([o.gradV(s) for s in sep])
    g2 = np.array([o.grad2V(s) for s in sep])
    assert np.array_equal(V, np.array(p["V"]))
    assert np.array_equal(g, np.array(p["gradV"]))
    assert np.array_equal(g2, np.array(p["grad2V"]))


def _oracle_for(oracle_lib, c, extent=None):
    n, m, T, L = c["n"], c["m"], c["temperature"], c["side"]
    tau = 1.0 / (m * T)
    cfg = wl.seeded_worldlines(n, m, L, LAM, tau, c["seed"], extent=extent)
    o = oracle_lib.Oracle(L, m, extent or n, tau, LAM, rc=c.get("rc"), action=c.get("action", "primitive"),
                          mu=c.get("mu", 0.0))
    o.load(cfg)
    return o


@pytest.mark.parametrize("case", FIX["actions"], ids=[c["name"] for c in FIX["actions"]])
def test_actions_and_estimators_match_reference(oracle_lib, case):
    o = _oracle_for(oracle_lib, case)
    beads = np.array(case["beads"])
    for shift in (1, 2):
        o.set_shift(shift)
        want = case["shift%d" % shift]
        for mode, key in ((0, "full"), (1, "bare"), (2, "corr")):
            got = [o.bead_action(int(t), int(p), mode=mode) for t, p in beads]
            assert _rel(got, want[key]) <= REL, (shift, key)
    o.set_shift(1)
    assert _rel(o.full_action(), case["full_action"]) <= REL
    assert _rel(o.kinetic_action(), case["kinetic_action"]) <= REL
    assert _rel(o.energy(), case["energy"]) <= REL
    assert _rel(o.virial(quirk=True), case["virial"]) <= 1e-11
    q = _qvectors(oracle_lib, case["side"])
    assert _rel(o.ssf_pairwise(q), case["ssf"]) <= REL
    assert _rel(o.isf_cpu_form(q).ravel(), case["isf"]) <= REL


def _check_trace(oracle_lib, c):
    ne = max(c["extent"], 3 * c["n"])
    o = _oracle_for(oracle_lib, c, extent=ne)
    mt = oracle_lib.MT(c["mt_seed"])
    r = o.run_worm_steps(mt, c["steps"], mbar=c["mbar"], temperature=c["temperature"],
                         initial_num_particles=c["n"], window=c["window"], mu=c["mu"],
                         diagonal_move=1 if c["staging"] else 0)
    assert list(r["attempted"]) == c["attempted"]
    assert list(r["accepted"]) == c["accepted"]
    p = o.path()
    e = c["extent"]
    assert p["nbs"].tolist() == c["nbs"]
    assert p["worm"].tolist() == c["worm"]
    assert np.array_equal(p["on"][:, :e], np.array(c["on"], dtype=np.uint8))
    assert not p["on"][:, e:].any()
    assert np.array_equal(p["next"][:, :e], np.array(c["next"]))
    assert np.array_equal(p["prev"][:, :e], np.array(c["prev"]))
    on = np.array(c["on"], dtype=bool)
    assert np.max(np.abs(p["pos"][:, :e][on] - np.array(c["pos"])[on])) <= 1e-12
    assert np.array_equal(mt.save(), np.array(c["rng"], dtype=np.uint32))
    want = np.array([np.nan if x is None else x for x in c["energies"]])
    closed = ~np.isnan(want)
    assert np.array_equal(closed, ~np.isnan(r["energies"]))
    if closed.any():
        assert _rel(r["energies"][closed], want[closed]) <= 1e-10


@pytest.mark.parametrize("case", FIX["traces"], ids=[c["name"] for c in FIX["traces"]])
def test_worm_steps_match_reference(oracle_lib, case):
    _check_trace(oracle_lib, case)


# ---- live cross-check on further configurations (reference tree only) ----

def _ref_or_skip():
    import pyref
    if not pyref.available():
        pytest.skip("the reference tree is absent")
    return pyref


@pytest.mark.parametrize("seed,action,rc", [(31, "gsf", None), (32, "gsf", 5.0), (33, "primitive", 3.5)])
def test_actions_match_live_reference(oracle_lib, seed, action, rc):
    pyref = _ref_or_skip()
    n, m, T = 20, 10, 2.5
    L = wl.box_side(n)
    tau = 1.0 / (m * T)
    cfg = wl.seeded_worldlines(n, m, L, LAM, tau, seed)
    r = pyref.Reference(cfg["pos"], L, T, LAM, rc=rc, gsf=(action == "gsf"))
    o = oracle_lib.Oracle(L, m, n, tau, LAM, rc=rc, action=action)
    o.load(cfg)
    for t in range(m):
        for p in range(0, n, 3):
            assert _rel(o.bead_action(t, p), r.bead_action(t, p)) <= REL
    assert _rel(o.energy(), r.estimator("energy")) <= REL
    assert _rel(o.virial(), r.estimator("virial")) <= 1e-11
    r.close()


@pytest.mark.parametrize("staging,canonical,mu", [(False, True, 0.0), (False, False, -1.0), (True, False, -3.0)])
def test_worm_steps_match_live_reference(oracle_lib, staging, canonical, mu):
    pyref = _ref_or_skip()
    n, m, T, mbar, steps = 10, 24, 2.0, 6, 15
    L = wl.box_side(n)
    tau = 1.0 / (m * T)
    cfg = wl.seeded_worldlines(n, m, L, LAM, tau, 41)
    r = pyref.Reference(cfg["pos"], L, T, LAM, mbar=mbar, staging=staging, canonical=canonical,
                        window=1 if canonical else -1, mu=mu, seed=77)
    closed, en = r.run_steps(steps)
    att, acc = r.move_stats()
    p = r.path()
    case = dict(n=n, m=m, temperature=T, seed=41, side=L, mt_seed=77, mbar=mbar, staging=staging,
                window=1 if canonical else -1, mu=mu, steps=steps, attempted=att.tolist(),
                accepted=acc.tolist(), extent=int(p["pos"].shape[1]), nbs=p["nbs"].tolist(),
                worm=p["worm"].tolist(), on=p["on"].tolist(), next=p["next"].tolist(),
                prev=p["prev"].tolist(), pos=p["pos"].tolist(), rng=r.rng_state().tolist(),
                energies=[None if not math.isfinite(x) else x for x in en])
    r.close()
    _check_trace(oracle_lib, case)

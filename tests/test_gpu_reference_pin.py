"""The plain FP64 GPU form against outputs of the reference itself.

tests/golden/reference_golden.json was computed by the reference's own
sources (tests/golden/make_ref_golden.py); the inputs are regenerated from
their seeds.  Through the C ABI on the GPU:

* per-bead potential actions (full, bare, correction; shifts 1 and 2), the
  full-path and kinetic actions and one energy, virial, S(q) and F(q,tau)
  sample, primitive and GSF, the cutoff at the box side and below it: within
  1e-12 relative (1e-11 for the 19 virial columns, products of several sums);
  F(q,tau) as the reference's GPU layout tau in [0, M/2], compared with the
  reference's CPU estimator, which is symmetric in tau -> M - tau;
* PathIntegralMonteCarlo::step() with the default move list from the same
  worldlines and MTRand seed, run by the plain form (host moves, FP64 device
  actions): the same per-move counts, links, active flags, worm locators and
  generator state, positions within 1e-12.
"""
import json
import os

import numpy as np
import pytest

from pimc_gb300 import worldlines as wl

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = json.load(open(os.path.join(HERE, "golden", "reference_golden.json")))
LAM = FIX["lambda"]
REL = 1e-12


def _rel(a, b, floor=1.0):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if a.size else 0.0


def _action(pgb, c, extent=None):
    n, m, T, L = c["n"], c["m"], c["temperature"], c["side"]
    tau = 1.0 / (m * T)
    cfg = wl.seeded_worldlines(n, m, L, LAM, tau, c["seed"], extent=extent)
    a = pgb.Action(L, m, extent or n, tau, LAM, rc=c.get("rc"), action=c.get("action", "primitive"),
                   precision=pgb.PGB_FP64, mu=c.get("mu", 0.0))
    a.load(cfg)
    return a


@pytest.mark.parametrize("case", FIX["actions"], ids=[c["name"] for c in FIX["actions"]])
def test_plain_form_actions_and_estimators_match_reference(pgb, case):
    a = _action(pgb, case)
    beads = np.array(case["beads"], dtype=np.int32)
    for shift in (1, 2):
        want = case["shift%d" % shift]
        for mode, key in ((pgb.PGB_ACTION_FULL, "full"), (pgb.PGB_ACTION_BARE, "bare"),
                          (pgb.PGB_ACTION_CORR, "corr")):
            got, _ = a.bead_actions(beads, shift=shift, mode=mode)
            assert _rel(got, want[key]) <= REL, (shift, key)
    assert _rel(a.full_action(), case["full_action"]) <= REL
    assert _rel(a.kinetic_action(), case["kinetic_action"]) <= REL
    assert _rel(a.energy(), case["energy"]) <= REL
    assert _rel(a.virial(cvcov2_quirk=True), case["virial"]) <= 1e-11
    q = pgb.qvectors("int", FIX["q_int"], [case["side"]] * 3)
    assert _rel(a.ssf(q), case["ssf"]) <= REL
    m = case["m"]
    isf_ref = np.array(case["isf"]).reshape(len(q), m)[:, :m // 2 + 1]
    assert _rel(a.isf(q, mode=0), isf_ref) <= REL
    a.close()


@pytest.mark.parametrize("case", FIX["traces"], ids=[c["name"] for c in FIX["traces"]])
def test_plain_form_worm_steps_match_reference(pgb, case):
    ne = max(case["extent"], 3 * case["n"])
    a = _action(pgb, case, extent=ne)
    a.plain_seed(case["mt_seed"])
    r = a.plain_worm_run(case["steps"], mbar=case["mbar"], temperature=case["temperature"],
                         initial_num_particles=case["n"], window=case["window"], mu=case["mu"],
                         diagonal_move=1 if case["staging"] else 0)
    assert list(r["attempted"]) == case["attempted"]
    assert list(r["accepted"]) == case["accepted"]
    p = a.path()
    e = case["extent"]
    assert p["nbs"].tolist() == case["nbs"]
    assert p["worm"].tolist() == case["worm"]
    assert np.array_equal(p["on"][:, :e], np.array(case["on"], dtype=np.uint8))
    assert np.array_equal(p["next"][:, :e], np.array(case["next"]))
    assert np.array_equal(p["prev"][:, :e], np.array(case["prev"]))
    on = np.array(case["on"], dtype=bool)
    assert np.max(np.abs(p["pos"][:, :e][on] - np.array(case["pos"])[on])) <= 1e-12
    assert np.array_equal(a.rng_state(), np.array(case["rng"], dtype=np.uint32))
    a.close()

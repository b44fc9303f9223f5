"""Golden fixtures computed by the reference itself.

Runs the reference's own sources (compiled unchanged by oracle/Makefile.ref
into oracle/_ref/libpimc_ref.so, see oracle/ref_harness.cpp) on seeded
inputs and writes reference_golden.json next to this script.  The inputs are
regenerated from their seeds by pimc_gb300.worldlines (a deterministic numpy
Philox stream), so the file holds only the reference's outputs:

* the Aziz potential V, gradV, grad2V (direct table lookup) at the
  separation samples of tools/benchmarks/potential_benchmark.cpp and the
  tail correction;
* per-bead potential actions (LocalAction::potentialAction, bare and
  correction parts, shifts 1 and 2), the full-path potential action, the
  kinetic action and one sample of the energy and virial estimators, for the
  primitive and GSF actions with the cutoff at the box side and below it
  (where the reference's LookupTable cell grid builds the neighbour lists);
* one sample of the S(q) and F(q,tau) estimators (CPU forms);
* PathIntegralMonteCarlo::step() from seeded worldlines and an MTRand seed
  with the default move list: per-move attempted/accepted counts, the energy
  of every step that ended closed, and the final path (links, active
  flags, worm locators, positions).

Usage: python tests/golden/make_ref_golden.py   (needs the reference tree)
"""
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

from pimc_gb300 import worldlines as wl  # noqa: E402

# lambda as the reference derives it from its mass parameter (24.24 / m)
LAM = 24.24 / (24.24 / wl.LAMBDA_HE4)

ACTION_CASES = [
    # name, N, M, T, cfg seed, action, rc (None: the box side)
    ("primitive_rcL", 16, 16, 2.0, 3, "primitive", None),
    ("gsf_rcL", 16, 16, 2.0, 4, "gsf", None),
    ("gsf_rc4", 24, 12, 2.0, 5, "gsf", 4.0),
    ("primitive_rc4", 24, 12, 2.0, 6, "primitive", 4.0),
]
Q_INT = "1 0 0  0 1 0  1 1 0  2 0 1  -1 2 1  3 1 -2"
TRACE_CASES = [
    # name, N, M, T, cfg seed, MTRand seed, Mbar, staging, canonical, window, mu, steps
    ("staging_canonical", 8, 16, 2.0, 3, 11, 4, True, True, 1, 0.0, 20),
    ("bisection_canonical", 8, 16, 2.0, 3, 11, 4, False, True, 1, 0.0, 20),
    ("bisection_grand_canonical", 8, 16, 2.0, 3, 11, 4, False, False, -1, -2.0, 20),
    ("bisection_canonical_n12", 12, 20, 2.5, 7, 23, 4, False, True, 1, 0.0, 12),
]


def tau_of(m, t):
    return 1.0 / (m * t)


def action_beads(m, n):
    rng = np.random.Generator(np.random.Philox(99))
    return np.stack([rng.integers(0, m, 24), rng.integers(0, n, 24)], 1).astype(int)


def main():
    import pyref
    from helpers import benchmark_samples
    if not pyref.available():
        raise SystemExit("the reference tree is absent: nothing to generate")
    out = {"lambda": LAM, "q_int": Q_INT}

    # potential
    n, m, T = 16, 16, 2.0
    L = wl.box_side(n)
    cfg = wl.seeded_worldlines(n, m, L, LAM, tau_of(m, T), 3)
    r = pyref.Reference(cfg["pos"], L, T, LAM)
    sep = benchmark_samples(count=512)
    V, g, g2 = r.potential(sep)
    out["potential"] = dict(n=n, side=L, table_length=r.table_length(), tailV=r.tail_v(),
                            V=V.tolist(), gradV=g.tolist(), grad2V=g2.tolist())
    r.close()

    # actions and estimators
    out["actions"] = []
    for name, n, m, T, seed, action, rc in ACTION_CASES:
        L = wl.box_side(n)
        cfg = wl.seeded_worldlines(n, m, L, LAM, tau_of(m, T), seed)
        r = pyref.Reference(cfg["pos"], L, T, LAM, rc=rc, gsf=(action == "gsf"),
                            wavevector=Q_INT, wavevector_type="int")
        beads = action_beads(m, n)
        per = {}
        for shift in (1, 2):
            r.set_shift(shift)
            per[shift] = dict(full=[r.bead_action(int(t), int(p)) for t, p in beads],
                              bare=[r.bare_action(int(t), int(p)) for t, p in beads],
                              corr=[r.correction(int(t), int(p)) for t, p in beads])
        r.set_shift(1)
        out["actions"].append(dict(
            name=name, n=n, m=m, temperature=T, seed=seed, action=action, rc=rc, side=L,
            beads=beads.tolist(), shift1=per[1], shift2=per[2],
            full_action=r.full_action(), kinetic_action=r.kinetic_action(),
            energy=r.estimator("energy").tolist(), virial=r.estimator("virial").tolist(),
            ssf=r.estimator("ssf").tolist(), isf=r.estimator("isf").tolist()))
        r.close()

    # worm-algorithm steps
    out["traces"] = []
    for name, n, m, T, seed, mt_seed, mbar, staging, canonical, window, mu, steps in TRACE_CASES:
        L = wl.box_side(n)
        cfg = wl.seeded_worldlines(n, m, L, LAM, tau_of(m, T), seed)
        r = pyref.Reference(cfg["pos"], L, T, LAM, mbar=mbar, staging=staging, canonical=canonical,
                            window=window, mu=mu, seed=mt_seed)
        closed, en = r.run_steps(steps)
        att, acc = r.move_stats()
        p = r.path()
        out["traces"].append(dict(
            name=name, n=n, m=m, temperature=T, seed=seed, mt_seed=mt_seed, mbar=mbar,
            staging=staging, canonical=canonical, window=window, mu=mu, steps=steps, side=L,
            attempted=att.tolist(), accepted=acc.tolist(), closed=closed,
            energies=[None if not math.isfinite(e) else e for e in en],
            extent=int(p["pos"].shape[1]), nbs=p["nbs"].tolist(), worm=p["worm"].tolist(),
            next=p["next"].tolist(), prev=p["prev"].tolist(), on=p["on"].tolist(),
            pos=p["pos"].tolist(), rng=r.rng_state().tolist()))
        r.close()
    path = os.path.join(HERE, "reference_golden.json")
    with open(path, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()

"""Generate tests/golden/oracle_golden.json from the FP64 oracle.

The reference cannot be built in this image, so these fixtures pin the
oracle's own outputs: the oracle is compiled with -ffp-contract=off and must
reproduce them on every host (x86-64 here, aarch64 next to the GPU).

    python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]


def compute(pyoracle):
    from helpers import benchmark_samples
    from pimc_gb300 import worldlines
    out = {}
    s = benchmark_samples(256)
    out["aziz1979"] = [list(pyoracle.aziz_values(1979, float(np.sqrt((x ** 2).sum())))) for x in s[:64]]
    mt = pyoracle.MT(139853)
    out["mt_rand"] = [mt.rand() for _ in range(16)]
    out["mt_norm"] = [mt.randnorm(0.0, 1.0) for _ in range(16)]
    n, m, L, lam, tau = 10, 12, 7.5, 6.0596, 0.01
    cfg = worldlines.seeded_worldlines(n, m, L, lam, tau, 11)
    o = pyoracle.Oracle(L, m, n, tau, lam, action="gsf")
    o.load(cfg)
    out["energy_gsf"] = list(o.energy())
    out["virial_gsf"] = list(o.virial(True))
    out["full_action_gsf"] = [o.full_action()]
    out["bead_actions_gsf"] = [o.bead_action(sl, p) for sl in range(0, m, 3) for p in range(0, n, 3)]
    q = pyoracle.qvectors("max_int", "1 1 1", [L, L, L])
    out["ssf"] = list(o.ssf_pairwise(q))
    out["isf"] = o.isf_rhoq(q[:4]).ravel().tolist()
    return out


if __name__ == "__main__":
    import pyoracle
    pyoracle.build()
    res = compute(pyoracle)
    with open(os.path.join(HERE, "oracle_golden.json"), "w") as f:
        json.dump(res, f, indent=1)
    print("wrote", sum(len(v) for v in res.values()), "values")

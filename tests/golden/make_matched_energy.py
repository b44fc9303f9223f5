"""FP64 reference energies for the matched-energy check of the batched walkers.

The batched walkers (FP32 pair sums, Philox streams) are compared with the
FP64 oracle's worm engine (MT19937) at three points of the walker mix.  The
oracle side costs hours of host time at bench sizes, so it is computed once by
this script and committed as matched_energy.json; bench.py and the tests run
only the GPU side and compare with it.

Each point runs `replicas` independent oracle walkers from seeded closed
worldlines (uniform centres, N(0, 2 lambda tau) jitter): `pre` diagonal
pre-equilibration steps (staging and 5 % centre-of-mass moves, which relax
the overlapping particles of the seeded start), then the reference's default
move list (bisection as the diagonal move, worm constant C0 = 1) with a
canonical window of one particle, `equil` unsampled steps and `sweeps`
sampled steps.  Per replica it stores the mean E/N over the sampled steps
that ended closed (None when none did).

Usage: python tests/golden/make_matched_energy.py [--threads T] [--quick]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from pimc_gb300 import worldlines as wl  # noqa: E402

TAU = 0.004
# (N, T, replicas, pre-equilibration steps, equilibration steps, sampled steps)
POINTS = [(128, 1.0, 64, 100, 50, 200), (64, 2.0, 128, 60, 40, 300), (8, 4.0, 256, 60, 100, 600)]
WORM_CONSTANT = 1.0


def run_point(n, t, replicas, pre, equil, sweeps, threads, diagonal_move=0, seed0=20000):
    import pyoracle
    m = wl.even_slices(t, TAU)
    L = wl.box_side(n)
    mbar = wl.default_mbar(n, L ** 3, wl.LAMBDA_HE4, TAU, m)
    t0 = time.time()
    r = pyoracle.worm_walkers_cpu(np.full(replicas, n), np.full(replicas, m), np.full(replicas, L),
                                  np.full(replicas, mbar),
                                  np.arange(replicas, dtype=np.uint32) + seed0 + 1000 * n,
                                  TAU, wl.LAMBDA_HE4, sweeps, threads, nequil=equil, window=1,
                                  diagonal_move=diagonal_move, worm_constant=WORM_CONSTANT, npre=pre)
    e = r["energy"]
    ok = ~np.isnan(e)
    return dict(n=n, m=m, temperature=1.0 / (m * TAU), side=L, mbar=mbar, replicas=replicas,
                pre=pre, equil=equil, sweeps=sweeps, diagonal_move=diagonal_move,
                worm_constant=WORM_CONSTANT,
                energy_per_replica=[None if not np.isfinite(x) else float(x) for x in e],
                mean=float(e[ok].mean()), stderr=float(e[ok].std(ddof=1) / np.sqrt(ok.sum())),
                closed_replicas=int(ok.sum()), failed=int(r["failed"]),
                seconds=round(time.time() - t0, 1))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--quick", action="store_true", help="tiny sizes, to time the script")
    ap.add_argument("--out", default=os.path.join(HERE, "matched_energy.json"))
    a = ap.parse_args()
    import pyoracle
    pyoracle.build()
    res = []
    for (n, t, rep, pre, eq, sw) in POINTS:
        if a.quick:
            rep, pre, eq, sw = 8, 5, 5, 10
        r = run_point(n, t, rep, pre, eq, sw, a.threads)
        print("N=%d T=%.3f: E/N = %.5f +- %.5f (%d/%d closed replicas, %.0f s)"
              % (n, r["temperature"], r["mean"], r["stderr"], r["closed_replicas"], rep, r["seconds"]),
              flush=True)
        res.append(r)
    if not a.quick:
        json.dump({"tau": TAU, "lambda": wl.LAMBDA_HE4, "window": 1, "points": res},
                  open(a.out, "w"), indent=1)


if __name__ == "__main__":
    main()

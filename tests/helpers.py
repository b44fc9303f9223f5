"""Shared inputs for the parity tests."""
import math

import numpy as np


def benchmark_samples(count=4096, rmin=0.25, rmax=5.0):
    """Deterministic separation vectors of tools/benchmarks/potential_benchmark.cpp
    (sampleVector, lines 103-117) plus its six fixed GPU-check points (129-150)."""
    out = []
    for i in range(count):
        t = (i % count) / (count - 1) if count > 1 else 0.0
        radius = rmin + (rmax - rmin) * t
        r = [radius * math.sin(0.731 * (i + 1) * (d + 1)) for d in range(3)]
        if r[0] * r[0] + r[1] * r[1] + r[2] * r[2] < 1.0e-7:
            r[0] = rmin
        out.append(r)
    out += [[0.1, 0.2, 1.0], [3.1, 0.0, 1.9], [-4.0, 2.5, -3.0], [5.5, 0.25, 6.75],
            [-6.0, -3.0, 7.5], [0.0, 6.5, -6.6]]
    return np.array(out, dtype=np.float64)


def rel_err(a, b, floor=1.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))


def random_beads(rng, m, n, k):
    return np.stack([rng.integers(0, m, size=k), rng.integers(0, n, size=k)], axis=1).astype(np.int32)


def make_pair(pgb, oracle, cfg, side, m, ne, tau, lam, rc=None, action="primitive",
              precision=0, mu=0.0):
    a = pgb.Action(side, m, ne, tau, lam, rc=rc, action=action, precision=precision, mu=mu)
    o = oracle.Oracle(side, m, ne, tau, lam, rc=rc, action=action, mu=mu)
    a.load(cfg)
    o.load(cfg)
    return a, o

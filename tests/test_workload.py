"""The bench's synthetic workloads on CPU: the batched-walker mix follows the
reference's rules for its parameters (M even, T reset to 1/(M tau), Mbar
from setup.cpp:1079-1104), and the F(q,tau) q list holds lattice vectors
inside |q| <= 4 1/A, distinct, in a fixed order."""
import math

import numpy as np

from pimc_gb300 import worldlines as wl


def test_walker_mix_follows_the_reference_rules():
    w = wl.workload_walkers(num=1024, seed=0)
    n, m, t, side, mbar = w["n"], w["m"], w["temperature"], w["side"], w["mbar"]
    assert len(n) == 1024 and n.min() >= 8 and n.max() <= 128
    assert np.all(m % 2 == 0)                               # the reference forces M even
    assert np.allclose(t, 1.0 / (m * w["tau"]))
    assert np.all((t >= 0.9) & (t <= 4.2))
    assert np.allclose(side ** 3, n / wl.DENSITY)            # Prism(density, N)
    # Mbar = int(ell^2 / (16 lambda tau)), ell = (N / V)^(-1/3), made even:
    # 32 at the bench's density, tau and lambda
    ell = wl.DENSITY ** (-1.0 / 3.0)
    assert int(ell * ell / (16 * wl.LAMBDA_HE4 * w["tau"])) == 32
    assert np.all(mbar == 32)
    assert np.all(mbar < m)
    # the same seed gives the same mix
    w2 = wl.workload_walkers(num=1024, seed=0)
    assert np.array_equal(w2["n"], n) and np.array_equal(w2["m"], m)


def test_default_mbar_edge_cases():
    lam, tau = wl.LAMBDA_HE4, 0.004
    # a dense box gives an update length below 2: raised to 2
    assert wl.default_mbar(1000, 10.0, lam, tau, 64) == 2
    # a dilute box gives one above M: M / 2, then made even
    assert wl.default_mbar(1, 1.0e6, lam, tau, 20) == 10
    assert wl.default_mbar(1, 1.0e6, lam, tau, 22) == 12


def test_isf_qvectors_are_distinct_lattice_vectors():
    L = wl.box_side(512)
    q, nvec = wl.isf_qvectors(L, count=2048, seed=0)
    assert q.shape == (2048, 3) and nvec.shape == (2048, 3)
    assert np.allclose(q, 2 * math.pi / L * nvec)
    assert np.all(np.sqrt((q ** 2).sum(1)) <= 4.0 + 1e-12)
    assert len({tuple(v) for v in nvec.tolist()}) == 2048
    q2, _ = wl.isf_qvectors(L, count=2048, seed=0)
    assert np.array_equal(q, q2)

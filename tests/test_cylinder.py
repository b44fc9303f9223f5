"""Cylinder structure factor (CylinderStaticStructureFactorEstimator and its
GPU counterpart) and the shell q-vectors of getQVectors2.

The device sums the densities of the beads inside x^2 + y^2 < R^2; the
oracle restates the reference CPU estimator's pair loop.  The q lists are
lattice vectors (the line geometry's q = (0, 0, n 2 pi / L_z) and max_float
lists), for which the min-image and raw separations give the same cosine.
"""
import numpy as np
import pytest

from helpers import make_pair


def test_qvector_shells_match_oracle(pgb, oracle_lib):
    for L in (9.0, 17.3, 28.6):
        for sphere in (False, True):
            q, sh = pgb.qvectors_shells(2 * np.pi / L, 4.0, sphere)
            oq, osh = oracle_lib.qvectors_shells(2 * np.pi / L, 4.0, sphere)
            assert np.array_equal(q, oq) and np.array_equal(sh, osh)
            assert np.array_equal(q[0], [0.0, 0.0, 0.0]) and sh[-1] == int(4.0 / (2 * np.pi / L) + 1e-7)
    q, sh = pgb.qvectors_shells(2 * np.pi / 10.0, 4.0, False)
    assert len(q) == sh[-1] + 1 and np.all(q[:, :2] == 0.0)


def _cyl_case(pgb, seed=5):
    n, m, L, lam, tau = 64, 24, 12.0, 6.0596, 0.004
    cfg = pgb.worldlines.seeded_worldlines(n, m, L, lam, tau, seed)
    qline, _ = pgb.qvectors_shells(2 * np.pi / L, 4.0, False)
    qlat = pgb.qvectors("max_float", "1.6 0 0", [L, L, L])
    return n, m, L, lam, tau, cfg, np.concatenate([qline, qlat])


@pytest.mark.gpu
@pytest.mark.parametrize("max_r", [2.0, 3.5, 100.0])
def test_ssf_cylinder_fp64(pgb, oracle_lib, max_r):
    n, m, L, lam, tau, cfg, q = _cyl_case(pgb)
    a, o = make_pair(pgb, oracle_lib, cfg, L, m, n, tau, lam)
    got, n0 = a.ssf_cylinder(q, max_r)
    want, on0 = o.ssf_cylinder(q, max_r)
    assert n0 == on0
    scale = np.maximum(np.abs(want), 1.0)
    assert np.max(np.abs(got - want) / scale) <= 1e-10
    if max_r >= L:
        # every bead inside: the prism S(q) times N
        assert n0 == n
        assert np.max(np.abs(got / n - a.ssf(q)) / np.maximum(np.abs(a.ssf(q)), 1.0)) <= 1e-12


@pytest.mark.gpu
def test_ssf_cylinder_mixed(pgb, oracle_lib):
    n, m, L, lam, tau, cfg, q = _cyl_case(pgb, seed=9)
    a, o = make_pair(pgb, oracle_lib, cfg, L, m, n, tau, lam, precision=pgb.PGB_MIXED)
    for max_r in (2.5, 4.0):
        got, n0 = a.ssf_cylinder(q, max_r)
        want, on0 = o.ssf_cylinder(q, max_r)
        assert n0 == on0 and n0 > 0
        # FP32 phases: absolute error against values O(n_inside)
        assert np.max(np.abs(got - want)) <= 2e-4 * max(n0, 1)
    # the unmasked path is unchanged by the masked one
    s = a.ssf(q)
    assert np.max(np.abs(s - o.ssf_pairwise(q))) <= 2e-4


@pytest.mark.gpu
def test_ssf_cylinder_empty_and_argument_errors(pgb, oracle_lib):
    n, m, L, lam, tau, cfg, q = _cyl_case(pgb)
    a, _ = make_pair(pgb, oracle_lib, cfg, L, m, n, tau, lam)
    got, n0 = a.ssf_cylinder(q, 1e-6)
    assert n0 == 0 and np.all(got == 0.0)
    with pytest.raises(pgb.PgbError):
        a.ssf_cylinder(q, 0.0)

"""F(q,tau) on the tensor cores (tcgen05, split-BF16 DFT GEMMs) against the FP64
oracle's rho_q form and against the CUDA-core correlation.

Tolerance: 2e-4 absolute on F(q,tau) values of order one (FP32 densities plus
split-BF16 products with FP32 accumulation, relative error ~1e-5 per term)."""
import numpy as np
import pytest

from helpers import make_pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,m,nq", [(48, 128, 150), (96, 256, 300), (64, 512, 129)])
def test_isf_tensor_core_matches_oracle(pgb, oracle_lib, n, m, nq):
    lam, tau = pgb.worldlines.LAMBDA_HE4, 0.004
    L = pgb.worldlines.box_side(n)
    cfg = pgb.worldlines.seeded_worldlines(n, m, L, lam, tau, 17)
    a, o = make_pair(pgb, oracle_lib, cfg, L, m, n, tau, lam, precision=pgb.PGB_MIXED)
    q, _ = pgb.worldlines.isf_qvectors(L, count=nq, seed=5)
    want = o.isf_rhoq(q, threads=8)
    got_tc = a.isf(q, mode=1)
    got_cc = a.isf(q, mode=0)
    assert np.all(np.isfinite(got_tc))
    assert np.max(np.abs(got_tc - want)) <= 2e-4
    assert np.max(np.abs(got_tc - got_cc)) <= 2e-4


def test_isf_tensor_core_rejects_unsupported_m(pgb, oracle_lib):
    n, m = 16, 100
    L = pgb.worldlines.box_side(n)
    cfg = pgb.worldlines.seeded_worldlines(n, m, L, 6.0596, 0.004, 1)
    a = pgb.Action(L, m, n, 0.004, 6.0596, precision=pgb.PGB_MIXED)
    a.load(cfg)
    q, _ = pgb.worldlines.isf_qvectors(L, count=8)
    with pytest.raises(pgb.PgbError):
        a.isf(q, mode=1)

"""Failure detection on the GPU without a fault: a bounded wait that runs out.

The tensor-core F(q,tau) pipeline (tcgen05 MMAs fed by bulk copies through
mbarriers) bounds every wait to about a second.  pgb_test_isf_tc_stall makes
the first GEMM's producer stop before its last K chunk: no arrival and no copy
for that chunk, so the MMA thread's wait runs out (a barrier that nothing
completes).  Every copy that was issued has been consumed, so the CTA frees
its tensor memory and returns with the pipeline's error word set; the host
reads it and returns PGB_ETIMEOUT.  The context stays usable: with the switch
off, the next call matches the FP64 oracle again.
"""
import time

import numpy as np
import pytest

from helpers import make_pair

pytestmark = pytest.mark.gpu


def test_isf_tensor_core_wait_runs_out_and_context_survives(pgb, oracle_lib):
    n, m, nq = 16, 128, 40
    lam, tau = pgb.worldlines.LAMBDA_HE4, 0.004
    L = pgb.worldlines.box_side(n)
    cfg = pgb.worldlines.seeded_worldlines(n, m, L, lam, tau, 23)
    a, o = make_pair(pgb, oracle_lib, cfg, L, m, n, tau, lam, precision=pgb.PGB_MIXED)
    q, _ = pgb.worldlines.isf_qvectors(L, count=nq, seed=3)
    want = o.isf_rhoq(q, threads=4)
    assert np.max(np.abs(a.isf(q, mode=1) - want)) <= 2e-4
    lib = pgb._lib.load()
    lib.pgb_test_isf_tc_stall(1)
    try:
        t0 = time.perf_counter()
        with pytest.raises(pgb.PgbError) as e:
            a.isf(q, mode=1)
        waited = time.perf_counter() - t0
    finally:
        lib.pgb_test_isf_tc_stall(0)
    assert e.value.code == pgb._lib.PGB_ETIMEOUT
    assert "wait ran out" in str(e.value)
    assert waited < 30.0
    got = a.isf(q, mode=1)
    assert np.max(np.abs(got - want)) <= 2e-4
    assert np.max(np.abs(a.isf(q, mode=0) - want)) <= 2e-4
    a.close()

"""pgb_isf_static: F(q,tau) with no device allocation inside the call.

It serves callers that may not call cudaMalloc when they measure (device
memory reserved up front by a pool they do not own, or work allowed only
after set-up).  The test drives it through the C ABI with device buffers it
owns and checks two calls in a row against pgb_isf (mode 0, mixed precision)
on the same worldlines, within the mixed-path tolerance of the other tests
(2e-4 absolute on F(q,tau) values of order one).  The second call uses fewer
q-vectors, so a stale density left in the shared static array by the first
call would show up as a mismatch.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import make_pair

pytestmark = pytest.mark.gpu

TOL = 2e-4


def test_isf_static_matches_isf(pgb, oracle_lib):
    torch = pytest.importorskip("torch")
    lib = pgb._lib.load()
    n, m = 96, 64
    L = pgb.worldlines.box_side(n)
    lam, tau = pgb.worldlines.LAMBDA_HE4, 0.004
    cfg = pgb.worldlines.seeded_worldlines(n, m, L, lam, tau, 8)
    a, _ = make_pair(pgb, oracle_lib, cfg, L, m, n, tau, lam, precision=pgb.PGB_MIXED)
    q, _ = pgb.worldlines.isf_qvectors(L, count=200, seed=3)

    dev = torch.device("cuda", 0)
    d_beads = torch.from_numpy(np.ascontiguousarray(cfg["pos"])).to(dev)
    side = np.array([L, L, L])
    for nq in (200, 57):                      # two calls in a row on the shared array
        want = a.isf(q[:nq], mode=0)
        d_q = torch.from_numpy(np.ascontiguousarray(q[:nq])).to(dev)
        d_out = torch.full((nq, m // 2 + 1), float("nan"), dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        rc = lib.pgb_isf_static(C.c_void_p(d_beads.data_ptr()), m, n, n,
                                side.ctypes.data_as(C.POINTER(C.c_double)),
                                C.c_void_p(d_q.data_ptr()), nq, C.c_void_p(d_out.data_ptr()),
                                C.c_void_p(stream))
        assert rc == 0, lib.pgb_last_error(None)
        torch.cuda.synchronize(dev)
        got = d_out.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert np.max(np.abs(got - want)) <= TOL

    # sizes beyond the static limit are rejected with a message, nothing launched
    big = 1 << 16
    rc = lib.pgb_isf_static(C.c_void_p(d_beads.data_ptr()), m, n, n,
                            side.ctypes.data_as(C.POINTER(C.c_double)),
                            C.c_void_p(d_q.data_ptr()), big, C.c_void_p(d_out.data_ptr()), None)
    assert rc == -1 and b"static scratch limit" in lib.pgb_last_error(None)

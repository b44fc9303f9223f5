"""pgb_isf_static: F(q,tau) with no device allocation inside the call.

It serves callers that may not call cudaMalloc when they measure (device
memory reserved up front by a pool they do not own, or work allowed only
after set-up).  The test drives it through the C ABI with device buffers it
owns and checks two calls in a row against the oracle's FP64 rho_q form of
F(q,tau) on the same worldlines, within the mixed-path tolerance of the other
tests (2e-4 absolute on F(q,tau) values of order one).  The second call uses
other worldlines and other q-vectors than the first, and more of them, so a
density left in the shared static array by the first call and read again by
the second would show up as a mismatch.  The pgb_isf mode 0 value, which the
entry point is documented to equal, is checked beside the oracle.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import make_pair

pytestmark = pytest.mark.gpu

TOL = 2e-4


def test_isf_static_matches_oracle(pgb, oracle_lib):
    torch = pytest.importorskip("torch")
    lib = pgb._lib.load()
    n, m = 96, 64
    L = pgb.worldlines.box_side(n)
    lam, tau = pgb.worldlines.LAMBDA_HE4, 0.004
    dev = torch.device("cuda", 0)
    side = np.array([L, L, L])
    # two calls in a row on the shared array: different worldlines (seeds 8
    # and 9), different q-vectors (seeds 3 and 5), the second call larger
    for cfg_seed, q_seed, nq in ((8, 3, 120), (9, 5, 200)):
        cfg = pgb.worldlines.seeded_worldlines(n, m, L, lam, tau, cfg_seed)
        a, o = make_pair(pgb, oracle_lib, cfg, L, m, n, tau, lam, precision=pgb.PGB_MIXED)
        q, _ = pgb.worldlines.isf_qvectors(L, count=nq, seed=q_seed)
        want = o.isf_rhoq(q, threads=4)
        d_beads = torch.from_numpy(np.ascontiguousarray(cfg["pos"])).to(dev)
        d_q = torch.from_numpy(np.ascontiguousarray(q)).to(dev)
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
        assert np.max(np.abs(got - a.isf(q, mode=0))) <= TOL
        a.close()

    # sizes beyond the static limit are rejected with a message, nothing launched
    big = 1 << 16
    rc = lib.pgb_isf_static(C.c_void_p(d_beads.data_ptr()), m, n, n,
                            side.ctypes.data_as(C.POINTER(C.c_double)),
                            C.c_void_p(d_q.data_ptr()), big, C.c_void_p(d_out.data_ptr()), None)
    assert rc == -1 and b"static scratch limit" in lib.pgb_last_error(None)

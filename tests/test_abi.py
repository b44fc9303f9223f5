"""CPU tests of the C ABI boundary: the library builds for sm_103a, loads,
exports every entry point declared in include/pimc_gb300.h, and fails loudly
(an error code and message, never a CPU fallback) when no GPU is present."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "pimc_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pgb_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_what_binding_binds(pgb):
    assert declared_symbols() == pgb._lib.exported_symbols()


def test_library_exports_every_declared_symbol(pgb):
    lib = pgb._lib.load()
    out = subprocess.run(["nm", "-D", "--defined-only", pgb._lib.LIB_PATH],
                         capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (pgb_[a-z0-9_]+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    for s in declared_symbols():
        assert getattr(lib, s) is not None


def test_library_targets_sm103a(pgb):
    out = subprocess.run(["/usr/local/cuda/bin/cuobjdump", "--list-elf", pgb._lib.LIB_PATH],
                         capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    assert "sm_103a" in out.stdout


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device error path")
def test_create_fails_loudly_without_gpu(pgb):
    with pytest.raises(pgb.PgbError) as ei:
        pgb.Action(9.0, 4, 4, 0.004, 6.0596)
    assert ei.value.code == -2
    assert "CUDA" in str(ei.value) or "device" in str(ei.value)


def test_argument_validation_without_gpu(pgb):
    lib = pgb._lib.load()
    p = pgb._lib.PgbParams()
    h = C.c_void_p()
    assert lib.pgb_create(C.byref(p), C.byref(h)) == -1          # zero sizes
    assert b"invalid" in lib.pgb_last_error(None)
    assert lib.pgb_bead_actions(None, None, 0, 1, 0, None, None) == -1
    n = C.c_int()
    side = np.array([9.0, 9.0, 9.0])
    assert lib.pgb_qvectors(b"bogus", b"1 2 3", side.ctypes.data_as(C.POINTER(C.c_double)),
                            None, 0, C.byref(n)) == -1


def test_qvectors_host_logic_matches_oracle(pgb, oracle_lib):
    """getQVectors restated on the product host side equals the oracle's."""
    L = 9.0107
    for kind, text in [("max_float", "4 0 0"), ("max_int", "2 1 3"), ("int", "1 0 0 0 -2 3"),
                       ("float", "0.1 0.2 0.3")]:
        a = pgb.qvectors(kind, text, [L, L, L])
        b = oracle_lib.qvectors(kind, text, [L, L, L])
        assert a.shape == b.shape and np.array_equal(a, b), kind


def test_isf_static_rejects_sizes_on_the_host(pgb):
    """The allocation-free F(q,tau) checks its sizes before any CUDA call:
    too many slices for one q's densities in shared memory, too many
    particles for one slice, too many densities for the static array.  The
    pointers are placeholders that the host never dereferences."""
    lib = pgb._lib.load()
    side = np.array([9.0, 9.0, 9.0])
    sp = side.ctypes.data_as(C.POINTER(C.c_double))
    fake = C.c_void_p(0x1000)
    assert lib.pgb_isf_static(fake, 25602, 16, 16, sp, fake, 1, fake, None) == -1
    assert b"num_slices" in lib.pgb_last_error(None)
    assert lib.pgb_isf_static(fake, 64, 7000, 7000, sp, fake, 1, fake, None) == -1
    assert b"num_ptcl" in lib.pgb_last_error(None)
    assert lib.pgb_isf_static(fake, 64, 16, 16, sp, fake, 1 << 16, fake, None) == -1
    assert b"static scratch limit" in lib.pgb_last_error(None)
    assert lib.pgb_isf_static(fake, 64, 16, 8, sp, fake, 4, fake, None) == -1   # extent < N

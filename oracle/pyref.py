"""ctypes binding of oracle/_ref/libpimc_ref.so: the reference's own sources
compiled by oracle/Makefile.ref (test infrastructure only).

The library exists only where the reference tree is present (it is built from
its sources); `available()` says whether it could be built.  The tests that
pin the oracle to the reference skip without it, and the committed fixtures
in tests/golden/ carry its outputs to machines without the tree.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libpimc_ref.so")
REF = os.environ.get("PIMC_REFERENCE", "/root/reference")

_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int32)
_lib = None


class RefParams(C.Structure):
    _fields_ = [("side", C.c_double), ("temperature", C.c_double), ("lambda_", C.c_double),
                ("rc", C.c_double), ("mu", C.c_double), ("worm_constant", C.c_double),
                ("num_slices", C.c_int), ("num_ptcl", C.c_int), ("mbar", C.c_int),
                ("window", C.c_int), ("canonical", C.c_int), ("gsf", C.c_int), ("staging", C.c_int),
                ("virial_window", C.c_int), ("aziz_year", C.c_int), ("seed", C.c_uint32),
                ("wavevector", C.c_char_p), ("wavevector_type", C.c_char_p)]


def build():
    """Compile the reference's sources into oracle/_ref (a no-op when up to
    date).  Returns False when the reference tree is absent."""
    if not os.path.isdir(os.path.join(REF, "src")):
        return False
    r = subprocess.run(["make", "-s", "-j8", "-f", "Makefile.ref", "REF=" + REF], cwd=HERE,
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stderr[-4000:])
    return True


def available():
    try:
        return build() and os.path.exists(LIB)
    except RuntimeError:
        return False


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB) and not build():
        raise RuntimeError("the reference tree is absent: oracle/_ref cannot be built")
    lib = C.CDLL(LIB)
    sig = {
        "ref_last_error": (C.c_char_p, []),
        "ref_create": (C.c_void_p, [C.POINTER(RefParams), _DP]),
        "ref_destroy": (None, [C.c_void_p]),
        "ref_table_length": (C.c_int, [C.c_void_p]),
        "ref_tail_v": (C.c_double, [C.c_void_p]),
        "ref_potential": (None, [C.c_void_p, _DP, C.c_int, _DP, _DP, _DP]),
        "ref_set_shift": (None, [C.c_void_p, C.c_int]),
        "ref_potential_action_bead": (C.c_double, [C.c_void_p, C.c_int, C.c_int]),
        "ref_bare_potential_action": (C.c_double, [C.c_void_p, C.c_int, C.c_int]),
        "ref_potential_action_correction": (C.c_double, [C.c_void_p, C.c_int, C.c_int]),
        "ref_potential_action_full": (C.c_double, [C.c_void_p]),
        "ref_kinetic_action": (C.c_double, [C.c_void_p]),
        "ref_update_bead": (None, [C.c_void_p, C.c_int, C.c_int, _DP]),
        "ref_estimator": (C.c_int, [C.c_void_p, C.c_int, _DP, C.c_int]),
        "ref_run_steps": (C.c_int, [C.c_void_p, C.c_int, _DP]),
        "ref_move_stats": (None, [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
        "ref_extent": (C.c_int, [C.c_void_p]),
        "ref_get_path": (None, [C.c_void_p, C.c_int, _DP, _IP, _IP, C.POINTER(C.c_uint8), _IP, _IP]),
        "ref_rng_state": (None, [C.c_void_p, C.POINTER(C.c_uint32)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _d(a):
    return a.ctypes.data_as(_DP)


def mass_lambda(lam):
    """The lambda the reference computes from its mass parameter,
    lambda = 24.24 / m with m = 24.24 / lam (constants.cpp:121-122)."""
    return 24.24 / (24.24 / lam)


class Reference:
    """One reference system (constants, Prism, LookupTable, Aziz, Path,
    LocalAction, the default move list and PathIntegralMonteCarlo) built
    from closed identity worldlines pos [M][N][3].  Only one may exist at a
    time: the reference's parameters live in a process-wide singleton."""

    def __init__(self, pos, side, temperature, lam, rc=None, mu=0.0, worm_constant=1.0, mbar=8,
                 window=-1, canonical=False, gsf=False, staging=False, seed=1, virial_window=5,
                 wavevector=None, wavevector_type=None, aziz_year=1979):
        self.lib = load()
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        self.M, self.N = pos.shape[0], pos.shape[1]
        self._wv = None if wavevector is None else wavevector.encode()
        self._wt = None if wavevector_type is None else wavevector_type.encode()
        p = RefParams(side, temperature, lam, side if rc is None else rc, mu, worm_constant,
                      self.M, self.N, mbar, window, 1 if canonical else 0, 1 if gsf else 0,
                      1 if staging else 0, virial_window, aziz_year, seed, self._wv, self._wt)
        self.h = self.lib.ref_create(C.byref(p), _d(pos))
        if not self.h:
            raise RuntimeError("reference set-up failed: %s" % self.lib.ref_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.ref_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def potential(self, sep):
        sep = np.ascontiguousarray(sep, dtype=np.float64).reshape(-1, 3)
        n = len(sep)
        V, g, g2 = np.zeros(n), np.zeros((n, 3)), np.zeros(n)
        self.lib.ref_potential(self.h, _d(sep), n, _d(V), _d(g), _d(g2))
        return V, g, g2

    def table_length(self):
        return self.lib.ref_table_length(self.h)

    def tail_v(self):
        return self.lib.ref_tail_v(self.h)

    def set_shift(self, shift):
        self.lib.ref_set_shift(self.h, shift)

    def bead_action(self, t, p):
        return self.lib.ref_potential_action_bead(self.h, t, p)

    def bare_action(self, t, p):
        return self.lib.ref_bare_potential_action(self.h, t, p)

    def correction(self, t, p):
        return self.lib.ref_potential_action_correction(self.h, t, p)

    def full_action(self):
        return self.lib.ref_potential_action_full(self.h)

    def kinetic_action(self):
        return self.lib.ref_kinetic_action(self.h)

    def update_bead(self, t, p, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        self.lib.ref_update_bead(self.h, t, p, _d(r))

    def estimator(self, kind, cap=1 << 20):
        out = np.zeros(cap)
        n = self.lib.ref_estimator(self.h, {"energy": 0, "virial": 1, "ssf": 2, "isf": 3}[kind],
                                   _d(out), cap)
        if n < 0:
            raise RuntimeError(self.lib.ref_last_error().decode())
        return out[:n]

    def run_steps(self, nsteps):
        en = np.zeros(max(nsteps, 1))
        closed = self.lib.ref_run_steps(self.h, nsteps, _d(en))
        return closed, en[:nsteps]

    def move_stats(self):
        att = np.zeros(12, dtype=np.int64)
        acc = np.zeros(12, dtype=np.int64)
        self.lib.ref_move_stats(self.h, att.ctypes.data_as(C.POINTER(C.c_longlong)),
                                acc.ctypes.data_as(C.POINTER(C.c_longlong)))
        return att, acc

    def path(self, ne=None):
        ne = self.lib.ref_extent(self.h) if ne is None else ne
        M = self.M
        pos = np.zeros((M, ne, 3))
        nxt = np.zeros((M, ne, 2), dtype=np.int32)
        prv = np.zeros((M, ne, 2), dtype=np.int32)
        on = np.zeros((M, ne), dtype=np.uint8)
        worm = np.zeros(8, dtype=np.int32)
        nbs = np.zeros(M, dtype=np.int32)
        self.lib.ref_get_path(self.h, ne, _d(pos), nxt.ctypes.data_as(_IP), prv.ctypes.data_as(_IP),
                              on.ctypes.data_as(C.POINTER(C.c_uint8)), worm.ctypes.data_as(_IP),
                              nbs.ctypes.data_as(_IP))
        return dict(pos=pos, next=nxt, prev=prv, on=on, worm=worm, nbs=nbs)

    def rng_state(self):
        out = np.zeros(625, dtype=np.uint32)
        self.lib.ref_rng_state(self.h, out.ctypes.data_as(C.POINTER(C.c_uint32)))
        return out

"""pimc_gb300 -- GB300-native WA-PIMC hot path (pair action + path-wide estimators).

Python mirror of the reference plugin surface for this path, over the C ABI
of libpimc_gb300.so (include/pimc_gb300.h):

  * ``Action``   -- AzizPotential + LocalAction + the estimator-facing
                    ActionBase virtuals (include/action.h:30-145) for one path
  * ``qvectors`` -- EstimatorBase::getQVectors (estimator.cpp:439-570)
  * ``Walkers``  -- many independent canonical chains in one persistent kernel

Every call runs on the GPU; a missing library or device raises.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import (PGB_FP64, PGB_MIXED, PGB_ACTION_FULL, PGB_ACTION_BARE, PGB_ACTION_CORR,
                   PgbError, dptr, iptr, u8ptr)
from . import worldlines

__all__ = ["Action", "Walkers", "WormWalkers", "Server", "qvectors", "device_info", "PGB_FP64", "PGB_MIXED",
           "PGB_ACTION_FULL", "PGB_ACTION_BARE", "PGB_ACTION_CORR", "PgbError", "worldlines",
           "action_factors"]


def action_factors(kind):
    """VFactor, gradVFactor, period of Setup::action (src/setup.cpp:1230-1253)."""
    if kind == "gsf":
        return (2.0 / 3.0, 4.0 / 3.0), (0.0, 2.0 / 9.0), 2
    if kind == "li_broughton":
        return (1.0, 1.0), (1.0 / 12.0, 1.0 / 12.0), 2
    return (1.0, 1.0), (0.0, 0.0), 1


def device_info():
    lib = _lib.load()
    name = C.create_string_buffer(256)
    sm, cc = C.c_int(), C.c_int()
    _lib.check(lib.pgb_device_info(name, 256, C.byref(sm), C.byref(cc)))
    return dict(name=name.value.decode(), sm_count=sm.value, cc=cc.value)


def qvectors(kind, text, side):
    lib = _lib.load()
    side = np.ascontiguousarray(np.broadcast_to(np.asarray(side, dtype=np.float64), (3,)))
    n = C.c_int()
    _lib.check(lib.pgb_qvectors(kind.encode(), text.encode(), dptr(side), None, 0, C.byref(n)))
    q = np.zeros((max(n.value, 1), 3))
    _lib.check(lib.pgb_qvectors(kind.encode(), text.encode(), dptr(side), dptr(q), n.value,
                                C.byref(n)))
    return q[:n.value]


def qvectors_shells(dq, qmax, sphere=False):
    """EstimatorBase::getQVectors2: (q [n][3], shell index [n])."""
    lib = _lib.load()
    n = C.c_int()
    _lib.check(lib.pgb_qvectors_shells(dq, qmax, 1 if sphere else 0, None, None, 0, C.byref(n)))
    q = np.zeros((max(n.value, 1), 3))
    sh = np.zeros(max(n.value, 1), dtype=np.int32)
    _lib.check(lib.pgb_qvectors_shells(dq, qmax, 1 if sphere else 0, dptr(q),
                                       sh.ctypes.data_as(C.POINTER(C.c_int)), n.value,
                                       C.byref(n)))
    return q[:n.value], sh[:n.value]


class Action:
    """One path on the device with its Aziz tables and LocalAction factors."""

    def __init__(self, side, num_slices, num_ptcl_ext, tau, lam, rc=None, action="primitive",
                 precision=PGB_FP64, aziz_year=1979, virial_window=5, mu=0.0):
        self.lib = _lib.load()
        side = np.broadcast_to(np.asarray(side, dtype=np.float64), (3,))
        vf, gf, period = action_factors(action)
        p = _lib.PgbParams()
        for i in range(3):
            p.side[i] = side[i]
        p.num_slices, p.num_ptcl_ext = int(num_slices), int(num_ptcl_ext)
        p.tau, p.lambda_ = float(tau), float(lam)
        p.rc = float(side[2] if rc is None else rc)
        p.vfactor[0], p.vfactor[1] = vf
        p.gradvfactor[0], p.gradvfactor[1] = gf
        p.period, p.aziz_year, p.virial_window = period, aziz_year, virial_window
        p.precision, p.mu = precision, mu
        self.params = p
        self.M, self.Ne = int(num_slices), int(num_ptcl_ext)
        h = C.c_void_p()
        rc_ = self.lib.pgb_create(C.byref(p), C.byref(h))
        if rc_ != 0:
            raise PgbError(rc_, (self.lib.pgb_last_error(None) or b"").decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.pgb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        return _lib.check(rc, self.h)

    # ---- potential ----
    def table_info(self):
        n, dr, tail = C.c_int(), C.c_double(), C.c_double()
        self._chk(self.lib.pgb_table_info(self.h, C.byref(n), C.byref(dr), C.byref(tail)))
        return n.value, dr.value, tail.value

    def tables(self):
        n, _, _ = self.table_info()
        V, dV, d2V = np.zeros(n), np.zeros(n), np.zeros(n)
        self._chk(self.lib.pgb_copy_tables(self.h, dptr(V), dptr(dV), dptr(d2V)))
        return V, dV, d2V

    def V_batch(self, sep):
        sep = np.ascontiguousarray(sep, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(len(sep))
        self._chk(self.lib.pgb_potential_batch(self.h, dptr(sep), dptr(out), len(sep)))
        return out

    def gradV_batch(self, sep):
        sep = np.ascontiguousarray(sep, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((len(sep), 3))
        self._chk(self.lib.pgb_gradv_batch(self.h, dptr(sep), dptr(out), len(sep)))
        return out

    def grad2V_batch(self, sep):
        sep = np.ascontiguousarray(sep, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(len(sep))
        self._chk(self.lib.pgb_grad2v_batch(self.h, dptr(sep), dptr(out), len(sep)))
        return out

    # ---- worldlines ----
    def load(self, cfg):
        pos = np.ascontiguousarray(cfg["pos"], dtype=np.float64)
        nxt = np.ascontiguousarray(cfg["next"], dtype=np.int32)
        prv = np.ascontiguousarray(cfg["prev"], dtype=np.int32)
        on = np.ascontiguousarray(cfg["on"], dtype=np.uint8)
        worm = np.ascontiguousarray(cfg.get("worm", np.full(8, -1)), dtype=np.int32)
        self._chk(self.lib.pgb_load_path(self.h, dptr(pos), iptr(nxt), iptr(prv), u8ptr(on),
                                         iptr(worm)))

    def update_positions(self, pos):
        """All bead positions (AoS [M][Ne][3]) with links and worm unchanged."""
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(self.M, self.Ne, 3)
        self._keep = pos                    # the copy is asynchronous
        self._chk(self.lib.pgb_update_positions(self.h, dptr(pos)))

    def update_beads(self, beads, pos):
        beads = np.ascontiguousarray(beads, dtype=np.int32).reshape(-1, 2)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        self._chk(self.lib.pgb_update_beads(self.h, iptr(beads), dptr(pos), len(beads)))

    def positions(self):
        out = np.zeros((self.M, self.Ne, 3))
        self._chk(self.lib.pgb_get_positions(self.h, dptr(out)))
        return out

    # ---- action ----
    def bead_actions(self, beads, shift=1, mode=PGB_ACTION_FULL):
        beads = np.ascontiguousarray(beads, dtype=np.int32).reshape(-1, 2)
        per = np.zeros(len(beads))
        tot = C.c_double()
        self._chk(self.lib.pgb_bead_actions(self.h, iptr(beads), len(beads), shift, mode,
                                            dptr(per), C.byref(tot)))
        return per, tot.value

    def trial_actions(self, beads, pos, shift=1, mode=PGB_ACTION_FULL):
        beads = np.ascontiguousarray(beads, dtype=np.int32).reshape(-1, 2)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(len(beads))
        self._chk(self.lib.pgb_trial_actions(self.h, iptr(beads), dptr(pos), len(beads), shift, mode,
                                             dptr(out)))
        return out

    def range_action(self, start, end, shift=1):
        out = C.c_double()
        self._chk(self.lib.pgb_range_action(self.h, start[0], start[1], end[0], end[1], shift,
                                            C.byref(out)))
        return out.value

    def full_action(self):
        out = C.c_double()
        self._chk(self.lib.pgb_full_action(self.h, C.byref(out)))
        return out.value

    def kinetic_action(self):
        out = C.c_double()
        self._chk(self.lib.pgb_kinetic_action(self.h, C.byref(out)))
        return out.value

    def slice_terms(self, tmatrix=True):
        arrs = {k: np.zeros(self.M) for k in ("vint", "g2", "r1", "r2", "d1", "d2", "kin", "xch")}
        st = _lib.PgbSliceTerms()
        for k, a in arrs.items():
            if tmatrix or k not in ("r2", "d2"):
                setattr(st, k, dptr(a))
        self._chk(self.lib.pgb_slice_terms_compute(self.h, C.byref(st)))
        return arrs

    # ---- estimators ----
    def energy(self):
        out = np.zeros(9)
        self._chk(self.lib.pgb_energy(self.h, dptr(out)))
        return out

    def virial(self, cvcov2_quirk=True):
        out = np.zeros(19)
        self._chk(self.lib.pgb_virial(self.h, 1 if cvcov2_quirk else 0, dptr(out)))
        return out

    def ssf(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(len(q))
        self._chk(self.lib.pgb_ssf(self.h, dptr(q), len(q), dptr(out)))
        return out

    def ssf_cylinder(self, q, max_r):
        """(1/M) sum_t |sum_{j inside} exp(i q.r_j)|^2 per q, and the number
        of slice-0 beads inside x^2 + y^2 < max_r^2."""
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(len(q))
        n0 = C.c_int()
        self._chk(self.lib.pgb_ssf_cylinder(self.h, dptr(q), len(q), max_r, dptr(out),
                                            C.byref(n0)))
        return out, n0.value

    def isf(self, q, mode=0):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((len(q), self.M // 2 + 1))
        self._chk(self.lib.pgb_isf(self.h, dptr(q), len(q), mode, dptr(out)))
        return out

    def pair_correlation(self, slice=-1):
        out = np.zeros(50)
        self._chk(self.lib.pgb_pair_correlation(self.h, slice, dptr(out)))
        return out

    def superfluid(self):
        out = np.zeros(26)
        self._chk(self.lib.pgb_superfluid(self.h, dptr(out)))
        return out

    def permutation_cycles(self):
        out = np.zeros(40)
        self._chk(self.lib.pgb_permutation_cycles(self.h, dptr(out)))
        return out

    def rhoq(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((len(q), self.M, 2))
        self._chk(self.lib.pgb_rhoq(self.h, dptr(q), len(q), dptr(out)))
        return out

    # ---- plain form (host-driven moves, FP64 device actions) ----
    def plain_seed(self, seed):
        self._chk(self.lib.pgb_plain_seed(self.h, seed))

    def rng_state(self):
        """The plain form's MT19937 state, MTRand::save layout (625 words)."""
        out = np.zeros(625, dtype=np.uint32)
        self._chk(self.lib.pgb_plain_get_rng(self.h, out.ctypes.data_as(C.POINTER(C.c_uint32))))
        return out

    def set_rng_state(self, words):
        words = np.ascontiguousarray(words, dtype=np.uint32)
        if words.shape != (625,):
            raise ValueError("an MT19937 state has 625 words")
        self._chk(self.lib.pgb_plain_set_rng(self.h, words.ctypes.data_as(C.POINTER(C.c_uint32))))

    def plain_worm_run(self, nsteps, mbar, temperature, initial_num_particles, mu=0.0,
                       worm_constant=1.0, window=-1, gaussian_sd=0.0, diagonal_move=1,
                       var_updates=1, max_wind=1, num_updates=0, trace_cap=0):
        """The worm-algorithm step loop (default PIMC move list) in the plain form."""
        wp = _lib.PgbWormParams(mbar, diagonal_move, var_updates, max_wind, temperature, mu,
                                worm_constant, window, gaussian_sd, num_updates,
                                initial_num_particles)
        trace = np.zeros((max(trace_cap, 1), 2), dtype=np.int32)
        ntr = C.c_int()
        en = np.zeros(max(nsteps, 1))
        npart = np.zeros(max(nsteps, 1), dtype=np.int32)
        st = _lib.PgbWormStats()
        self._chk(self.lib.pgb_plain_worm_run(self.h, C.byref(wp), nsteps, iptr(trace), trace_cap,
                                              C.byref(ntr), dptr(en), iptr(npart), C.byref(st)))
        return dict(trace=trace[:ntr.value], energies=en[:nsteps], num_particles=npart[:nsteps],
                    attempted=list(st.attempted), accepted=list(st.accepted),
                    bead_updates=st.bead_updates, diagonal=st.diagonal)

    def path(self):
        """Links, active flags and worm locators of the host mirror, with positions."""
        nxt = np.zeros((self.M, self.Ne, 2), dtype=np.int32)
        prv = np.zeros((self.M, self.Ne, 2), dtype=np.int32)
        on = np.zeros((self.M, self.Ne), dtype=np.uint8)
        worm = np.zeros(8, dtype=np.int32)
        self._chk(self.lib.pgb_get_path(self.h, iptr(nxt), iptr(prv), u8ptr(on), iptr(worm)))
        return dict(next=nxt, prev=prv, on=on, worm=worm, nbs=on.sum(axis=1).astype(np.int32),
                    pos=self.positions())

    def set_beads(self, beads, pos, nxt, prv, on):
        beads = np.ascontiguousarray(beads, dtype=np.int32).reshape(-1, 2)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        nxt = np.ascontiguousarray(nxt, dtype=np.int32).reshape(-1, 2)
        prv = np.ascontiguousarray(prv, dtype=np.int32).reshape(-1, 2)
        on = np.ascontiguousarray(on, dtype=np.uint8).reshape(-1)
        self._chk(self.lib.pgb_set_beads(self.h, iptr(beads), dptr(pos), iptr(nxt), iptr(prv),
                                         u8ptr(on), len(beads)))

    def set_worm(self, worm8):
        w = np.ascontiguousarray(worm8, dtype=np.int32)
        self._chk(self.lib.pgb_set_worm(self.h, iptr(w)))

    def plain_run(self, nsteps, mbar, temperature, diagonal_move=1, var_updates=1, max_wind=1,
                  p_com=0.05, num_updates=0, trace_cap=0):
        mp = _lib.PgbMoveParams(mbar, diagonal_move, var_updates, max_wind, temperature, p_com,
                                num_updates)
        trace = np.zeros((max(trace_cap, 1), 2), dtype=np.int32)
        ntr = C.c_int()
        en = np.zeros(max(nsteps, 1))
        st = _lib.PgbMoveStats()
        self._chk(self.lib.pgb_plain_run(self.h, C.byref(mp), nsteps, iptr(trace), trace_cap,
                                         C.byref(ntr), dptr(en), C.byref(st)))
        return dict(trace=trace[:ntr.value], energies=en[:nsteps],
                    attempted=list(st.attempted), accepted=list(st.accepted),
                    bead_updates=st.bead_updates)


class Walkers:
    """Independent canonical walkers advanced together on the device."""

    def __init__(self, n, m, temperature, side, mbar, tau, lam, seed=0, p_com=0.05,
                 threads_per_walker=0, var_updates=1, aziz_year=1979):
        self.lib = _lib.load()
        self.n = np.ascontiguousarray(n, dtype=np.int32)
        self.m = np.ascontiguousarray(m, dtype=np.int32)
        self.t = np.ascontiguousarray(temperature, dtype=np.float64)
        self.side = np.ascontiguousarray(side, dtype=np.float64)
        self.mbar = np.ascontiguousarray(mbar, dtype=np.int32)
        p = _lib.PgbWalkersParams()
        p.num_walkers = len(self.n)
        p.num_ptcl = self.n.ctypes.data_as(C.POINTER(C.c_int))
        p.num_slices = self.m.ctypes.data_as(C.POINTER(C.c_int))
        p.temperature = dptr(self.t)
        p.side = dptr(self.side)
        p.mbar = self.mbar.ctypes.data_as(C.POINTER(C.c_int))
        p.tau, p.lambda_, p.p_com, p.seed = tau, lam, p_com, seed
        p.aziz_year, p.threads_per_walker, p.var_updates = aziz_year, threads_per_walker, var_updates
        h = C.c_void_p()
        rc = self.lib.pgb_walkers_create(C.byref(p), C.byref(h))
        if rc != 0:
            raise PgbError(rc, (self.lib.pgb_walkers_last_error(None) or b"").decode())
        self.h = h
        self.W = len(self.n)

    def _chk(self, rc):
        return _lib.check(rc, self.h, walkers=True)

    def close(self):
        if getattr(self, "h", None):
            self.lib.pgb_walkers_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init(self):
        self._chk(self.lib.pgb_walkers_init(self.h))

    def set_positions(self, w, pos):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        self._chk(self.lib.pgb_walkers_set_positions(self.h, w, dptr(pos)))

    def positions(self, w):
        out = np.zeros((int(self.m[w]), int(self.n[w]), 3))
        self._chk(self.lib.pgb_walkers_get_positions(self.h, w, dptr(out)))
        return out

    def all_positions(self):
        """Every walker's positions, concatenated (walker w's [M_w][N_w][3])."""
        out = np.zeros(int(self.lib.pgb_walkers_state_bytes(self.h)) // 8)
        self._chk(self.lib.pgb_walkers_get_all_positions(self.h, dptr(out)))
        return out

    def set_all_positions(self, pos):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        self._keep = pos
        self._chk(self.lib.pgb_walkers_set_all_positions(self.h, dptr(pos)))

    def sweeps_done(self):
        out = np.zeros(self.W, dtype=np.uint64)
        self._chk(self.lib.pgb_walkers_get_sweeps(self.h, out.ctypes.data_as(C.POINTER(C.c_ulonglong))))
        return out

    def set_sweeps_done(self, sweeps):
        s = np.ascontiguousarray(sweeps, dtype=np.uint64)
        self._chk(self.lib.pgb_walkers_set_sweeps(self.h, s.ctypes.data_as(C.POINTER(C.c_ulonglong))))

    def run(self, sweeps, measure=1, sync=True):
        self._chk(self.lib.pgb_walkers_run_async(self.h, sweeps, measure))
        if sync:
            self._chk(self.lib.pgb_walkers_sync(self.h))

    def sync(self):
        self._chk(self.lib.pgb_walkers_sync(self.h))

    def stats(self):
        st = (_lib.PgbWalkerStats * self.W)()
        self._chk(self.lib.pgb_walkers_stats(self.h, st))
        return [dict(energy_sum=s.energy_sum, energy_sumsq=s.energy_sumsq, samples=s.samples,
                     bead_updates=s.bead_updates, attempted=list(s.attempted),
                     accepted=list(s.accepted)) for s in st]

    # numpy view of pgb_walker_stats, one record per walker
    STATS_DTYPE = np.dtype([("energy_sum", "<f8"), ("energy_sumsq", "<f8"), ("samples", "<i8"),
                            ("bead_updates", "<i8"), ("attempted", "<i8", (2,)),
                            ("accepted", "<i8", (2,))])

    def stats_array(self, out=None):
        """The per-walker accumulators as a structured array (columns
        energy_sum, energy_sumsq, samples, bead_updates, attempted[2],
        accepted[2]); `out` (from a previous call) is filled in place."""
        if out is None:
            out = np.zeros(self.W, dtype=self.STATS_DTYPE)
        assert out.dtype == self.STATS_DTYPE and out.itemsize == C.sizeof(_lib.PgbWalkerStats)
        self._chk(self.lib.pgb_walkers_stats(self.h, C.cast(out.ctypes.data,
                                                            C.POINTER(_lib.PgbWalkerStats))))
        return out

    def reset_stats(self):
        self._chk(self.lib.pgb_walkers_reset_stats(self.h))

    def energy(self, precision=PGB_MIXED):
        out = np.zeros(self.W)
        self._chk(self.lib.pgb_walkers_energy(self.h, precision, dptr(out)))
        return out

    def launch_count(self):
        return self.lib.pgb_walkers_launch_count(self.h)

    def threads(self):
        return self.lib.pgb_walkers_threads(self.h)

    def tuning(self):
        n = self.lib.pgb_walkers_tuning(self.h, None, None, 0)
        sc = (C.c_int * max(n, 1))()
        ms = (C.c_float * max(n, 1))()
        self.lib.pgb_walkers_tuning(self.h, sc, ms, n)
        return {int(sc[i]): float(ms[i]) for i in range(n)}

    def stream(self):
        return self.lib.pgb_walkers_stream(self.h)


class WormWalkers:
    """Device-resident worm-algorithm walkers (one warp per small walker, a
    team of two or four warps from N0 = 32 and 64): the reference's
    default PIMC move list on independent paths (grand canonical, or
    canonical with a particle window)."""

    STATS_DTYPE = np.dtype([("energy_sum", "<f8"), ("energy_sumsq", "<f8"), ("n_sum", "<f8"),
                            ("n_sumsq", "<f8"), ("samples", "<i8"), ("attempted", "<i8", (12,)),
                            ("accepted", "<i8", (12,)), ("bead_updates", "<i8"), ("sweeps", "<i8"),
                            ("error", "<i4"), ("pad", "<i4")])

    def __init__(self, n, m, side, mbar, tau, lam, mu=None, capacity=None, worm_constant=1.0,
                 window=-1, seed=0, aziz_year=1979, diagonal_move=0):
        """diagonal_move: 0 bisection (the reference's default), 1 staging;
        worm_constant: C0 for every walker, or one per walker."""
        self.lib = _lib.load()
        self.n = np.ascontiguousarray(n, dtype=np.int32)
        self.W = len(self.n)
        self.m = np.ascontiguousarray(np.broadcast_to(m, self.W), dtype=np.int32)
        self.side = np.ascontiguousarray(np.broadcast_to(side, self.W), dtype=np.float64)
        self.mbar = np.ascontiguousarray(np.broadcast_to(mbar, self.W), dtype=np.int32)
        self.mu = np.ascontiguousarray(np.broadcast_to(0.0 if mu is None else mu, self.W), dtype=np.float64)
        cap = 2 * self.n + 8 if capacity is None else np.broadcast_to(capacity, self.W)
        self.capacity = np.ascontiguousarray(cap, dtype=np.int32)
        p = _lib.PgbWormWalkersParams()
        p.num_walkers = self.W
        p.num_ptcl = self.n.ctypes.data_as(C.POINTER(C.c_int))
        p.num_slices = self.m.ctypes.data_as(C.POINTER(C.c_int))
        p.side = dptr(self.side)
        p.mu = dptr(self.mu)
        p.mbar = self.mbar.ctypes.data_as(C.POINTER(C.c_int))
        p.capacity = self.capacity.ctypes.data_as(C.POINTER(C.c_int))
        p.tau, p.lambda_, p.worm_constant, p.window, p.seed, p.aziz_year = (
            tau, lam, float(np.ravel(worm_constant)[0]), window, seed, aziz_year)
        p.diagonal_move = int(diagonal_move)
        self.diagonal_move = int(diagonal_move)
        if np.ndim(worm_constant) > 0:
            self.c0 = np.ascontiguousarray(np.broadcast_to(worm_constant, self.W), dtype=np.float64)
            p.worm_constants = dptr(self.c0)
            p.worm_constant = float(self.c0[0])
        h = C.c_void_p()
        rc = self.lib.pgb_worm_walkers_create(C.byref(p), C.byref(h))
        if rc != 0:
            raise PgbError(rc, (self.lib.pgb_worm_walkers_last_error(None) or b"").decode())
        self.h = h
        self.tau, self.lam = tau, lam

    def _chk(self, rc):
        return _lib.check(rc, self.h, worm=True)

    def close(self):
        if getattr(self, "h", None):
            self.lib.pgb_worm_walkers_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, w, pos):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(int(self.m[w]), int(self.n[w]), 3)
        self._chk(self.lib.pgb_worm_walkers_load(self.h, w, dptr(pos)))

    def load_seeded(self, seed=0):
        """Every walker from seeded closed worldlines (uniform centres, Gaussian jitter)."""
        from . import worldlines as wl
        for w in range(self.W):
            cfg = wl.seeded_worldlines(int(self.n[w]), int(self.m[w]), float(self.side[w]), self.lam,
                                       self.tau, seed * 100003 + w)
            self.load(w, cfg["pos"])

    def run(self, sweeps, sync=True):
        if sync:
            self._chk(self.lib.pgb_worm_walkers_run(self.h, sweeps))
        else:
            self._chk(self.lib.pgb_worm_walkers_run_async(self.h, sweeps))

    def synchronize(self):
        self._chk(self.lib.pgb_worm_walkers_synchronize(self.h))

    def equilibrate(self, sweeps):
        """Diagonal pre-equilibration: centre-of-mass and diagonal moves only."""
        self._chk(self.lib.pgb_worm_walkers_equilibrate(self.h, sweeps))

    def stream(self):
        return self.lib.pgb_worm_walkers_stream(self.h)

    def launch_count(self):
        return int(self.lib.pgb_worm_walkers_launch_count(self.h))

    def seed_device(self, seed=0):
        """Every walker from seeded closed worldlines made on the device."""
        self._chk(self.lib.pgb_worm_walkers_seed(self.h, seed))

    def state_bytes(self):
        return int(self.lib.pgb_worm_walkers_state_bytes(self.h))

    def get_state(self, image):
        """Copy the whole device state into `image` (a writable buffer of
        state_bytes() bytes, e.g. a pinned tensor's numpy view)."""
        self._chk(self.lib.pgb_worm_walkers_get_state(self.h, C.c_void_p(image.ctypes.data)))

    def set_state_async(self, image):
        self._chk(self.lib.pgb_worm_walkers_set_state_async(self.h, C.c_void_p(image.ctypes.data)))

    def stats_async(self, out):
        self._chk(self.lib.pgb_worm_walkers_stats_async(self.h, C.cast(out.ctypes.data,
                                                                       C.POINTER(_lib.PgbWormWalkerStats))))

    def bead_actions(self, w, beads):
        """Bare potential action of beads [k][2] of walker w by the walkers'
        own FP32 pair sums."""
        beads = np.ascontiguousarray(beads, dtype=np.int32).reshape(-1, 2)
        out = np.zeros(len(beads))
        self._chk(self.lib.pgb_worm_walkers_bead_actions(self.h, w, iptr(beads), len(beads), dptr(out)))
        return out

    def stats(self):
        out = np.zeros(self.W, dtype=self.STATS_DTYPE)
        assert out.itemsize == C.sizeof(_lib.PgbWormWalkerStats)
        self._chk(self.lib.pgb_worm_walkers_stats(self.h, C.cast(out.ctypes.data,
                                                                 C.POINTER(_lib.PgbWormWalkerStats))))
        return out

    def reset_stats(self):
        self._chk(self.lib.pgb_worm_walkers_reset_stats(self.h))

    def path(self, w):
        M, ne = int(self.m[w]), int(self.capacity[w])
        pos = np.zeros((M, ne, 3))
        nxt = np.zeros((M, ne, 2), dtype=np.int32)
        prv = np.zeros((M, ne, 2), dtype=np.int32)
        on = np.zeros((M, ne), dtype=np.uint8)
        worm = np.zeros(8, dtype=np.int32)
        self._chk(self.lib.pgb_worm_walkers_get_path(self.h, w, dptr(pos), iptr(nxt), iptr(prv),
                                                     u8ptr(on), iptr(worm)))
        return dict(pos=pos, next=nxt, prev=prv, on=on, worm=worm,
                    nbs=on.sum(axis=1).astype(np.int32))


class Server:
    """Continuous-batching job server: jobs arrive, are admitted when their
    worldlines fit the HBM budget, run together in shared launches and stream
    estimator bins back."""

    def __init__(self, hbm_budget_bytes, max_active=1024, sweeps_per_round=10, bin_sweeps=100,
                 tau=0.004, lam=None, p_com=0.05, aziz_year=1979, round_seconds=0.0,
                 grand_canonical=False, diagonal_move=0):
        """grand_canonical: every job a device worm walker at its mu
        (pgb_worm_server_*), diagonal_move 0 bisection (the reference's
        default) or 1 staging; otherwise canonical staging + COM chains."""
        self.lib = _lib.load()
        lam = worldlines.LAMBDA_HE4 if lam is None else lam
        p = _lib.PgbServerParams(float(hbm_budget_bytes), max_active, sweeps_per_round, bin_sweeps,
                                 tau, lam, p_com, aziz_year, float(round_seconds), int(diagonal_move))
        self.gc = bool(grand_canonical)
        self.pre = "pgb_worm_server_" if self.gc else "pgb_server_"
        h = C.c_void_p()
        rc = getattr(self.lib, self.pre + "create")(C.byref(p), C.byref(h))
        if rc != 0:
            raise PgbError(rc, (getattr(self.lib, self.pre + "last_error")(None) or b"").decode())
        self.h = h

    def _f(self, name):
        return getattr(self.lib, self.pre + name)

    def _chk(self, rc):
        return _lib.check(rc, self.h, server=not self.gc, worm_server=self.gc)

    def close(self):
        if getattr(self, "h", None):
            self._f("destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, n, temperature, sweeps, seed, arrival=0.0, mu=0.0,
               density=worldlines.DENSITY):
        spec = _lib.PgbJobSpec(int(n), float(temperature), float(mu), float(density), int(sweeps),
                               int(seed), float(arrival))
        jid = C.c_int()
        self._chk(self._f("submit")(self.h, C.byref(spec), C.byref(jid)))
        return jid.value

    def step(self):
        a, q = C.c_int(), C.c_int()
        self._chk(self._f("step")(self.h, C.byref(a), C.byref(q)))
        return a.value, q.value

    def bins(self):
        out = []
        buf = (_lib.PgbBin * 1024)()
        while True:
            n = C.c_int()
            self._chk(self._f("poll_bins")(self.h, buf, 1024, C.byref(n)))
            out += [dict(job=b.job, bin=b.bin, energy=b.energy_per_particle, samples=b.samples,
                         time=b.time) for b in buf[:n.value]]
            if n.value < 1024:
                return out

    def job(self, jid):
        i = _lib.PgbJobInfo()
        self._chk(self._f("job_info")(self.h, jid, C.byref(i)))
        return dict(state=i.state, arrival=i.arrival, admitted=i.admitted, first_bin=i.first_bin,
                    completed=i.completed, sweeps_done=i.sweeps_done, n=i.n, m=i.m, bytes=i.bytes)

    def clock(self):
        return self._f("clock")(self.h)

    def bead_updates(self):
        t = C.c_longlong()
        self._chk(self._f("active_bead_updates")(self.h, C.byref(t)))
        return t.value

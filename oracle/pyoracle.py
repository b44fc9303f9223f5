"""ctypes binding of the FP64 CPU oracle (oracle/_build/libpimc_oracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py as the checker.  The product never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libpimc_oracle.so")


class OrcParams(C.Structure):
    _fields_ = [("side", C.c_double * 3), ("num_slices", C.c_int), ("num_ptcl_ext", C.c_int),
                ("tau", C.c_double), ("lambda_", C.c_double), ("rc", C.c_double),
                ("vfactor", C.c_double * 2), ("gradvfactor", C.c_double * 2),
                ("aziz_year", C.c_int), ("virial_window", C.c_int), ("mu", C.c_double)]


class OrcGpParams(C.Structure):
    _fields_ = [("matern_nu", C.c_double), ("ell", C.c_double * 3), ("norm_offset", C.c_double * 3),
                ("norm_scale", C.c_double * 3), ("standard_mean", C.c_double),
                ("standard_std", C.c_double), ("mean", C.c_double), ("sigma2", C.c_double),
                ("side", C.c_double * 3), ("periodic", C.c_int * 3)]


class OrcWormParams(C.Structure):
    _fields_ = [("mbar", C.c_int), ("diagonal_move", C.c_int), ("var_updates", C.c_int),
                ("max_wind", C.c_int), ("temperature", C.c_double), ("mu", C.c_double),
                ("worm_constant", C.c_double), ("window", C.c_int), ("gaussian_sd", C.c_double),
                ("num_updates", C.c_int), ("initial_num_particles", C.c_int)]


class OrcWormStats(C.Structure):
    _fields_ = [("attempted", C.c_longlong * 12), ("accepted", C.c_longlong * 12),
                ("bead_updates", C.c_longlong), ("diagonal", C.c_int)]


class OrcMoveParams(C.Structure):
    _fields_ = [("mbar", C.c_int), ("diagonal_move", C.c_int), ("var_updates", C.c_int),
                ("max_wind", C.c_int), ("temperature", C.c_double), ("p_com", C.c_double),
                ("num_updates", C.c_int)]


class OrcMoveStats(C.Structure):
    _fields_ = [("attempted", C.c_longlong * 3), ("accepted", C.c_longlong * 3),
                ("bead_updates", C.c_longlong)]


_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int32)
_VP = C.c_void_p
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        build()
    lib = C.CDLL(LIB)
    sig = {
        "orc_aziz_values": (None, [C.c_int, C.c_double, _DP]),
        "orc_create": (_VP, [C.POINTER(OrcParams)]),
        "orc_destroy": (None, [_VP]),
        "orc_table_length": (C.c_int, [_VP]),
        "orc_table_dr": (C.c_double, [_VP]),
        "orc_tailV": (C.c_double, [_VP]),
        "orc_copy_tables": (None, [_VP, _DP, _DP, _DP]),
        "orc_V": (C.c_double, [_VP, _DP]),
        "orc_gradV": (None, [_VP, _DP, _DP]),
        "orc_grad2V": (C.c_double, [_VP, _DP]),
        "orc_load_path": (None, [_VP, _DP, _IP, _IP, C.POINTER(C.c_uint8), _IP]),
        "orc_get_positions": (None, [_VP, _DP]),
        "orc_update_bead": (None, [_VP, C.c_int, C.c_int, _DP]),
        "orc_set_shift": (None, [_VP, C.c_int]),
        "orc_potential_action_bead": (C.c_double, [_VP, C.c_int, C.c_int]),
        "orc_bare_potential_action": (C.c_double, [_VP, C.c_int, C.c_int]),
        "orc_potential_action_correction": (C.c_double, [_VP, C.c_int, C.c_int]),
        "orc_potential_action_range": (C.c_double, [_VP, C.c_int, C.c_int, C.c_int, C.c_int]),
        "orc_potential_action_list": (C.c_double, [_VP, _IP, C.c_int]),
        "orc_potential_action_full": (C.c_double, [_VP]),
        "orc_kinetic_action_full": (C.c_double, [_VP]),
        "orc_Vnn": (C.c_double, [_VP, C.c_int, C.c_int]),
        "orc_gradVnnSquared": (C.c_double, [_VP, C.c_int, C.c_int]),
        "orc_V_slice": (None, [_VP, C.c_int, _DP]),
        "orc_gradVSquared_slice": (C.c_double, [_VP, C.c_int]),
        "orc_gradVSquared_bead": (C.c_double, [_VP, C.c_int, C.c_int]),
        "orc_deriv_tau": (C.c_double, [_VP, C.c_int]),
        "orc_deriv_lambda": (C.c_double, [_VP, C.c_int]),
        "orc_second_deriv_tau": (C.c_double, [_VP, C.c_int]),
        "orc_rdotgradU1": (C.c_double, [_VP, C.c_int]),
        "orc_rdotgradU2": (C.c_double, [_VP, C.c_int]),
        "orc_deltadotgradU1": (C.c_double, [_VP, C.c_int]),
        "orc_deltadotgradU2": (C.c_double, [_VP, C.c_int]),
        "orc_virial_kin_corr": (C.c_double, [_VP, C.c_int]),
        "orc_energy": (None, [_VP, _DP]),
        "orc_virial": (None, [_VP, C.c_int, _DP]),
        "orc_qvectors": (C.c_int, [C.c_char_p, C.c_char_p, _DP, _DP, C.c_int]),
        "orc_ssf_pairwise": (None, [_VP, _DP, C.c_int, _DP]),
        "orc_ssf_rhoq": (None, [_VP, _DP, C.c_int, _DP]),
        "orc_isf_cpu_form": (None, [_VP, _DP, C.c_int, _DP]),
        "orc_isf_gpu_form": (None, [_VP, _DP, C.c_int, _DP]),
        "orc_isf_rhoq": (None, [_VP, _DP, C.c_int, C.c_int, _DP]),
        "orc_rhoq": (None, [_VP, _DP, C.c_int, _DP]),
        "orc_pair_correlation": (None, [_VP, C.c_int, _DP]),
        "orc_superfluid": (None, [_VP, _DP]),
        "orc_permutation_cycles": (None, [_VP, _DP]),
        "orc_run_worm_steps": (C.c_int, [_VP, _VP, C.POINTER(OrcWormParams), C.c_int, _IP, C.c_int,
                                         _DP, _IP, C.POINTER(OrcWormStats)]),
        "orc_get_path": (None, [_VP, _IP, _IP, C.POINTER(C.c_uint8), _IP, _IP]),
        "orc_gp_eval": (None, [C.POINTER(OrcGpParams), _DP, C.c_int, _DP, C.c_int, _DP]),
        "orc_gp_benzene": (None, [C.POINTER(OrcGpParams), _DP, C.c_int, _DP, C.c_int, _DP]),
        "orc_ssf_cylinder": (None, [_VP, _DP, C.c_int, C.c_double, _DP, C.POINTER(C.c_int)]),
        "orc_qvectors_shells": (C.c_int, [C.c_double, C.c_double, C.c_int, _DP,
                                          C.POINTER(C.c_int), C.c_int]),
        "orc_format_state": (C.c_long, [_DP, _IP, _IP, C.POINTER(C.c_uint8), C.c_int, C.c_int,
                                        C.POINTER(C.c_longlong), C.c_int, C.POINTER(C.c_uint32),
                                        C.c_char_p, C.c_long]),
        "orc_mt_create": (_VP, [C.c_uint32]),
        "orc_mt_destroy": (None, [_VP]),
        "orc_mt_randint": (C.c_uint32, [_VP]),
        "orc_mt_randint_n": (C.c_uint32, [_VP, C.c_uint32]),
        "orc_mt_rand": (C.c_double, [_VP]),
        "orc_mt_randexc": (C.c_double, [_VP]),
        "orc_mt_randnorm": (C.c_double, [_VP, C.c_double, C.c_double]),
        "orc_mt_save": (None, [_VP, C.POINTER(C.c_uint32)]),
        "orc_mt_load": (None, [_VP, C.POINTER(C.c_uint32)]),
        "orc_run_steps": (C.c_int, [_VP, _VP, C.POINTER(OrcMoveParams), C.c_int, _IP, C.c_int,
                                    _DP, C.POINTER(OrcMoveStats)]),
        "orc_walkers_cpu": (C.c_double, [C.c_int, _IP, _IP, _DP, _DP, C.POINTER(C.c_uint32),
                                         C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, _DP,
                                         C.POINTER(C.c_longlong), _DP]),
        "orc_worm_walkers_cpu": (C.c_double, [C.c_int, _IP, _IP, _DP, _IP, _DP, C.POINTER(C.c_uint32),
                                              C.c_double, C.c_double, C.c_int, C.c_int, C.c_int,
                                              C.c_int, C.c_int, C.c_int, _DP, C.POINTER(C.c_longlong),
                                              _DP, _IP]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _d(a):
    return a.ctypes.data_as(_DP)


def _i(a):
    return a.ctypes.data_as(_IP)


def aziz_values(year, r):
    out = np.zeros(3)
    load().orc_aziz_values(year, r, _d(out))
    return out


def action_factors(kind):
    if kind == "gsf":
        return (2.0 / 3.0, 4.0 / 3.0), (0.0, 2.0 / 9.0)
    if kind == "li_broughton":
        return (1.0, 1.0), (1.0 / 12.0, 1.0 / 12.0)
    return (1.0, 1.0), (0.0, 0.0)


class Oracle:
    """FP64 CPU restatement of AzizPotential + LocalAction + estimators."""

    def __init__(self, side, num_slices, num_ptcl_ext, tau, lam, rc=None, action="primitive",
                 aziz_year=1979, virial_window=5, mu=0.0):
        self.lib = load()
        side = np.broadcast_to(np.asarray(side, dtype=np.float64), (3,))
        vf, gf = action_factors(action)
        p = OrcParams()
        for i in range(3):
            p.side[i] = side[i]
        p.num_slices, p.num_ptcl_ext = int(num_slices), int(num_ptcl_ext)
        p.tau, p.lambda_ = float(tau), float(lam)
        p.rc = float(side[2] if rc is None else rc)
        p.vfactor[0], p.vfactor[1] = vf
        p.gradvfactor[0], p.gradvfactor[1] = gf
        p.aziz_year, p.virial_window, p.mu = aziz_year, virial_window, mu
        self.M, self.Ne = int(num_slices), int(num_ptcl_ext)
        self.side = np.array(side)
        self.h = self.lib.orc_create(C.byref(p))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def load(self, cfg):
        pos = np.ascontiguousarray(cfg["pos"], dtype=np.float64)
        nxt = np.ascontiguousarray(cfg["next"], dtype=np.int32)
        prv = np.ascontiguousarray(cfg["prev"], dtype=np.int32)
        on = np.ascontiguousarray(cfg["on"], dtype=np.uint8)
        worm = np.ascontiguousarray(cfg.get("worm", np.full(8, -1)), dtype=np.int32)
        self.lib.orc_load_path(self.h, _d(pos), _i(nxt), _i(prv),
                               on.ctypes.data_as(C.POINTER(C.c_uint8)), _i(worm))

    def positions(self):
        out = np.zeros((self.M, self.Ne, 3))
        self.lib.orc_get_positions(self.h, _d(out))
        return out

    def update_bead(self, s, p, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        self.lib.orc_update_bead(self.h, s, p, _d(r))

    def set_shift(self, shift):
        self.lib.orc_set_shift(self.h, shift)

    def table_length(self):
        return self.lib.orc_table_length(self.h)

    def tailV(self):
        return self.lib.orc_tailV(self.h)

    def tables(self):
        n = self.table_length()
        V, dV, d2V = np.zeros(n), np.zeros(n), np.zeros(n)
        self.lib.orc_copy_tables(self.h, _d(V), _d(dV), _d(d2V))
        return V, dV, d2V

    def V(self, sep):
        sep = np.ascontiguousarray(sep, dtype=np.float64)
        return self.lib.orc_V(self.h, _d(sep))

    def gradV(self, sep):
        sep = np.ascontiguousarray(sep, dtype=np.float64)
        out = np.zeros(3)
        self.lib.orc_gradV(self.h, _d(sep), _d(out))
        return out

    def grad2V(self, sep):
        sep = np.ascontiguousarray(sep, dtype=np.float64)
        return self.lib.orc_grad2V(self.h, _d(sep))

    def bead_action(self, s, p, mode=0):
        if mode == 0:
            return self.lib.orc_potential_action_bead(self.h, s, p)
        if mode == 1:
            return self.lib.orc_bare_potential_action(self.h, s, p)
        return self.lib.orc_potential_action_correction(self.h, s, p)

    def range_action(self, start, end):
        return self.lib.orc_potential_action_range(self.h, start[0], start[1], end[0], end[1])

    def list_action(self, beads):
        b = np.ascontiguousarray(beads, dtype=np.int32).reshape(-1, 2)
        return self.lib.orc_potential_action_list(self.h, _i(b), len(b))

    def full_action(self):
        return self.lib.orc_potential_action_full(self.h)

    def kinetic_action(self):
        return self.lib.orc_kinetic_action_full(self.h)

    def slice_fn(self, name, s):
        return getattr(self.lib, "orc_" + name)(self.h, s)

    def V_slice(self, s):
        out = np.zeros(2)
        self.lib.orc_V_slice(self.h, s, _d(out))
        return out

    def energy(self):
        out = np.zeros(9)
        self.lib.orc_energy(self.h, _d(out))
        return out

    def virial(self, quirk=True):
        out = np.zeros(19)
        self.lib.orc_virial(self.h, 1 if quirk else 0, _d(out))
        return out

    def ssf_pairwise(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(len(q))
        self.lib.orc_ssf_pairwise(self.h, _d(q), len(q), _d(out))
        return out

    def ssf_rhoq(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(len(q))
        self.lib.orc_ssf_rhoq(self.h, _d(q), len(q), _d(out))
        return out

    def isf_cpu_form(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((len(q), self.M))
        self.lib.orc_isf_cpu_form(self.h, _d(q), len(q), _d(out))
        return out

    def isf_gpu_form(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((len(q), self.M // 2 + 1))
        self.lib.orc_isf_gpu_form(self.h, _d(q), len(q), _d(out))
        return out

    def isf_rhoq(self, q, threads=1):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((len(q), self.M // 2 + 1))
        self.lib.orc_isf_rhoq(self.h, _d(q), len(q), threads, _d(out))
        return out

    def pair_correlation(self, slice=-1):
        out = np.zeros(50)
        self.lib.orc_pair_correlation(self.h, slice, _d(out))
        return out

    def superfluid(self):
        out = np.zeros(26)
        self.lib.orc_superfluid(self.h, _d(out))
        return out

    def permutation_cycles(self):
        out = np.zeros(40)
        self.lib.orc_permutation_cycles(self.h, _d(out))
        return out

    def ssf_cylinder(self, q, max_r):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(len(q))
        n0 = C.c_int()
        self.lib.orc_ssf_cylinder(self.h, _d(q), len(q), max_r, _d(out), C.byref(n0))
        return out, n0.value

    def rhoq(self, q):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((len(q), self.M, 2))
        self.lib.orc_rhoq(self.h, _d(q), len(q), _d(out))
        return out

    def run_worm_steps(self, mt, nsteps, mbar, temperature, mu=0.0, worm_constant=1.0, window=-1,
                       gaussian_sd=0.0, diagonal_move=1, var_updates=1, max_wind=1, num_updates=0,
                       initial_num_particles=None, trace_cap=0):
        wp = OrcWormParams(mbar, diagonal_move, var_updates, max_wind, temperature, mu,
                           worm_constant, window, gaussian_sd, num_updates,
                           self.Ne if initial_num_particles is None else initial_num_particles)
        trace = np.zeros((max(trace_cap, 1), 2), dtype=np.int32)
        en = np.zeros(max(nsteps, 1))
        npart = np.zeros(max(nsteps, 1), dtype=np.int32)
        st = OrcWormStats()
        n = self.lib.orc_run_worm_steps(self.h, mt.h, C.byref(wp), nsteps, _i(trace), trace_cap,
                                        _d(en), _i(npart), C.byref(st))
        if n < 0:
            raise RuntimeError("worm steps failed (%d)" % n)
        return dict(trace=trace[:n], energies=en[:nsteps], num_particles=npart[:nsteps],
                    attempted=list(st.attempted), accepted=list(st.accepted),
                    bead_updates=st.bead_updates, diagonal=st.diagonal)

    def path(self):
        nb = self.M * self.Ne
        nxt = np.zeros((self.M, self.Ne, 2), dtype=np.int32)
        prv = np.zeros((self.M, self.Ne, 2), dtype=np.int32)
        on = np.zeros((self.M, self.Ne), dtype=np.uint8)
        worm = np.zeros(8, dtype=np.int32)
        nbs = np.zeros(self.M, dtype=np.int32)
        self.lib.orc_get_path(self.h, _i(nxt), _i(prv), on.ctypes.data_as(C.POINTER(C.c_uint8)),
                              _i(worm), _i(nbs))
        return dict(next=nxt, prev=prv, on=on, worm=worm, nbs=nbs, pos=self.positions())

    def run_steps(self, mt, nsteps, mbar, temperature, diagonal_move=1, var_updates=1,
                  max_wind=1, p_com=0.05, num_updates=0, trace_cap=0):
        mp = OrcMoveParams(mbar, diagonal_move, var_updates, max_wind, temperature, p_com,
                           num_updates)
        trace = np.zeros((max(trace_cap, 1), 2), dtype=np.int32)
        en = np.zeros(max(nsteps, 1))
        st = OrcMoveStats()
        n = self.lib.orc_run_steps(self.h, mt.h, C.byref(mp), nsteps, _i(trace), trace_cap,
                                   _d(en), C.byref(st))
        return dict(trace=trace[:n], energies=en[:nsteps], attempted=list(st.attempted),
                    accepted=list(st.accepted), bead_updates=st.bead_updates)


def gp_eval(training, pos, benzene=False, **kw):
    """GaussianProcessPotential::GP (or GPHeBenzenePotential::V) on the CPU;
    kw: matern_nu, ell, norm_offset, norm_scale, standard_mean, standard_std,
    mean, sigma2, side, periodic."""
    lib = load()
    p = OrcGpParams()
    p.matern_nu = kw["matern_nu"]
    for d in range(3):
        for k in ("ell", "norm_offset", "norm_scale", "side"):
            getattr(p, k)[d] = np.broadcast_to(kw[k], 3)[d]
        p.periodic[d] = int(np.broadcast_to(kw.get("periodic", 1), 3)[d])
    p.standard_mean, p.standard_std = kw["standard_mean"], kw["standard_std"]
    p.mean, p.sigma2 = kw["mean"], kw["sigma2"]
    t = np.ascontiguousarray(training, dtype=np.float64).reshape(-1, 4)
    x = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    out = np.zeros(len(x))
    fn = lib.orc_gp_benzene if benzene else lib.orc_gp_eval
    fn(C.byref(p), _d(t), len(t), _d(x), len(x), _d(out))
    return out


def qvectors_shells(dq, qmax, sphere=False):
    lib = load()
    n = lib.orc_qvectors_shells(dq, qmax, 1 if sphere else 0, None, None, 0)
    q = np.zeros((max(n, 1), 3))
    sh = np.zeros(max(n, 1), dtype=np.int32)
    lib.orc_qvectors_shells(dq, qmax, 1 if sphere else 0, _d(q), sh.ctypes.data_as(C.POINTER(C.c_int)), n)
    return q[:n], sh[:n]


def qvectors(kind, text, side):
    lib = load()
    side = np.ascontiguousarray(np.broadcast_to(np.asarray(side, dtype=np.float64), (3,)))
    n = lib.orc_qvectors(kind.encode(), text.encode(), _d(side), None, 0)
    q = np.zeros((max(n, 1), 3))
    lib.orc_qvectors(kind.encode(), text.encode(), _d(side), _d(q), n)
    return q[:n]


class MT:
    """MT19937 with the reference conversions (include/MersenneTwister.h)."""

    def __init__(self, seed):
        self.lib = load()
        self.h = self.lib.orc_mt_create(seed)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_mt_destroy(self.h)
            self.h = None

    def randint(self, n=None):
        return self.lib.orc_mt_randint(self.h) if n is None else self.lib.orc_mt_randint_n(self.h, n)

    def rand(self):
        return self.lib.orc_mt_rand(self.h)

    def randexc(self):
        return self.lib.orc_mt_randexc(self.h)

    def randnorm(self, mean=0.0, sd=1.0):
        return self.lib.orc_mt_randnorm(self.h, mean, sd)

    def save(self):
        out = np.zeros(625, dtype=np.uint32)
        self.lib.orc_mt_save(self.h, out.ctypes.data_as(C.POINTER(C.c_uint32)))
        return out

    def load(self, words):
        w = np.ascontiguousarray(words, dtype=np.uint32)
        self.lib.orc_mt_load(self.h, w.ctypes.data_as(C.POINTER(C.c_uint32)))


def format_state(cfg, rng_words, counts):
    """The state text as the reference's C++ streams write it."""
    lib = load()
    pos = np.ascontiguousarray(cfg["pos"], dtype=np.float64)
    nxt = np.ascontiguousarray(cfg["next"], dtype=np.int32)
    prv = np.ascontiguousarray(cfg["prev"], dtype=np.int32)
    on = np.ascontiguousarray(cfg["on"], dtype=np.uint8)
    m, ne = on.shape
    cnt = np.ascontiguousarray(counts, dtype=np.int64).reshape(-1, 2)
    w = np.ascontiguousarray(rng_words, dtype=np.uint32)
    args = (_d(pos), _i(nxt), _i(prv), on.ctypes.data_as(C.POINTER(C.c_uint8)), m, ne,
            cnt.ctypes.data_as(C.POINTER(C.c_longlong)), len(cnt),
            w.ctypes.data_as(C.POINTER(C.c_uint32)))
    n = lib.orc_format_state(*args, None, 0)
    buf = C.create_string_buffer(n + 1)
    lib.orc_format_state(*args, buf, n + 1)
    return buf.value.decode()


def walkers_cpu(n, m, temperature, side, seeds, tau, lam, nsteps, threads, nequil=0,
                with_setup=False):
    """Canonical staging + COM walkers on `threads` host threads.  Returns the
    wall seconds of the nsteps timed steps (set-up and the nequil unsampled
    steps excluded), per-walker mean E/N and bead updates of the timed steps,
    and with with_setup the set-up seconds as a fourth value."""
    lib = load()
    n = np.ascontiguousarray(n, dtype=np.int32)
    m = np.ascontiguousarray(m, dtype=np.int32)
    t = np.ascontiguousarray(temperature, dtype=np.float64)
    L = np.ascontiguousarray(side, dtype=np.float64)
    s = np.ascontiguousarray(seeds, dtype=np.uint32)
    en = np.zeros(len(n))
    bu = np.zeros(len(n), dtype=np.int64)
    setup = C.c_double()
    sec = lib.orc_walkers_cpu(len(n), _i(n), _i(m), _d(t), _d(L),
                              s.ctypes.data_as(C.POINTER(C.c_uint32)), tau, lam, nequil, nsteps,
                              threads,
                              _d(en), bu.ctypes.data_as(C.POINTER(C.c_longlong)), C.byref(setup))
    return (sec, en, bu, setup.value) if with_setup else (sec, en, bu)


def worm_walkers_cpu(n, m, side, mbar, seeds, tau, lam, nsteps, threads, nequil=0, window=1,
                     diagonal_move=0, worm_constant=1.0, npre=0):
    """Worm-engine walkers (the reference's default move list; diagonal_move 0
    bisection, 1 staging) on `threads` host threads.  Returns a dict with the
    timed wall seconds of nsteps steps of every walker, the set-up seconds
    (system, tables, seeded worldlines and nequil untimed steps), per-walker
    bead updates and mean E/N over the timed steps that ended diagonal, and
    the number of walkers that outgrew their bead extent.  npre diagonal
    pre-equilibration steps (centre of mass and diagonal moves only) come
    before the nequil steps, untimed."""
    lib = load()
    n = np.ascontiguousarray(n, dtype=np.int32)
    m = np.ascontiguousarray(m, dtype=np.int32)
    L = np.ascontiguousarray(side, dtype=np.float64)
    mb = np.ascontiguousarray(mbar, dtype=np.int32)
    c0 = np.ascontiguousarray(np.broadcast_to(worm_constant, len(n)), dtype=np.float64)
    s = np.ascontiguousarray(seeds, dtype=np.uint32)
    en = np.zeros(len(n))
    bu = np.zeros(len(n), dtype=np.int64)
    setup = C.c_double()
    failed = C.c_int()
    sec = lib.orc_worm_walkers_cpu(len(n), _i(n), _i(m), _d(L), _i(mb), _d(c0),
                                   s.ctypes.data_as(C.POINTER(C.c_uint32)), tau, lam, window,
                                   diagonal_move, npre, nequil, nsteps, threads, _d(en),
                                   bu.ctypes.data_as(C.POINTER(C.c_longlong)), C.byref(setup),
                                   C.byref(failed))
    return dict(seconds=sec, setup_seconds=setup.value, bead_updates=bu, energy=en,
                failed=failed.value)

"""ctypes binding of libpimc_gb300.so (the C ABI declared in include/pimc_gb300.h).

The shared library is built in-tree by pimc_gb300/build.py.  Loading fails
loudly when it is missing: there is no CPU fallback for any entry point.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpimc_gb300.so")

PGB_OK, PGB_EINVAL, PGB_ECUDA, PGB_ENOMEM, PGB_ESTATE, PGB_ETIMEOUT = 0, -1, -2, -3, -4, -5
PGB_FP64, PGB_MIXED = 0, 1
PGB_ACTION_FULL, PGB_ACTION_BARE, PGB_ACTION_CORR = 0, 1, 2


class PgbParams(C.Structure):
    _fields_ = [("side", C.c_double * 3), ("num_slices", C.c_int), ("num_ptcl_ext", C.c_int),
                ("tau", C.c_double), ("lambda_", C.c_double), ("rc", C.c_double),
                ("vfactor", C.c_double * 2), ("gradvfactor", C.c_double * 2),
                ("period", C.c_int), ("aziz_year", C.c_int), ("virial_window", C.c_int),
                ("precision", C.c_int), ("mu", C.c_double)]


class PgbSliceTerms(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_double)) for n in
                ("vint", "g2", "r1", "r2", "d1", "d2", "kin", "xch")]


class PgbWalkersParams(C.Structure):
    _fields_ = [("num_walkers", C.c_int), ("num_ptcl", C.POINTER(C.c_int)),
                ("num_slices", C.POINTER(C.c_int)), ("temperature", C.POINTER(C.c_double)),
                ("side", C.POINTER(C.c_double)), ("mbar", C.POINTER(C.c_int)),
                ("tau", C.c_double), ("lambda_", C.c_double), ("p_com", C.c_double),
                ("seed", C.c_uint64), ("aziz_year", C.c_int),
                ("threads_per_walker", C.c_int), ("var_updates", C.c_int)]


class PgbWalkerStats(C.Structure):
    _fields_ = [("energy_sum", C.c_double), ("energy_sumsq", C.c_double),
                ("samples", C.c_longlong), ("bead_updates", C.c_longlong),
                ("attempted", C.c_longlong * 2), ("accepted", C.c_longlong * 2)]


class PgbMoveParams(C.Structure):
    _fields_ = [("mbar", C.c_int), ("diagonal_move", C.c_int), ("var_updates", C.c_int),
                ("max_wind", C.c_int), ("temperature", C.c_double), ("p_com", C.c_double),
                ("num_updates", C.c_int)]


class PgbMoveStats(C.Structure):
    _fields_ = [("attempted", C.c_longlong * 3), ("accepted", C.c_longlong * 3),
                ("bead_updates", C.c_longlong)]


class PgbServerParams(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_double), ("max_active", C.c_int),
                ("sweeps_per_round", C.c_int), ("bin_sweeps", C.c_int), ("tau", C.c_double),
                ("lambda_", C.c_double), ("p_com", C.c_double), ("aziz_year", C.c_int),
                ("round_seconds", C.c_double), ("diagonal_move", C.c_int)]


class PgbGpParams(C.Structure):
    _fields_ = [("matern_nu", C.c_double), ("ell", C.c_double * 3), ("norm_offset", C.c_double * 3),
                ("norm_scale", C.c_double * 3), ("standard_mean", C.c_double),
                ("standard_std", C.c_double), ("mean", C.c_double), ("sigma2", C.c_double),
                ("side", C.c_double * 3), ("periodic", C.c_int * 3), ("precision", C.c_int)]


class PgbWormParams(C.Structure):
    _fields_ = [("mbar", C.c_int), ("diagonal_move", C.c_int), ("var_updates", C.c_int),
                ("max_wind", C.c_int), ("temperature", C.c_double), ("mu", C.c_double),
                ("worm_constant", C.c_double), ("window", C.c_int), ("gaussian_sd", C.c_double),
                ("num_updates", C.c_int), ("initial_num_particles", C.c_int)]


class PgbWormStats(C.Structure):
    _fields_ = [("attempted", C.c_longlong * 12), ("accepted", C.c_longlong * 12),
                ("bead_updates", C.c_longlong), ("diagonal", C.c_int)]


class PgbWormWalkersParams(C.Structure):
    _fields_ = [("num_walkers", C.c_int), ("num_ptcl", C.POINTER(C.c_int)),
                ("num_slices", C.POINTER(C.c_int)), ("side", C.POINTER(C.c_double)),
                ("mu", C.POINTER(C.c_double)), ("mbar", C.POINTER(C.c_int)),
                ("capacity", C.POINTER(C.c_int)), ("tau", C.c_double), ("lambda_", C.c_double),
                ("worm_constant", C.c_double), ("window", C.c_int), ("seed", C.c_uint64),
                ("aziz_year", C.c_int), ("diagonal_move", C.c_int),
                ("worm_constants", C.POINTER(C.c_double))]


class PgbWormWalkerStats(C.Structure):
    _fields_ = [("energy_sum", C.c_double), ("energy_sumsq", C.c_double), ("n_sum", C.c_double),
                ("n_sumsq", C.c_double), ("samples", C.c_longlong), ("attempted", C.c_longlong * 12),
                ("accepted", C.c_longlong * 12), ("bead_updates", C.c_longlong),
                ("sweeps", C.c_longlong), ("error", C.c_int), ("pad", C.c_int)]


class PgbJobSpec(C.Structure):
    _fields_ = [("n", C.c_int), ("temperature", C.c_double), ("mu", C.c_double),
                ("density", C.c_double), ("sweeps", C.c_longlong), ("seed", C.c_uint64),
                ("arrival", C.c_double)]


class PgbBin(C.Structure):
    _fields_ = [("job", C.c_int), ("bin", C.c_int), ("energy_per_particle", C.c_double),
                ("samples", C.c_longlong), ("time", C.c_double)]


class PgbJobInfo(C.Structure):
    _fields_ = [("state", C.c_int), ("arrival", C.c_double), ("admitted", C.c_double),
                ("first_bin", C.c_double), ("completed", C.c_double), ("sweeps_done", C.c_longlong),
                ("n", C.c_int), ("m", C.c_int), ("bytes", C.c_size_t)]


_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int32)
_FP = C.POINTER(C.c_float)
_U8 = C.POINTER(C.c_uint8)
_VP = C.c_void_p

_SIGS = {
    "pgb_create": (C.c_int, [C.POINTER(PgbParams), C.POINTER(_VP)]),
    "pgb_destroy": (C.c_int, [_VP]),
    "pgb_last_error": (C.c_char_p, [_VP]),
    "pgb_device_info": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "pgb_table_info": (C.c_int, [_VP, C.POINTER(C.c_int), _DP, _DP]),
    "pgb_copy_tables": (C.c_int, [_VP, _DP, _DP, _DP]),
    "pgb_potential_batch": (C.c_int, [_VP, _DP, _DP, C.c_int]),
    "pgb_gradv_batch": (C.c_int, [_VP, _DP, _DP, C.c_int]),
    "pgb_grad2v_batch": (C.c_int, [_VP, _DP, _DP, C.c_int]),
    "pgb_load_path": (C.c_int, [_VP, _DP, _IP, _IP, _U8, _IP]),
    "pgb_update_beads": (C.c_int, [_VP, _IP, _DP, C.c_int]),
    "pgb_get_positions": (C.c_int, [_VP, _DP]),
    "pgb_bead_actions": (C.c_int, [_VP, _IP, C.c_int, C.c_int, C.c_int, _DP, _DP]),
    "pgb_trial_actions": (C.c_int, [_VP, _IP, _DP, C.c_int, C.c_int, C.c_int, _DP]),
    "pgb_trial_actions_device_async": (C.c_int, [_VP, _VP, _VP, C.c_int, C.c_int, C.c_int, _VP, _VP]),
    "pgb_range_action": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _DP]),
    "pgb_full_action": (C.c_int, [_VP, _DP]),
    "pgb_kinetic_action": (C.c_int, [_VP, _DP]),
    "pgb_slice_terms_compute": (C.c_int, [_VP, C.POINTER(PgbSliceTerms)]),
    "pgb_energy": (C.c_int, [_VP, _DP]),
    "pgb_virial": (C.c_int, [_VP, C.c_int, _DP]),
    "pgb_qvectors": (C.c_int, [C.c_char_p, C.c_char_p, _DP, _DP, C.c_int, C.POINTER(C.c_int)]),
    "pgb_ssf": (C.c_int, [_VP, _DP, C.c_int, _DP]),
    "pgb_isf": (C.c_int, [_VP, _DP, C.c_int, C.c_int, _DP]),
    "pgb_test_isf_tc_stall": (None, [C.c_int]),
    "pgb_rhoq": (C.c_int, [_VP, _DP, C.c_int, _DP]),
    "pgb_isf_device_async": (C.c_int, [_VP, _VP, C.c_int, C.c_int, _VP]),
    "pgb_update_positions": (C.c_int, [_VP, _DP]),
    "pgb_pair_correlation": (C.c_int, [_VP, C.c_int, _DP]),
    "pgb_ssf_cylinder": (C.c_int, [_VP, _DP, C.c_int, C.c_double, _DP, C.POINTER(C.c_int)]),
    "pgb_qvectors_shells": (C.c_int, [C.c_double, C.c_double, C.c_int, _DP, C.POINTER(C.c_int),
                                      C.c_int, C.POINTER(C.c_int)]),
    "pgb_plain_get_rng": (C.c_int, [_VP, C.POINTER(C.c_uint32)]),
    "pgb_worm_server_create": (C.c_int, [C.POINTER(PgbServerParams), C.POINTER(C.c_void_p)]),
    "pgb_worm_server_destroy": (C.c_int, [_VP]),
    "pgb_worm_server_submit": (C.c_int, [_VP, C.POINTER(PgbJobSpec), C.POINTER(C.c_int)]),
    "pgb_worm_server_step": (C.c_int, [_VP, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "pgb_worm_server_poll_bins": (C.c_int, [_VP, C.POINTER(PgbBin), C.c_int, C.POINTER(C.c_int)]),
    "pgb_worm_server_job_info": (C.c_int, [_VP, C.c_int, C.POINTER(PgbJobInfo)]),
    "pgb_worm_server_clock": (C.c_double, [_VP]),
    "pgb_worm_server_active_bead_updates": (C.c_int, [_VP, C.POINTER(C.c_longlong)]),
    "pgb_worm_server_last_error": (C.c_char_p, [_VP]),
    "pgb_worm_walkers_create": (C.c_int, [C.POINTER(PgbWormWalkersParams), C.POINTER(C.c_void_p)]),
    "pgb_worm_walkers_destroy": (C.c_int, [_VP]),
    "pgb_worm_walkers_last_error": (C.c_char_p, [_VP]),
    "pgb_worm_walkers_load": (C.c_int, [_VP, C.c_int, _DP]),
    "pgb_worm_walkers_run": (C.c_int, [_VP, C.c_int]),
    "pgb_worm_walkers_run_async": (C.c_int, [_VP, C.c_int]),
    "pgb_worm_walkers_equilibrate": (C.c_int, [_VP, C.c_int]),
    "pgb_worm_walkers_synchronize": (C.c_int, [_VP]),
    "pgb_worm_walkers_stream": (_VP, [_VP]),
    "pgb_worm_walkers_launch_count": (C.c_longlong, [_VP]),
    "pgb_worm_walkers_seed": (C.c_int, [_VP, C.c_uint64]),
    "pgb_worm_walkers_state_bytes": (C.c_longlong, [_VP]),
    "pgb_worm_walkers_get_state": (C.c_int, [_VP, _VP]),
    "pgb_worm_walkers_set_state_async": (C.c_int, [_VP, _VP]),
    "pgb_worm_walkers_stats_async": (C.c_int, [_VP, C.POINTER(PgbWormWalkerStats)]),
    "pgb_worm_walkers_bead_actions": (C.c_int, [_VP, C.c_int, _IP, C.c_int, _DP]),
    "pgb_worm_walkers_stats": (C.c_int, [_VP, C.POINTER(PgbWormWalkerStats)]),
    "pgb_worm_walkers_reset_stats": (C.c_int, [_VP]),
    "pgb_worm_walkers_get_path": (C.c_int, [_VP, C.c_int, _DP, _IP, _IP, C.POINTER(C.c_uint8), _IP]),
    "pgb_worm_normals_check": (C.c_int, [C.c_uint64, C.c_int, C.c_int, _FP, _FP, _IP]),
    "pgb_plain_worm_run": (C.c_int, [_VP, C.POINTER(PgbWormParams), C.c_int, _IP, C.c_int,
                                     C.POINTER(C.c_int), _DP, _IP, C.POINTER(PgbWormStats)]),
    "pgb_set_beads": (C.c_int, [_VP, _IP, _DP, _IP, _IP, C.POINTER(C.c_uint8), C.c_int]),
    "pgb_set_worm": (C.c_int, [_VP, _IP]),
    "pgb_get_path": (C.c_int, [_VP, _IP, _IP, C.POINTER(C.c_uint8), _IP]),
    "pgb_gp_create": (C.c_int, [C.POINTER(PgbGpParams), _DP, C.c_int, C.POINTER(C.c_void_p)]),
    "pgb_gp_destroy": (C.c_int, [_VP]),
    "pgb_gp_last_error": (C.c_char_p, [_VP]),
    "pgb_gp_stream": (C.c_void_p, [_VP]),
    "pgb_gp_eval": (C.c_int, [_VP, _DP, _DP, C.c_int]),
    "pgb_gp_eval_device_async": (C.c_int, [_VP, _VP, _VP, C.c_int]),
    "pgb_gp_benzene_v": (C.c_int, [_VP, _DP, _DP, C.c_int]),
    "pgb_plain_set_rng": (C.c_int, [_VP, C.POINTER(C.c_uint32)]),
    "pgb_walkers_get_all_positions": (C.c_int, [_VP, _DP]),
    "pgb_walkers_get_sweeps": (C.c_int, [_VP, C.POINTER(C.c_ulonglong)]),
    "pgb_walkers_set_sweeps": (C.c_int, [_VP, C.POINTER(C.c_ulonglong)]),
    "pgb_superfluid": (C.c_int, [_VP, _DP]),
    "pgb_permutation_cycles": (C.c_int, [_VP, _DP]),
    "pgb_ssf_device_async": (C.c_int, [_VP, _VP, C.c_int, _VP]),
    "pgb_load_positions_device_async": (C.c_int, [_VP, _VP]),
    "pgb_stream": (_VP, [_VP]),
    "pgb_isf_static": (C.c_int, [_VP, C.c_int, C.c_int, C.c_int, _DP, _VP, C.c_int, _VP, _VP]),
    "pgb_walkers_create": (C.c_int, [C.POINTER(PgbWalkersParams), C.POINTER(_VP)]),
    "pgb_walkers_destroy": (C.c_int, [_VP]),
    "pgb_walkers_init": (C.c_int, [_VP]),
    "pgb_walkers_set_positions": (C.c_int, [_VP, C.c_int, _DP]),
    "pgb_walkers_get_positions": (C.c_int, [_VP, C.c_int, _DP]),
    "pgb_walkers_set_all_positions": (C.c_int, [_VP, _DP]),
    "pgb_walkers_state_bytes": (C.c_size_t, [_VP]),
    "pgb_walkers_run_async": (C.c_int, [_VP, C.c_int, C.c_int]),
    "pgb_walkers_sync": (C.c_int, [_VP]),
    "pgb_walkers_stats": (C.c_int, [_VP, C.POINTER(PgbWalkerStats)]),
    "pgb_walkers_reset_stats": (C.c_int, [_VP]),
    "pgb_walkers_launch_count": (C.c_longlong, [_VP]),
    "pgb_walkers_threads": (C.c_int, [_VP]),
    "pgb_walkers_tuning": (C.c_int, [_VP, C.POINTER(C.c_int), C.POINTER(C.c_float), C.c_int]),
    "pgb_walkers_energy": (C.c_int, [_VP, C.c_int, _DP]),
    "pgb_walkers_stream": (_VP, [_VP]),
    "pgb_walkers_last_error": (C.c_char_p, [_VP]),
    "pgb_server_create": (C.c_int, [C.POINTER(PgbServerParams), C.POINTER(_VP)]),
    "pgb_server_destroy": (C.c_int, [_VP]),
    "pgb_server_submit": (C.c_int, [_VP, C.POINTER(PgbJobSpec), C.POINTER(C.c_int)]),
    "pgb_server_step": (C.c_int, [_VP, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "pgb_server_poll_bins": (C.c_int, [_VP, C.POINTER(PgbBin), C.c_int, C.POINTER(C.c_int)]),
    "pgb_server_job_info": (C.c_int, [_VP, C.c_int, C.POINTER(PgbJobInfo)]),
    "pgb_server_clock": (C.c_double, [_VP]),
    "pgb_server_bead_updates": (C.c_longlong, [_VP]),
    "pgb_server_active_bead_updates": (C.c_int, [_VP, C.POINTER(C.c_longlong)]),
    "pgb_server_last_error": (C.c_char_p, [_VP]),
    "pgb_plain_seed": (C.c_int, [_VP, C.c_uint32]),
    "pgb_plain_run": (C.c_int, [_VP, C.POINTER(PgbMoveParams), C.c_int, _IP, C.c_int,
                                C.POINTER(C.c_int), _DP, C.POINTER(PgbMoveStats)]),
}

_lib = None


def exported_symbols():
    """Names of every entry point the C ABI header declares."""
    return sorted(_SIGS)


def load():
    """Load the in-tree library (raises OSError if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OSError("libpimc_gb300.so not found at %s: run "
                      "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class PgbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("pgb error %d: %s" % (code, msg))
        self.code = code


def dptr(a):
    return a.ctypes.data_as(_DP)


def iptr(a):
    return a.ctypes.data_as(_IP)


def u8ptr(a):
    return a.ctypes.data_as(_U8)


def check(rc, handle=None, walkers=False, server=False, gp=False, worm=False, worm_server=False):
    if rc != PGB_OK:
        lib = load()
        if worm_server:
            msg = lib.pgb_worm_server_last_error(handle)
        elif worm:
            msg = lib.pgb_worm_walkers_last_error(handle)
        elif gp:
            msg = lib.pgb_gp_last_error(handle)
        elif server:
            msg = lib.pgb_server_last_error(handle)
        elif walkers:
            msg = lib.pgb_walkers_last_error(handle)
        else:
            msg = lib.pgb_last_error(handle)
        raise PgbError(rc, (msg or b"").decode())
    return rc

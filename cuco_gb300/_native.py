"""ctypes binding of libcuco_gb300.so (the C ABI in include/cuco_gb300.h).

The library is built in-tree (cuco_gb300/_lib/) by cuco_gb300.build.  There is
no fallback: if the library is missing or fails to load, every entry point
raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libcuco_gb300.so")


class CucoError(RuntimeError):
    pass


class CucoConfig(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("pm_grid", ctypes.c_int), ("cell_grid", ctypes.c_int),
                ("boxsize", ctypes.c_float), ("mass", ctypes.c_float), ("G", ctypes.c_double),
                ("asmth", ctypes.c_float), ("rcut", ctypes.c_float), ("softening", ctypes.c_float),
                ("mode", ctypes.c_int), ("device", ctypes.c_int)]


class SimParam(ctypes.Structure):
    _fields_ = [("shortrange_table", ctypes.c_float * 1000), ("boxsize", ctypes.c_float),
                ("boxhalf", ctypes.c_float), ("to_grid_fac", ctypes.c_float), ("rcut", ctypes.c_float),
                ("rcut2", ctypes.c_float), ("asmth", ctypes.c_float), ("asmthfac", ctypes.c_float),
                ("mass", ctypes.c_float), ("G", ctypes.c_float)]


class SoftParam(ctypes.Structure):
    _fields_ = [("h", ctypes.c_float), ("h_inv", ctypes.c_float), ("h3_inv", ctypes.c_float)]


class Particle(ctypes.Structure):
    _fields_ = [("Pos", ctypes.c_float * 3), ("Mass", ctypes.c_float), ("Vel", ctypes.c_float * 3),
                ("GravAccel", ctypes.c_float * 3), ("GravPM", ctypes.c_float * 3),
                ("Ti_endstep", ctypes.c_int), ("Ti_begstep", ctypes.c_int)]


class Header(ctypes.Structure):
    _fields_ = [("NumPart", ctypes.c_int), ("Mass", ctypes.c_float), ("Time", ctypes.c_float),
                ("Redshift", ctypes.c_float), ("BoxSize", ctypes.c_float), ("Omega0", ctypes.c_float),
                ("OmegaLambda", ctypes.c_float), ("HubbleParam", ctypes.c_float)]


class All(ctypes.Structure):
    _fields_ = [("NumPart", ctypes.c_int), ("BoxSize", ctypes.c_float), ("Mass", ctypes.c_float),
                ("G", ctypes.c_double), ("UnitTime_in_s", ctypes.c_double),
                ("UnitMass_in_kg", ctypes.c_double), ("UnitVelocity_in_m_per_s", ctypes.c_double),
                ("UnitLength_in_m", ctypes.c_double), ("UnitTime_in_Megayears", ctypes.c_double),
                ("Hubble", ctypes.c_float), ("Omega0", ctypes.c_float), ("OmegaLambda", ctypes.c_float),
                ("OmegaBaryon", ctypes.c_float), ("HubbleParam", ctypes.c_float),
                ("Time", ctypes.c_float), ("TimeBegin", ctypes.c_float), ("TimeStep", ctypes.c_float),
                ("TimeMax", ctypes.c_float), ("Timebase_interval", ctypes.c_double),
                ("Ti_Current", ctypes.c_int), ("Ti_nextoutput", ctypes.c_int),
                ("PM_Ti_endstep", ctypes.c_int), ("PM_Ti_begstep", ctypes.c_int),
                ("Asmth", ctypes.c_float), ("Rcut", ctypes.c_float),
                ("ErrTolIntAccuracy", ctypes.c_float), ("MaxSizeTimestep", ctypes.c_float),
                ("MinSizeTimestep", ctypes.c_float), ("SofteningHalo", ctypes.c_float),
                ("SofteningHaloMaxPhys", ctypes.c_float), ("SofteningTable", ctypes.c_float),
                ("ForceSoftening", ctypes.c_float), ("NumCurrentTiStep", ctypes.c_int),
                ("SnapshotFileCount", ctypes.c_int), ("OutputListTimes", ctypes.c_float * 500),
                ("OutputListLength", ctypes.c_int), ("InitCondFile", ctypes.c_char * 250),
                ("OutputDir", ctypes.c_char * 250), ("SnapshotFileBase", ctypes.c_char * 250),
                ("OutputListFilename", ctypes.c_char * 250)]


# Every function include/cuco_gb300.h declares, with its ctypes signature.
_P = ctypes.c_void_p
_I = ctypes.c_int
_U = ctypes.c_uint
_D = ctypes.c_double
SIGNATURES = {
    # gravlist.cu / radixsort names
    "cudaInit": (None, []),
    "allocateArray": (None, [ctypes.POINTER(_P), ctypes.c_size_t]),
    "freeArray": (None, [_P]),
    "copyArrayFromDevice": (None, [_P, _P, _I]),
    "copyArrayToDevice": (None, [_P, _P, _I, _I]),
    "setSimParam": (None, [ctypes.POINTER(SimParam)]),
    "setSoftParam": (None, [ctypes.POINTER(SoftParam)]),
    "copyPosToDevice": (None, []),
    "copyAccelFromDevice": (None, []),
    "calcHash": (None, [_P, _P, _P, _U]),
    "reorderDataAndFindCellStart": (None, [_P, _P, _P, _P, _P, _P, _U, _U]),
    "cudaForceEvaluateShortrange": (None, [_P, _P, _P, _P, _P, _U, _U]),
    "radixSort": (None, [_P, _P, _P, _P, _P, _P, _P, ctypes.c_size_t, _U, _U, ctypes.c_bool]),
    "radixSortKeysOnly": (None, [_P, _P, _P, _P, _P, ctypes.c_size_t, _U, _U, ctypes.c_bool]),
    "radixSortFloatKeys": (None, [_P, _P, _P, _P, _P, _P, _P, ctypes.c_size_t, _U, _U, ctypes.c_bool]),
    "radixSortFloatKeysOnly": (None, [_P, _P, _P, _P, _P, ctypes.c_size_t, _U, _U, ctypes.c_bool]),
    "cuco_radixsort_overflow": (None, [_U, _U]),
    "cuco_box_selftest_timeout": (_I, [_P, _D]),
    "cuco_debug_bounds_violations": (_I, [_P]),
    "read_ic": (None, [ctypes.c_char_p]),
    "savepositions": (None, [_I]),
    "cuco_box_load_snapshot": (_I, [_P, ctypes.c_char_p, _I, _P]),
    "cuco_box_save_snapshot": (_I, [_P, ctypes.c_char_p, _P]),
    "initDeviceParameters": (None, []),
    "checkCudaError": (None, [ctypes.c_char_p]),
    # host force / integrator names
    "cuco_dropin_configure": (None, [_I, _I]),
    "long_range_init": (None, []),
    "long_range_force": (None, []),
    "pm_init_periodic": (None, []),
    "pm_init_periodic_allocate": (None, []),
    "pm_init_periodic_free": (None, []),
    "pmforce_periodic": (None, []),
    "set_softenings": (None, []),
    "linklist_init": (None, []),
    "gravity_linklist_cuda": (None, []),
    "compute_accelerations": (None, []),
    "move_particles": (None, [_I, _I]),
    "do_box_wrapping": (None, []),
    "advance_and_find_timesteps": (None, []),
    "get_timestep": (_I, [_I]),
    "cuco_dropin_min_ti_endstep": (_I, []),
    "cuco_dropin_host_access": (_I, []),
    "init_drift_table": (None, []),
    "drift_integ": (_D, [_D, _P]),
    "gravkick_integ": (_D, [_D, _P]),
    "get_drift_factor": (_D, [_I, _I]),
    "get_gravkick_factor": (_D, [_I, _I]),
    # engine
    "cuco_config_reference": (_I, [ctypes.POINTER(CucoConfig)]),
    "cuco_box_create": (_I, [ctypes.POINTER(CucoConfig), ctypes.POINTER(_P)]),
    "cuco_box_destroy": (_I, [_P]),
    "cuco_box_set_state": (_I, [_P, _P, _P, _I]),
    "cuco_box_get_state": (_I, [_P, _P, _P, _P, _P, _I]),
    "cuco_box_set_state_fixed": (_I, [_P, _P, _P, _I]),
    "cuco_box_get_state_fixed": (_I, [_P, _P, _I]),
    "cuco_box_set_softening": (_I, [_P, ctypes.c_float]),
    "cuco_box_forces": (_I, [_P, _I, _I]),
    "cuco_box_step": (_I, [_P, _D, _D, _D]),
    "cuco_box_run": (_I, [_P, _I, _P, _P, _P]),
    "cuco_box_sync": (_I, [_P]),
    "cuco_box_stream": (_I, [_P, ctypes.POINTER(_P)]),
    "cuco_box_enable_timing": (_I, [_P, _I]),
    "cuco_box_timings": (_I, [_P, _P]),
    "cuco_box_phase_totals": (_I, [_P, _P, _I]),
    "cuco_box_debug": (_I, [_P, _P, _P, _P, _P]),
    "cuco_box_cell_order": (_I, [_P, _P, _P]),
    "cuco_box_launches_per_step": (_I, [_P]),
    "cuco_box_count_pairs": (_I, [_P, _I]),
    "cuco_box_pair_count": (_I, [_P, ctypes.POINTER(ctypes.c_uint64), _I]),
    "cuco_box_timer": (_I, [_P, _I, ctypes.POINTER(ctypes.c_float)]),
    "cuco_ensemble_create": (_I, [ctypes.POINTER(CucoConfig), _I, ctypes.POINTER(_P)]),
    "cuco_ensemble_destroy": (_I, [_P]),
    "cuco_ensemble_reshape": (_I, [_P, ctypes.POINTER(CucoConfig), _I, _P]),
    "cuco_ensemble_cell_grid": (_I, [_P, _I, _P, _P, _P]),
    "cuco_ensemble_set_state": (_I, [_P, _I, _P, _P]),
    "cuco_ensemble_get_state": (_I, [_P, _I, _P, _P, _P, _P]),
    "cuco_ensemble_forces": (_I, [_P]),
    "cuco_ensemble_step": (_I, [_P, _P, _P, _P]),
    "cuco_ensemble_sync": (_I, [_P]),
    "cuco_ensemble_timer": (_I, [_P, _I, ctypes.POINTER(ctypes.c_float)]),
    "cuco_ensemble_count_pairs": (_I, [_P, _I, _P]),
    "cuco_ensemble_launches_per_step": (_I, [_P]),
    "cuco_ensemble_copy_state": (_I, [_P, _I, _P, _I]),
    "cuco_ensemble_footprint": (_I, [ctypes.POINTER(CucoConfig), _I, _P]),
    "cuco_pinned_alloc": (_I, [ctypes.c_size_t, ctypes.POINTER(_P)]),
    "cuco_pinned_free": (_I, [_P]),
    "cuco_fp32_peak": (_I, [_I, ctypes.POINTER(_D)]),
    "cuco_radix_sort_noalloc": (_I, [_P, _P, _U, _U, _P]),
    "cuco_cosmo_factors": (_I, [_D, _D, _D, _D, _D, ctypes.POINTER(_D), ctypes.POINTER(_D)]),
    "cuco_last_error": (ctypes.c_char_p, []),
    "cuco_version": (ctypes.c_char_p, []),
}

_lib = None


def load(path: str | None = None):
    """Load the native library (once).  Raises CucoError if it is not built.
    $CUCO_LIBRARY selects another build of it (the debug build with bounds
    checks, libcuco_gb300_debug.so)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("CUCO_LIBRARY") or LIB_PATH
    if not os.path.isfile(path):
        raise CucoError(f"{path} is missing: build it with cuco_gb300.build.build() "
                        "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, what: str = "") -> None:
    if status != 0:
        msg = load().cuco_last_error().decode(errors="replace")
        raise CucoError(f"{what}: status {status}: {msg}")


def ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)

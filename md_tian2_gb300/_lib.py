"""ctypes binding of libmdt_gpu.so (include/mdt_gpu.h).

The CUDA library is the only implementation of the hot path: if it is missing or a GPU
is absent, calls raise :class:`EngineError` instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as ct
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libmdt_gpu.so"

c_double_p = ct.POINTER(ct.c_double)
c_int32_p = ct.POINTER(ct.c_int32)
c_uint8_p = ct.POINTER(ct.c_uint8)


class EngineError(RuntimeError):
    """Error status returned by libmdt_gpu."""


class PropParams(ct.Structure):
    _fields_ = [("step", ct.c_double), ("Tsurf", ct.c_double), ("Tproj", ct.c_double),
                ("pile_tau", ct.c_double), ("andersen_time", ct.c_double), ("gamma_const", ct.c_double),
                ("pul", ct.c_double), ("pll", ct.c_double), ("seed", ct.c_uint64),
                ("use_exit", ct.c_int32), ("rng_mode", ct.c_int32)]


class RefillParams(ct.Structure):
    """mdt_refill_params (include/mdt_gpu.h)."""
    _fields_ = [("z0", ct.c_double), ("einc_min", ct.c_double), ("einc_max", ct.c_double),
                ("polar_min", ct.c_double), ("polar_max", ct.c_double), ("azimuth", ct.c_double),
                ("seed", ct.c_uint64)]


class TrajSummary(ct.Structure):
    _fields_ = [("status", ct.c_int32), ("steps_done", ct.c_int32), ("epot", ct.c_double),
                ("ekin_p", ct.c_double), ("ekin_l", ct.c_double), ("ebead", ct.c_double)]


class NNModelC(ct.Structure):
    """mdt_nn_model (include/mdt_gpu.h)."""
    _fields_ = [("nelem", ct.c_int32), ("z", ct.c_void_p), ("maxsf", ct.c_int32), ("nsf", ct.c_void_p),
                ("sftype", ct.c_void_p), ("eta", ct.c_void_p), ("rshift", ct.c_void_p), ("lambda_", ct.c_void_p),
                ("zeta", ct.c_void_p), ("rc", ct.c_void_p), ("e1", ct.c_void_p), ("e2", ct.c_void_p),
                ("smin", ct.c_void_p), ("smax", ct.c_void_p), ("savg", ct.c_void_p),
                ("scalesym", ct.c_int32), ("centersym", ct.c_int32), ("scmin", ct.c_double), ("scmax", ct.c_double),
                ("cutoff_type", ct.c_int32), ("cutoff_alpha", ct.c_double), ("nlayers", ct.c_int32),
                ("maxnodes", ct.c_int32), ("nodes", ct.c_void_p), ("act", ct.c_void_p), ("maxweights", ct.c_int32),
                ("weights", ct.c_void_p), ("normnodes", ct.c_int32), ("remove_atom_energies", ct.c_int32),
                ("atom_energy", ct.c_void_p)]


class TrainOpts(ct.Structure):
    """mdt_train_opts (include/mdt_gpu.h)."""
    _fields_ = [("w_energy", ct.c_double), ("w_force", ct.c_double), ("lr", ct.c_double), ("beta1", ct.c_double),
                ("beta2", ct.c_double), ("eps", ct.c_double), ("precision", ct.c_int32)]


# name -> (restype, argtypes); every symbol declared in include/mdt_gpu.h
SIGNATURES = {
    "mdt_create": (ct.c_int32, [ct.c_int32, ct.POINTER(ct.c_void_p)]),
    "mdt_destroy": (ct.c_int32, [ct.c_void_p]),
    "mdt_last_error": (ct.c_char_p, [ct.c_void_p]),
    "mdt_synchronize": (ct.c_int32, [ct.c_void_p]),
    "mdt_set_stream": (ct.c_int32, [ct.c_void_p, ct.c_void_p]),
    "mdt_emt_set_params": (ct.c_int32, [ct.c_void_p, ct.c_int32] + [c_double_p] * 7 + [c_int32_p]),
    "mdt_batch_define": (ct.c_int32, [ct.c_void_p, ct.c_int32, c_int32_p, c_int32_p, c_int32_p, c_double_p,
                                      c_uint8_p, c_double_p, ct.c_int32, c_int32_p, c_uint8_p]),
    "mdt_state_upload": (ct.c_int32, [ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    "mdt_state_download": (ct.c_int32, [ct.c_void_p] + [ct.c_void_p] * 6),
    "mdt_calc_force": (ct.c_int32, [ct.c_void_p, ct.c_int32, ct.c_int32, ct.POINTER(PropParams)]),
    "mdt_propagate_1": (ct.c_int32, [ct.c_void_p, ct.POINTER(PropParams)]),
    "mdt_propagate_2": (ct.c_int32, [ct.c_void_p, ct.POINTER(PropParams)]),
    "mdt_md_steps": (ct.c_int32, [ct.c_void_p, ct.c_int32, ct.c_int32, ct.POINTER(PropParams)]),
    "mdt_set_random_arrays": (ct.c_int32, [ct.c_void_p] + [ct.c_void_p] * 4),
    "mdt_query": (ct.c_int32, [ct.c_void_p, ct.POINTER(PropParams), ct.POINTER(TrajSummary)]),
    "mdt_device_state": (ct.c_int32, [ct.c_void_p, ct.POINTER(ct.c_void_p), ct.POINTER(ct.c_int64)]),
    "mdt_launch_count": (ct.c_int64, [ct.c_void_p]),
    "mdt_peak_fma": (ct.c_int32, [ct.c_int32, ct.c_int32, c_double_p]),
    "mdt_wait_check": (ct.c_int32, [ct.c_int32, ct.c_int32, ct.POINTER(ct.c_int32), c_double_p]),
    "mdt_rng_deviates": (ct.c_int32, [ct.c_int32, ct.c_uint64, ct.c_int32, ct.c_int32, ct.c_int32, ct.c_int64,
                                      c_double_p]),
    "mdt_nn_set_model": (ct.c_int32, [ct.c_void_p, ct.POINTER(NNModelC), ct.c_int32, c_int32_p, ct.c_int32]),
    "mdt_set_pes": (ct.c_int32, [ct.c_void_p, ct.c_int32, ct.c_double]),
    "mdt_nn_fast_path": (ct.c_int32, [ct.c_void_p, ct.c_int32]),
    "mdt_nn_radial_kernel": (ct.c_int32, [ct.c_void_p, ct.c_int32]),
    "mdt_nn_radial_block": (ct.c_int32, [ct.c_void_p, ct.c_int32]),
    "mdt_traj_observables": (ct.c_int32, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    "mdt_traj_bounces": (ct.c_int32, [ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.POINTER(PropParams)]),
    "mdt_set_adsorption": (ct.c_int32, [ct.c_void_p, ct.c_double, ct.c_double]),
    "mdt_nn_repack": (ct.c_int32, [ct.c_void_p, ct.c_void_p]),
    "mdt_refill_draws": (ct.c_int32, [ct.c_void_p, ct.c_void_p]),
    "mdt_autotune": (ct.c_int32, [ct.c_void_p, ct.c_int32, ct.c_int32, ct.POINTER(PropParams), ct.c_void_p,
                                  ct.c_void_p, ct.c_void_p]),
    "mdt_set_step_limit": (ct.c_int32, [ct.c_void_p, ct.c_int32]),
    "mdt_refill": (ct.c_int32, [ct.c_void_p, ct.POINTER(RefillParams), ct.c_void_p, ct.POINTER(ct.c_int32)]),
    "mdt_nn_set_skin": (ct.c_int32, [ct.c_void_p, ct.c_double]),
    "mdt_nn_stats": (ct.c_int32, [ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    "mdt_nn_neighbors": (ct.c_int32, [ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    "mdt_nn_descriptors": (ct.c_int32, [ct.c_void_p, ct.c_int32, ct.c_void_p]),
    "mdt_train_set_labels": (ct.c_int32, [ct.c_void_p, ct.c_void_p, ct.c_void_p]),
    "mdt_train_step": (ct.c_int32, [ct.c_void_p, ct.POINTER(TrainOpts), ct.c_void_p, ct.c_int32, ct.c_void_p]),
    "mdt_train_gradient": (ct.c_int32, [ct.c_void_p, ct.POINTER(TrainOpts), ct.c_void_p, ct.c_int32, ct.c_void_p]),
    "mdt_train_commit": (ct.c_int32, [ct.c_void_p, ct.c_void_p]),
    "mdt_emt_force_noalloc": (ct.c_int32, [ct.c_int32] + [ct.c_void_p] * 5 + [ct.c_int32] + [ct.c_void_p] * 8 +
                              [ct.c_void_p] * 5 + [ct.c_void_p]),
}

_lib = None


def load(path: Path | str | None = None) -> ct.CDLL:
    """Load libmdt_gpu.so (building it is ``md_tian2_gb300.build.build()``)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise EngineError(f"{p} is missing: build the CUDA engine first (python -m md_tian2_gb300.build)")
    lib = ct.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib

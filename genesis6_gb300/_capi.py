"""ctypes binding of libg6gpu.so (the C ABI declared in include/g6gpu.h).

The library is built in-tree (genesis6_gb300/libg6gpu.so).  Loading it never
falls back to anything else: a missing library raises, and every call that
needs the GPU raises G6Error when the CUDA runtime reports no device.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libg6gpu.so")

G6_OK, G6_ERR_ARG, G6_ERR_CUDA, G6_ERR_CAPACITY, G6_ERR_NONFINITE = range(5)
G6_ERR_STATE = 6   # (5 is unused)
TIP4P, TIP5P, ST2, SPCE, OPLSMEOH = 1, 2, 3, 4, 5
MODELS = {"TIP4P": TIP4P, "TIP5P": TIP5P, "ST2": ST2, "SPCE": SPCE, "OPLSMEOH": OPLSMEOH}
PATH_STD, PATH_CUSTOM = 0, 1
PATHS = {"std": PATH_STD, "custom": PATH_CUSTOM}
FP64, MIXED = 0, 1
PRECISIONS = {"fp64": FP64, "mixed": MIXED}
NVE, NOSE, ANDERSEN = 0, 1, 2
MC_PLAIN, MC_LEARNED, MC_COLLECT = 0, 1, 2
OP_EP, OP_Q6, OP_TRIANGLE, OP_NBIN = 0, 1, 2, 21   # g6gpu.h G6_OP_*
MLP_NPARAM, MLP_NFEAT, MLP_RECORD = 5890, 24, 51
LOG_WIDTH = 10
REC = 53

# Exported symbols (kept in step with include/g6gpu.h; a test checks both).
SYMBOLS = [
    "g6_version", "g6_last_error", "g6_status_string", "g6_model_info", "g6_ctx_create", "g6_ctx_destroy",
    "g6_system", "g6_set_cutoff", "g6_set_grid", "g6_set_skin", "g6_set_box", "g6_upload_state",
    "g6_download_state", "g6_upload_poses", "g6_cells", "g6_pairsearch", "g6_get_pairs", "g6_force", "g6_step_forces",
    "g6_molecule_energies", "g6_rdf", "g6_hbonds", "g6_force_sites", "g6_pair_potential", "g6_pairsearch_hetero",
    "g6_force_sites_hetero", "g6_md_run", "g6_md_step_host",
    "g6_replica_exchange", "g6_replica_exchange_umbrella", "g6_exchange_plan", "g6_replica_scale", "g6_last_epot",
    "g6_md_begin", "g6_md_advance", "g6_md_end", "g6_stream",
    "g6_time_force", "g6_tune", "g6_set_lpi", "g6_tune_shape", "g6_get_shape", "g6_set_shape", "g6_set_step_timing", "g6_step_times", "g6_force_noalloc", "g6_mc_run", "g6_order_parameter", "g6_mc_run_umbrella", "g6_mlp_set", "g6_mlp_get", "g6_mlp_objective", "g6_mlp_widths",
    "g6_mlp_records", "g6_mlp_grad", "g6_mlp_train",
]


class G6Error(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("g6 status %d: %s" % (status, msg))
        self.status = status


class Thermostat(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("temp", ctypes.c_double), ("q", ctypes.c_double),
                ("dump", ctypes.c_double), ("zeta", ctypes.c_double * 5), ("zetasum", ctypes.c_double),
                ("collision_rate", ctypes.c_double), ("seed", ctypes.c_uint64)]


class Shape(ctypes.Structure):
    _fields_ = [("lpi", ctypes.c_int), ("step_lpi", ctypes.c_int), ("step_mpw", ctypes.c_int),
                ("skin", ctypes.c_double), ("cap", ctypes.c_int), ("step_ms", ctypes.c_double),
                ("step_half", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


TUNE_SKIN = 1

_lib = None


def lib():
    """Load libg6gpu.so (building it first if the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    from . import build as _build
    _build.build()
    L = ctypes.CDLL(LIB_PATH)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    vp = ctypes.c_void_p
    i64 = ctypes.c_int64
    L.g6_version.restype = ctypes.c_int
    L.g6_last_error.restype = ctypes.c_char_p
    L.g6_last_error.argtypes = [vp]
    L.g6_status_string.restype = ctypes.c_char_p
    L.g6_status_string.argtypes = [ctypes.c_int]
    L.g6_model_info.argtypes = [ctypes.c_int, ip, dp, dp, dp]
    L.g6_ctx_create.argtypes = [ctypes.c_int, ctypes.POINTER(vp)]
    L.g6_ctx_destroy.argtypes = [vp]
    L.g6_system.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip, dp]
    L.g6_set_cutoff.argtypes = [vp, ctypes.c_double, ctypes.c_double]
    L.g6_set_grid.argtypes = [vp, ctypes.c_double]
    L.g6_set_skin.argtypes = [vp, ctypes.c_double]
    L.g6_set_box.argtypes = [vp, ctypes.c_int, dp]
    L.g6_upload_state.argtypes = [vp, dp]
    L.g6_download_state.argtypes = [vp, dp]
    L.g6_upload_poses.argtypes = [vp, dp, dp]
    L.g6_cells.argtypes = [vp, ip]
    L.g6_pairsearch.argtypes = [vp, ctypes.POINTER(i64)]
    L.g6_get_pairs.argtypes = [vp, i64, ip, ip, dp, dp, dp, dp, dp]
    L.g6_force.argtypes = [vp, dp, dp, dp, dp]
    L.g6_step_forces.argtypes = [vp, dp, dp, dp]
    L.g6_molecule_energies.argtypes = [vp, dp]
    L.g6_rdf.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.POINTER(i64)]
    L.g6_hbonds.argtypes = [vp, i64, ip, ip, ip, ctypes.POINTER(i64)]
    L.g6_force_sites.argtypes = [vp, ctypes.c_int, dp, dp, dp, dp, dp, dp, i64, ip, ip, dp, dp, dp, dp, dp, dp, dp]
    L.g6_pair_potential.argtypes = [vp, ctypes.c_int, dp, dp, dp, i64, ip, ip, dp, dp, dp, dp, dp]
    L.g6_pairsearch_hetero.argtypes = [vp, dp, ctypes.c_int, dp, ctypes.c_int, dp, ctypes.POINTER(i64)]
    L.g6_force_sites_hetero.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, dp,
                                        dp, ctypes.c_int, ctypes.c_int, i64, ip, ip, dp, dp, dp, dp, dp, dp, dp]
    L.g6_md_run.argtypes = [vp, ctypes.c_double, ctypes.c_int, ctypes.POINTER(Thermostat), dp]
    L.g6_md_step_host.argtypes = [vp, ctypes.c_double, ctypes.POINTER(Thermostat), dp, dp]
    # the same entry point with every pointer an integer address: the per-step
    # host-buffer call pays no typed-pointer conversions (RigidWater.md_step_host)
    L.md_step_host_addr = ctypes.CFUNCTYPE(ctypes.c_int, vp, ctypes.c_double, vp, vp, vp)(
        ctypes.cast(L.g6_md_step_host, vp).value)
    L.g6_replica_exchange.argtypes = [vp, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, dp,
                                      ctypes.POINTER(Thermostat), ip]
    L.g6_replica_exchange_umbrella.argtypes = [vp, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, dp,
                                               ctypes.POINTER(Thermostat), ctypes.c_int, dp, dp, ip]
    L.g6_exchange_plan.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, dp, dp, dp,
                                   ctypes.c_int, dp, dp, dp, ip]
    L.g6_replica_scale.argtypes = [vp, dp]
    L.g6_last_epot.argtypes = [vp, dp]
    L.g6_md_begin.argtypes = [vp, ctypes.c_double, ctypes.c_int, ctypes.POINTER(Thermostat), ctypes.c_int]
    L.g6_md_advance.argtypes = [vp, ctypes.c_int]
    L.g6_md_end.argtypes = [vp, ctypes.POINTER(Thermostat), dp]
    L.g6_stream.argtypes = [vp, ctypes.POINTER(vp)]
    L.g6_force_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, vp, vp, vp, vp, vp, vp]
    L.g6_mc_run.argtypes = [vp, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, dp, dp, dp, ctypes.c_int,
                            ctypes.c_int, dp, ctypes.POINTER(ctypes.c_int64), dp, dp]
    L.g6_order_parameter.argtypes = [vp, ctypes.c_int, dp, ctypes.c_int, dp]
    L.g6_mc_run_umbrella.argtypes = [vp, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, dp, dp, dp, ctypes.c_int, dp,
                                     dp, ctypes.c_int, dp, ctypes.c_int, dp, dp, ctypes.POINTER(ctypes.c_int64), dp,
                                     dp]
    fp = ctypes.POINTER(ctypes.c_float)
    L.g6_mlp_set.argtypes = [vp, fp, fp, fp, ctypes.c_double, ctypes.c_double]
    L.g6_mlp_get.argtypes = [vp, fp, fp, fp]
    L.g6_mlp_objective.argtypes = [vp, ctypes.c_double, ctypes.c_double]
    L.g6_mlp_widths.argtypes = [vp, fp, ctypes.c_int64, dp, dp]
    L.g6_mlp_records.argtypes = [vp, fp, i64, ctypes.POINTER(i64)]
    L.g6_mlp_grad.argtypes = [vp, fp, i64, fp, dp]
    L.g6_mlp_train.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_uint64, ctypes.c_double,
                               ctypes.c_double, dp]
    L.g6_time_force.argtypes = [vp, dp]
    L.g6_set_step_timing.argtypes = [vp, ctypes.c_int]
    L.g6_step_times.argtypes = [vp, dp, dp]
    L.g6_tune.argtypes = [vp, ip]
    L.g6_set_lpi.argtypes = [vp, ctypes.c_int]
    L.g6_tune_shape.argtypes = [vp, ctypes.c_int, ctypes.POINTER(Shape)]
    L.g6_get_shape.argtypes = [vp, ctypes.POINTER(Shape)]
    L.g6_set_shape.argtypes = [vp, ctypes.POINTER(Shape)]
    for name in SYMBOLS:
        if name not in ("g6_last_error", "g6_status_string"):
            getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


def dptr(a):
    """Pointer to a C-contiguous float64 array (None -> NULL)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def fptr(a):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def iptr(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def model_info(model: str):
    """Body-frame sites, site parameters (q, eps, sig), mass and principal moments (host only)."""
    L = lib()
    ns = ctypes.c_int()
    body = np.zeros(18)
    param = np.zeros(18)
    mi = np.zeros(4)
    st = L.g6_model_info(MODELS[model], ctypes.byref(ns), dptr(body), dptr(param), dptr(mi))
    if st != G6_OK:
        raise G6Error(st, "unknown model %s" % model)
    n = ns.value
    return {"nsite": n, "body": body[:3 * n].reshape(n, 3).copy(), "param": param[:3 * n].reshape(n, 3).copy(),
            "mass": float(mi[0]), "inertia": mi[1:].copy()}

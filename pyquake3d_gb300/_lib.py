"""ctypes binding of libpq3d.so (the C ABI declared in include/pq3d.h).

The library is built in-tree by ``pyquake3d_gb300.build``.  There is no CPU
fallback: if the library is missing or CUDA is unavailable, the calls that
need it raise.
"""
from __future__ import annotations

import ctypes
import os
import re

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libpq3d.so")
HEADER = os.path.join(os.path.dirname(_PKG), "include", "pq3d.h")

c_double_p = ctypes.POINTER(ctypes.c_double)
c_float_p = ctypes.POINTER(ctypes.c_float)
c_i64_p = ctypes.POINTER(ctypes.c_int64)
c_void_p = ctypes.c_void_p
c_i64 = ctypes.c_int64
c_int = ctypes.c_int
c_dbl = ctypes.c_double
c_size = ctypes.c_size_t
c_bool = ctypes.c_bool

PQ3D_OK = 0
PQ3D_ERR_ARG = 1
PQ3D_ERR_CUDA = 2
PQ3D_ERR_TIMEOUT = 3
PQ3D_ERR_STEP = 4
PQ3D_ERR_UNSUPPORTED = 5


class PQ3DError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("pq3d error %d: %s" % (code, msg))
        self.code = code


class DenseSim(ctypes.Structure):
    """Mirror of pq3d_dense_sim."""
    _fields_ = [("N", c_i64)] + \
        [(n, c_void_p) for n in ("Tno", "Tt1o", "Tt2o", "state",
                                 "slipv1", "slipv2", "slipv", "rake", "slip1", "slip2", "slip", "Tt", "fric",
                                 "a", "b", "dc", "f0", "shear_loading", "normal_loading", "rake0",
                                 "rates", "vprime", "cand", "K64", "K32", "ctrl")] + \
        [("V0", c_dbl), ("Vpl", c_dbl), ("eta", c_dbl), ("fix_Tn", c_int), ("ndepth", ctypes.c_int32)] + \
        [(n, c_void_p) for n in ("P", "dPdt", "Parr", "dila")]


class RunCtrl(ctypes.Structure):
    """Mirror of pq3d_run_ctrl (88 bytes)."""
    _fields_ = [("h", c_dbl), ("time", c_dbl), ("t_end", c_dbl), ("h_last", c_dbl), ("attempts", c_i64),
                ("steps", c_i64), ("max_steps", c_i64), ("err1_bits", ctypes.c_uint64), ("err2_bits", ctypes.c_uint64),
                ("status", ctypes.c_int32), ("active", ctypes.c_int32), ("nrjct", ctypes.c_int32),
                ("accepted", ctypes.c_int32)]


class BatchSim(ctypes.Structure):
    """Mirror of pq3d_batch_sim."""
    _fields_ = [("N", c_i64), ("B", ctypes.c_int32), ("precision", ctypes.c_int32)] + \
        [(n, c_void_p) for n in ("Tno", "Tt1o", "Tt2o", "state", "slipv1", "slipv2", "slipv", "slip1", "slip2",
                                 "a", "b", "dc", "f0", "shear_loading", "normal_loading", "cos_rake0", "sin_rake0",
                                 "rates")] + \
        [("nsplit", ctypes.c_int32), ("tc_ctas", ctypes.c_int32), ("cand", c_void_p), ("vop", c_void_p), ("K", c_void_p),
         ("ctrl", c_void_p), ("V0", c_dbl), ("Vpl", c_dbl), ("eta", c_dbl), ("fix_Tn", ctypes.c_int32),
         ("attempt64", ctypes.c_int32), ("N_total", c_i64), ("cell0", c_i64), ("base", c_void_p),
         ("fix_order", c_void_p), ("fix_pos", c_void_p)]


class HMat(ctypes.Structure):
    """Mirror of pq3d_hmat."""
    _fields_ = [("N", c_i64), ("nblocks", ctypes.c_int32), ("nleaves", ctypes.c_int32), ("t_rows", c_i64)] + \
        [(n, c_void_p) for n in ("perm", "blk", "rank", "off", "data", "lr_ids", "t_info", "t_off", "leaf", "leaf_ptr",
                                 "leaf_blocks", "t_sched")] + [("t_nlong", c_i64), ("t_grp", c_void_p), ("t_ngrp", c_i64)]


PQ3D_BATCH_FP64 = 0
PQ3D_BATCH_FP32 = 1
PQ3D_BATCH_BF16X6 = 2
PQ3D_BATCH_HMAT = 3
PQ3D_BATCH_BF16X18 = 4
PQ3D_BATCH_BASE_FIELDS = 24   # floats per cell and run of pq3d_batch_sim.base


class StepCtrl(ctypes.Structure):
    """Mirror of pq3d_step_ctrl (104 bytes)."""
    _fields_ = [("dttry", c_dbl), ("time", c_dbl), ("maxv", c_dbl), ("status", ctypes.c_int32),
                ("steps_done", ctypes.c_int32), ("attempts", c_i64), ("err_slot", ctypes.c_uint64 * 6),
                ("maxv_bits", ctypes.c_uint64), ("bar_count", ctypes.c_uint32), ("bar_gen", ctypes.c_uint32)]


_SIGS = {
    "pq3d_last_error": (ctypes.c_char_p, []),
    "pq3d_version": (c_int, []),
    "TDstressFS_C": (None, [c_double_p, c_double_p, c_double_p, c_size, c_double_p, c_double_p, c_double_p,
                            c_dbl, c_dbl, c_dbl, c_dbl, c_dbl, c_bool, c_double_p, c_double_p]),
    "TDstressEachSourceAtReceiver_C": (None, [c_dbl, c_dbl, c_dbl, c_double_p, c_double_p, c_double_p, c_size,
                                              c_dbl, c_dbl, c_dbl, c_dbl, c_dbl, c_bool, c_double_p, c_double_p]),
    "TDstressFS_C1": (None, [c_double_p, c_double_p, c_double_p, c_size, c_double_p, c_double_p, c_double_p,
                             c_dbl, c_dbl, c_dbl, c_dbl, c_dbl] + [c_double_p] * 12),
    "pq3d_gf_workspace_bytes": (c_size, [c_i64]),
    "pq3d_assemble_dense": (c_int, [c_void_p, c_void_p, c_i64, c_i64, c_i64, c_dbl, c_dbl, c_int,
                                    c_void_p, c_void_p, c_void_p, c_size, c_void_p]),
    "pq3d_assemble_dense_noalloc": (c_int, [c_void_p, c_void_p, c_i64, c_i64, c_i64, c_dbl, c_dbl, c_int,
                                            c_void_p, c_void_p, c_void_p]),
    "pq3d_assemble_dense_host": (c_int, [c_void_p, c_i64, c_void_p, c_i64, c_dbl, c_dbl, c_int, c_void_p, c_void_p]),
    "pq3d_dense_matvec_f64": (c_int, [c_void_p, c_i64, c_void_p, c_void_p, c_void_p]),
    "pq3d_dense_matvec_f32": (c_int, [c_void_p, c_i64, c_void_p, c_void_p, c_void_p]),
    "pq3d_dense_step": (c_int, [ctypes.POINTER(DenseSim), c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "pq3d_dilatancy_table_len": (c_size, [c_int]),
    "pq3d_dilatancy_table": (c_int, [c_void_p, c_int, c_dbl, c_dbl, c_dbl, c_dbl, c_dbl, c_void_p]),
    "pq3d_batch_operator_bytes": (c_size, [c_i64]),
    "pq3d_batch_pack_operator": (c_int, [c_void_p, c_i64, c_void_p, c_void_p]),
    "pq3d_batch_rhs_bytes": (c_size, [c_i64, c_int]),
    "pq3d_batch_gemm_bf16x6": (c_int, [c_void_p, c_void_p, c_i64, c_int, c_int, c_int, c_void_p, c_void_p, c_size,
                                       c_void_p]),
    "pq3d_batch_gemm_bf16x6_plan": (c_int, [c_int, c_int, c_void_p]),
    "pq3d_batch_operator_fix_bytes": (c_size, [c_i64]),
    "pq3d_batch_pack_operator_fix": (c_int, [c_void_p, c_i64, c_void_p, c_void_p, c_void_p]),
    "pq3d_batch_rhs_fix_bytes": (c_size, [c_i64, c_int]),
    "pq3d_batch_pack_rhs_fix": (c_int, [c_void_p, c_i64, c_int, c_void_p, c_void_p, c_void_p]),
    "pq3d_batch_gemm_bf16x18": (c_int, [c_void_p, c_void_p, c_i64, c_int, c_int, c_void_p, c_void_p, c_size,
                                        c_void_p]),
    "pq3d_batch_workspace_bytes": (c_size, [ctypes.POINTER(BatchSim)]),
    "pq3d_gf_setup": (c_int, [c_void_p, c_void_p, c_i64, c_int, c_void_p, c_size, c_void_p]),
    "pq3d_hmat_aca": (c_int, [c_void_p, c_i64, c_void_p, c_int, c_void_p, c_void_p, c_dbl, c_dbl, c_dbl, c_int,
                              c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "pq3d_hmat_dense_blocks": (c_int, [c_void_p, c_i64, c_void_p, c_void_p, c_void_p, c_int, c_dbl, c_dbl, c_int,
                                       c_void_p, c_void_p, c_void_p]),
    "pq3d_hmat_pack_factors": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p,
                                       c_void_p, c_void_p]),
    "pq3d_hmat_workspace_bytes": (c_size, [ctypes.POINTER(HMat), c_int]),
    "pq3d_hmat_apply": (c_int, [ctypes.POINTER(HMat), c_void_p, c_int, c_void_p, c_void_p, c_size, c_void_p]),
    "pq3d_hmat_apply_masked": (c_int, [ctypes.POINTER(HMat), c_void_p, c_int, c_void_p, c_void_p, c_int, c_void_p,
                                       c_size, c_void_p]),
    "pq3d_batch_prepare": (c_int, [ctypes.POINTER(BatchSim), c_void_p]),
    "pq3d_batch_iterate": (c_int, [ctypes.POINTER(BatchSim), c_void_p, c_size, c_void_p]),
    "pq3d_batch_iterate_begin": (c_int, [ctypes.POINTER(BatchSim), c_void_p, c_size, c_void_p]),
    "pq3d_batch_iterate_end": (c_int, [ctypes.POINTER(BatchSim), c_void_p]),
    "pq3d_hmat_cluster_order": (c_int, [c_void_p, c_i64, c_int, c_void_p, c_void_p, c_void_p]),
    "pq3d_hmat_partition": (c_int, [c_void_p, c_i64, c_int, c_int, c_dbl, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_i64, c_void_p, c_void_p, c_void_p]),
    "pq3d_selftest_barrier_timeout": (c_int, [c_int, c_int, ctypes.c_uint, c_void_p]),
    "pq3d_selftest_mbar_timeout": (c_int, [ctypes.c_uint, c_void_p]),
    "pq3d_selftest_ff_conversions": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "pq3d_selftest_tri_mode": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
}

_lib = None


def header_functions():
    """Names of the functions declared in include/pq3d.h."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", txt, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "while", "defined")))


def load(build_if_missing: bool = True):
    """Load libpq3d.so (building it first if it is absent and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError("libpq3d.so is not built (run python -m pyquake3d_gb300.build)")
        from . import build as _b
        _b.build()
    L = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc: int):
    if rc != PQ3D_OK:
        raise PQ3DError(rc, load().pq3d_last_error().decode())

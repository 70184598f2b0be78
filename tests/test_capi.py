"""The C-ABI library loads without a GPU and exports every function that
include/pq3d.h declares (no compute call is made here)."""
import ctypes

from pyquake3d_gb300 import _lib


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    names = _lib.header_functions()
    assert "TDstressFS_C" in names and "pq3d_assemble_dense" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_reference_ctypes_signatures_bind():
    """The reference binds TDstressFS_C / TDstressEachSourceAtReceiver_C with
    these argtypes (src/Hmatrix.py:32-56); the same declarations bind here."""
    lib = ctypes.CDLL(_lib.LIB_PATH)
    D = ctypes.POINTER(ctypes.c_double)
    lib.TDstressFS_C.argtypes = [D, D, D, ctypes.c_size_t, D, D, D, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_bool, D, D]
    lib.TDstressEachSourceAtReceiver_C.argtypes = [ctypes.c_double] * 3 + [D, D, D, ctypes.c_size_t] + \
        [ctypes.c_double] * 5 + [ctypes.c_bool, D, D]
    assert lib.pq3d_version() == 1


def test_error_text_starts_empty():
    assert _lib.load().pq3d_last_error() == b""


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors have the sizes and field offsets of include/pq3d.h."""
    import os
    import subprocess
    src = tmp_path / "probe.c"
    fields = {"pq3d_batch_sim": ("BatchSim", ["N", "B", "precision", "Tno", "rates", "nsplit", "tc_ctas", "cand", "vop", "K",
                                              "ctrl", "V0", "eta", "fix_Tn", "attempt64", "N_total", "cell0", "base",
                                              "fix_order", "fix_pos"]),
              "pq3d_dense_sim": ("DenseSim", ["N", "Tno", "fric", "a", "rake0", "rates", "cand", "K64", "K32", "ctrl",
                                              "V0", "eta", "fix_Tn", "ndepth", "P", "Parr", "dila"]),
              "pq3d_run_ctrl": ("RunCtrl", ["h", "time", "attempts", "max_steps", "err2_bits", "status", "accepted"]),
              "pq3d_step_ctrl": ("StepCtrl", ["dttry", "status", "attempts", "err_slot", "maxv_bits", "bar_gen"]),
              "pq3d_hmat": ("HMat", ["N", "nblocks", "nleaves", "t_rows", "perm", "data", "t_info", "t_sched", "t_nlong", "t_grp", "t_ngrp", "leaf_blocks"])}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "pq3d.h"', "int main(void){"]
    for cname, (_, fl) in fields.items():
        lines.append('printf("%%zu\\n", sizeof(%s));' % cname)
        for f in fl:
            lines.append('printf("%%zu\\n", offsetof(%s, %s));' % (cname, f))
    lines.append('printf("%d\\n", PQ3D_BATCH_BASE_FIELDS);')
    lines.append("return 0;}")
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.check_call(["gcc", "-I", os.path.dirname(_lib.HEADER), "-o", str(exe), str(src)])
    vals = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    k = 0
    for cname, (pyname, fl) in fields.items():
        cls = getattr(_lib, pyname)
        assert ctypes.sizeof(cls) == vals[k], cname
        k += 1
        for f in fl:
            assert getattr(cls, f).offset == vals[k], (cname, f)
            k += 1
    assert vals[k] == _lib.PQ3D_BATCH_BASE_FIELDS


def test_batch_structure_checks_need_no_gpu():
    """pq3d_batch_prepare validates the simulation structure before any CUDA
    call: K-slice counts per product, the CTA count and the attempt flag."""
    import numpy as np
    L = _lib.load()
    buf = np.zeros(64, dtype=np.float64)          # 16-byte aligned stand-in pointers (never dereferenced)
    p = buf.ctypes.data

    def sim(**kw):
        S = _lib.BatchSim()
        S.N, S.B, S.precision, S.nsplit = 8, 2, _lib.PQ3D_BATCH_FP64, 1
        for k in ("Tno", "rates", "cand", "vop", "K", "ctrl", "base"):
            setattr(S, k, p)
        for k, v in kw.items():
            setattr(S, k, v)
        return S

    cases = [(dict(nsplit=2), "nsplit"),
             (dict(precision=_lib.PQ3D_BATCH_FP32, nsplit=65), "64 K slices"),
             (dict(precision=_lib.PQ3D_BATCH_BF16X6, tc_ctas=4), "tc_ctas"),
             (dict(precision=_lib.PQ3D_BATCH_FP32, attempt64=3), "attempt64"),
             (dict(precision=_lib.PQ3D_BATCH_FP32, base=None), "base array")]
    for kw, text in cases:
        S = sim(**kw)
        assert L.pq3d_batch_prepare(ctypes.byref(S), None) == _lib.PQ3D_ERR_ARG, kw
        assert text in L.pq3d_last_error().decode(), (kw, L.pq3d_last_error())


def test_tensor_core_launch_arguments_checked_without_gpu():
    import numpy as np
    L = _lib.load()
    plan = np.zeros(2, dtype=np.int32)
    assert L.pq3d_batch_gemm_bf16x6_plan(0, 2, plan.ctypes.data) == _lib.PQ3D_ERR_ARG
    assert L.pq3d_batch_gemm_bf16x6_plan(64, 4, plan.ctypes.data) == _lib.PQ3D_ERR_ARG
    buf = np.zeros(64, dtype=np.float64)
    p = buf.ctypes.data
    # CTAs per SM outside 0..3, then a K-slice count above the column blocks (N = 64: 4 blocks)
    assert L.pq3d_batch_gemm_bf16x6(p, p, 64, 16, 1, 4, p, p, 256, None) == _lib.PQ3D_ERR_ARG
    assert "ctas_per_sm" in L.pq3d_last_error().decode()
    assert L.pq3d_batch_gemm_bf16x6(p, p, 64, 16, 5, 2, p, p, 256, None) == _lib.PQ3D_ERR_ARG
    assert "nsplit" in L.pq3d_last_error().decode()

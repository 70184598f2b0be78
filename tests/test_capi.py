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

"""Comparison helpers shared by the parity tests."""
import numpy as np


def normwise_rel(ref, got, axis=-1):
    """max_i |ref_i - got_i| / max_i |ref_i| along ``axis``; rows whose
    reference is all zero compare absolutely."""
    ref = np.asarray(ref, dtype=np.float64)
    got = np.asarray(got, dtype=np.float64)
    scale = np.max(np.abs(ref), axis=axis, keepdims=True)
    scale = np.where(scale == 0, 1.0, scale)
    return float(np.nanmax(np.abs(ref - got) / scale)) if ref.size else 0.0

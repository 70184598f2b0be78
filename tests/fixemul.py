"""NumPy model of the fixed-point slices of the BF16x18 tensor-core product
(test helper): the same digits and the same retained slice products as
pyquake3d_gb300/csrc/gemm_fix.cu, summed in FP64."""
import numpy as np

K_CHUNK = 1024     # operator columns sharing one exponent per row
V_CHUNK = 256      # right-hand-side columns sharing one exponent per run (one exact span)
K_SLICES, V_SLICES, MAX_LEVEL = 4, 6, 5


def chunk_exponents(X, chunk):
    """(R, C) -> (R, nchunks) ints e with |X| < 2^e over each chunk of
    `chunk` columns (0 for an all-zero chunk)."""
    R, C = X.shape
    nch = (C + chunk - 1) // chunk
    Xp = np.zeros((R, nch * chunk))
    Xp[:, :C] = np.abs(X)
    m = Xp.reshape(R, nch, chunk).max(axis=2)
    _, e = np.frexp(m)
    return np.where(m > 0, e, 0).astype(np.int64)


def digits(X, n, chunk):
    """Balanced base-256 digits of round(X 2^(8n-1-e)) per (row, chunk):
    (digits list of n int64 arrays (R, C), exponents broadcast to (R, C))."""
    R, C = X.shape
    e = np.repeat(chunk_exponents(X, chunk), chunk, axis=1)[:, :C]
    Xi = np.rint(np.ldexp(X, 8 * n - 1 - e)).astype(np.int64)
    out = [None] * n
    for p in range(n - 1, 0, -1):
        t = ((Xi + 128) & 255) - 128
        out[p] = t
        Xi = (Xi - t) >> 8
    out[0] = Xi
    return out, e


def slices(X, n, chunk):
    """Slice values d_p 2^(e-7-8p) (exact in BF16)."""
    d, e = digits(X, n, chunk)
    return [np.ldexp(d[p].astype(np.float64), e - 7 - 8 * p) for p in range(n)]


def product(K, V):
    """(B, 3N): sum over the retained slice pairs (p + q <= 5) of V_q K_p^T,
    i.e. what the tensor-core product computes, in FP64."""
    Ks = slices(np.asarray(K, dtype=np.float64), K_SLICES, K_CHUNK)
    Vs = slices(np.asarray(V, dtype=np.float64), V_SLICES, V_CHUNK)
    R = np.zeros((V.shape[0], K.shape[0]))
    for p in range(K_SLICES):
        vv = sum(Vs[q] for q in range(V_SLICES) if p + q <= MAX_LEVEL)
        R += vv @ Ks[p].T
    return R

"""The kernels' division shortcuts, checked on the host (no GPU):

- the masked pyrDown (CudaPyramid2.cu:436-542) divides S << 8 by
  alpha = 256 m, i.e. floor(S / m), as umulhi(S << 8, ceil(2^24 / m)) for
  1 <= m <= 256 and S <= 65280 (16 * 16 * 255), checked exhaustively;
- the weighted normalisation (:775-791) divides by the weight sum in fp32
  with one remainder correction (divTrunc), checked for every weight sum up
  to 64 * 256 next to every multiple of it.
"""
import numpy as np


def _umulhi(a, b):
    return (a.astype(np.uint64) * np.uint64(b)) >> np.uint64(32)


def test_pyrdown_division_by_alpha():
    s = np.arange(65281, dtype=np.uint64)
    for m in range(1, 257):
        mg = ((1 << 24) + m - 1) // m
        assert np.array_equal(_umulhi(s << np.uint64(8), mg), s // np.uint64(m)), m


def _fmul_rz(a, b):
    """fp32 product rounded toward zero (the kernels' __fmul_rz): the exact product of two fp32 values fits
    in a double, so round that to fp32 and step back toward zero when the rounding went outward."""
    x = a.astype(np.float64) * b.astype(np.float64)
    f = x.astype(np.float32)
    out = np.abs(f.astype(np.float64)) > np.abs(x)
    f[out] = np.nextafter(f[out], np.float32(0))
    return f


def test_normalisation_division_by_weight_sum():
    """divTrunc (the weighted normalisation's a / W, truncating): the fp32 quotient from __frcp_rn(W) and
    __fmul_rz, then one remainder correction, equals the integer quotient.  Every W up to 64 * 256 (64
    cameras with overlapping custom masks), numerators next to each multiple of W up to 255 W."""
    k = np.arange(256, dtype=np.int64)
    for d in range(1, 64 * 256 + 1):
        m = np.concatenate([k * d, k * d + 1, np.maximum(k * d - 1, 0), np.minimum(k * d + d - 1, 255 * d)])
        rcp = np.float32(1) / np.float32(d)  # correctly rounded, as __frcp_rn
        q = _fmul_rz(m.astype(np.float32), np.full(m.shape, rcp, np.float32)).astype(np.int64)
        r = m - q * d
        q += (r >= d).astype(np.int64) - (r < 0).astype(np.int64)
        assert np.array_equal(q, m // d), d

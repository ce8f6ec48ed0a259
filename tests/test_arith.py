"""The integer shortcut of the masked pyrDown (CudaPyramid2.cu:436-542),
checked exhaustively on the host (no GPU): S << 8 divided by alpha = 256 m,
i.e. floor(S / m), is taken as umulhi(S << 8, ceil(2^24 / m)) for
1 <= m <= 256 and S <= 65280 (16 * 16 * 255).
"""
import numpy as np


def _umulhi(a, b):
    return (a.astype(np.uint64) * np.uint64(b)) >> np.uint64(32)


def test_pyrdown_division_by_alpha():
    s = np.arange(65281, dtype=np.uint64)
    for m in range(1, 257):
        mg = ((1 << 24) + m - 1) // m
        assert np.array_equal(_umulhi(s << np.uint64(8), mg), s // np.uint64(m)), m

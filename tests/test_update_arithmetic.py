"""Host-side checks of two pieces of the FP32 update kernel
(rheocell_gb300/csrc/rc_cells_f32.cu, cell_update_bulk) that need no GPU:

* the 16-byte aligned bulk-copy windows: for every chunk of every possible
  cell start and size, the window covers the chunk, starts and ends on
  16-byte boundaries, fits the stage's buffers and never leaves the padded
  allocation (S_cap + 8 elements, rc_engine.cu);
* the short double -> float conversion (d2f_fast, rc_common.cuh), restated
  bit for bit in numpy: equal to IEEE round-to-nearest-even (numpy's own
  conversion) except at exact ties, where it rounds away from zero; zero
  below the FP32 normal range; NaN beyond it.  The same function is checked
  against CUDA's conversion on the device in test_gpu_conversions.py."""
from __future__ import annotations

import numpy as np

CH, PAD = 512, 8
FW, DW = CH + 8, CH + 4


def windows(start, n):
    """(float window, double window) per chunk: [first, end) element ranges."""
    out = []
    for c in range((n + CH - 1) // CH):
        i0 = start + c * CH
        cnt = min(CH, n - c * CH)
        fa, fe = i0 & ~3, (i0 + cnt + 3) & ~3
        da, de = i0 & ~1, (i0 + cnt + 1) & ~1
        out.append((i0, cnt, fa, fe, da, de))
    return out


def test_bulk_copy_windows():
    for S_pad_start in range(0, 8):
        for n in (1, 2, 3, 5, 511, 512, 513, 1023, 1024, 1681, 4096, 16384):
            start = 1000 + S_pad_start
            S = start + n  # this cell is the last one: the tightest case
            for i0, cnt, fa, fe, da, de in windows(start, n):
                assert fa <= i0 and i0 + cnt <= fe and da <= i0 and i0 + cnt <= de
                assert (fa * 4) % 16 == 0 and ((fe - fa) * 4) % 16 == 0     # floats
                assert (da * 8) % 16 == 0 and ((de - da) * 8) % 16 == 0     # doubles
                assert fe - fa <= FW and de - da <= DW                       # stage buffers
                assert fe <= S + PAD and de <= S + PAD                       # padded allocation
                assert i0 - fa <= 3 and i0 - da <= 1                         # slack before the chunk


def d2f_fast(x: np.ndarray) -> np.ndarray:
    """The kernel's short conversion, restated on uint32 halves."""
    u = x.astype(np.float64).view(np.uint64)
    hi = (u >> np.uint64(32)).astype(np.uint32)
    lo = (u & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    mag = hi & np.uint32(0x7FFFFFFF)
    sign = hi ^ mag
    funnel = ((hi << np.uint32(3)) | (lo >> np.uint32(29))).astype(np.uint32)
    b = (funnel - np.uint32(384 << 23) + ((lo >> np.uint32(28)) & np.uint32(1))).astype(np.uint32)
    b = np.where(mag < np.uint32(897 << 20), np.uint32(0), b)
    b = np.where(mag >= np.uint32(1151 << 20), np.uint32(0x7FC00000), b)
    return (b | sign).astype(np.uint32).view(np.float32)


def test_short_conversion_rounds_to_nearest():
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.standard_normal(300000),
                        rng.uniform(-1, 1, 200000) * 10.0 ** rng.uniform(-37, 37, 200000)])
    f = rng.standard_normal(50000).astype(np.float32)
    ties = np.concatenate([f.astype(np.float64) + 0.5 * np.spacing(np.abs(f)).astype(np.float64),
                           f.astype(np.float64) - 0.5 * np.spacing(np.abs(f)).astype(np.float64)])
    x = np.concatenate([x, ties])
    with np.errstate(over="ignore"):
        rn = x.astype(np.float32)
    got = d2f_fast(x)
    normal = (np.abs(rn) >= np.float32(2.0 ** -126)) & np.isfinite(rn) & (np.abs(x) >= 2.0 ** -126)
    diff = normal & (got.view(np.uint32) != rn.view(np.uint32))
    # differences only at exact ties, one ulp away from zero
    assert np.all(np.abs(x[diff] - rn[diff].astype(np.float64)) == np.abs(x[diff] - got[diff].astype(np.float64)))
    assert np.all(np.abs(got[diff]).astype(np.float64) > np.abs(rn[diff]).astype(np.float64))
    assert 0 < diff.sum() < ties.size
    # below the normal range: signed zero; beyond the range and non-finite: NaN
    small = np.array([1e-39, -1e-39, 1e-300, -0.0, 0.0])
    assert np.all(d2f_fast(small) == 0) and np.array_equal(np.signbit(d2f_fast(small)), np.signbit(small))
    assert np.all(np.isnan(d2f_fast(np.array([1e39, -1e300, np.inf, -np.inf, np.nan]))))

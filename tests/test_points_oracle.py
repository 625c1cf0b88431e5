"""Pins the oracle's voxelisation of points (no GPU).

The reference maps a point p of grid b to ijk = VoxelCoordTransform(1/w, -o/w).apply(p).round()
in the points' arithmetic type (src/fvdb/detail/ops/BuildGridFromPoints.cu:27-43): double for
FP64 points, float for FP32 / FP16 ones.  Here that rule is restated a second time with exact
rational arithmetic (one rounding of p*s + t to the target type, then floor(v + 1/2) in that
type) and compared with the oracle on points placed on and next to half-voxel boundaries,
where the two precisions give different voxels.
"""

from fractions import Fraction
import math

import numpy as np

from oracle import oracle as orc


def round_to_f32(fr: Fraction) -> float:
    """fr rounded to the nearest float32 (ties to even), as a Python float."""
    if fr == 0:
        return 0.0
    sign = -1 if fr < 0 else 1
    a = abs(fr)
    e = math.floor(math.log2(a.numerator) - math.log2(a.denominator))
    while Fraction(2) ** e > a:
        e -= 1
    while Fraction(2) ** (e + 1) <= a:
        e += 1
    e = max(e, -126)  # subnormal range keeps the exponent of the smallest normal
    scaled = a / Fraction(2) ** (e - 23)  # 24-bit significand
    q, r = divmod(scaled.numerator, scaled.denominator)
    twice = 2 * r
    if twice > scaled.denominator or (twice == scaled.denominator and q % 2 == 1):
        q += 1
    return sign * float(Fraction(q) * Fraction(2) ** (e - 23))


def exact_ijk(p: float, w: float, o: float, precision: str) -> int:
    if precision == "f64":
        s, t = 1.0 / w, -o / w
        v = float(Fraction(p) * Fraction(s) + Fraction(t))  # one rounding (fused multiply-add)
        return math.floor(v + 0.5)
    s = round_to_f32(Fraction(1.0 / w))
    t = round_to_f32(Fraction(-o / w))
    v = round_to_f32(Fraction(np.float32(p).item()) * Fraction(s) + Fraction(t))
    return math.floor(round_to_f32(Fraction(v) + Fraction(1, 2)))


def boundary_points(n: int, w: float, o: float, seed: int) -> np.ndarray:
    """Points at (k + 1/2) w + o and a few double / float ulps either side of it."""
    rng = np.random.default_rng(seed)
    k = rng.integers(-300, 300, size=(n, 3))
    base = (k + 0.5) * w + o
    nudge = rng.integers(-3, 4, size=(n, 3))
    kind = rng.integers(0, 3, size=(n, 3))
    f64_step = np.spacing(np.abs(base))
    f32_step = np.spacing(np.abs(base).astype(np.float32)).astype(np.float64)
    return np.where(kind == 0, base, np.where(kind == 1, base + nudge * f64_step, base + nudge * f32_step))


def test_points_match_exact_restatement():
    for w, o, seed in ((0.1, 0.0, 0), (1 / 256, 0.0, 1), (0.05, 0.37, 2), (0.3, -1.25, 3)):
        pts = boundary_points(400, w, o, seed)
        for prec in ("f64", "f32"):
            src = pts if prec == "f64" else pts.astype(np.float32).astype(np.float64)
            got = orc.points_to_ijk(src, [0, src.shape[0]], [w] * 3, [o] * 3, prec)
            expect = np.array([[exact_ijk(v, w, o, prec) for v in row] for row in src], dtype=np.int32)
            assert np.array_equal(got, expect), (w, o, prec)


def test_precisions_differ_near_boundaries():
    """FP64 points next to a half-voxel boundary land in voxels that the FP32 rule misplaces:
    a case that rounding FP64 points to float would get wrong."""
    pts = boundary_points(2000, 0.1, 0.0, 7)
    d = orc.points_to_ijk(pts, [0, pts.shape[0]], [0.1] * 3, [0.0] * 3, "f64")
    f = orc.points_to_ijk(pts.astype(np.float32).astype(np.float64), [0, pts.shape[0]], [0.1] * 3, [0.0] * 3, "f32")
    assert (d != f).any()


def test_points_per_grid_transforms():
    pts = np.array([[0.26, 0.26, 0.26], [0.26, 0.26, 0.26]])
    out = orc.points_to_ijk(pts, [0, 1, 2], [[0.5, 0.5, 0.5], [0.1, 0.2, 0.4]], [[0, 0, 0], [0.06, 0.0, 0.0]], "f64")
    assert out.tolist() == [[1, 1, 1], [2, 1, 1]]

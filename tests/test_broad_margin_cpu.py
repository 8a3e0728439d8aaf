"""The FP64 form's sweep margin, restated with exact arithmetic on the CPU (no GPU needed).

k_broad_small keeps each world's fat boxes in shared memory in FP32: lower corners rounded down,
upper corners rounded up. A candidate whose FP32 boxes overlap is confirmed on the exact FP64 boxes
unless it is "sure": a's FP32 box shrunk by slack = 4 eps M on every side (M the largest magnitude
of a coordinate of the world's FP32 boxes, eps = 2^-23; lower + slack rounded up, upper - slack
rounded down) still overlaps b's with strict compares. The kernel takes a sure hit without reading
the exact boxes, so a sure hit must always have overlapping exact boxes. This test checks that on
random boxes built to touch within a few ulps, at coordinate scales from millimetres to kilometres.
"""
from fractions import Fraction

import numpy as np

F32 = np.float32
EPS32 = F32(1.1920929e-07)  # EpsOf<float>::v


def down_f(x: float) -> np.float32:
    """The largest float32 <= x (__double2float_rd)."""
    f = F32(x)
    if float(f) > x:
        f = np.nextafter(f, F32(-np.inf))
    return f


def up_f(x: float) -> np.float32:
    """The smallest float32 >= x (__double2float_ru)."""
    f = F32(x)
    if float(f) < x:
        f = np.nextafter(f, F32(np.inf))
    return f


def add_ru(a: np.float32, b: np.float32) -> np.float32:
    """a + b rounded up to float32 (__fadd_ru), from the exact sum."""
    exact = Fraction(float(a)) + Fraction(float(b))
    f = F32(float(exact))
    while Fraction(float(f)) < exact:
        f = np.nextafter(f, F32(np.inf))
    while Fraction(float(np.nextafter(f, F32(-np.inf)))) >= exact:
        f = np.nextafter(f, F32(-np.inf))
    return f


def sub_rd(a: np.float32, b: np.float32) -> np.float32:
    """a - b rounded down to float32 (__fsub_rd), from the exact difference."""
    exact = Fraction(float(a)) - Fraction(float(b))
    f = F32(float(exact))
    while Fraction(float(f)) > exact:
        f = np.nextafter(f, F32(-np.inf))
    while Fraction(float(np.nextafter(f, F32(np.inf)))) <= exact:
        f = np.nextafter(f, F32(np.inf))
    return f


def test_sure_hits_overlap_on_the_exact_boxes():
    rng = np.random.default_rng(7)
    sure_hits = tight_sure = not_overlapping = wrong_without_margin = 0
    for scale in (1e-3, 0.5, 5.0, 40.0, 3000.0):
        for _ in range(700):
            a_lo = rng.uniform(-scale, scale, 3)
            a_hi = a_lo + rng.uniform(0.05, 1.0, 3) * scale * 0.1
            # b's lower corner within a few FP64 ulps and a few FP32 ulps of a's upper corner on
            # random axes, elsewhere well inside: near-touching along some axes
            b_lo = a_lo + rng.uniform(0.0, 0.5, 3) * (a_hi - a_lo)
            for k in range(3):
                if rng.random() < 0.6:
                    step = rng.choice([np.spacing(a_hi[k]), float(np.spacing(F32(a_hi[k])))])
                    b_lo[k] = a_hi[k] + rng.integers(-12, 13) * step
            b_hi = b_lo + rng.uniform(0.05, 1.0, 3) * scale * 0.1
            qa = [down_f(x) for x in a_lo] + [up_f(x) for x in a_hi]
            qb = [down_f(x) for x in b_lo] + [up_f(x) for x in b_hi]
            m = max(abs(float(x)) for x in qa + qb)  # the world's M is at least the pair's
            slack = F32(F32(4.0) * EPS32) * F32(m) + F32(1e-30)
            qs = [add_ru(qa[k], slack) for k in range(3)] + [sub_rd(qa[k + 3], slack) for k in range(3)]
            hit32 = all(qb[k] <= qa[k + 3] and qb[k + 3] >= qa[k] for k in range(3))
            sure = all(qb[k] < qs[k + 3] and qb[k + 3] > qs[k] for k in range(3))
            exact = all(b_lo[k] <= a_hi[k] and b_hi[k] >= a_lo[k] for k in range(3))
            if not exact:
                not_overlapping += 1
                # with no margin, strict FP32 overlap would take these unconfirmed
                if all(qb[k] < qa[k + 3] and qb[k + 3] > qa[k] for k in range(3)):
                    wrong_without_margin += 1
            if sure:
                assert hit32, "a sure hit is an FP32 hit"
                assert exact, (scale, a_lo, a_hi, b_lo, b_hi)
                sure_hits += 1
                gap = min(float(qa[k + 3]) - float(qb[k]) for k in range(3))
                if gap < 64 * float(slack):
                    tight_sure += 1
    # the cases are near the boundary: many sure hits within a few slacks of it, many pairs whose
    # exact boxes do not overlap, and some that FP32 boxes with no margin would wrongly take
    assert sure_hits > 250 and tight_sure > 60 and not_overlapping > 1000, (sure_hits, tight_sure, not_overlapping)
    assert wrong_without_margin > 20, wrong_without_margin

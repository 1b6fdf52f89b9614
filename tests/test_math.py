"""The project-owned FP64 functions of nbg_math.h (shared by the oracle and
the kernels) against glibc: accuracy in ulps and the special cases that Go's
math package and C99 define."""
import math

import numpy as np
import pytest

from nbodygo_gb300.workloads import SplitMix64
from oracle.oracle import math_eval

SIN, COS, TAN, ASIN, ACOS, ATAN, ATAN2, GOMIN = range(8)


def ulps(got, ref):
    if math.isnan(ref):
        return 0.0 if math.isnan(got) else math.inf
    if ref == 0.0:
        return abs(got) / math.ulp(0.0)
    return abs(got - ref) / math.ulp(ref)


def worst(fn, args, ref):
    return max(ulps(math_eval(fn, *a), ref(*a)) for a in args)


rng = SplitMix64(2024)
ANG = [(x, 0.0) for x in rng.uniform(4000, -2 * math.pi, 2 * math.pi)]
SMALL = [(x, 0.0) for x in rng.uniform(500, -1e-6, 1e-6)]
UNIT = [(x, 0.0) for x in rng.uniform(4000, -1.0, 1.0)]
NEAR1 = [(x, 0.0) for x in 1.0 - rng.log_uniform(500, 1e-15, 1e-2)]
WIDE = [(x, 0.0) for x in rng.normal(3000, 0.0, 50.0)]
PAIRS = list(zip(rng.normal(4000, 0, 10), rng.normal(4000, 0, 10)))


@pytest.mark.parametrize("fn,ref,args,bound", [
    (SIN, math.sin, ANG + SMALL, 2.0),
    (COS, math.cos, ANG + SMALL, 2.0),
    (TAN, math.tan, [(x, 0.0) for x, _ in ANG if abs(math.cos(x)) > 0.05] + SMALL, 4.0),
    (ASIN, math.asin, UNIT + NEAR1 + SMALL, 3.0),
    (ACOS, math.acos, UNIT + NEAR1 + SMALL, 3.0),
    (ATAN, math.atan, WIDE + UNIT + SMALL, 2.0),
    (ATAN2, math.atan2, PAIRS, 3.0),
])
def test_accuracy_against_glibc(fn, ref, args, bound):
    w = worst(fn, args, lambda a, b: ref(a, b) if fn == ATAN2 else ref(a))
    assert w <= bound, f"worst error {w} ulp"


def test_special_cases():
    nan, inf = math.nan, math.inf
    for fn in (SIN, COS, TAN, ASIN, ACOS, ATAN):
        assert math.isnan(math_eval(fn, nan))
    for fn in (SIN, COS, TAN):
        assert math.isnan(math_eval(fn, inf)) and math.isnan(math_eval(fn, -inf))
    for fn in (SIN, TAN, ASIN, ATAN):
        assert math.copysign(1.0, math_eval(fn, -0.0)) == -1.0
    assert math.isnan(math_eval(ASIN, 1.0000000000000002)) and math.isnan(math_eval(ACOS, -1.5))
    assert math_eval(ACOS, 1.0) == 0.0 and math_eval(ACOS, -1.0) == math.pi
    assert math_eval(ASIN, 1.0) == math.pi / 2 and math_eval(ATAN, inf) == math.pi / 2
    # atan2 quadrants and signed zeros (C99 F.10.1.4, Go math.Atan2)
    assert math_eval(ATAN2, 0.0, -0.0) == math.pi and math_eval(ATAN2, -0.0, -0.0) == -math.pi
    assert math.copysign(1, math_eval(ATAN2, -0.0, 0.0)) == -1 and math_eval(ATAN2, 0.0, 0.0) == 0.0
    assert math_eval(ATAN2, 1.0, 0.0) == math.pi / 2 and math_eval(ATAN2, -1.0, -0.0) == -math.pi / 2
    assert math_eval(ATAN2, inf, inf) == math.pi / 4 and math_eval(ATAN2, -inf, -inf) == -3 * math.pi / 4
    assert math_eval(ATAN2, 2.0, -inf) == math.pi and math_eval(ATAN2, -2.0, inf) == 0.0
    assert math.isnan(math_eval(ATAN2, nan, 1.0)) and math.isnan(math_eval(ATAN2, 1.0, nan))
    for y, x in PAIRS[:200]:
        assert abs(math_eval(ATAN2, y, x) - math.atan2(y, x)) <= 4 * math.ulp(math.atan2(y, x))


def test_go_min():
    assert math_eval(GOMIN, 3.0, 2000.0) == 3.0
    assert math_eval(GOMIN, 2500.0, 2000.0) == 2000.0
    assert math.isnan(math_eval(GOMIN, math.nan, 2000.0))
    assert math.copysign(1.0, math_eval(GOMIN, 0.0, -0.0)) == -1.0
    assert math_eval(GOMIN, -math.inf, 5.0) == -math.inf


def test_deterministic_bits():
    """Same argument, same bits, every call (no state, no rounding mode)."""
    xs = np.array([a for a, _ in ANG[:100]])
    a = [math_eval(SIN, x) for x in xs]
    b = [math_eval(SIN, x) for x in xs]
    assert a == b

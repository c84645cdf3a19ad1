"""The oracle's own elementary functions (Tang's table-driven exp/log, pow,
acos) against libm: accuracy bounds and the exact values the Riemann solver
relies on (log 1 = 0, exp 0 = 1, pow(1, y) = 1)."""
import math

import numpy as np
import pytest

import oracle_binding as orc

EPS = np.finfo(np.float64).eps


def ulp_err(got, ref):
    return abs(got - ref) / (abs(ref) * EPS) if ref != 0 else abs(got)


def test_exact_points():
    L = orc.lib()
    assert L.oracle_log(1.0) == 0.0
    assert L.oracle_exp(0.0) == 1.0
    for y in (0.1428571, 1.0 / 1.4, 2.5, -3.0, 7.0):
        assert L.oracle_pow(1.0, y) == 1.0
    assert L.oracle_pow(0.0, 2.0) == 0.0
    assert L.oracle_pow(5.0, 0.0) == 1.0


def test_exp_accuracy():
    L = orc.lib()
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.uniform(-700, 700, 4000), rng.uniform(-1, 1, 4000), rng.uniform(-1e-8, 1e-8, 500)])
    worst = max(ulp_err(L.oracle_exp(float(x)), math.exp(float(x))) for x in xs)
    assert worst < 2.0, worst


def test_log_accuracy():
    L = orc.lib()
    rng = np.random.default_rng(2)
    xs = np.concatenate([np.exp(rng.uniform(-700, 700, 4000)), rng.uniform(0.5, 2.0, 4000),
                         1.0 + rng.uniform(-1e-6, 1e-6, 500), [5e-324, 1e-310, 1e300]])
    worst = 0.0
    for x in xs:
        ref = math.log(float(x))
        got = L.oracle_log(float(x))
        # relative to |log x| with an absolute floor of one ulp of 1 near x = 1
        worst = max(worst, abs(got - ref) / (max(abs(ref), 1e-300) * EPS))
    assert worst < 3.0, worst


def test_pow_accuracy():
    L = orc.lib()
    rng = np.random.default_rng(3)
    xs = np.exp(rng.uniform(-8, 8, 6000))
    ys = rng.uniform(-6, 6, 6000)
    worst = 0.0
    for x, y in zip(xs, ys):
        ref = float(x) ** float(y)
        got = L.oracle_pow(float(x), float(y))
        bound = 2.0 + abs(y * math.log(x))
        worst = max(worst, ulp_err(got, ref) / bound)
    assert worst < 1.5, worst


def test_acos_accuracy_and_monotone():
    L = orc.lib()
    xs = np.linspace(-1.0, 1.0, 20001)
    vals = np.array([L.oracle_acos(float(x)) for x in xs])
    ref = np.arccos(xs)
    assert np.max(np.abs(vals - ref)) < 8 * EPS
    assert np.all(np.diff(vals) <= 0.0)
    assert L.oracle_acos(1.0) == 0.0


@pytest.mark.parametrize("x", [-1.0, float("nan")])
def test_log_domain(x):
    L = orc.lib()
    assert math.isnan(L.oracle_log(x))
    assert L.oracle_log(0.0) == -math.inf


def test_exp_range_ends():
    """Arguments around the fast path's |x| < 704 limit, down to subnormal
    and zero results and up to the overflow threshold."""
    L = orc.lib()
    xs = np.concatenate([np.linspace(-745.1, -690.0, 3001), np.linspace(690.0, 709.78, 2001),
                         [703.999999, 704.0, -703.999999, -704.0, -708.4, -708.39641853226408]])
    for x in xs:
        ref = math.exp(float(x))
        got = L.oracle_exp(float(x))
        if ref < 2.2250738585072014e-308:   # subnormal result: absolute error in units of the smallest subnormal
            assert abs(got - ref) <= 5e-324 * 2, (x, got, ref)
        else:
            assert ulp_err(got, ref) < 2.0, (x, got, ref)
    assert L.oracle_exp(709.79) == math.inf and L.oracle_exp(-745.3) == 0.0


def test_log_table_ties_and_boundaries():
    """Mantissas exactly halfway between two table points (rounded away from
    zero), and the 0.75 / 1.5 split of the reduced mantissa."""
    L = orc.lib()
    xs = [1.0 + (2 * k + 1) / 256.0 for k in range(64)] + [0.5 + (2 * k + 1) / 512.0 for k in range(32)]
    xs += [1.5, np.nextafter(1.5, 0.0), 0.75, np.nextafter(0.75, 0.0), 3.0, np.nextafter(3.0, 0.0)]
    for x in xs:
        ref = math.log(float(x))
        got = L.oracle_log(float(x))
        assert abs(got - ref) <= 3.0 * abs(ref) * EPS + 1e-300, (x, got, ref)

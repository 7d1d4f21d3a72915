"""The kinetics kernels' own FP64 exp and log (ember_gb300/csrc/emath.cuh).

CPU: the oracle's restatement (oracle/oracle_chem.c: oracle_exp, oracle_log)
against the C library's exp (within 1 ulp) and log (within 2 ulp), with the C
library's special values. GPU: the device functions
(ember_math_eval) bit for bit against the restatement, on edge values (zeros,
subnormals, sqrt 2 and the overflow and underflow thresholds with their
neighbours, the rounding boundaries of the exponent reduction, infinities,
NaN) and seeded values over the whole range.
log10 and exp10 are log(x) log10(e) and exp(x ln 10), as the Troe falloff
evaluates them.
"""
import math

import numpy as np
import pytest

LOG10E = 0.4342944819032518
LN10 = 2.302585092994046


def _around(v, k=3):
    out = [v]
    lo = hi = v
    for _ in range(k):
        lo, hi = np.nextafter(lo, -np.inf), np.nextafter(hi, np.inf)
        out += [lo, hi]
    return out


def exp_inputs(seed=1):
    rng = np.random.default_rng(seed)
    edge = [0.0, -0.0, 5e-324, -5e-324, 1e-300, -1e-300, np.inf, -np.inf, np.nan, 800.0, -800.0, 1e308, -1e308]
    for v in (708.0, -708.0, 709.782712893384, -745.1332191019412, -708.3964185322641, 709.0, -744.0, 1.0, -1.0):
        edge += _around(v)
    ln2 = math.log(2.0)
    for k in range(-1075, 1025, 7):  # x log2(e) near k + 1/2: the reduction's rounding boundaries
        edge += _around((k + 0.5) * ln2, 2)
    x = np.concatenate([np.array(edge), rng.uniform(-750.0, 715.0, 20000), rng.normal(0.0, 1.0, 5000),
                        rng.normal(0.0, 30.0, 5000), -np.exp(rng.uniform(-40.0, 6.5, 3000))])
    return x.astype(np.float64)


def log_inputs(seed=2):
    rng = np.random.default_rng(seed)
    sqrt2 = 1.4142135623730951
    edge = [0.0, -0.0, -1.0, -5e-324, 5e-324, 1e-320, np.inf, -np.inf, np.nan, np.finfo(np.float64).max]
    for v in (1.0, sqrt2, sqrt2 / 2, 2.0, 0.5, 2.2250738585072014e-308, 10.0, 0.1):
        edge += _around(v)
    for k in range(-1070, 1020, 13):  # m on either side of sqrt 2 at many exponents
        edge += _around(math.ldexp(sqrt2, k), 2)
    x = np.concatenate([np.array(edge), np.exp(rng.uniform(-740.0, 709.0, 20000)),
                        1.0 + rng.normal(0.0, 1e-3, 3000), rng.uniform(0.0, 4.0, 3000),
                        rng.uniform(-1.0, 0.0, 200)])
    return x.astype(np.float64)


def oracle_eval(op, x):
    from oracle import chem
    lib = chem._lib()
    f = lib.oracle_exp if op in (0, 3) else lib.oracle_log
    out = np.empty_like(x)
    for i, v in enumerate(x.tolist()):
        if op == 0:
            out[i] = f(v)
        elif op == 1:
            out[i] = f(v)
        elif op == 2:
            out[i] = f(v) * LOG10E
        else:
            out[i] = f(v * LN10)
    return out


def _c_exp(v):
    try:
        return math.exp(v)
    except OverflowError:
        return math.inf


def ulps(a, b):
    """|a - b| in units of the spacing of doubles at b (finite b)."""
    return np.abs(a - b) / np.spacing(np.abs(b))


def test_oracle_exp_and_log_against_the_c_library():
    x = exp_inputs()
    got = oracle_eval(0, x)
    ref = np.array([_c_exp(v) for v in x.tolist()])
    same_special = np.isnan(got) == np.isnan(ref)
    assert same_special.all()
    fin = np.isfinite(ref) & (ref != 0.0)
    assert np.array_equal(got[~fin & ~np.isnan(ref)], ref[~fin & ~np.isnan(ref)])  # inf and 0 where the C library gives them
    assert ulps(got[fin], ref[fin]).max() <= 1.0

    x = log_inputs()
    got = oracle_eval(1, x)
    ref = np.array([(math.log(v) if v > 0 else (-math.inf if v == 0 else math.nan)) if not math.isnan(v) else math.nan
                    for v in x.tolist()])
    assert (np.isnan(got) == np.isnan(ref)).all()
    fin = np.isfinite(ref) & (ref != 0.0)
    assert np.array_equal(got[~fin & ~np.isnan(ref)], ref[~fin & ~np.isnan(ref)])  # log 1 = 0, log 0 = -inf, log inf = inf
    assert ulps(got[fin], ref[fin]).max() <= 2.0

    # exp10 over the arguments the Troe blending gives it (|log10 F| of a few):
    # the rounded constant ln 10 and the rounding of x ln 10 each shift the
    # result by up to |x ln 10| ulp, on top of exp's own error (measured: 2 ulp
    # at |x| <= 0.5, 9 at |x| <= 3)
    xs = np.random.default_rng(3).uniform(-3.0, 3.0, 2000)
    got = oracle_eval(3, xs)
    assert (ulps(got, np.array([10.0 ** v for v in xs.tolist()])) <= 3.0 + 2.0 * np.abs(xs) * LN10).all()


@pytest.mark.gpu
@pytest.mark.parametrize("op", [0, 1, 2, 3])
def test_device_exp_and_log_match_the_oracle_bitwise(gpu_lib, op):
    from ember_gb300 import _lib
    if op in (0, 3):
        x = exp_inputs() if op == 0 else exp_inputs(4) / LN10
    else:
        x = log_inputs(2 + op)
    y = np.empty_like(x)
    rc = _lib.lib().ember_math_eval(op, x.ctypes.data, y.ctypes.data, x.size)
    assert rc == 0, _lib.last_error()
    ref = oracle_eval(op, x)
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(y), nan)
    assert np.array_equal(y[~nan].view(np.int64), ref[~nan].view(np.int64))


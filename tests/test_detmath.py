"""detmath (the synthetic cases' elementary functions from IEEE basic operations):
accurate to a few ulp against 200-bit mpmath, exact where the result is exact, and the
signed-zero conventions of numpy's atan2."""

import numpy as np
import pytest

from mpas_dycore_pytorch_gb300 import detmath as dm


def _ulps(got, ref):
    return float(np.max(np.abs(got - ref) / np.spacing(np.abs(ref))))


@pytest.mark.parametrize("name,lo,hi,bound", [("exp", -30.0, 30.0, 2), ("sin", -20.0, 20.0, 2),
                                              ("cos", -20.0, 20.0, 2), ("log", 1e-6, 1e6, 3),
                                              ("asin", -1.0, 1.0, 6)])
def test_accuracy(name, lo, hi, bound):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    x = np.random.default_rng(11).uniform(lo, hi, 1500)
    if name == "log":
        x = np.exp(np.random.default_rng(11).uniform(np.log(lo), np.log(hi), 1500))
    ref = np.array([float(getattr(mpmath, name)(mpmath.mpf(v))) for v in x])
    assert _ulps(getattr(dm, name)(x), ref) <= bound


def test_atan2_and_pow_accuracy():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    rng = np.random.default_rng(12)
    y, x = rng.normal(size=1500), rng.normal(size=1500)
    ref = np.array([float(mpmath.atan2(mpmath.mpf(a), mpmath.mpf(b))) for a, b in zip(y, x)])
    assert _ulps(dm.atan2(y, x), ref) <= 6
    a = rng.uniform(0.2, 1.2, 1500)
    ref = np.array([float(mpmath.power(mpmath.mpf(v), mpmath.mpf(3.5))) for v in a])
    assert _ulps(dm.pow(a, 3.5), ref) <= 10


def test_exact_values_and_conventions():
    assert dm.exp(np.array(0.0)) == 1.0 and dm.log(np.array(1.0)) == 0.0
    assert dm.sin(np.array(0.0)) == 0.0 and dm.cos(np.array(0.0)) == 1.0
    assert dm.atan2(0.0, -1.0) == np.pi and dm.atan2(-0.0, -1.0) == -np.pi
    assert dm.atan2(1.0, 0.0) == np.pi / 2 and dm.atan2(0.0, 0.0) == 0.0
    assert dm.asin(np.array(1.0)) == np.pi / 2

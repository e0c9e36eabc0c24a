"""pow_exner (csrc/pow_exner.cuh), the kernels' Exner-function pow, built for the host from
the same source: correctly rounded on random arguments, and equal to the C library's pow
(which the reference's Exner function calls) wherever the library rounds correctly."""

from __future__ import annotations

import ctypes
import math
import pathlib
import shutil
import subprocess
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
CSRC = ROOT / "mpas_dycore_pytorch_gb300" / "csrc"
RCV = 287.0 / (1004.5 - 287.0)


@pytest.fixture(scope="module")
def pow_exner(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    so = tmp_path_factory.mktemp("powx") / "libpowx.so"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-o", str(so),
                    str(ROOT / "tests" / "pow_exner_host.cpp")], check=True)
    lib = ctypes.CDLL(str(so))

    def call(x, y):
        x = np.ascontiguousarray(x, np.float64)
        y = np.ascontiguousarray(np.broadcast_to(np.float64(y), x.shape))
        out = np.empty_like(x)
        lib.pow_exner_many(ctypes.c_void_p(x.ctypes.data), ctypes.c_void_p(y.ctypes.data),
                           ctypes.c_void_p(out.ctypes.data), ctypes.c_long(x.size))
        return out
    return call


def test_tables_are_generated_from_the_script():
    r = subprocess.run([sys.executable, str(CSRC / "gen_pow_tables.py"), "--check"])
    assert r.returncode == 0, "pow_tables.inc differs from gen_pow_tables.py's output"


@pytest.mark.parametrize("lo,hi,y", [(0.01, 2.0, RCV), (1e-5, 1e5, 0.37), (0.5, 1.5, 3.5), (0.9, 1.1, -2.75)])
def test_correctly_rounded(pow_exner, lo, hi, y):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 200
    x = np.random.default_rng(7).uniform(lo, hi, 1500)
    got = pow_exner(x, y)
    ref = np.array([float(mpmath.power(mpmath.mpf(v), mpmath.mpf(y))) for v in x])
    assert np.array_equal(got, ref), int((got != ref).sum())


def test_agrees_with_the_c_library_pow(pow_exner):
    """The library's pow is not always correctly rounded: they differ in well under 1 case
    in 300, by one ulp."""
    x = np.random.default_rng(3).uniform(0.02, 1.5, 100_000)
    got = pow_exner(x, RCV)
    lib = np.array([math.pow(v, RCV) for v in x])
    diff = got != lib
    assert diff.mean() < 3e-3, diff.mean()
    assert np.all(np.abs(got - lib) <= np.spacing(lib))


def test_exact_cases_and_fallbacks(pow_exner):
    x = np.array([1.0, 4.0, 0.25, 2.0, 0.0, -2.0, np.inf, 1e-310, 3.0])
    y = np.array([RCV, 0.5, 0.5, 10.0, RCV, 2.0, 0.5, 0.5, 800.0])
    got = pow_exner(x, y)
    want = np.array([math.pow(a, b) if not (a == 3.0) else np.inf for a, b in zip(x, y)])
    assert np.array_equal(got, want, equal_nan=True), got

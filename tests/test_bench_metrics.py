"""bench.py's error metric (pure numpy): relative L2 per field, and pressure
against the dynamic pressure with each field's mean removed, because a
streamwise-periodic channel fixes the pressure level only through the path
to the fixed point."""
import os
import sys
from types import SimpleNamespace

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _out(U, p, k, om, nut):
    return SimpleNamespace(state={"U": U, "p": p, "k": k, "omega": om, "nuT": nut})


def test_pressure_level_is_not_an_error():
    rng = np.random.default_rng(3)
    n = 64
    U = np.zeros((n, 3))
    U[:, 0] = 20.0 + rng.standard_normal(n)
    p, k, om, nut = rng.standard_normal(n), rng.random(n), rng.random(n) + 1, rng.random(n)
    a = _out(U, p + 123.0, k, om, nut)           # same fields, pressure shifted by a constant
    b = _out(U, p, k, om, nut)
    e = bench._field_errors([a], [b])
    for f in ("U", "k", "omega", "nuT", "p"):
        assert e[f]["max"] < 1e-14, (f, e[f])


def test_pressure_difference_is_an_error():
    n = 64
    U = np.zeros((n, 3))
    U[:, 0] = 20.0
    p = np.linspace(0.0, 1.0, n)
    q = 0.5 * 20.0 ** 2
    a = _out(U, p + 1e-3 * q * np.sign(np.arange(n) - n / 2 + 0.5), np.ones(n), np.ones(n), np.ones(n))
    b = _out(U, p, np.ones(n), np.ones(n), np.ones(n))
    e = bench._field_errors([a], [b])
    assert abs(e["p"]["max"] - 1e-3) < 1e-12
    assert e["U"]["max"] == 0.0

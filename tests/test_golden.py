"""The committed golden fixtures (tests/golden/*.npz, made by
tests/golden/make_golden.py from the FP64 oracle) are reproduced by the
oracle on this machine: the fixed-point scatter exactly, FP64 values to
1e-10 relative (libm may differ in the last bits between hosts). This pins
the oracle the GPU parity tests compare against."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden as G  # noqa: E402
from oracle import ffi  # noqa: E402


def rel(a, b):
    s = float(np.max(np.abs(b))) or 1.0
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)))) / s


@pytest.mark.parametrize("name", sorted(G.CASES))
def test_oracle_reproduces_golden(name):
    fx = np.load(os.path.join(HERE, "golden", name + ".npz"))
    _, _, over, gamma = G.CASES[name]
    o = ffi.Oracle(G.problem_of(name), G.params(over))
    for tag in ("initial", "spread"):
        c = fx[tag + "_coords"]
        phys, fill, ov, cnt = o.scatter_fixed(c)
        assert np.array_equal(phys, fx[tag + "_phys"])
        assert np.array_equal(fill, fx[tag + "_fill"])
        assert np.array_equal(ov, fx[tag + "_overflow_fixed"])
        assert np.array_equal(cnt.astype(np.int64), fx[tag + "_overflow_bins"])
        ev = o.evaluate(c, float(fx["gamma"]))
        for k in ("density", "potential", "field_gradient", "wa_gradient"):
            assert rel(ev[k], fx[tag + "_" + k]) <= 1e-10, k
        assert rel(ev["wirelength"], fx[tag + "_wirelength"]) <= 1e-10
        assert rel([f.energy for f in ev["fields"]], fx[tag + "_energy"]) <= 1e-10

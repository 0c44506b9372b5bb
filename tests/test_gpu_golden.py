"""The CUDA engine against the committed golden fixtures (the FP64 oracle's
outputs at FP32-representable positions), through the C ABI: density grids,
overflow sums and overflowed-bin counts bit-exact; density, potential, field
and WA gradients within 1e-5 normwise relative; WA value and energies within
1e-5 relative."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden as G  # noqa: E402
from texo_gb300.placer import Placer, default_params  # noqa: E402

pytestmark = pytest.mark.gpu
TOL = 1e-5


def normwise(a, b):
    s = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) / s if s else float(np.max(np.abs(a)))


@pytest.mark.parametrize("name", sorted(G.CASES))
def test_engine_matches_golden(name):
    fx = np.load(os.path.join(HERE, "golden", name + ".npz"))
    _, _, over, _ = G.CASES[name]
    gamma = float(fx["gamma"])
    with Placer(G.problem_of(name), default_params(**over)) as g:
        for tag in ("initial", "spread"):
            c = fx[tag + "_coords"]
            phys, fill = g.scatter(c)
            assert np.array_equal(phys, fx[tag + "_phys"])
            assert np.array_equal(fill, fx[tag + "_fill"])
            d = g.evaluate(c, gamma)
            for f in range(g.num_fields):
                assert d["fields"][f].overflow_fixed == fx[tag + "_overflow_fixed"][f]
                assert d["fields"][f].overflow_bins == fx[tag + "_overflow_bins"][f]
                e = fx[tag + "_energy"][f]
                assert abs(d["fields"][f].energy - e) <= TOL * max(abs(e), 1e-30)
            for k in ("density", "potential", "field_gradient", "wa_gradient"):
                assert normwise(d[k], fx[tag + "_" + k]) <= TOL, k
            w = float(fx[tag + "_wirelength"])
            assert abs(d["wirelength"] - w) <= TOL * abs(w)

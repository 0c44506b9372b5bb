"""Generates the golden parity fixtures in this folder from the FP64 oracle
(oracle/, the CPU restatement of the reference path; test infrastructure).

Each fixture holds one problem (the seeded synthetic generator's arguments,
or the small mixed-field case), FP32-representable positions (the device
holds FP32 coordinates), and the oracle's outputs at those positions: the
fixed-point density grids, overflow sums and counts (bit-exact targets), the
FP64 density, potential, field and WA gradients, energies and WA value
(1e-5 normwise targets). Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ffi  # noqa: E402
from texo_gb300 import abi, problem as P  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def mixed_problem():
    cap = np.zeros((2, 12), np.uint32)
    cap[0, 0:4] = 1
    cap[1, 4:8] = 1
    units = [(1.25, 0.25, [(0, 0.0, 0.0, 1.0), (1, 0.5, 0.5, 1.0)]),
             (2.5, 0.75, [(0, 0.0, 0.0, 1.25)]),
             (0.3, 1.1, [(1, 0.0, 0.0, 1.0)])]
    return P.density_problem(4, 3, [(abi.KIND_LUT, 4), (abi.KIND_REGISTER, 0)], cap, units,
                             nets=[[0, 2], [1, 3, 2]])


# name: (problem factory, synthetic args or None, params overrides, gamma)
CASES = {
    "mixed-4x3": (mixed_problem, None, {}, 0.5),
    "ecp5-2k-tiles": (None, (48, 2000, 96, 2400, 6.0, 0), {}, 8.0),
    "ecp5-2k-bins64-td0.9": (None, (48, 2000, 96, 2400, 6.0, 0),
                             dict(bins_x=64, bins_y=64, target_density=0.9, gamma_base=4.0), 3.0),
}


def params(overrides):
    p = abi.default_params_py()
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def problem_of(name):
    make, synth, _, _ = CASES[name]
    return make() if make else P.synthetic(*synth)


def positions(o, seed):
    c, lo, hi = o.initial()
    if seed is not None:
        rng = np.random.default_rng(seed)
        c = lo + (hi - lo) * rng.random(c.size)
    return c.astype(np.float32).astype(np.float64)


def make(name):
    _, _, over, gamma = CASES[name]
    o = ffi.Oracle(problem_of(name), params(over))
    out = {"gamma": np.float64(gamma)}
    for tag, seed in (("initial", None), ("spread", 5)):
        c = positions(o, seed)
        phys, fill, ov, cnt = o.scatter_fixed(c)
        ev = o.evaluate(c, gamma)
        out.update({
            tag + "_coords": c, tag + "_phys": phys, tag + "_fill": fill, tag + "_overflow_fixed": ov,
            tag + "_overflow_bins": cnt.astype(np.int64), tag + "_density": ev["density"],
            tag + "_potential": ev["potential"], tag + "_field_gradient": ev["field_gradient"],
            tag + "_wa_gradient": ev["wa_gradient"], tag + "_wirelength": np.float64(ev["wirelength"]),
            tag + "_energy": np.array([f.energy for f in ev["fields"]]),
        })
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


if __name__ == "__main__":
    for n in CASES:
        make(n)
        print("wrote", n)

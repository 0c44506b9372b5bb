"""GPU parity at the benchmark sizes, against the FP64 oracle.

  * lfe5u-85-42k (42,000 cells + 365 IO, 50,000 nets, 256^2 bins, target
    density 0.9): scatter grids, overflow sums and overflowed-bin counts
    bit-exact; density, potential, field and WA gradients normwise within
    1e-5 of FP64 at spread positions; a full device-engine placement
    converges (overflow <= 0.10) with final HPWL within 1% of the oracle's.
  * stress-1m (1,000,000 cells + 4,096 IO, 1,200,000 nets, 1024^2 bins):
    scatter bit-exact; density, potential, field and WA gradients within
    1e-5 (the double-float FFT form: field gradient 7.9e-6 measured).
Both evaluations run with the default FP32 form (the FFT on these
power-of-two grids) and with the tensor-core form (integer slices, exact
accumulation), each held to the same 1e-5 bounds.
"""
import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi, problem as P
from texo_gb300.placer import Placer, default_params

pytestmark = pytest.mark.gpu

CONFIGS = {
    "lfe5u-85-42k": ((210, 42000, 365, 50000, 12.0), 256, 1e-5),
    "stress-1m": ((1024, 1000000, 4096, 1200000, 24.0), 1024, 1e-5),
}


def normwise(a, b):
    return float(np.max(np.abs(a - b))) / float(np.max(np.abs(b)))


DCT = {"fp32": abi.DCT_FP32, "tensor": abi.DCT_TENSOR}
_PROBLEMS = {}


def make(name, engine=abi.ENGINE_HOST, dct=abi.DCT_FP32):
    (side, cells, io, nets, sigma), bins, field_tol = CONFIGS[name]
    if name not in _PROBLEMS:
        _PROBLEMS.clear()
        _PROBLEMS[name] = P.synthetic(side, cells, io, nets, sigma, 0)
    prob = _PROBLEMS[name]
    prm = default_params(bins_x=bins, bins_y=bins, target_density=0.9, gamma_base=4.0, max_iterations=1000,
                         best_effort=1, engine=engine, dct_mode=dct)
    return prob, prm, field_tol


@pytest.mark.parametrize("dct", sorted(DCT))
@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_full_size_scatter_and_evaluation(name, dct):
    prob, prm, field_tol = make(name, dct=DCT[dct])
    o = ffi.Oracle(prob, prm)
    c, lo, hi = o.initial()
    c = (lo + (hi - lo) * np.random.default_rng(11).random(c.size)).astype(np.float32).astype(np.float64)
    with Placer(prob, prm) as g:
        phys, fill = g.scatter(c)
        d = g.evaluate(c, 4.0)
    rp, rf, rov, rcnt = o.scatter_fixed(c)
    assert np.array_equal(phys, rp) and np.array_equal(fill, rf)
    assert d["fields"][0].overflow_fixed == rov[0] and d["fields"][0].overflow_bins == rcnt[0]
    r = o.evaluate(c, 4.0, threads=5)
    assert normwise(d["density"], r["density"]) <= 1e-5
    assert normwise(d["potential"], r["potential"]) <= 1e-5
    assert normwise(d["wa_gradient"], r["wa_gradient"]) <= 1e-5
    assert normwise(d["field_gradient"], r["field_gradient"]) <= field_tol
    assert abs(d["wirelength"] - r["wirelength"]) <= 1e-5 * abs(r["wirelength"])
    a, b = d["fields"][0], r["fields"][0]
    assert abs(a.energy - b.energy) <= 1e-5 * abs(b.energy)
    assert abs(a.force_l1 - b.force_l1) <= 1e-5 * b.force_l1


def test_config1_device_placement_matches_oracle_hpwl():
    prob, prm, _ = make("lfe5u-85-42k", engine=abi.ENGINE_DEVICE)
    st, _, _, s_ref = ffi.Oracle(prob, prm).place(threads=5)
    assert st == 0 and s_ref.converged
    with Placer(prob, prm) as g:
        _, _, s = g.run()
    assert s["converged"] and s["overflow"][0] <= 0.10
    assert abs(s["hpwl"] - s_ref.hpwl) <= 0.01 * s_ref.hpwl

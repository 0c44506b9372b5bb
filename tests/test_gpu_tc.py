"""The tensor-core (tcgen05) DCT form against the FP64 oracle.

Every operand value is cut into four 8-bit integer slices with one
power-of-two scale per row, and the slice products are summed exactly in
FP32, so the form meets the same bounds as the FP32 forms:
  * potential (normwise relative, max|a-b|/max|b|) <= 1e-5,
  * field gradient (normwise relative) <= 1e-5,
  * energy (relative) <= 1e-5,
  * a full placement converges with final HPWL within 1% of the oracle's,
and results are bit-for-bit repeatable. The benchmark-size evaluations (42k
and 1M cells) are in test_gpu_parity_full.py.
"""
import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi, problem as P
from texo_gb300.placer import Placer, default_params

pytestmark = pytest.mark.gpu

TOL = 1e-5


def normwise(a, b):
    s = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) / s


def tc_params(**kw):
    return default_params(dct_mode=abi.DCT_TENSOR, engine=abi.ENGINE_HOST, **kw)


@pytest.mark.parametrize("W,H,matrix", [(127, 96, True), (64, 64, True), (256, 256, False), (1024, 1024, False),
                                        (200, 72, False)])
def test_poisson_tensor_matches_fp64(W, H, matrix):
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 0)
    i = np.arange(W * H)
    d = ((i * 31 + 7) % 101) - 50.0 + ((i * 13 + 5) % 17) / 17.0
    ref, er = ffi.poisson(W, H, d, matrix=matrix)
    with Placer(prob, tc_params(bins_x=W, bins_y=H)) as g:
        assert g.dct_form() == 2   # tensor cores
        pot, e = g.poisson(d)
        pot2, e2 = g.poisson(d)
    assert normwise(pot, ref) <= TOL
    assert abs(e - er) <= TOL * abs(er)
    assert np.array_equal(pot, pot2) and e == e2


def test_poisson_tensor_wide_dynamic_range():
    # a smooth large-scale mode plus a small fine-scale term: the per-row
    # scales keep the small term's bits
    W = H = 128
    y, x = np.mgrid[0:H, 0:W]
    d = 1e4 * np.cos(np.pi * (x + 0.5) / W) + 1e-2 * (((x * 7 + y * 13) % 11) - 5.0)
    ref, er = ffi.poisson(W, H, d.ravel(), matrix=True)
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 0)
    with Placer(prob, tc_params(bins_x=W, bins_y=H)) as g:
        pot, e = g.poisson(d.ravel())
    assert normwise(pot, ref) <= TOL
    assert abs(e - er) <= TOL * abs(er)


@pytest.mark.parametrize("kw", [{}, dict(bins_x=64, bins_y=64, target_density=0.9, gamma_base=4.0)])
def test_evaluation_tensor_matches_fp64(kw):
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 0)
    prm = abi.default_params_py()
    for k, v in kw.items():
        setattr(prm, k, v)
    o = ffi.Oracle(prob, prm)
    c, lo, hi = o.initial()
    c = (lo + (hi - lo) * np.random.default_rng(1).random(c.size)).astype(np.float32).astype(np.float64)
    r = o.evaluate(c, 2.5)
    with Placer(prob, tc_params(**kw)) as g:
        d = g.evaluate(c, 2.5)
        # the density side does not depend on the DCT form: still exact
        phys, _ = g.scatter(c)
    assert np.array_equal(phys, o.scatter_fixed(c)[0])
    assert normwise(d["potential"], r["potential"]) <= TOL
    assert normwise(d["field_gradient"], r["field_gradient"]) <= TOL
    assert normwise(d["wa_gradient"], r["wa_gradient"]) <= TOL
    e, er = d["fields"][0].energy, r["fields"][0].energy
    assert abs(e - er) <= TOL * abs(er)


def test_placement_tensor_matches_oracle_hpwl():
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 0)
    prm = default_params(best_effort=1, max_iterations=400)
    st, _, _, s_ref = ffi.Oracle(prob, prm).place()
    assert st == 0
    prm = tc_params(best_effort=1, max_iterations=400)
    with Placer(prob, prm) as g:
        t, c, s = g.run()
        g.reset()
        t2, c2, _ = g.run()
    assert s["converged"] and s["overflow"][0] <= 0.10
    assert abs(s["hpwl"] - s_ref.hpwl) <= 0.01 * s_ref.hpwl
    assert np.array_equal(t, t2) and np.array_equal(c, c2)

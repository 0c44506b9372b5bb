"""The DCT-form autotuner and tile families on the GPU: an autotuned handle
runs one of the admissible forms and keeps the parity bounds of that form;
jobs of different tile families share a batch and still finish exactly as
they do alone."""
import ctypes as C

import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi, problem as P
from texo_gb300.placer import Batch, Placer, default_params

pytestmark = pytest.mark.gpu


def normwise(a, b):
    s = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) / s


def form(g):
    f = C.c_int32()
    abi.check(g.lib.texo_gp_dct_form(g.h, C.byref(f)), "texo_gp_dct_form")
    return f.value


def test_autotuned_fp32_form_keeps_the_fp32_bound():
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 0)
    o = ffi.Oracle(prob, abi.default_params_py())
    c, lo, hi = o.initial()
    c = (lo + (hi - lo) * np.random.default_rng(3).random(c.size)).astype(np.float32).astype(np.float64)
    r = o.evaluate(c, 2.0)
    with Placer(prob, default_params(autotune=1, engine=abi.ENGINE_HOST)) as g:
        assert form(g) in (0, 1)      # 48 x 48 tiles: not a power of two
        d = g.evaluate(c, 2.0)
        d2 = g.evaluate(c, 2.0)
    for k in ("potential", "field_gradient"):
        assert normwise(d[k], r[k]) <= 1e-5
        assert np.array_equal(d[k], d2[k])


def test_autotune_may_choose_the_tensor_cores_only_when_allowed():
    prob = P.synthetic(64, 3000, 100, 3600, 6.0, 4)
    with Placer(prob, default_params(autotune=1, bins_x=1024, bins_y=1024, engine=abi.ENGINE_HOST,
                                     dct_mode=abi.DCT_BF16X3)) as g:
        assert form(g) in (0, 1, 2, 3)
    with Placer(prob, default_params(autotune=1, bins_x=1024, bins_y=1024, engine=abi.ENGINE_HOST)) as g:
        assert form(g) in (0, 1, 3)
    # the fixed rules: the FFT form on power-of-two grids, else the GEMM form
    # with 64x64 tiles from 1024 blocks of 32 x 32 bins up
    with Placer(prob, default_params(bins_x=1024, bins_y=1024)) as g:
        assert form(g) == 3
    with Placer(prob, default_params(bins_x=1000, bins_y=1000)) as g:
        assert form(g) == 1
    with Placer(prob, default_params(bins_x=250, bins_y=250)) as g:
        assert form(g) == 0
    with Placer(prob, default_params(bins_x=1024, bins_y=1024, dct_mode=abi.DCT_BF16X3,
                                     engine=abi.ENGINE_HOST)) as g:
        assert form(g) == 2


def test_tile_families_share_a_batch_and_match_alone():
    prm = lambda **kw: default_params(best_effort=1, max_iterations=120, engine=abi.ENGINE_DEVICE, **kw)
    jobs = [(P.synthetic(48, 2000, 96, 2400, 6.0, 5), prm(bins_x=1024, bins_y=1024)),
            (P.synthetic(36, 1100, 60, 1300, 6.0, 6), prm()),
            (P.synthetic(24, 400, 40, 480, 6.0, 7), prm())]
    alone = []
    for p, q in jobs:
        with Placer(p, q) as g:
            alone.append(g.run(allow_nonconverged=True))
    b = Batch(prm())
    for i, (p, q) in enumerate(jobs):
        assert b.admit(p, i, q)
    got = {}
    for _ in range(500):
        b.advance(9)
        while True:
            r = b.retire()
            if r is None:
                break
            got[r[0]] = r
        if len(got) == len(jobs):
            break
    assert len(got) == len(jobs)
    for i, (t, _, s) in enumerate(alone):
        assert np.array_equal(got[i][1], t), "job %d differs in the mix" % i
        assert got[i][2]["hpwl"] == s["hpwl"]


@pytest.mark.parametrize("workload", ["rich", "lfe5u-85-42k"])
def test_autotuned_wa_lanes_keep_the_bound(workload):
    # the autotuner also picks the WA lanes per net of each degree class (and
    # the scatter form): whichever it picks, WA and the density stay within
    # 1e-5 of FP64 and repeat bit for bit
    from rich_problems import rich_problem
    if workload == "rich":
        prob, kw = rich_problem(0), {}
    else:
        prob = P.synthetic(210, 42000, 365, 50000, 12.0, 0)
        kw = dict(bins_x=256, bins_y=256, target_density=0.9, gamma_base=4.0)
    prm = default_params(autotune=1, engine=abi.ENGINE_HOST, **kw)
    o = ffi.Oracle(prob, prm)
    c, lo, hi = o.initial()
    c = (lo + (hi - lo) * np.random.default_rng(5).random(c.size)).astype(np.float32).astype(np.float64)
    r = o.evaluate(c, 1.5)
    with Placer(prob, prm) as g:
        d = g.evaluate(c, 1.5)
        d2 = g.evaluate(c, 1.5)
    assert abs(d["wirelength"] - r["wirelength"]) <= 1e-5 * abs(r["wirelength"])
    for k in ("wa_gradient", "density", "potential", "field_gradient"):
        assert normwise(d[k], r[k]) <= 1e-5, k
        assert np.array_equal(d[k], d2[k])

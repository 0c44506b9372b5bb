"""The tiled (shared-memory privatised) density scatter of the host engine
against the direct one and the oracle, through the C ABI.

Both forms deposit int64 2^-32 fixed point, so the bound is bit-exact: the
physical and filler grids, the overflow sums and counts, and everything
downstream of them (potential, field, the whole placement) must be identical
word for word, at clustered positions (every object in a few tiles: long
runs of one key, heavy collisions) and at spread ones, with one and two
density fields, and bin grids equal to or different from the tile grid.
"""
import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi, problem as P
from texo_gb300.placer import Placer, default_params

from rich_problems import rich_problem

pytestmark = pytest.mark.gpu

CASES = {
    "ecp5-2k-bins64": (lambda: P.synthetic(48, 2000, 96, 2400, 6.0, 0),
                       dict(bins_x=64, bins_y=64, target_density=1.0, gamma_base=4.0)),
    "rich-2field": (lambda: rich_problem(0), {}),
    "lfe5u-85-42k": (lambda: P.synthetic(210, 42000, 365, 50000, 12.0, 0),
                     dict(bins_x=256, bins_y=256, target_density=0.9, gamma_base=4.0)),
    "odd-bins-100x70": (lambda: P.synthetic(100, 9000, 120, 10000, 6.0, 3), dict(bins_x=100, bins_y=70)),
}


def positions(o, spread, seed):
    c, lo, hi = o.initial()
    if spread:
        c = lo + (hi - lo) * np.random.default_rng(seed).random(c.size)
    return c.astype(np.float32).astype(np.float64)


@pytest.mark.parametrize("spread", [False, True])
@pytest.mark.parametrize("name", sorted(CASES))
def test_tiled_scatter_is_bit_exact(name, spread):
    make, kw = CASES[name]
    prob = make()
    o = ffi.Oracle(prob, default_params(**kw))
    c = positions(o, spread, 7)
    rp, rf, rov, rcnt = o.scatter_fixed(c)
    out = {}
    for mode in (abi.SCATTER_DIRECT, abi.SCATTER_TILED):
        with Placer(prob, default_params(scatter_mode=mode, **kw)) as g:
            phys, fill = g.scatter(c)
            d = g.evaluate(c, 2.0)
        assert np.array_equal(phys, rp) and np.array_equal(fill, rf)
        for f in range(len(prob.fields)):
            assert d["fields"][f].overflow_fixed == rov[f] and d["fields"][f].overflow_bins == rcnt[f]
        out[mode] = d
    a, b = out[abi.SCATTER_DIRECT], out[abi.SCATTER_TILED]
    for k in ("density", "potential", "field_gradient", "wa_gradient"):
        assert np.array_equal(a[k], b[k]), k
    assert a["wirelength"] == b["wirelength"]


def test_tiled_scatter_placement_identical_to_direct():
    prob, kw = rich_problem(1), dict(best_effort=1, max_iterations=400)
    res = []
    for mode in (abi.SCATTER_DIRECT, abi.SCATTER_TILED):
        with Placer(prob, default_params(scatter_mode=mode, **kw)) as g:
            res.append(g.run())
    (t0, c0, s0), (t1, c1, s1) = res
    assert s0["converged"] and np.array_equal(t0, t1) and np.array_equal(c0, c1)
    assert s0["iterations"] == s1["iterations"] and s0["hpwl"] == s1["hpwl"]


def test_autotuned_scatter_changes_nothing():
    # the DCT half of the autotuner is cached per grid, so both runs get the
    # same DCT form; the scatter half may pick either form
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 0)
    kw = dict(best_effort=1, max_iterations=60, autotune=1)
    with Placer(prob, default_params(scatter_mode=abi.SCATTER_DIRECT, **kw)) as g:
        t0, c0, _ = g.run()
    with Placer(prob, default_params(scatter_mode=abi.SCATTER_AUTO, **kw)) as g:
        t1, c1, _ = g.run()
    assert np.array_equal(t0, t1) and np.array_equal(c0, c1)

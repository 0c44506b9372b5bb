"""texo_gp_scatter_static (the density scatter that allocates nothing) against
texo_gp_scatter, both called through the C ABI.

Tolerance: bit-exact. Both entry points produce int64 2^-32 fixed-point grids
whose sums are exact in any order, so every word must agree. Two calls in a
row with different coordinates check that no state leaks from one call into
the next through the shared scratch.
"""
import ctypes as C

import numpy as np
import pytest

from texo_gb300 import abi, problem as P
from texo_gb300.placer import Placer, default_params

pytestmark = pytest.mark.gpu

SCRATCH_GRID_WORDS = 131072


def _params(**kw):
    p = default_params()
    for k, v in kw.items():
        setattr(p, k, v)
    return p


CASES = {
    "tiles-2k": (lambda: P.synthetic(48, 2000, 96, 2400, 6.0, 0), {}),
    "bins64-td0.9": (lambda: P.synthetic(48, 2000, 96, 2400, 6.0, 0),
                     dict(bins_x=64, bins_y=64, target_density=0.9)),
    "prime-side-127": (lambda: P.synthetic(127, 9000, 120, 10000, 6.0, 7), {}),
}


def _coords(g, seed):
    c, lo, hi = g.initial()
    if seed is None:
        return c
    rng = np.random.default_rng(seed)
    return lo + (hi - lo) * rng.random(c.size)


def _static(lib, g, coords):
    n = g.num_fields * g.bins
    phys = np.full(n, -7, np.int64)
    fill = np.full(n, -7, np.int64)
    code = lib.texo_gp_scatter_static(g.h, abi.ptr(coords, C.c_double), abi.ptr(phys, C.c_int64),
                                      abi.ptr(fill, C.c_int64))
    abi.check(code, "texo_gp_scatter_static")
    return phys.reshape(g.num_fields, g.bins), fill.reshape(g.num_fields, g.bins)


@pytest.mark.parametrize("name", sorted(CASES))
def test_static_scatter_matches_scatter_twice(name):
    make, kw = CASES[name]
    lib = abi.load()
    with Placer(make(), _params(**kw)) as g:
        assert g.num_fields * g.bins <= SCRATCH_GRID_WORDS
        for seed in (None, 3):  # two calls in a row, different coordinates
            c = np.ascontiguousarray(_coords(g, seed))
            sp, sf = _static(lib, g, c)
            rp, rf = g.scatter(c)
            assert np.array_equal(sp, rp)
            assert np.array_equal(sf, rf)
            assert np.any(sp != 0) and np.any(sf != 0)


def test_static_scatter_rejects_oversized_grid():
    lib = abi.load()
    with Placer(P.synthetic(400, 2000, 96, 2400, 6.0, 1)) as g:
        assert g.num_fields * g.bins > SCRATCH_GRID_WORDS
        c = np.ascontiguousarray(g.initial()[0])
        phys = np.zeros(g.num_fields * g.bins, np.int64)
        code = lib.texo_gp_scatter_static(g.h, abi.ptr(c, C.c_double), abi.ptr(phys, C.c_int64), None)
        assert code == abi.CODE["UNSUPPORTED"]
        assert b"static scratch limit" in lib.texo_gp_last_error()
        # the handle still works through the ordinary entry point
        rp, _ = g.scatter(c)
        assert rp.shape == (g.num_fields, g.bins)


def test_static_scatter_rejects_too_many_objects():
    # a small bin grid (fits the grid limit) with more than 131072 units + fillers
    lib = abi.load()
    with Placer(P.synthetic(400, 2000, 96, 2400, 6.0, 1), _params(bins_x=64, bins_y=64)) as g:
        assert g.num_fields * g.bins <= SCRATCH_GRID_WORDS
        assert g.units + g.num_fillers > 131072
        c = np.ascontiguousarray(g.initial()[0])
        phys = np.zeros(g.num_fields * g.bins, np.int64)
        code = lib.texo_gp_scatter_static(g.h, abi.ptr(c, C.c_double), abi.ptr(phys, C.c_int64), None)
        assert code == abi.CODE["UNSUPPORTED"]
        assert b"units + fillers" in lib.texo_gp_last_error()


def test_static_scatter_allocates_nothing_after_the_first_call():
    torch = pytest.importorskip("torch")
    lib = abi.load()
    make, kw = CASES["bins64-td0.9"]
    with Placer(make(), _params(**kw)) as g:
        c = np.ascontiguousarray(_coords(g, 5))
        _static(lib, g, c)                      # the first call on the device reserves the array
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        for _ in range(3):
            _static(lib, g, c)
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0


def test_static_scatter_leaves_the_handle_alone():
    # evaluate(x) is the same whether or not a static scatter at other
    # coordinates came between two evaluations
    lib = abi.load()
    make, kw = CASES["tiles-2k"]
    with Placer(make(), _params(**kw)) as g:
        x = np.ascontiguousarray(_coords(g, 9))
        a = g.evaluate(x, 4.0)
        _static(lib, g, np.ascontiguousarray(_coords(g, 10)))
        b = g.evaluate(x, 4.0)
    for k in ("density", "potential", "wa_gradient", "field_gradient"):
        assert np.array_equal(a[k], b[k])
    assert a["wirelength"] == b["wirelength"]

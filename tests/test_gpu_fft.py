"""The FFT-based DCT form (the default FP32 form on power-of-two grids up to
1024, double-float butterflies) against the FP64 oracle: potential normwise
<= 1e-6 at every size (the transforms are exact to FP32; what remains is the
FP32 storage between passes), energy <= 1e-6 relative, field gradient <=
1e-5 on identical positions; the compensated GEMM form meets the 1e-5 bounds
too. Results repeat bit for bit."""
import ctypes as C

import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi, problem as P
from texo_gb300.placer import Placer, default_params

pytestmark = pytest.mark.gpu


def normwise(a, b):
    s = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) / s


def form(g):
    f = C.c_int32()
    abi.check(g.lib.texo_gp_dct_form(g.h, C.byref(f)), "texo_gp_dct_form")
    return f.value


@pytest.mark.parametrize("W,H,tol", [(64, 64, 1e-6), (256, 256, 1e-6), (256, 64, 1e-6), (32, 128, 1e-6),
                                     (1024, 1024, 1e-6)])
def test_fft_poisson_matches_fp64(W, H, tol):
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 0)
    i = np.arange(W * H)
    d = ((i * 31 + 7) % 101) - 50.0 + ((i * 13 + 5) % 17) / 17.0
    ref, er = ffi.poisson(W, H, d, matrix=W * H <= 4096)
    with Placer(prob, default_params(bins_x=W, bins_y=H, engine=abi.ENGINE_HOST)) as g:
        assert form(g) == 3
        pot, e = g.poisson(d)
        pot2, _ = g.poisson(d)
    assert normwise(pot, ref) <= tol
    assert abs(e - er) <= 1e-6 * abs(er)
    assert np.array_equal(pot, pot2)


@pytest.mark.parametrize("mode,forms", [(abi.DCT_FP32, (3,)), (abi.DCT_FP32_GEMM, (0, 1))])
def test_fp32_forms_match_fp64_on_a_256_grid(mode, forms):
    prob = P.synthetic(96, 6000, 150, 7200, 8.0, 2)
    prm = abi.default_params_py()
    prm.bins_x = prm.bins_y = 256
    o = ffi.Oracle(prob, prm)
    c, lo, hi = o.initial()
    c = (lo + (hi - lo) * np.random.default_rng(7).random(c.size)).astype(np.float32).astype(np.float64)
    r = o.evaluate(c, 3.0)
    with Placer(prob, default_params(bins_x=256, bins_y=256, dct_mode=mode, engine=abi.ENGINE_HOST)) as g:
        assert form(g) in forms
        d = g.evaluate(c, 3.0)
    for k in ("density", "potential", "field_gradient", "wa_gradient"):
        assert normwise(d[k], r[k]) <= 1e-5, k
    assert abs(d["fields"][0].energy - r["fields"][0].energy) <= 1e-5 * abs(r["fields"][0].energy)

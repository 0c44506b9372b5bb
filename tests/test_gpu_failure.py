"""Failure detection on the GPU without a fault: the engine's bounded waits
(grid barrier, tensor-core mbarrier) run out against partners that never
arrive, report it, and leave the context usable; a failing request in the
serving loop is covered by test_gpu_server.py."""
import ctypes as C

import numpy as np
import pytest

from texo_gb300 import abi, problem as P
from texo_gb300.placer import Placer, default_params

pytestmark = pytest.mark.gpu


def test_bounded_waits_run_out_and_the_device_stays_usable():
    lib = abi.load()
    b, m = C.c_int32(-1), C.c_int32(-1)
    abi.check(lib.texo_gp_selftest_waits(0, C.byref(b), C.byref(m)), "texo_gp_selftest_waits")
    assert b.value == 1 and m.value == 1
    with Placer(P.synthetic(24, 400, 40, 480, 6.0, 1), default_params(max_iterations=50, best_effort=1)) as g:
        _, _, s = g.run(allow_nonconverged=True)
    assert s["iterations"] > 0 and np.isfinite(s["hpwl"])

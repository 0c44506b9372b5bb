"""The serving loop on the GPU: requests submitted while others are already
running join the resident batch, and every job's result is bit-identical to
the same job placed alone; admission never holds more device memory than the
HBM budget; a request that fails does not disturb the others."""
import time

import numpy as np
import pytest

from texo_gb300 import abi, problem as P
from texo_gb300.placer import Placer, Server, default_params

pytestmark = pytest.mark.gpu

SIZES = [(24, 400, 40, 480, 1), (48, 2000, 96, 2400, 2), (64, 3500, 100, 4200, 3), (36, 1100, 60, 1300, 4),
         (30, 700, 50, 840, 5), (56, 2800, 100, 3400, 6)]


def params(**kw):
    p = default_params(best_effort=1, max_iterations=300, engine=abi.ENGINE_DEVICE)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def problems():
    return [P.synthetic(side, cells, io, nets, 6.0, seed) for side, cells, io, nets, seed in SIZES]


def alone(probs):
    out = []
    for p in probs:
        with Placer(p, params()) as g:
            t, _, s = g.run()
        out.append((t, s))
    return out


def drain(server, n, timeout_s=120.0):
    got = {}
    t_end = time.time() + timeout_s
    while len(got) < n and time.time() < t_end:
        r = server.poll(wait_ms=200)
        if r is not None:
            got[r[0]] = r
    return got


def test_staggered_requests_match_results_alone():
    probs = problems()
    ref = alone(probs)
    with Server(params(), chunk_iterations=5, admission_threads=2) as s:
        s.submit(probs[0], 0)
        s.submit(probs[1], 1)
        first = s.poll(wait_ms=-1)       # the others arrive while work is in flight
        for i in range(2, len(probs)):
            s.submit(probs[i], i)
        got = drain(s, len(probs) - 1)
        got[first[0]] = first
    assert len(got) == len(probs)
    for i, (t, st) in enumerate(ref):
        jid, tb, info = got[i]
        assert info["status"] == st["status"]
        assert np.array_equal(t, tb), "job %d differs when served" % i
        assert info["iterations"] == st["iterations"] and info["hpwl"] == st["hpwl"]
        assert info["submit_ms"] <= info["admit_ms"] <= info["finish_ms"]


def test_admission_keeps_within_the_hbm_budget():
    probs = problems()
    from texo_gb300.placer import Batch
    probe = Batch(params())
    assert probe.admit(probs[2], 0)
    _, _, one = probe.counts()
    probe.close()
    budget = int(one * 1.2)      # one job of this size at a time
    with Server(params(), hbm_budget=budget, chunk_iterations=10, admission_threads=3) as s:
        for i in range(4):
            s.submit(probs[2], i)
        peak, got = 0, {}
        t_end = time.time() + 120
        while len(got) < 4 and time.time() < t_end:
            peak = max(peak, s.counts()[3])
            r = s.poll(wait_ms=5)
            if r is not None:
                got[r[0]] = r
    assert len(got) == 4
    assert peak <= budget
    hp = {got[i][2]["hpwl"] for i in range(4)}
    assert len(hp) == 1


def test_a_failing_request_does_not_disturb_the_others():
    probs = problems()
    ref = alone(probs[:2])
    cap = np.zeros((1, 4 * 3), np.uint32)
    cap[0, :2] = 1   # two sites for three units: INSUFFICIENT_CAPACITY
    bad = P.density_problem(4, 3, [(abi.KIND_LUT, 4)], cap,
                            [(0.5, 0.5, [(0, 0.0, 0.0, 1.0)]), (1.5, 0.5, [(0, 0.0, 0.0, 1.0)]),
                             (2.5, 0.5, [(0, 0.0, 0.0, 1.0)])], nets=[[0, 1, 2]])
    with Server(params(), chunk_iterations=7) as s:
        s.submit(probs[0], 10)
        s.submit(bad, 11)
        s.submit(probs[1], 12)
        got = drain(s, 3)
    assert got[11][1] is None and got[11][2]["status"] == "INSUFFICIENT_CAPACITY"
    for jid, (t, st) in zip((10, 12), ref):
        assert np.array_equal(got[jid][1], t)

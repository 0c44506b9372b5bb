"""The oracle's per-iteration controller trace (the records the GPU
controller's trace is compared with) agrees with the run statistics it
summarises, on the smallest benchmark configuration and on the two-field
macro problem."""
import pytest

from oracle import ffi
from texo_gb300 import problem as P
from texo_gb300.placer import default_params

from rich_problems import rich_problem


@pytest.mark.parametrize("which", ["config0", "rich"])
def test_trace_matches_run_statistics(which):
    if which == "config0":
        prob = P.synthetic(48, 2000, 96, 2400, 6.0, 0, lib=ffi.lib())
        prm = default_params(bins_x=64, bins_y=64, target_density=1.0, gamma_base=4.0, best_effort=1)
    else:
        prob = rich_problem(0)
        prm = default_params(best_effort=1)
    o = ffi.Oracle(prob, prm)
    st, _, _, s = o.place(threads=5, max_iterations=12)
    assert st == 0
    tr = o.trace()
    assert [r.iteration for r in tr] == list(range(1, 13))
    assert sum(r.trials for r in tr) == s.line_search_trials
    assert tr[-1].gamma == s.gamma and tr[-1].objective == s.objective
    assert all(r.trials >= 1 and r.lipschitz > 0 and r.momentum >= 1.0 for r in tr)
    K = len(prob.fields)
    assert all(r.lambda_[f] > 0 and r.energy_scale[f] >= 1.0 for r in tr for f in range(K))
    # a second run replaces the trace
    o.place(threads=1, max_iterations=3)
    assert len(o.trace()) == 3

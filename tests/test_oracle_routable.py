"""The oracle's routability-driven rounds (eplace::place with a routing
capacity map, eplace.rs:320-420) on the two-kind routability case: rounds
stop at AreaAdjustmentReady until a proposal grows nothing, the installed
areas conserve every kind's member + filler total, and the last round
converges to the final targets."""
import numpy as np

from texo_gb300 import abi, routability as R

from routable_rounds import OracleRounds, routability_case


def test_oracle_rounds_on_the_routability_case():
    prob, ch, cv, ctl = routability_case()
    prm = abi.default_params_py()
    prm.best_effort = 1
    rounds = OracleRounds(prob, prm)
    f0, q0 = rounds.fillers()
    t, c, info = R.place_routable(prob, prm, ch, cv, register_controls=ctl, rounds=rounds)
    stops = [r["stop"] for r in info["rounds"]]
    assert stops[-1] == "final" and all(s == "area_ready" for s in stops[:-1])
    assert info["area_rounds"] >= 1 and info["rounds"][0]["relative_increase"] > 0.01
    assert info["rounds"][-2]["relative_increase"] < 0.01
    assert not info["rounds"][-1]["exhausted"]
    # charge conservation per field (instance_area.rs postconditions)
    m0 = np.asarray(prob.member_charge, dtype=np.float64)
    for f in range(len(prob.fields)):
        before = m0[prob.member_field == f].sum() + q0[f0 == f].sum()
        after = info["member_charge"][prob.member_field == f].sum() + info["filler_charge"][f0 == f].sum()
        assert abs(after - before) <= 1e-9 * before
    assert np.all(info["member_charge"] >= m0)
    o = rounds.o
    ev = o.evaluate(c, 4.0)
    assert all(fr.normalized_overflow <= 0.10 for fr in ev["fields"])

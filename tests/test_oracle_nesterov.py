"""Pins the oracle's dynamic Nesterov step and eplace scalar rules against the
reference's tests (crates/texo-pnr/src/global_placement.rs:714-1139 and
crates/texo-pnr/src/eplace.rs:1620-1915)."""
import ctypes as C
import math
import struct

import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi

NAME = abi.STATUS


def bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def quad1(target):
    def f(c):
        d = c[0] - target
        return 0.5 * d * d, [d]
    return f


B1 = ([-10.0], [10.0])


def step(state, bounds, metric, evaluate):
    return ffi.nesterov_step(state, bounds[0], bounds[1], metric, evaluate)


# global_placement.rs:746-764
def test_dynamic_step_returns_the_accepted_candidate_payload():
    s = ffi.NesterovState.new([2.0], *B1)
    st, out = step(s, B1, [1.0], lambda c: (*quad1(0.0)(c), bits(c[0]) >> 1))
    assert st == 0 and out.stationary == 0
    assert list(s.x) == [0.0]
    assert out.payload == bits(0.0) >> 1
    assert bits(out.objective) == bits(0.0)
    assert bits(out.stationarity) == bits(0.0)
    assert bits(out.coordinate_change) == bits(2.0)


# :766-796
def test_diagonal_metric_conditions_an_anisotropic_quadratic():
    s = ffi.NesterovState([2.0, 2.0], momentum=1.0, lipschitz=2.0)
    st, out = step(s, ([-10.0, -10.0], [10.0, 10.0]), [1.0, 100.0],
                   lambda c: (0.5 * c[0] ** 2 + 50.0 * c[1] ** 2, [c[0], 100.0 * c[1]], 0))
    assert st == 0 and out.stationary == 0
    assert list(s.x) == [0.0, 0.0]
    assert out.trials == 1


# :798-809
def test_metric_kkt_residual_scales_active_components_and_keeps_bound_signs():
    r = ffi.box_metric_kkt([3.0, -40.0, -50.0, 6.0], [0.0, 0.0, 2.0, 2.0], [0.0] * 4, [2.0] * 4,
                           [9.0, 100.0, 25.0, 4.0])
    assert bits(r) == bits(4.0)


# :811-828
def test_unchanged_candidate_reduces_lipschitz_before_declaring_stationarity():
    s = ffi.NesterovState([1.0], lipschitz=2.0 ** 60)
    st, out = step(s, B1, [1.0], lambda c: (*quad1(0.0)(c), 0))
    assert st == 0 and out.stationary == 0
    assert out.coordinate_change > 0 and out.trials > 1


# :830-847
def test_overflowing_metric_step_denominator_is_transactional():
    s = ffi.NesterovState([1.0], lipschitz=np.finfo(float).max)
    before = s.key()
    st, _ = step(s, B1, [4.0], lambda c: (*quad1(0.0)(c), 0))
    assert NAME[st] == "LINE_SEARCH_OVERFLOW"
    assert s.key() == before


# :849-873
def test_dynamic_step_re_evaluates_a_changed_objective_and_keeps_momentum():
    s = ffi.NesterovState.new([2.0], *B1)
    step(s, B1, [1.0], lambda c: (*quad1(0.0)(c), 0))
    m1 = s.momentum
    old = s.x[0]
    old_obj = quad1(3.0)([old])[0]
    seen = []

    def ev(c):
        seen.append(list(c))
        v, g = quad1(3.0)(c)
        return v, g, len(seen)
    st, out = step(s, B1, [1.0], ev)
    assert seen[0] == [old]
    assert st == 0 and out.stationary == 0 and out.objective <= old_obj
    assert s.momentum > m1


# :875-901 — fault injection: the evaluator fails on its second call.
def test_evaluator_failure_leaves_dynamic_state_bit_identical():
    s = ffi.NesterovState.new([2.0], *B1)
    step(s, B1, [1.0], lambda c: (*quad1(0.0)(c), 0))
    before = s.key()
    calls = [0]

    def ev(c):
        calls[0] += 1
        if calls[0] == 2:
            return 7     # injected evaluator failure
        return (*quad1(3.0)(c), 0)
    st, out = step(s, B1, [1.0], ev)
    assert NAME[st] == "EVALUATION" and out.inner == 7
    assert calls[0] == 2
    assert s.key() == before


# :903-928
def test_stationary_status_carries_the_origin_payload_and_a_new_objective_moves():
    s = ffi.NesterovState.new([1.0], *B1)
    st, out = step(s, B1, [1.0], lambda c: (*quad1(1.0)(c), bits(c[0]) >> 1))
    assert st == 0 and out.stationary == 1
    assert out.payload == bits(1.0) >> 1 and out.trials == 0
    st, out = step(s, B1, [1.0], lambda c: (*quad1(2.0)(c), 0))
    assert st == 0 and out.stationary == 0
    assert list(s.x) == [2.0]


# :930-968
def test_restart_backtracks_instead_of_repeating_a_rejected_candidate():
    s = ffi.NesterovState([0.0], previous=[-10.0], momentum=2.0, lipschitz=100.0)
    n = [0]

    def ev(c):
        n[0] += 1
        v = {1: 0.0, 2: 100.0, 3: 99.98, 4: 1.0, 5: 1.0}.get(n[0], c[0])
        return v, [1.0], n[0]
    st, out = step(s, ([-20.0], [20.0]), [1.0], ev)
    assert st == 0 and out.stationary == 0
    assert n[0] == 6 and out.payload == 6 and out.trials == 4
    assert list(s.x) == [-0.01]


# :970-1011
def test_malformed_bounds_and_nonfinite_initial_coordinates_are_typed_errors():
    s = ffi.NesterovState.new([0.5], [], [1.0])
    before = s.key()
    calls = [0]

    def ev(c):
        calls[0] += 1
        return 0.0, [0.0], 0
    st, _ = step(s, ([], [1.0]), [1.0], ev)
    assert NAME[st] == "INVALID_BOUNDS" and calls[0] == 0 and s.key() == before
    s2 = ffi.NesterovState.new([float("nan")], [0.0], [1.0])
    st, out = step(s2, ([0.0], [1.0]), [1.0], ev)
    assert NAME[st] == "INVALID_INITIAL_COORDINATE" and out.error_index == 0
    assert math.isnan(s2.x[0])


# :1013-1056
def test_invalid_diagonal_metrics_are_rejected_before_evaluation():
    s = ffi.NesterovState.new([1.0], *B1)
    before = s.key()
    calls = [0]

    def ev(c):
        calls[0] += 1
        return 0.0, [0.0], 0
    st, out = step(s, B1, [], ev)
    assert NAME[st] == "INVALID_METRIC_LENGTH" and (out.expected, out.actual) == (1, 0)
    for m in (0.0, -1.0, float("nan"), float("inf")):
        st, out = step(s, B1, [m], ev)
        assert NAME[st] == "NONPOSITIVE_METRIC" and out.error_index == 0
    assert calls[0] == 0 and s.key() == before


# :1058-1075
def test_invalid_dynamic_evaluation_is_transactional():
    s = ffi.NesterovState.new([2.0], *B1)
    before = s.key()
    st, _ = step(s, B1, [1.0], lambda c: (float("nan"), [0.0], 0))
    assert NAME[st] == "INVALID_OBJECTIVE" and s.key() == before


# :1077-1116
def test_invalid_dynamic_parameters_are_rejected_before_evaluation():
    calls = [0]

    def ev(c):
        calls[0] += 1
        return 0.0, [0.0], 0
    s = ffi.NesterovState.new([2.0], *B1)
    s.momentum = 0.5
    st, _ = step(s, B1, [1.0], ev)
    assert NAME[st] == "INVALID_MOMENTUM_PARAMETER"
    s.momentum = 1.0
    s.lipschitz = float("inf")
    st, _ = step(s, B1, [1.0], ev)
    assert NAME[st] == "INVALID_LIPSCHITZ_ESTIMATE" and calls[0] == 0


def test_gradient_length_and_nonfinite_gradient_are_typed_errors():
    s = ffi.NesterovState.new([2.0], *B1)
    st, out = step(s, B1, [1.0], lambda c: (0.0, [0.0, 1.0], 0))
    assert NAME[st] == "INVALID_GRADIENT_LENGTH" and (out.expected, out.actual) == (1, 2)
    st, out = step(s, B1, [1.0], lambda c: (0.0, [float("inf")], 0))
    assert NAME[st] == "NONFINITE_GRADIENT" and out.error_index == 0


# :1118-1139
def test_dynamic_steps_are_bit_deterministic():
    a = ffi.NesterovState.new([2.0], *B1)
    b = ffi.NesterovState.new([2.0], *B1)
    ra = step(a, B1, [1.0], lambda c: (*quad1(-3.0)(c), bits(c[0]) >> 1))[1]
    rb = step(b, B1, [1.0], lambda c: (*quad1(-3.0)(c), bits(c[0]) >> 1))[1]
    assert bytes(ra) == bytes(rb) and a.key() == b.key()


# ---- eplace scalar rules ----------------------------------------------------
def _aug(e, e0, lam, beta=2000.0):
    v, c = C.c_double(), C.c_double()
    ffi.lib().orc_augmented(e, e0, lam, beta, C.byref(v), C.byref(c))
    return v.value, c.value


# eplace.rs:1667-1685
def test_raw_phi_augmented_objective_and_gradient_have_matching_units():
    v, c = _aug(12.5, 50.0, 0.75)
    assert abs(v - 0.75 * (12.5 + 0.5 * 2000.0 * 12.5 * 12.5 / 50.0)) <= 1e-12
    assert abs(c - 0.75 * (1.0 + 2000.0 * 12.5 / 50.0)) <= 1e-12


def _growth(lg):
    g = C.c_double()
    st = ffi.lib().orc_multiplier_growth(lg, 1.05, 1.06, C.byref(g))
    return st, g.value


# :1698-1723
def test_multiplier_growth_matches_elfplace_endpoints_and_initial_step():
    p = abi.default_params_py()
    assert bits(p.alpha_low) == bits(1.05) and bits(p.alpha_high) == bits(1.06)
    step_v = C.c_double()
    m = np.array([3.0, 4.0])
    assert ffi.lib().orc_area_adjusted_multiplier_step(ffi.P(m), 2, 1.06, C.byref(step_v)) == 0
    assert abs(step_v.value - 0.30) <= 1e-15
    assert bits(_growth(0.0)[1]) == bits(1.05)
    assert bits(_growth(np.finfo(float).max)[1]) == bits(1.06)
    assert abs(_growth(1.0)[1] - 1.055) <= 1e-15
    assert NAME[_growth(-1.0)[0]] == "INVALID_NORMALIZATION"


# :1725-1739
@pytest.mark.parametrize("target", [0.10, 0.20])
def test_heterogeneous_field_gamma_hits_target_and_unit_overflow_endpoints(target):
    g = C.c_double()
    assert ffi.lib().orc_field_gamma(target, target, 8.0, C.byref(g)) == 0
    assert abs(g.value - 0.8) <= 1e-14
    assert ffi.lib().orc_field_gamma(1.0, target, 8.0, C.byref(g)) == 0
    assert abs(g.value - 80.0) <= 1e-12


# :1741-1749
def test_global_gamma_is_pin_weighted_field_mean():
    out = C.c_double()
    g, w = np.array([2.0, 10.0]), np.array([1.0, 3.0])
    assert ffi.lib().orc_weighted_gamma_mean(ffi.P(g), ffi.P(w), 2, 8.0, C.byref(out)) == 0
    assert out.value == 8.0
    g, w = np.array([80.0]), np.array([0.0])
    assert ffi.lib().orc_weighted_gamma_mean(ffi.P(g), ffi.P(w), 1, 8.0, C.byref(out)) == 0
    assert out.value == 8.0


# :1751-1758 and :1300-1308
def test_scarce_memory_overflow_has_an_independent_stop_condition():
    t = ffi.lib().orc_overflow_target
    assert t(abi.KIND_LUT) == 0.10 and t(abi.KIND_REGISTER) == 0.10
    assert t(abi.KIND_MEMORY) == 0.20 and t(abi.KIND_DSP) == 0.20
    assert t(abi.KIND_IO) == 0.0

    def converged(fields):
        return all(o <= t(k) for k, o in fields)
    assert not converged([(abi.KIND_LUT, 0.09), (abi.KIND_MEMORY, 0.21)])
    assert converged([(abi.KIND_LUT, 0.09), (abi.KIND_MEMORY, 0.20)])


# :1866-1875
def test_checkpoint_retains_the_lowest_field_overflow_excess():
    better = ffi.lib().orc_checkpoint_better
    best = (0.40 - 0.20, 0.40 - 0.20)
    cand = (0.25 - 0.20, 0.25 - 0.20)
    assert better(*cand, *best) == 1
    best = cand
    worse = (0.30 - 0.20, 0.30 - 0.20)
    assert better(*worse, *best) == 0
    assert better(*best, *best) == 0


# :1860-1864 (cap as a parameter; default equals the reference constant)
def test_paper_iteration_cap_default():
    assert abi.default_params_py().max_iterations == 3000


# :1760-1776
def test_area_adjustment_starts_at_lut_and_register_fifteen_percent():
    ready = ffi.lib().orc_area_adjustment_ready

    def is_ready(fields):
        k = np.array([f[0] for f in fields], np.uint32)
        o = np.array([f[1] for f in fields], np.float64)
        return ready(len(fields), ffi.P(k, C.c_uint32), ffi.P(o)) == 1
    assert is_ready([(abi.KIND_LUT, 0.15), (abi.KIND_REGISTER, 0.149), (abi.KIND_MEMORY, 0.99)])
    assert not is_ready([(abi.KIND_LUT, 0.151), (abi.KIND_REGISTER, 0.149)])


# :1799-1822
def test_area_adjusted_multiplier_matches_elfplace_force_balance():
    energy = np.array([5.0, 10.0])
    force = np.array([2.0, 3.0])
    initial = np.array([10.0, 20.0])
    wa = np.array([3.0, 4.0, -1.0, 0.0])     # units (3, 4) and (-1, 0): x then y per unit
    out = np.zeros(2)
    assert ffi.lib().orc_area_adjusted_multipliers(2, ffi.P(energy), ffi.P(force), ffi.P(initial), 2000.0,
                                                   ffi.P(wa), 2, ffi.P(out)) == 0
    assert abs(out[0] - out[1]) <= 1e-15
    # equation (27): <sum_i q_i ||xi_i||_1, lambda'> = eta' ||grad W||_1
    assert abs(2.0 * out[0] + 3.0 * out[1] - 0.8) <= 1e-14
    # a non-finite energy is the reference's DensityFieldChanged
    bad = np.array([np.nan, 10.0])
    assert ffi.lib().orc_area_adjusted_multipliers(2, ffi.P(bad), ffi.P(force), ffi.P(initial), 2000.0,
                                                   ffi.P(wa), 2, ffi.P(out)) == abi.CODE["DENSITY_FIELD_CHANGED"]

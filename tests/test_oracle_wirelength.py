"""Pins the oracle's weighted-average wirelength and preconditioners against
the reference's tests (crates/texo-pnr/src/analytical_placement.rs:817-1183)."""
import math

import numpy as np

from oracle import ffi
from texo_gb300.problem import Problem

GAMMA = 0.25   # TEST_GLOBAL_GAMMA, analytical_placement.rs:826


def wa_problem(n_units, cell_unit, nets, fixed=None, offsets=None, arcs=()):
    """Logic-only problem (no density fields): pure WA evaluation."""
    C = len(cell_unit)
    fixed = fixed or [None] * C
    offsets = offsets or [(0.0, 0.0)] * C
    net_ptr, pins = [0], []
    for net in nets:
        pins.extend(net)
        net_ptr.append(len(pins))
    cf = np.array([0 if f is None else 1 for f in fixed], np.uint8)
    cfxy = np.array([(0.0, 0.0) if f is None else f for f in fixed], np.float64)
    big = 1.0e7
    return Problem(
        64, 64, [], np.zeros((0, 64 * 64), np.uint32),
        np.zeros((n_units, 2)), np.full((n_units, 2), -big), np.full((n_units, 2), big),
        np.zeros(n_units + 1, np.uint32), [], np.zeros((0, 2)), [], [],
        cell_unit, np.array(offsets, np.float64), cf, cfxy, net_ptr, pins,
        [a[0] for a in arcs], [a[1] for a in arcs], [a[2] for a in arcs])


def wide_net(fanout, critical=None):
    """analytical_placement.rs:828-847: one source and `fanout` sinks."""
    n = fanout + 1
    arcs = [(0, 1, critical - 1)] if critical and critical > 1 else []
    return wa_problem(n, list(range(n)), [list(range(n))], arcs=arcs)


def wa(problem, positions, gamma=GAMMA):
    o = ffi.Oracle(problem)
    c = np.array(positions, np.float64).ravel()
    r = o.evaluate(c, gamma)
    g = r["wa_gradient"].reshape(-1, 2)
    return r["wirelength"], g[:, 0], g[:, 1]


def assert_rel(actual, expected, tol):
    assert abs(actual - expected) <= tol * max(abs(expected), 1.0), (actual, expected)


# :857-870
def test_wirelength_preconditioner_counts_movable_nets_and_timing_weight():
    o = ffi.Oracle(wide_net(3, 7))
    p = o.wirelength_preconditioner()
    assert p[0] == 6.0 + 1.0 / 3.0 and p[1] == 6.0 + 1.0 / 3.0
    assert p[2] == 1.0 / 3.0 and p[3] == 1.0 / 3.0
    # baseline (timing excluded) is exactly 1/fanout per incident net
    assert np.all(ffi.Oracle(wide_net(3)).wirelength_preconditioner() == 1.0 / 3.0)


# :872-882
def test_baseline_preconditioner_is_inverse_fanout():
    assert ffi.Oracle(wide_net(1)).wirelength_preconditioner()[0] == 1.0
    assert ffi.Oracle(wide_net(4)).wirelength_preconditioner()[0] == 0.25
    w = ffi.Oracle(wide_net(4)).cell_incidence_weights()
    assert np.all(w == 0.25)


# :884-900
def test_weighted_average_two_pin_value_matches_closed_form():
    v, gx, gy = wa(wide_net(1), [(0.0, 1.0), (4.0, -2.0)])
    expected = 4.0 * math.tanh(4.0 / (2 * GAMMA)) + 3.0 * math.tanh(3.0 / (2 * GAMMA))
    assert_rel(v, expected, 1e-14)
    assert abs(gx.sum()) <= 1e-14 and abs(gy.sum()) <= 1e-14


# :902-936
def test_weighted_average_multi_pin_objective_is_translation_invariant_and_deterministic():
    pos = np.array([(-3.0, 7.0), (11.0, -2.0), (1.0, 5.0), (4.0, 15.0), (8.0, 0.0)])
    p = wide_net(4)
    first = wa(p, pos)
    repeated = wa(p, pos)
    shifted = wa(p, pos + np.array([1_000_000.0, -2_000_000.0]))
    for a, b, c in zip(first, repeated, shifted):
        assert np.array_equal(a, b) and np.array_equal(a, c)


# :938-988
def test_weighted_average_gradient_matches_finite_differences():
    p = wide_net(3, 7)
    pos = np.array([(0.00, 0.18), (0.08, 0.02), (0.15, 0.11), (0.22, 0.27)])
    _, gx, gy = wa(p, pos)
    step = 1e-6
    for u in range(4):
        for axis, g in ((0, gx), (1, gy)):
            lo, hi = pos.copy(), pos.copy()
            lo[u, axis] -= step
            hi[u, axis] += step
            fd = (wa(p, hi)[0] - wa(p, lo)[0]) / (2 * step)
            assert_rel(g[u], fd, 2e-8)


# :990-1062
def test_weighted_average_uses_fixed_coordinates_and_macro_offsets():
    # cells: root(0) and member(1) in unit 0, fixed sink (2) in unit 1, moving sink (3) in unit 2
    p = wa_problem(3, [0, 0, 1, 2], [[1, 2, 3]],
                   fixed=[None, None, (10.0, 5.0), None],
                   offsets=[(0.0, 0.0), (3.0, -2.0), (0.0, 0.0), (-1.0, 1.0)])
    pos = [(2.0, 4.0), (99.0, 99.0), (7.0, 8.0)]
    v, gx, gy = wa(p, pos)
    ref = wa_problem(3, [0, 1, 2], [[0, 1, 2]], fixed=[None, (10.0, 5.0), None])
    rv, rgx, rgy = wa(ref, [(5.0, 2.0), (0.0, 0.0), (6.0, 9.0)])
    assert_rel(v, rv, 1e-14)
    for u in (0, 2):
        assert_rel(gx[u], rgx[u], 1e-14)
        assert_rel(gy[u], rgy[u], 1e-14)
    assert gx[1] == 0.0 and gy[1] == 0.0
    moved = list(pos)
    moved[1] = (-1000.0, -1000.0)
    v2, gx2, gy2 = wa(p, moved)
    assert v == v2 and np.array_equal(gx, gx2) and np.array_equal(gy, gy2)


# :1106-1183
def test_weighted_average_timing_overlay_is_exactly_sink_local():
    pos = [(0.0, 0.0), (2.0, 1.0), (-1.0, 3.0)]
    base = wa(wide_net(2), pos)
    crit = wa(wide_net(2, 5), pos)
    arc = wa(wide_net(1), pos[:2])
    assert_rel(crit[0] - base[0], 4.0 * arc[0], 1e-14)
    for u in range(2):
        assert_rel(crit[1][u] - base[1][u], 4.0 * arc[1][u], 1e-14)
        assert_rel(crit[2][u] - base[2][u], 4.0 * arc[2][u], 1e-14)
    assert_rel(crit[1][2], base[1][2], 1e-14)
    assert_rel(crit[2][2], base[2][2], 1e-14)


def test_hpwl_is_the_pin_span_sum():
    p = wa_problem(3, [0, 1, 2], [[0, 1, 2], [1, 2]])
    o = ffi.Oracle(p)
    c = np.array([0.0, 0.0, 4.0, 1.0, 2.0, 5.0])
    # net0: x span 4, y span 5; net1: x span 2, y span 4
    assert o.hpwl(c) == 15.0

"""The coarse quadratic seed with macro units and timed arcs (CPU: the
system assembly with the oracle's solve).

`analytical_axis_equations` (lib.rs:4464-4527) places a macro member at its
unit origin plus the member's offset, so an edge between members of two
units pulls the origins apart by the offsets' difference, and an edge to a
fixed unit pulls towards the fixed cell's coordinate minus the own offset.
Pinned by the reference's own case (`analytical_placement_accounts_for_
group_member_offsets`, lib.rs:14975-15003: a two-cell macro on a 9 x 1
device whose far member drives a lone sink ends next to it) and by
stationarity of the B2B objective at the solution, computed from the edges
directly rather than from the assembled system.
"""
import numpy as np

from oracle import ffi
from texo_gb300 import abi, problem as P, seed

from rich_problems import rich_problem


def oracle_solver(d, ptr, idx, w, rhs, x0):
    x, st, ok = ffi.solve_quadratic(d, ptr, idx, w, rhs, x0)
    assert ok
    return x, st


def macro_offsets_case():
    # cells: 0 macro_root, 1 macro_far (3 sites right of the root), 2 sink;
    # net far -> sink; units: the macro (roots 0..5) and the sink (0..8)
    return P.Problem(
        width=9, height=1, fields=[(abi.KIND_LOGIC, 0)], capacity=np.ones(9, np.uint32),
        initial_xy=[4.0, 0.0, 4.0, 0.0], lower_xy=[0.0, 0.0, 0.0, 0.0], upper_xy=[5.0, 0.0, 8.0, 0.0],
        member_ptr=[0, 2, 3], member_field=[0, 0, 0], member_offset_xy=[0.0, 0.0, 3.0, 0.0, 0.0, 0.0],
        member_charge=[1.0, 1.0, 1.0], member_cell=[0, 1, 2],
        cell_unit=[0, 0, 1], cell_offset_xy=[0.0, 0.0, 3.0, 0.0, 0.0, 0.0], cell_fixed=[0, 0, 0],
        cell_fixed_xy=np.zeros(6), net_ptr=[0, 2], pin_cell=[1, 2])


def test_group_member_offsets_known_answer():
    prob = macro_offsets_case()
    center = np.array([[4.0, 0.0], [4.0, 0.0]])
    x, _ = seed.solve_axis(prob, center, 0, 4, solver=oracle_solver)
    y, _ = seed.solve_axis(prob, center, 1, 0, solver=oracle_solver)
    # one floating component {macro, sink}: far member (origin + 3) meets
    # the sink, and the component is centred on the device's middle column
    assert np.allclose(x, [2.5, 5.5], atol=1e-12, rtol=0)
    assert np.allclose(y, [0.0, 0.0], atol=1e-12, rtol=0)
    assert abs((x[0] + 3.0) - x[1]) <= 1e-12


def b2b_gradient(prob, positions, axis, x):
    """Gradient of sum_e w_e ((x_l + o_l) - (x_r + o_r))^2 / 2 over the movable
    units (fixed units at their origins, fixed cells at their coordinates),
    from the edges themselves."""
    l, r, w, lc, rc = seed.b2b_edges(prob, positions, axis, with_cells=True)
    fixed, origin = seed.fixed_units(prob, axis)
    off = np.asarray(prob.cell_offset_xy, dtype=np.float64).reshape(-1, 2)[:, axis]
    fxy = np.asarray(prob.cell_fixed_xy, dtype=np.float64).reshape(-1, 2)[:, axis]
    cfix = np.asarray(prob.cell_fixed, dtype=bool)
    xx = np.where(fixed, origin, x)

    def at(u, c):
        return fxy[c] if cfix[c] else xx[u] + off[c]
    g = np.zeros(len(x))
    scale = np.zeros(len(x))
    for a, b, ww, ca, cb in zip(l, r, w, lc, rc):
        res = at(a, ca) - at(b, cb)
        g[a] += ww * res
        g[b] -= ww * res
        scale[a] += ww * (abs(at(a, ca)) + abs(at(b, cb)))
        scale[b] += ww * (abs(at(a, ca)) + abs(at(b, cb)))
    return np.where(fixed, 0.0, g), np.maximum(scale, 1.0)


def exact_solver(d, ptr, idx, w, rhs, x0):
    from scipy.sparse import csr_matrix, diags
    from scipy.sparse.linalg import spsolve
    A = (diags(d) - csr_matrix((w, idx, ptr), shape=(len(d), len(d)))).tocsc()
    return spsolve(A, rhs), None


def test_seed_is_stationary_with_macros_and_timed_arcs():
    """With an exact sparse solve the assembled system's solution (gauges
    and recentring included) zeroes the edge-wise gradient to rounding; the
    oracle's CG stops by the reference's residual rule, close to it."""
    prob = rich_problem(0)
    assert np.any(np.asarray(prob.cell_offset_xy) != 0) and len(prob.arc_driver_cell) > 0
    pos = np.asarray(prob.initial_xy).reshape(-1, 2)
    for axis, center in ((0, prob.width // 2), (1, prob.height // 2)):
        xe, _ = seed.solve_axis(prob, pos, axis, center, solver=exact_solver)
        g, scale = b2b_gradient(prob, pos, axis, xe)
        assert np.max(np.abs(g) / scale) <= 1e-12, axis
        x, _ = seed.solve_axis(prob, pos, axis, center, solver=oracle_solver)
        assert np.max(np.abs(x - xe)) <= 1e-4 * np.max(np.abs(xe)), axis


def test_timed_arcs_add_overlay_edges():
    prob = rich_problem(0)
    pos = np.asarray(prob.initial_xy).reshape(-1, 2)
    l, r, w, lc, rc = seed.b2b_edges(prob, pos, 0, with_cells=True)
    drv = np.asarray(prob.arc_driver_cell, dtype=np.int64)
    snk = np.asarray(prob.arc_sink_cell, dtype=np.int64)
    cu = np.asarray(prob.cell_unit, dtype=np.int64)
    keep = cu[drv] != cu[snk]
    n = int(keep.sum())
    assert n > 0
    # the overlay edges come last, driver to sink, 64 * extra / separation
    assert np.array_equal(lc[-n:], drv[keep]) and np.array_equal(rc[-n:], snk[keep])
    coord = seed._cell_coordinates(prob, pos, 0)
    sep = np.maximum(np.abs(coord[drv[keep]] - coord[snk[keep]]), 1.0)
    extra = np.asarray(prob.arc_extra_weight, dtype=np.float64)[keep]
    assert np.array_equal(w[-n:], 64.0 * extra / sep)


def test_anchor_pulls_a_free_unit_to_its_incumbent():
    """add_anchor (lib.rs:4410-4415): a unit with no edges but an anchor sits
    on the anchor; the weights follow lib.rs:4094-4105."""
    prob = macro_offsets_case()
    pos = np.array([[4.0, 0.0], [4.0, 0.0]])
    anchor = np.array([[1.0, 0.0], [7.0, 0.0]])
    dx = seed.axis_system(prob, pos, 0)[0]
    dy = seed.axis_system(prob, pos, 1)[0]
    wx, wy = seed.anchor_weights(prob, pos, anchor, 3, dx, dy)
    # distances 3 and 3; diagonals max(d, 1); 0.1 * 3 / 3
    assert np.allclose(wx, np.maximum(dx, 1.0) * 0.1, rtol=0, atol=1e-15)
    assert np.allclose(wy, np.maximum(dy, 1.0) * 0.1, rtol=0, atol=1e-15)
    # the anchored system: no floating component any more, both units pulled
    x, _ = seed.solve_axis(prob, pos, 0, 4, solver=exact_solver, anchors=(wx, anchor[:, 0]))
    d, ptr, idx, w, rhs, _ = seed.axis_system(prob, pos, 0)
    # stationarity of edges + anchors: the gradient of the edge part equals
    # the anchors' pull
    g, _ = b2b_gradient(prob, pos, 0, x)
    assert np.allclose(g + wx * (x - anchor[:, 0]), 0.0, atol=1e-9)
    # an explicit fixed mask overrides the collapsed-bounds rule
    fixed = np.array([True, False])
    f, c = seed.fixed_units(prob, 0, fixed)
    assert list(f) == [True, False] and c[0] == 0.0

"""The coarse quadratic seed of Texo's analytical placer, per axis, on the GPU.

Restates the host side of `solve_analytical_axis` (crates/texo-pnr/src/
lib.rs:4410-4560): the bound-to-bound edges of every net at the current
positions and the timed arcs' overlay edges (`linearize_axis`,
analytical_placement.rs:283-356, with `axis_bounds`, :793-815), the equations
they give with fixed units anchored and macro members at their offsets from
the unit origin (`analytical_axis_equations`, lib.rs:4464-4527), the gauge of
each floating component (`finalize_component_gauges`, lib.rs:4419-4460), and
the recentering after the solve. The solve itself is `texo_gp_quadratic_solve`
(the GPU restatement of `solve_quadratic`, lib.rs:4586-4752).

A unit is fixed when its bounds collapse (lower == upper, the problem's
convention for a unit with one placement choice); its origin is then that
point, and its cells sit at their fixed coordinates.
"""
import numpy as np

from .placer import quadratic_solve

PLACEMENT_WEIGHT_SCALE = 64.0   # analytical_placement.rs:13


def _axis_bounds(units, pos):
    """axis_bounds (analytical_placement.rs:793-815): the lowest pin (first on
    ties) and the highest (last on ties); when they coincide on one unit, the
    last pin of another unit. None when every pin is on one unit."""
    if np.all(units == units[0]):
        return None
    lower = int(np.argmin(pos))
    upper = len(pos) - 1 - int(np.argmax(pos[::-1]))
    if pos[lower] == pos[upper] and units[lower] == units[upper]:
        other = np.nonzero(units != units[lower])[0]
        upper = int(other[-1])
    return lower, upper


def _cell_coordinates(problem, positions, axis):
    fixed = np.asarray(problem.cell_fixed, dtype=bool)
    fixed_xy = np.asarray(problem.cell_fixed_xy, dtype=np.float64).reshape(-1, 2)
    offset_xy = np.asarray(problem.cell_offset_xy, dtype=np.float64).reshape(-1, 2)
    cell_unit = np.asarray(problem.cell_unit, dtype=np.int64)
    pos = np.asarray(positions, dtype=np.float64).reshape(-1, 2)
    return np.where(fixed, fixed_xy[:, axis], pos[cell_unit, axis] + offset_xy[:, axis])


def b2b_edges(problem, positions, axis, with_cells=False):
    """Bound-to-bound edges (left unit, right unit, weight) of every net at
    `positions` ([U, 2] unit origins) along `axis` (0 = x, 1 = y), in the
    reference's order: nets in order, pins in order, lower bound before upper;
    then one edge per timed arc whose driver and sink are on different units
    (weight 64 * extra_weight / separation, analytical_placement.rs:331-352).
    with_cells=True also returns the cells at the two ends."""
    net_ptr = np.asarray(problem.net_ptr, dtype=np.int64)
    pin_cell = np.asarray(problem.pin_cell, dtype=np.int64)
    cell_unit = np.asarray(problem.cell_unit, dtype=np.int64)
    coord = _cell_coordinates(problem, positions, axis)
    left, right, lcell, rcell, weight = [], [], [], [], []
    for e in range(len(net_ptr) - 1):
        cells = pin_cell[net_ptr[e]:net_ptr[e + 1]]
        units = cell_unit[cells]
        p = coord[cells]
        bounds = _axis_bounds(units, p)
        if bounds is None:
            continue
        lo, hi = bounds
        fanout = max(len(cells) - 1, 1)
        for i in range(len(cells)):
            for b in (lo, hi):
                if i == b or (i == hi and b == lo) or units[i] == units[b]:
                    continue
                sep = max(abs(p[i] - p[b]), 1.0)
                left.append(units[i])
                right.append(units[b])
                lcell.append(cells[i])
                rcell.append(cells[b])
                weight.append(PLACEMENT_WEIGHT_SCALE / (fanout * sep))
    drivers = np.asarray(problem.arc_driver_cell, dtype=np.int64).reshape(-1)
    sinks = np.asarray(problem.arc_sink_cell, dtype=np.int64).reshape(-1)
    extra = np.asarray(problem.arc_extra_weight, dtype=np.uint64).reshape(-1)
    for a in range(len(drivers)):
        dc, sc = int(drivers[a]), int(sinks[a])
        if cell_unit[dc] == cell_unit[sc]:
            continue
        sep = max(abs(coord[dc] - coord[sc]), 1.0)
        left.append(cell_unit[dc])
        right.append(cell_unit[sc])
        lcell.append(dc)
        rcell.append(sc)
        weight.append(PLACEMENT_WEIGHT_SCALE * float(extra[a]) / sep)
    out = (np.array(left, np.int64), np.array(right, np.int64), np.array(weight))
    if with_cells:
        return out + (np.array(lcell, np.int64), np.array(rcell, np.int64))
    return out


def fixed_units(problem, axis, fixed=None):
    """(fixed mask [U], origin coordinate along `axis` [U]) of the units;
    `fixed` (optional) overrides the collapsed-bounds rule (the reference's
    rule is one placement choice)."""
    lower = np.asarray(problem.lower_xy, dtype=np.float64).reshape(-1, 2)
    upper = np.asarray(problem.upper_xy, dtype=np.float64).reshape(-1, 2)
    if fixed is None:
        fixed = np.all(lower == upper, axis=1)
    fixed = np.asarray(fixed, dtype=bool)
    return fixed, np.where(fixed, lower[:, axis], 0.0)


def axis_system(problem, positions, axis, fixed=None):
    """(diagonal, adjacency CSR (ptr, index, weight), rhs, anchored) of one
    axis (`analytical_axis_equations`, lib.rs:4464-4527): a fixed unit holds
    its origin; an edge to a fixed unit adds to the diagonal and adds
    weight * (fixed cell's coordinate - own cell's offset) to the right-hand
    side; an edge between movable units adds to both diagonals, to both
    adjacency rows (in edge order) and weight * (other offset - own offset)
    to each right-hand side."""
    U = problem.num_units
    fixed_xy = np.asarray(problem.cell_fixed_xy, dtype=np.float64).reshape(-1, 2)
    offset = np.asarray(problem.cell_offset_xy, dtype=np.float64).reshape(-1, 2)[:, axis]
    unit_fixed, unit_coord = fixed_units(problem, axis, fixed)
    diag = np.where(unit_fixed, 1.0, 0.0)
    rhs = np.where(unit_fixed, unit_coord, 0.0)
    anchored = unit_fixed.copy()
    l, r, w, lc, rc = b2b_edges(problem, positions, axis, with_cells=True)
    rows, cols, ws = [], [], []
    for a, b, x, ca, cb in zip(l.tolist(), r.tolist(), w.tolist(), lc.tolist(), rc.tolist()):
        fa, fb = unit_fixed[a], unit_fixed[b]
        if fa and fb:
            continue
        if fa:
            diag[b] += x
            rhs[b] += x * (fixed_xy[ca, axis] - offset[cb])
            anchored[b] = True
        elif fb:
            diag[a] += x
            rhs[a] += x * (fixed_xy[cb, axis] - offset[ca])
            anchored[a] = True
        else:
            diag[a] += x
            diag[b] += x
            rows += [a, b]
            cols += [b, a]
            ws += [x, x]
            rhs[a] += x * (offset[cb] - offset[ca])
            rhs[b] += x * (offset[ca] - offset[cb])
    rows = np.array(rows, np.int64)
    order = np.argsort(rows, kind="stable")
    ptr = np.zeros(U + 1, np.int64)
    np.add.at(ptr, rows + 1, 1)
    ptr = np.cumsum(ptr)
    return diag, ptr, np.array(cols, np.int64)[order], np.array(ws)[order], rhs, anchored


def finalize_gauges(diag, ptr, index, weight, rhs, anchored):
    """finalize_component_gauges (lib.rs:4419-4460): every connected component
    without an anchored unit loses its smallest unit to a gauge (diagonal 1,
    right-hand side 0, no edges; its neighbours drop the edge from their rows
    and keep it in their diagonals). Returns the new system and the floating
    components (sorted unit lists)."""
    from scipy.sparse import csr_matrix
    from scipy.sparse.csgraph import connected_components
    n = len(diag)
    g = csr_matrix((np.ones(len(index)), index, ptr), shape=(n, n))
    ncomp, label = connected_components(g, directed=False)
    floating = []
    gauge = np.zeros(n, bool)
    has_anchor = np.zeros(ncomp, bool)
    np.logical_or.at(has_anchor, label, anchored)
    for c in np.nonzero(~has_anchor)[0]:
        comp = np.nonzero(label == c)[0]
        gauge[comp[0]] = True
        floating.append(comp)
    diag, rhs = diag.copy(), rhs.copy()
    diag[gauge] = 1.0
    rhs[gauge] = 0.0
    rows = np.repeat(np.arange(n), np.diff(ptr))
    keep = ~gauge[rows] & ~gauge[index]
    new_ptr = np.zeros(n + 1, np.int64)
    np.add.at(new_ptr, rows[keep] + 1, 1)
    return diag, np.cumsum(new_ptr), index[keep], weight[keep], rhs, floating


ANCHOR_ALPHA = 0.1   # lib.rs:4001


def anchor_weights(problem, solved, anchor_xy, iteration, diag_x, diag_y, fixed=None):
    """The incumbent anchors of a timing iteration (lib.rs:4084-4108): for
    every movable unit, weight max(diagonal, 1) * 0.1 * iteration /
    max(distance, 1) per axis, `distance` the Manhattan distance from the
    solved position to the incumbent's tile, `diag_*` the axis systems'
    diagonals before the anchors. Returns (wx, wy) [U], zero for fixed units."""
    fixed, _ = fixed_units(problem, 0, fixed)
    s = np.asarray(solved, dtype=np.float64).reshape(-1, 2)
    a = np.asarray(anchor_xy, dtype=np.float64).reshape(-1, 2)
    dist = np.maximum(np.abs(s[:, 0] - a[:, 0]) + np.abs(s[:, 1] - a[:, 1]), 1.0)
    scale = ANCHOR_ALPHA * float(iteration) / dist
    wx = np.where(fixed, 0.0, np.maximum(diag_x, 1.0) * scale)
    wy = np.where(fixed, 0.0, np.maximum(diag_y, 1.0) * scale)
    return wx, wy


def solve_axis(problem, positions, axis, center, device=0, solver=None, anchors=None, fixed=None):
    """solve_analytical_axis (lib.rs:4531-4560) for one axis: the system at
    `positions`, the gauges, the GPU solve from the current coordinates (each
    floating component shifted so its gauge sits at 0), and each floating
    component recentred on `center`. `solver(diag, ptr, index, weight, rhs,
    x0) -> (x, stats)` replaces the GPU solve (a checker passes its own).
    `anchors` (weights [U], coordinates [U]) are added first (`add_anchor`,
    lib.rs:4410-4415: weight on the diagonal, weight * coordinate on the
    right-hand side, the unit anchored) where the weight is positive.
    `fixed` as in `fixed_units`. Returns (coordinates [U], solve stats)."""
    diag, ptr, index, weight, rhs, anchored = axis_system(problem, positions, axis, fixed)
    if anchors is not None:
        w, c = (np.asarray(v, dtype=np.float64) for v in anchors)
        on = w > 0.0
        diag = diag + np.where(on, w, 0.0)
        rhs = rhs + np.where(on, w * c, 0.0)
        anchored = anchored | on
    diag, ptr, index, weight, rhs, floating = finalize_gauges(diag, ptr, index, weight, rhs, anchored)
    x = np.asarray(positions, dtype=np.float64).reshape(-1, 2)[:, axis].copy()
    for comp in floating:
        x[comp] -= x[comp[0]]
    if solver is None:
        x, stats = quadratic_solve(diag, ptr, index, weight, rhs, x, device=device)
    else:
        x, stats = solver(diag, ptr, index, weight, rhs, x)
    for comp in floating:
        x[comp] += float(center) - x[comp].sum() / len(comp)
    return x, stats

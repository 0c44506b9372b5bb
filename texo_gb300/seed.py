"""The coarse quadratic seed of Texo's analytical placer, per axis, on the GPU.

Restates for single-cell units the host side of `solve_analytical_axis`
(crates/texo-pnr/src/lib.rs:4410-4560): the bound-to-bound edges of every net
at the current positions (`linearize_axis`, analytical_placement.rs:277-352,
with `axis_bounds`, :793-815), the equations they give with fixed units
anchored (`analytical_axis_equations`, lib.rs:4466-4528), the gauge of each
floating component (`finalize_component_gauges`, lib.rs:4419-4460), and the
recentering after the solve. The solve itself is `texo_gp_quadratic_solve`
(the GPU restatement of `solve_quadratic`, lib.rs:4586-4752).
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


def b2b_edges(problem, positions, axis):
    """Bound-to-bound edges (left unit, right unit, weight) of every net at
    `positions` ([U, 2] unit origins) along `axis` (0 = x, 1 = y), in the
    reference's order: nets in order, pins in order, lower bound before upper."""
    net_ptr = np.asarray(problem.net_ptr, dtype=np.int64)
    pin_cell = np.asarray(problem.pin_cell, dtype=np.int64)
    cell_unit = np.asarray(problem.cell_unit, dtype=np.int64)
    fixed = np.asarray(problem.cell_fixed, dtype=bool)
    fixed_xy = np.asarray(problem.cell_fixed_xy, dtype=np.float64).reshape(-1, 2)
    offset_xy = np.asarray(problem.cell_offset_xy, dtype=np.float64).reshape(-1, 2)
    pos = np.asarray(positions, dtype=np.float64).reshape(-1, 2)
    coord = np.where(fixed, fixed_xy[:, axis], pos[cell_unit, axis] + offset_xy[:, axis])
    left, right, weight = [], [], []
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
                weight.append(PLACEMENT_WEIGHT_SCALE / (fanout * sep))
    return np.array(left, np.int64), np.array(right, np.int64), np.array(weight)


def axis_system(problem, positions, axis):
    """(diagonal, adjacency CSR (ptr, index, weight), rhs, anchored) of one
    axis: a fixed unit holds its coordinate; an edge to a fixed unit adds to
    the diagonal and the right-hand side; an edge between movable units adds
    to both diagonals and to both adjacency rows (in edge order)."""
    U = problem.num_units
    cell_unit = np.asarray(problem.cell_unit, dtype=np.int64)
    fixed_cell = np.asarray(problem.cell_fixed, dtype=bool)
    fixed_xy = np.asarray(problem.cell_fixed_xy, dtype=np.float64).reshape(-1, 2)
    unit_fixed = np.zeros(U, bool)
    unit_coord = np.zeros(U)
    unit_fixed[cell_unit[fixed_cell]] = True
    unit_coord[cell_unit[fixed_cell]] = fixed_xy[fixed_cell, axis]
    diag = np.where(unit_fixed, 1.0, 0.0)
    rhs = np.where(unit_fixed, unit_coord, 0.0)
    anchored = unit_fixed.copy()
    l, r, w = b2b_edges(problem, positions, axis)
    rows, cols, ws = [], [], []
    for a, b, x in zip(l.tolist(), r.tolist(), w.tolist()):
        fa, fb = unit_fixed[a], unit_fixed[b]
        if fa and fb:
            continue
        if fa:
            diag[b] += x
            rhs[b] += x * unit_coord[a]
            anchored[b] = True
        elif fb:
            diag[a] += x
            rhs[a] += x * unit_coord[b]
            anchored[a] = True
        else:
            diag[a] += x
            diag[b] += x
            rows += [a, b]
            cols += [b, a]
            ws += [x, x]
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


def solve_axis(problem, positions, axis, center, device=0):
    """solve_analytical_axis (lib.rs:4531-4560) for one axis: the system at
    `positions`, the gauges, the GPU solve from the current coordinates (each
    floating component shifted so its gauge sits at 0), and each floating
    component recentred on `center`. Returns (coordinates [U], solve stats)."""
    diag, ptr, index, weight, rhs, anchored = axis_system(problem, positions, axis)
    diag, ptr, index, weight, rhs, floating = finalize_gauges(diag, ptr, index, weight, rhs, anchored)
    x = np.asarray(positions, dtype=np.float64).reshape(-1, 2)[:, axis].copy()
    for comp in floating:
        x[comp] -= x[comp[0]]
    x, stats = quadratic_solve(diag, ptr, index, weight, rhs, x, device=device)
    for comp in floating:
        x[comp] += float(center) - x[comp].sum() / len(comp)
    return x, stats

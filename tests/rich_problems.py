"""Placement problems that exercise the drop-in features the synthetic
benchmark netlists leave out: two density fields (LUT and register), rigid
two-member macros (LUT + FF on one site, and two-LUT carry chains one site
apart), fixed exchangeable occupancy (BELs held by fixed units), and timed
arcs (sink weights > 1, `analytical_placement.rs:27-32, 547-573`).

Built from a seeded synthetic netlist (its nets and IO are kept; its movable
cells are regrouped into units), so the sizes stay those of the benchmark's
smallest workload (48 x 48 sites, 2,000 movable cells) while every feature
above is present at scale.
"""
import numpy as np

from oracle import ffi
from texo_gb300 import abi, problem as P

KIND_LUT = (abi.KIND_LUT, 4)
KIND_REG = (abi.KIND_REGISTER, 0)


def rich_problem(seed=0, side=48, cells=2000, io=96, nets=2400, sigma=6.0, macro_fraction=0.4,
                 register_fraction=0.35, fixed_fraction=0.04, timed_fraction=0.15, fields=2,
                 timed=True, macros=True, fixed=True, capacity=1):
    base = P.synthetic(side, cells, io, nets, sigma, seed, lib=ffi.lib())
    rng = np.random.default_rng(1000 + seed)
    W = H = side
    nc = base.num_cells
    movable = np.nonzero(base.cell_fixed == 0)[0]
    kinds = [KIND_LUT, KIND_REG][:fields]
    cell_field = np.zeros(nc, np.uint32)
    if fields > 1:
        cell_field[movable] = (rng.random(movable.size) < register_fraction).astype(np.uint32)
    # group movable cells into units: macros of two consecutive cells, else singles
    units = []          # (cells, offsets)
    i = 0
    mv = list(movable)
    while i < len(mv):
        c = mv[i]
        if macros and i + 1 < len(mv) and rng.random() < macro_fraction:
            d = mv[i + 1]
            if cell_field[c] != cell_field[d]:
                units.append(([c, d], [(0.0, 0.0), (0.0, 0.0)]))    # LUT + FF on one site
            else:
                units.append(([c, d], [(0.0, 0.0), (0.0, 1.0)]))    # carry chain: next site up
            i += 2
        else:
            units.append(([c], [(0.0, 0.0)]))
            i += 1
    fixed_cells = np.nonzero(base.cell_fixed != 0)[0]
    cell_unit = np.zeros(nc, np.uint32)
    cell_off = np.zeros((nc, 2))
    initial, lower, upper = [], [], []
    member_ptr, mfield, moff, mq, mcell = [0], [], [], [], []
    for cs, offs in units:
        u = len(initial)
        x0, y0 = base.initial_xy[base.cell_unit[cs[0]]]
        top = max(dy for _, dy in offs)
        initial.append((x0, min(y0, H - 1 - top)))
        lower.append((0.0, 0.0))
        upper.append((float(W - 1), float(H - 1 - top)))
        for c, (dx, dy) in zip(cs, offs):
            cell_unit[c] = u
            cell_off[c] = (dx, dy)
            mfield.append(int(cell_field[c]))
            moff.append((dx, dy))
            mq.append(1.0)
            mcell.append(int(c))
        member_ptr.append(len(mfield))
    for c in fixed_cells:   # fixed IO: units without density members, as in the benchmark netlists
        u = len(initial)
        xy = base.cell_fixed_xy[c]
        initial.append(tuple(xy))
        lower.append(tuple(xy))
        upper.append(tuple(xy))
        cell_unit[c] = u
        member_ptr.append(len(mfield))
    capacity = np.full((fields, W * H), capacity, np.uint32)
    occupancy = []
    if fixed:
        # BELs held by fixed units (exchangeable kinds): a few tiles of each field
        for f in range(fields):
            tiles = rng.choice(W * H, size=int(fixed_fraction * W * H), replace=False)
            for t in tiles:
                occupancy.append((f, int(t % W), int(t // W)))
    arcs_d, arcs_s, arcs_w = [], [], []
    if timed:
        net_ptr = base.net_ptr
        for e in range(base.num_nets):
            if rng.random() < timed_fraction and net_ptr[e + 1] - net_ptr[e] >= 2:
                k = int(rng.integers(net_ptr[e] + 1, net_ptr[e + 1]))
                arcs_d.append(int(base.pin_cell[net_ptr[e]]))
                arcs_s.append(int(base.pin_cell[k]))
                arcs_w.append(int(rng.integers(1, 4)))
    return P.Problem(W, H, kinds, capacity, initial, lower, upper, member_ptr, mfield,
                     np.array(moff).reshape(-1, 2), mq, mcell, cell_unit, cell_off, base.cell_fixed,
                     base.cell_fixed_xy, base.net_ptr, base.pin_cell, arcs_d, arcs_s, arcs_w,
                     fixed_occupancy=np.array(occupancy, np.uint32).reshape(-1, 3))

"""The analytical placement pass around the placement loop, on the GPU.

`analytical_place` (crates/texo-pnr/src/lib.rs:3990-4150) in the order the
reference runs it:

1. the coarse quadratic seed: both axes linearised at the device centre and
   solved (`solve_analytical_axis`, the GPU PCG of texo_gp_quadratic_solve);
2. for a timing iteration with an incumbent placement, the seed again at the
   solved positions with every movable unit anchored towards its incumbent
   tile (lib.rs:4066-4110);
3. the global placement: the seed rounded to tiles (coarse), or
   `eplace::place` from the seed (texo_gp_place, or with a routing-capacity
   map texo_gp_place_routable), best effort or not;
4. `project`: the relaxed projection (texo_gp_project) and its
   transactional repair (texo_gp_repair), a BEL for every cell.

A timing iteration's targets are projected from the incumbent when its BELs
are given (`project_anchored_targets`, lib.rs:4157-4231).
"""
import copy
from dataclasses import dataclass

import numpy as np

from . import abi, legalize, seed
from .placer import default_params, place, place_with_routing_capacity

COARSE = "coarse"
ELECTROSTATIC = "electrostatic"
ELECTROSTATIC_BEST_EFFORT = "electrostatic_best_effort"


@dataclass
class AnalyticalResult:
    seed_xy: np.ndarray        # [U, 2] solved seed positions (unit origins)
    targets: np.ndarray        # [U, 2] rounded tile targets handed to project
    preferred: np.ndarray      # [U] the projection's row per unit (-1: left to the repair)
    info: dict
    bels: np.ndarray = None    # [cells] the legal BEL of every cell (after the repair)


def _rounded(values, extent):
    t = np.trunc(values)
    r = t + np.where(np.abs(values - t) >= 0.5, np.sign(values), 0.0)
    return np.clip(np.where(np.isnan(r), 0.0, r), 0, extent - 1).astype(np.uint32)


def analytical_place(problem, units, bel_xy, mode=ELECTROSTATIC, params=None, anchor=None,
                     routing_capacity=None, register_controls=None, device=0):
    """One analytical placement pass. `problem` and `units` describe the same
    placement units (texo_gb300.ecp5.placement_problem builds both from a
    device snapshot); `bel_xy` [B, 2] the BEL tiles. `anchor`: (incumbent
    unit tiles [U, 2], timing iteration[, incumbent BEL of every cell]); with
    the BELs the targets are projected from the incumbent
    (`project_anchored_targets`), else afresh. `routing_capacity`: (horizontal,
    vertical) [H, W] channel capacities for the routability rounds."""
    W, H = problem.width, problem.height
    cx, cy = W // 2, H // 2
    U = problem.num_units
    if len(units) != U:
        raise ValueError("one placement unit per problem unit")
    bel_xy = np.asarray(bel_xy, dtype=np.float64).reshape(-1, 2)
    # the seed's view of the units: fixed where a unit has one choice, else
    # free within its choices' bounds (eplace's problem collapses the units
    # without density members, which the seed still moves)
    fixed = np.array([len(u.choices) == 1 for u in units], dtype=bool)
    lo = np.zeros((U, 2))
    hi = np.zeros((U, 2))
    bounds = {}
    for i, u in enumerate(units):
        key = id(u.choices)
        if key not in bounds:
            first = bel_xy[[a[0] for a in u.choices]]
            bounds[key] = (first.min(axis=0), first.max(axis=0))
        lo[i], hi[i] = bounds[key]
    seed_problem = copy.copy(problem)
    seed_problem.lower_xy = np.ascontiguousarray(lo)
    seed_problem.upper_xy = np.ascontiguousarray(hi)
    centre = np.where(fixed[:, None], lo, np.array([float(cx), float(cy)]))
    info = {"mode": mode}
    x, sx = seed.solve_axis(seed_problem, centre, 0, cx, device=device, fixed=fixed)
    y, sy = seed.solve_axis(seed_problem, centre, 1, cy, device=device, fixed=fixed)
    info["seed"] = {"x_iterations": sx["iterations"], "y_iterations": sy["iterations"]}
    solved = np.stack([x, y], 1)
    if anchor is not None:
        anchor_xy, iteration = anchor[0], anchor[1]
        dx = seed.axis_system(seed_problem, solved, 0, fixed)[0]
        dy = seed.axis_system(seed_problem, solved, 1, fixed)[0]
        wx, wy = seed.anchor_weights(seed_problem, solved, anchor_xy, iteration, dx, dy, fixed)
        a = np.asarray(anchor_xy, dtype=np.float64).reshape(-1, 2)
        x, _ = seed.solve_axis(seed_problem, solved, 0, cx, device=device, anchors=(wx, a[:, 0]), fixed=fixed)
        y, _ = seed.solve_axis(seed_problem, solved, 1, cy, device=device, anchors=(wy, a[:, 1]), fixed=fixed)
        solved = np.stack([x, y], 1)
        info["anchored"] = True
    if mode == COARSE or anchor is not None:
        targets = np.stack([_rounded(solved[:, 0], W), _rounded(solved[:, 1], H)], 1)
    else:
        prm = params or default_params()
        prm.best_effort = 1 if mode == ELECTROSTATIC_BEST_EFFORT else int(prm.best_effort)
        # eplace::place starts from the seed, clamped to each unit's bounds;
        # units without density members keep their seed coordinate
        plo = np.asarray(problem.lower_xy, dtype=np.float64).reshape(-1, 2)
        phi = np.asarray(problem.upper_xy, dtype=np.float64).reshape(-1, 2)
        still = np.all(plo == phi, axis=1) & ~fixed
        start = np.where(fixed[:, None], lo, np.clip(solved, plo, phi))
        start[still] = solved[still]
        gp = copy.copy(problem)
        gp.initial_xy = np.ascontiguousarray(start)
        gp.lower_xy = np.ascontiguousarray(np.where(still[:, None], solved, plo))
        gp.upper_xy = np.ascontiguousarray(np.where(still[:, None], solved, phi))
        if routing_capacity is None:
            targets, _, st = place(gp, prm)
        else:
            ch, cv = routing_capacity
            targets, _, st, rep = place_with_routing_capacity(gp, prm, ch, cv, register_controls)
            info["routable"] = rep
        info["placement"] = {"iterations": st["iterations"], "converged": st["converged"], "hpwl": st["hpwl"],
                             "overflow": st["overflow"]}
    if anchor is not None and len(anchor) > 2:
        # a timing iteration with the incumbent's cell BELs: project from it
        bels = legalize.project_anchored(W, H, bel_xy.astype(np.int64), units, targets, anchor[2])
        pos = {}
        preferred = np.full(U, -1, dtype=np.int64)
        for i, u in enumerate(units):
            key = id(u.choices)
            if key not in pos:
                pos[key] = {tuple(int(b) for b in a): c for c, a in enumerate(u.choices)}
            preferred[i] = pos[key][tuple(int(b) for b in bels[u.cells])]
        info["project"] = {"anchored": True}
        return AnalyticalResult(solved, np.asarray(targets, np.uint32).reshape(-1, 2), preferred, info,
                                np.asarray(bels, np.int64))
    proj = legalize.project(W, H, bel_xy, units, targets)
    info["project"] = proj.stats
    placed, info["repair"] = legalize.repair(W, H, bel_xy, units, targets, proj.preferred, fixed)
    return AnalyticalResult(solved, np.asarray(targets, np.uint32).reshape(-1, 2), proj.preferred, info, placed)

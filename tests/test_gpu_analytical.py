"""The analytical placement pass (`analytical_place`, lib.rs:3990-4150) on
the GPU over an ECP5-like fabric: the seed's two axis solves against the same
steps with the oracle's solve, and each mode (coarse, electrostatic, an
anchored timing iteration) through `project` to legal choices."""
import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi, analytical as A, ecp5, seed

pytestmark = pytest.mark.gpu


def fabric(seed_no=0, side=16):
    arch = ecp5.read_architecture(ecp5.synthetic_architecture(side, side))
    nc, units, kinds, nets = ecp5.synthetic_design(arch, seed_no, luts=500, ffs=250, lut_ff_pairs=150,
                                                   carry=((12, 4), (6, 6)), io=24)
    prob, _ = ecp5.placement_problem(arch, nc, units, nets, cell_kind=kinds)
    return arch, prob, units


def oracle_solver(d, ptr, idx, w, rhs, x0):
    x, st, ok = ffi.solve_quadratic(d, ptr, idx, w, rhs, x0)
    assert ok
    return x, st


def legal(res, units):
    bels = np.full(1 + max(c for u in units for c in u.cells), -1)
    for i, u in enumerate(units):
        if res.preferred[i] >= 0:
            bels[u.cells] = u.choices[res.preferred[i]]
    placed = bels[bels >= 0]
    return len(np.unique(placed)) == len(placed)


@pytest.mark.parametrize("mode", [A.COARSE, A.ELECTROSTATIC, A.ELECTROSTATIC_BEST_EFFORT])
def test_modes_reach_legal_choices(mode):
    arch, prob, units = fabric()
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    res = A.analytical_place(prob, units, bel_xy, mode=mode)
    assert np.all(res.preferred >= 0) and legal(res, units)
    # the repair keeps a complete, legal projection
    expected = np.full(len(res.bels), -1)
    for i, u in enumerate(units):
        expected[u.cells] = u.choices[res.preferred[i]]
    assert np.array_equal(res.bels, expected) and res.info["repair"]["initial_pending"] == 0
    if mode != A.COARSE:
        assert res.info["placement"]["converged"]


def test_seed_matches_the_oracle_path():
    arch, prob, units = fabric(1)
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    res = A.analytical_place(prob, units, bel_xy, mode=A.COARSE)
    # the same seed with the oracle's solve
    fixed = np.array([len(u.choices) == 1 for u in units])
    import copy
    sp = copy.copy(prob)
    lo = np.array([bel_xy[[a[0] for a in u.choices]].min(axis=0) for u in units], np.float64)
    hi = np.array([bel_xy[[a[0] for a in u.choices]].max(axis=0) for u in units], np.float64)
    sp.lower_xy, sp.upper_xy = lo, hi
    cx, cy = prob.width // 2, prob.height // 2
    centre = np.where(fixed[:, None], lo, np.array([float(cx), float(cy)]))
    x, _ = seed.solve_axis(sp, centre, 0, cx, solver=oracle_solver, fixed=fixed)
    y, _ = seed.solve_axis(sp, centre, 1, cy, solver=oracle_solver, fixed=fixed)
    ref = np.stack([x, y], 1)
    assert np.max(np.abs(res.seed_xy - ref)) <= 1e-8 * np.max(np.abs(ref))


def test_anchored_iteration_moves_towards_the_incumbent():
    arch, prob, units = fabric(2)
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    first = A.analytical_place(prob, units, bel_xy, mode=A.ELECTROSTATIC)
    incumbent = np.array([bel_xy[u.choices[c][0]] for u, c in zip(units, first.preferred)], np.float64)
    free = np.array([len(u.choices) > 1 for u in units])
    d0 = np.abs(first.seed_xy - incumbent).sum(axis=1)[free].sum()
    res = A.analytical_place(prob, units, bel_xy, anchor=(incumbent, 4))
    d1 = np.abs(res.seed_xy - incumbent).sum(axis=1)[free].sum()
    assert res.info.get("anchored") and d1 < d0
    assert np.all(res.preferred >= 0) and legal(res, units)


def test_anchored_iteration_projects_from_the_incumbent():
    arch, prob, units = fabric(3)
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    first = A.analytical_place(prob, units, bel_xy, mode=A.ELECTROSTATIC)
    bels = np.full(1 + max(c for u in units for c in u.cells), -1)
    for i, u in enumerate(units):
        bels[u.cells] = u.choices[first.preferred[i]]
    incumbent = np.array([bel_xy[bels[u.cells[0]]] for u in units], np.float64)
    res = A.analytical_place(prob, units, bel_xy, anchor=(incumbent, 4, bels))
    assert res.info["project"] == {"anchored": True}
    assert np.all(res.preferred >= 0) and legal(res, units)
    # a unit whose new target is its incumbent tile keeps its choice
    for i, u in enumerate(units):
        if len(u.choices) > 1 and np.array_equal(res.targets[i], incumbent[i].astype(np.uint32)):
            assert res.preferred[i] == first.preferred[i]


@pytest.mark.parametrize("engine", [abi.ENGINE_HOST, abi.ENGINE_DEVICE])
def test_routable_pass_ends_on_legal_bels(engine):
    """The whole pass with a routing-capacity map on either engine: the seed,
    the area rounds (RUDY, register clustering with the registers' control
    sets, instance areas), `project` and its repair with the control sets as
    shared-resource rules: a legal BEL for every cell."""
    from texo_gb300 import legalize
    from texo_gb300.placer import default_params
    arch, prob, units = fabric(4)
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    kinds = [None] * (1 + max(c for u in units for c in u.cells))
    for u in units:
        for c, b in zip(u.cells, u.choices[0]):
            kinds[c] = arch.bel_kind[b]
    sets = ecp5.synthetic_control_sets(kinds, seed=2)
    controls = {c: (clk, lsr, ce) for c, ce, clk, lsr in sets}
    cap = np.full((arch.height, arch.width), 8, np.uint32)
    res = A.analytical_place(prob, units, bel_xy, mode=A.ELECTROSTATIC,
                             params=default_params(best_effort=1, engine=engine),
                             routing_capacity=(cap, cap), register_controls=controls)
    assert res.info["routable"]["rounds"] >= 1
    placed = res.bels
    assert np.all(placed >= 0) and len(np.unique(placed)) == len(placed)
    # the control sets, checked on the repair's output with them as rules
    rules = ecp5.ff_control_set_rules(arch, sets)
    fixed = [len(u.choices) == 1 for u in units]
    legal_bels, _ = legalize.repair(arch.width, arch.height, bel_xy, units, res.targets, res.preferred, fixed,
                                    legalize.Legality(rules=rules))
    for cell_values, bel_res in rules:
        seen = {}
        for c, v in cell_values.items():
            assert seen.setdefault(bel_res[int(legal_bels[c])], v) == v

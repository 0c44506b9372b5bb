"""`project` up to its repair (legalization/mod.rs:322-389) with the oracle's
auctions: fixed units, shared-row families (disjoint ones auctioned,
overlapping ones seeded nearest-first), singletons, on the reference's
device fixture and on a seeded ECP5-like fabric.

The composition is host code shared by both auction backends; the oracle's
FIFO auction is the reference's, its parallel-round form the GPU's. Checked:
the known answer on the fixture (worked by hand from the rules), every
placed unit on free BELs with no BEL used twice, each family auction a
maximum matching whose reduced costs pass the epsilon-complementary-slackness
certificate, the overlapping seeding equal to a brute-force nearest free
row, and the parallel-round form within the reference's cost bound of the
FIFO's."""
import json
import os

import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi, ecp5, legalize as L

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "minimal_ecp5.json")


def oracle_auction(jacobi):
    def run(grid, kinds, targets, scale):
        code, a, _, st = ffi.auction_singletons(grid, kinds, targets, cost_scale=max(int(scale), 1), jacobi=jacobi)
        assert code == 0, code
        return a, st
    return run


def test_known_answer_on_the_fixture():
    with open(FIXTURE) as f:
        arch = ecp5.read_architecture(json.load(f))
    luts = ecp5.single_cell_choices(arch, ecp5.LUT4)
    units = [L.Unit([0, 1], ecp5.carry_chain_assignments(arch, 1)),
             L.Unit([2, 3], ecp5.lut_ff_assignments(arch)),
             L.Unit([4], luts, False),
             L.Unit([5], [[4]], False),
             L.Unit([6], [[7]], False)]
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    targets = [[0, 0]] * 5
    for jacobi in (False, True):
        pj = L.project(arch.width, arch.height, bel_xy, units, targets, cost_scale=1,
                       auction=oracle_auction(jacobi))
        # carry before LUT-FF (same scarcity and size, lower first cell):
        # carry takes BELs 0-1; LUT-FF's first row needs BEL 0, so it takes
        # row 1 (BELs 8, 10) at distance 1; the lone LUT takes BEL 2, the
        # lowest free COMB on the target tile
        assert list(pj.preferred) == [0, 1, 2, 0, 0]
        assert list(pj.bels(units)) == [0, 1, 8, 10, 2, 4, 7]
        assert pj.stats["disjoint_shared_families"] == 2 and pj.stats["fixed_units"] == 2


def test_fixed_conflict_is_an_error():
    units = [L.Unit([0], [[3]], False), L.Unit([1], [[3]], False)]
    with pytest.raises(L.ProjectionError):
        L.project(2, 2, [[0, 0], [1, 0], [0, 1], [1, 1]], units, [[0, 0], [0, 0]], auction=oracle_auction(False))


def fabric_case(seed=0, side=16):
    arch = ecp5.read_architecture(ecp5.synthetic_architecture(side, side))
    nc, units, kinds, nets = ecp5.synthetic_design(arch, seed, luts=500, ffs=250, lut_ff_pairs=150,
                                                   carry=((12, 4), (6, 6)), io=24)
    prob, _ = ecp5.placement_problem(arch, nc, units, nets, cell_kind=kinds)
    prm = abi.default_params_py()
    prm.best_effort = 1
    st, targets, _, _ = ffi.Oracle(prob, prm).place(threads=4)
    assert st == 0
    return arch, units, targets


def brute_nearest(unit, targets_u, occupied, bel_xy):
    best = None
    for c, a in enumerate(unit.choices):
        if occupied[np.asarray(a)].any():
            continue
        x, y = bel_xy[a[0]]
        key = (abs(int(x) - int(targets_u[0])) + abs(int(y) - int(targets_u[1])), (int(x), int(y)), c)
        best = key if best is None or key < best else best
    return None if best is None else best[2]


@pytest.mark.parametrize("seed", [0, 1])
def test_projection_on_a_fabric(seed):
    arch, units, targets = fabric_case(seed)
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    res = {}
    for name, jacobi in (("fifo", False), ("jacobi", True)):
        pj = L.project(arch.width, arch.height, bel_xy, units, targets, cost_scale=1, auction=oracle_auction(jacobi))
        bels = pj.bels(units)
        placed = bels[bels >= 0]
        assert len(np.unique(placed)) == len(placed)                 # no BEL twice
        assert pj.stats["relaxed_unmatched_units"] == 0 and np.all(pj.preferred >= 0)
        assert pj.stats["overlapping_shared_units"] == 6 and pj.stats["disjoint_shared_families"] == 2
        for u, unit in enumerate(units):                              # the choice is one of the unit's
            assert list(bels[unit.cells]) == list(unit.choices[pj.preferred[u]])
        res[name] = (pj, bels)
    # the parallel rounds meet the reference's bound: total base cost within
    # n (the bidder count, s = 1) of the FIFO's on every auctioned cohort
    cost = {}
    for name, (pj, _) in res.items():
        d = 0
        for u, unit in enumerate(units):
            if len(unit.choices) > 1:
                x, y = bel_xy[unit.choices[pj.preferred[u]][0]]
                d += abs(int(x) - int(targets[u][0])) + abs(int(y) - int(targets[u][1]))
        cost[name] = d
    n = sum(1 for u in units if len(u.choices) > 1)
    assert abs(cost["jacobi"] - cost["fifo"]) <= n


def test_overlapping_seeding_is_nearest_free_row():
    arch, units, targets = fabric_case(0)
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    pj = L.project(arch.width, arch.height, bel_xy, units, targets, cost_scale=1, auction=oracle_auction(False))
    # replay: fixed units, then the overlapping units in the seeding order
    occupied = np.zeros(len(bel_xy), bool)
    for unit in units:
        if len(unit.choices) == 1:
            occupied[np.asarray(unit.choices[0])] = True
    over = [u for u, unit in enumerate(units) if unit.is_shared() and len(unit.choices) > 1
            and len(unit.cells) == 12]
    over.sort(key=lambda u: (len(units[u].choices), -len(units[u].cells), units[u].cells[0]))
    for u in over:
        c = brute_nearest(units[u], targets[u], occupied, bel_xy)
        assert pj.preferred[u] == c
        occupied[np.asarray(units[u].choices[c])] = True


def grid_bels(w, h, per_tile=1):
    """BEL tiles of a w x h grid with `per_tile` BELs a tile, row-major."""
    return np.array([(x, y) for y in range(h) for x in range(w) for _ in range(per_tile)], np.int64)


@pytest.mark.parametrize("jacobi", [False, True])
def test_capacity_shortage_leaves_units_unmatched(jacobi):
    # 6 singleton units for 4 BELs: two go unmatched (the repair's), the rest
    # on distinct BELs
    bel_xy = grid_bels(2, 2)
    table = [[b] for b in range(4)]
    units = [L.Unit([u], table, False) for u in range(6)]
    pj = L.project(2, 2, bel_xy, units, [[0, 0]] * 6, cost_scale=1, auction=oracle_auction(jacobi))
    assert pj.stats["relaxed_unmatched_units"] == 2 and int(np.sum(pj.preferred < 0)) == 2
    placed = [table[c][0] for c in pj.preferred if c >= 0]
    assert sorted(placed) == [0, 1, 2, 3]


def test_family_rows_blocked_by_fixed_units():
    # a disjoint family of two-BEL rows whose every row touches a fixed BEL
    bel_xy = grid_bels(4, 1, 2)           # BELs 2x, 2x+1 on tile x
    rows = [[0, 1], [2, 3], [4, 5], [6, 7]]
    units = [L.Unit([0], [[1]], False), L.Unit([1], [[2]], False), L.Unit([2], [[5]], False),
             L.Unit([3], [[7]], False), L.Unit([4, 5], rows), L.Unit([6, 7], rows)]
    pj = L.project(4, 1, bel_xy, units, [[0, 0]] * 6, cost_scale=1, auction=oracle_auction(False))
    assert list(pj.preferred[:4]) == [0, 0, 0, 0]
    assert list(pj.preferred[4:]) == [-1, -1] and pj.stats["relaxed_unmatched_units"] == 2


def test_overlapping_seed_skips_a_blocked_row():
    # overlapping rows (sliding windows of two tiles); the nearest row to the
    # target holds a fixed BEL, so the unit takes the next ring's least point
    bel_xy = grid_bels(5, 1)
    rows = [[x, x + 1] for x in range(4)]     # rows overlap: BEL x+1 in two rows
    units = [L.Unit([0], [[2]], False), L.Unit([1, 2], rows)]
    pj = L.project(5, 1, bel_xy, units, [[0, 0], [2, 0]], cost_scale=1, auction=oracle_auction(False))
    # rows at x = 1 and 2 use BEL 2; at distance 1 from x = 2: rows 1 (blocked) and 3
    assert pj.preferred[1] == 3 and pj.stats["overlapping_shared_units"] == 1


def test_singletons_of_several_candidate_tables():
    # two kinds of singleton with their own candidate tables on one grid, one
    # auction: every unit on a BEL of its own table
    bel_xy = grid_bels(3, 3, 2)
    lut = [[b] for b in range(0, 18, 2)]
    ff = [[b] for b in range(1, 18, 2)]
    units = [L.Unit([u], lut if u % 2 else ff, False) for u in range(12)]
    targets = [[1, 1]] * 12
    for jacobi in (False, True):
        pj = L.project(3, 3, bel_xy, units, targets, cost_scale=1, auction=oracle_auction(jacobi))
        bels = pj.bels(units)
        assert np.all(bels >= 0) and len(set(bels.tolist())) == 12
        assert all((b % 2 == 0) == (u % 2 == 1) for u, b in enumerate(bels))


# ---- the reference's own projection tests (legalization/mod.rs:1205-1377) ----

def reference_case(coordinates, candidate_sets, targets):
    """projection_problem (mod.rs:1205-1241): Logic BELs on a one-row device
    at the given x, one single-cell unit per candidate set (its own table),
    targets on row 0."""
    width = max(coordinates) + 1
    bel_xy = np.array([(x, 0) for x in coordinates], np.int64)
    units = [L.Unit([c], [[b] for b in cands], False) for c, cands in enumerate(candidate_sets)]
    return width, 1, bel_xy, units, [[t, 0] for t in targets]


REFERENCE_CASES = [
    # singleton_projection_avoids_far_greedy_spill (:1272-1279)
    (([0, 1, 100], [[0, 1, 2], [0, 2]], [0, 0]), [1, 0]),
    # singleton_projection_avoids_false_no_bel_behind_fixed_owner (:1281-1291)
    (([0, 1, 100], [[0, 1], [0, 2], [2]], [0, 0, 100]), [1, 0, 2]),
    # projection_reaches_candidate_after_legacy_sixty_four_limit (:1302-1311)
    (([0] * 66, [[i] for i in range(65)] + [list(range(66))], [0] * 66), list(range(66))),
]


@pytest.mark.parametrize("case,expected", REFERENCE_CASES)
def test_reference_projection_cases(case, expected):
    w, h, bel_xy, units, targets = reference_case(*case)
    for jacobi in (False, True):
        pj = L.project(w, h, bel_xy, units, targets, cost_scale=1, auction=oracle_auction(jacobi))
        assert list(pj.bels(units)) == expected


def test_reference_four_real_bels_at_one_point():
    # projection_uses_four_real_bels_at_one_point (:1293-1300)
    w, h, bel_xy, units, targets = reference_case([0, 0, 0, 0], [[0, 1, 2, 3]] * 4, [0, 0, 0, 0])
    for jacobi in (False, True):
        pj = L.project(w, h, bel_xy, units, targets, cost_scale=1, auction=oracle_auction(jacobi))
        assert len(set(pj.bels(units).tolist())) == 4


def test_reference_composite_rows():
    # composite_slot_classification_requires_disjoint_complete_rows (:1313-1329)
    assert L._rows_disjoint([[0, 1], [2, 3]]) and not L._rows_disjoint([[0, 1], [1, 2]])
    # disjoint_composite_rows_remain_atomic_before_singleton_projection (:1331-1377)
    bel_xy = np.array([(0, 0), (0, 0), (1, 0), (1, 0), (2, 0)], np.int64)
    rows = [[0, 1], [2, 3]]
    units = [L.Unit([0, 1], rows), L.Unit([2, 3], rows), L.Unit([4], [[1], [4]], False)]
    for jacobi in (False, True):
        pj = L.project(3, 1, bel_xy, units, [[0, 0]] * 3, cost_scale=1, auction=oracle_auction(jacobi))
        bels = pj.bels(units)
        assert len(set(bels.tolist())) == 5 and bels[4] == 4
        for unit in units[:2]:
            assert list(bels[unit.cells]) in rows


def test_anchored_projection_keeps_or_improves_each_unit():
    """project_anchored_targets (lib.rs:4157-4231): a unit already on its
    target tile keeps its BELs; one whose target moved takes the first free
    choice strictly closer to the target in ring order; farther units go
    first."""
    bel_xy = grid_bels(6, 1)                  # one BEL a tile on a 6 x 1 row
    table = [[b] for b in range(6)]
    units = [L.Unit([0], table, False), L.Unit([1], table, False), L.Unit([2], [[5]], False)]
    incumbent = np.array([0, 1, 5])
    # unit 0: target 3 (distance 3): ring 0 at 3 is free -> BEL 3
    # unit 1: target 1 (distance 0): stays on BEL 1
    bels = L.project_anchored(6, 1, bel_xy, units, [[3, 0], [1, 0], [5, 0]], incumbent)
    assert list(bels) == [3, 1, 5]
    # both target tile 4 (unit 0 from 0 at distance 4, unit 1 from 1 at 3):
    # unit 0 goes first and takes BEL 4; unit 1 then finds 3 (distance 1 < 3)
    bels = L.project_anchored(6, 1, bel_xy, units, [[4, 0], [4, 0], [5, 0]], incumbent)
    assert list(bels) == [4, 3, 5]
    # a target past a fixed BEL with nothing free closer: the incumbent stays
    units2 = [L.Unit([0], [[0], [5]], False), L.Unit([1], [[5]], False)]
    bels = L.project_anchored(6, 1, bel_xy, units2, [[5, 0], [5, 0]], np.array([0, 5]))
    assert list(bels) == [0, 5]

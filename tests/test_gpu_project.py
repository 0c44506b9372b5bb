"""`project` with the GPU auctions on the adapter's ECP5-like fabric: the
same choices as with the oracle's parallel-round auctions (the GPU matches
that restatement bit for bit), and the whole path from the device snapshot
(adapter -> placement -> projection) on the GPU."""
import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi, ecp5, legalize as L
from texo_gb300.placer import default_params, place

from test_project import fabric_case, oracle_auction

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed,scale", [(0, 1), (1, 1), (0, 4)])
def test_gpu_projection_equals_the_parallel_restatement(seed, scale):
    arch, units, targets = fabric_case(seed)
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    g = L.project(arch.width, arch.height, bel_xy, units, targets, cost_scale=scale)
    o = L.project(arch.width, arch.height, bel_xy, units, targets, cost_scale=scale, auction=oracle_auction(True))
    assert np.array_equal(g.preferred, o.preferred)
    assert g.stats["bids"] == o.stats["bids"]
    assert np.all(g.preferred >= 0)


def test_device_snapshot_to_legal_choices_on_the_gpu():
    arch = ecp5.read_architecture(ecp5.synthetic_architecture(24, 24))
    nc, units, kinds, nets = ecp5.synthetic_design(arch, 3, luts=1200, ffs=600, lut_ff_pairs=400,
                                                   carry=((30, 4), (10, 6)), io=40)
    prob, _ = ecp5.placement_problem(arch, nc, units, nets, cell_kind=kinds)
    targets, _, st = place(prob, default_params(best_effort=1))
    prm = abi.default_params_py()
    prm.best_effort = 1
    _, _, _, rs = ffi.Oracle(prob, prm).place(threads=4)
    assert st["converged"] and abs(st["hpwl"] - rs.hpwl) <= 0.01 * rs.hpwl
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    pj = L.project(arch.width, arch.height, bel_xy, units, targets)
    bels = pj.bels(units)
    assert np.all(pj.preferred >= 0) and np.all(bels >= 0)
    assert len(np.unique(bels)) == len(bels)
    for u, unit in enumerate(units):
        assert list(bels[unit.cells]) == list(unit.choices[pj.preferred[u]])


def test_gpu_edge_cases_equal_the_parallel_restatement():
    """Capacity shortage (unmatched units), rows blocked by fixed BELs,
    several candidate tables in one singleton auction: the GPU composition
    gives the oracle's parallel-round composition's choices."""
    from test_project import grid_bels
    cases = []
    table = [[b] for b in range(4)]
    cases.append((2, 2, grid_bels(2, 2), [L.Unit([u], table, False) for u in range(6)], [[0, 0]] * 6))
    rows = [[0, 1], [2, 3], [4, 5], [6, 7]]
    cases.append((4, 1, grid_bels(4, 1, 2), [L.Unit([0], [[1]], False), L.Unit([1], [[2]], False),
                                             L.Unit([2, 3], rows), L.Unit([4, 5], rows), L.Unit([6, 7], rows)],
                  [[0, 0]] * 5))
    lut = [[b] for b in range(0, 18, 2)]
    ff = [[b] for b in range(1, 18, 2)]
    cases.append((3, 3, grid_bels(3, 3, 2), [L.Unit([u], lut if u % 2 else ff, False) for u in range(12)],
                  [[1, 1]] * 12))
    for w, h, bel_xy, units, targets in cases:
        g = L.project(w, h, bel_xy, units, targets, cost_scale=1)
        o = L.project(w, h, bel_xy, units, targets, cost_scale=1, auction=oracle_auction(True))
        assert np.array_equal(g.preferred, o.preferred), (w, h)
        assert g.stats["relaxed_unmatched_units"] == o.stats["relaxed_unmatched_units"]
        # the automatic scale: same unmatched count, no BEL twice
        a = L.project(w, h, bel_xy, units, targets)
        bels = a.bels(units)
        assert a.stats["relaxed_unmatched_units"] == o.stats["relaxed_unmatched_units"]
        assert len(np.unique(bels[bels >= 0])) == int(np.sum(bels >= 0))


def test_native_projection_equals_the_python_composition_with_gpu_auctions():
    """texo_gp_project (the composition in native code) against the same
    steps driven from Python with the same GPU auctions: identical choices
    and statistics."""
    arch, units, targets = fabric_case(1)
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    for scale in (0, 1):
        n = L.project(arch.width, arch.height, bel_xy, units, targets, cost_scale=scale)
        p = L.project(arch.width, arch.height, bel_xy, units, targets, cost_scale=scale, auction=L.gpu_auction)
        assert np.array_equal(n.preferred, p.preferred)
        for key in ("fixed_units", "overlapping_shared_units", "disjoint_shared_families", "singleton_units",
                    "relaxed_unmatched_units", "bids", "candidates_examined"):
            assert n.stats[key] == p.stats[key], key


def test_native_projection_conflict_is_an_error():
    units = [L.Unit([0], [[3]], False), L.Unit([1], [[3]], False)]
    with pytest.raises(L.ProjectionError):
        L.project(2, 2, [[0, 0], [1, 0], [0, 1], [1, 1]], units, [[0, 0], [0, 0]])


def test_reference_projection_cases_on_the_gpu():
    """The reference's own projection tests (legalization/mod.rs:1272-1377)
    through texo_gp_project: overlapping candidate tables (kinds that share
    BELs), a fixed owner, the candidate past the legacy 64 limit, four BELs
    at one point, disjoint composite rows before the singletons."""
    from test_project import REFERENCE_CASES, reference_case
    for case, expected in REFERENCE_CASES:
        w, h, bel_xy, units, targets = reference_case(*case)
        for scale in (0, 1):
            pj = L.project(w, h, bel_xy, units, targets, cost_scale=scale)
            assert list(pj.bels(units)) == expected, (case, scale)
    w, h, bel_xy, units, targets = reference_case([0, 0, 0, 0], [[0, 1, 2, 3]] * 4, [0, 0, 0, 0])
    assert len(set(L.project(w, h, bel_xy, units, targets).bels(units).tolist())) == 4
    bel_xy = np.array([(0, 0), (0, 0), (1, 0), (1, 0), (2, 0)], np.int64)
    rows = [[0, 1], [2, 3]]
    units = [L.Unit([0, 1], rows), L.Unit([2, 3], rows), L.Unit([4], [[1], [4]], False)]
    bels = L.project(3, 1, bel_xy, units, [[0, 0]] * 3).bels(units)
    assert len(set(bels.tolist())) == 5 and bels[4] == 4


def test_projection_at_scale_equals_the_parallel_restatement():
    """A 64 x 64-tile ECP5-like fabric (27,744 LUT and 27,744 FF BELs), 15,000
    singletons, 2,000 LUT-FF pairs, 160 carry chains of 4 and 40 of 6 pairs,
    at the oracle placement's targets: the native composition with the GPU
    auctions gives the choices of the Python composition with the oracle's
    parallel rounds, bit for bit, at the reference's scale and the automatic
    one."""
    arch = ecp5.read_architecture(ecp5.synthetic_architecture(64, 64))
    nc, units, kinds, nets = ecp5.synthetic_design(arch, 5, luts=10000, ffs=5000, lut_ff_pairs=2000,
                                                   carry=((160, 4), (40, 6)), io=100)
    prob, _ = ecp5.placement_problem(arch, nc, units, nets, cell_kind=kinds)
    prm = abi.default_params_py()
    prm.best_effort = 1
    st, targets, _, _ = ffi.Oracle(prob, prm).place(threads=8)
    assert st == 0
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    g = L.project(arch.width, arch.height, bel_xy, units, targets, cost_scale=1)
    o = L.project(arch.width, arch.height, bel_xy, units, targets, cost_scale=1, auction=oracle_auction(True))
    assert np.array_equal(g.preferred, o.preferred) and np.all(g.preferred >= 0)
    assert g.stats["bids"] == o.stats["bids"]
    a = L.project(arch.width, arch.height, bel_xy, units, targets)
    bels = a.bels(units)
    assert np.all(bels >= 0) and len(np.unique(bels)) == len(bels)


def test_project_and_repair_on_the_gpu():
    """The whole `project` (GPU auctions, then the transactional repair) on
    the 24 x 24 fabric: every cell on a BEL of its unit's rows, no BEL twice,
    and the repair keeps the projection where it was already legal; with
    more units than BELs of a kind, the repair's NoBel."""
    arch = ecp5.read_architecture(ecp5.synthetic_architecture(24, 24))
    nc, units, kinds, nets = ecp5.synthetic_design(arch, 3, luts=1200, ffs=600, lut_ff_pairs=400,
                                                   carry=((30, 4), (10, 6)), io=40)
    prob, _ = ecp5.placement_problem(arch, nc, units, nets, cell_kind=kinds)
    targets, _, st = place(prob, default_params(best_effort=1))
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    placed, ps, rs = L.project_and_repair(arch.width, arch.height, bel_xy, units, targets)
    assert np.all(placed >= 0) and len(np.unique(placed)) == len(placed)
    for unit in units:
        assert list(placed[unit.cells]) in [list(r) for r in unit.choices]
    pj = L.project(arch.width, arch.height, bel_xy, units, targets)
    assert np.array_equal(placed, pj.bels(units)) and rs["initial_pending"] == 0
    # with the registers' control sets as shared resources the repair
    # separates what the occupancy-only projection put together
    rules = ecp5.ff_control_set_rules(arch, ecp5.synthetic_control_sets(kinds, seed=4))
    placed, _, rs = L.project_and_repair(arch.width, arch.height, bel_xy, units, targets,
                                         legality=L.Legality(rules=rules))
    assert rs["initial_pending"] > 0 and np.all(placed >= 0) and len(np.unique(placed)) == len(placed)
    for cell_values, bel_res in rules:
        seen = {}
        for c, v in cell_values.items():
            assert seen.setdefault(bel_res[int(placed[c])], v) == v
    # more LUT singletons than the 8 LUT BELs of a 3 x 3 fabric
    small = ecp5.read_architecture(ecp5.synthetic_architecture(3, 3))
    luts = ecp5.single_cell_choices(small, ecp5.LUT4)
    assert len(luts) == 8
    many = [L.Unit([c], luts, False) for c in range(len(luts) + 1)]
    sxy = np.stack([small.bel_x, small.bel_y], 1)
    with pytest.raises(L.NoBelError):
        L.project_and_repair(small.width, small.height, sxy, many, [[0, 0]] * len(many))

"""The auction oracle against the reference's own auction tests
(crates/texo-pnr/src/legalization/auction.rs:341-505), the exact optimum of
small grid problems, and its epsilon-optimality certificate; plus the host
layout helpers of texo_gb300.legalize. CPU only."""
import numpy as np
import pytest

from auction_cases import (KNOWN_ANSWERS, brute_force, domains_of, exhaustive_families, grid_optimum, quality,
                           random_grid, sixty_six_domains)
from oracle import ffi
from texo_gb300 import abi, legalize

AUCTION = abi.CODE


@pytest.mark.parametrize("name,domains,objects,max_cost,expected", KNOWN_ANSWERS, ids=[k[0] for k in KNOWN_ANSWERS])
def test_known_answers(name, domains, objects, max_cost, expected):
    code, a, _, st = ffi.auction_explicit(domains, objects, max_cost)
    assert code == 0
    assert list(a) == expected
    assert st["unmatched"] == 0


def test_candidate_after_sixty_four_remains_visible():
    first = ffi.auction_explicit(sixty_six_domains(), 66, 0)
    second = ffi.auction_explicit(sixty_six_domains(), 66, 0)
    assert first[0] == 0
    assert list(first[1]) == list(second[1]) and first[3] == second[3]
    assert first[3]["unmatched"] == 0 and first[1][65] == 65


def test_dummy_reports_maximum_cardinality_deficiency():
    code, a, _, st = ffi.auction_explicit([[(0, 0)], [(0, 0)]], 1, 0)
    assert code == 0
    assert (a >= 0).sum() == 1 and st["unmatched"] == 1


def test_price_range_exhaustion_is_reported_before_bidding():
    code, *_ = ffi.auction_explicit([[]], 0, 2 ** 64 - 1)
    assert code == AUCTION["AUCTION_RANGE"]


def test_exhaustive_small_graphs_have_exact_cardinality_and_bounded_cost():
    cases = 0
    for nb, no, max_cost, costs in exhaustive_families():
        unmatched, optimum = brute_force(costs)
        got = np.full((len(costs), nb), -1)
        for i in range(len(costs)):
            code, a, _, _ = ffi.auction_explicit(domains_of(costs[i]), no, max_cost)
            assert code == 0
            got[i] = a
        q_unmatched, q_cost = quality(costs, got)
        assert np.array_equal(q_unmatched, unmatched), (nb, no)
        assert np.all(q_cost <= optimum + nb), (nb, no)
        cases += len(costs)
    assert cases == 91205


def test_malformed_domains():
    assert ffi.auction_explicit([[(3, 0)]], 2, 0)[0] == AUCTION["AUCTION_OBJECT_RANGE"]
    assert ffi.auction_explicit([[(0, 5)]], 1, 4)[0] == AUCTION["AUCTION_COST_RANGE"]
    assert ffi.auction_explicit([[(0, 0), (1, 0), (0, 1)]], 2, 1)[0] == AUCTION["AUCTION_DUPLICATE_OBJECT"]
    # the same object in two bidders' domains is the normal case
    assert ffi.auction_explicit([[(0, 0)], [(0, 0), (1, 1)]], 2, 1)[0] == 0


GRIDS = [   # (width, height, kinds, max BELs a tile, bidders, occupied fraction)
    (12, 10, 1, 1, 100, 0.0),
    (16, 16, 2, 2, 300, 0.1),
    (20, 8, 3, 3, 250, 0.2),
    (9, 9, 1, 1, 120, 0.3),    # more bidders than free BELs
    (1, 1, 1, 3, 5, 0.0),      # one tile
    (25, 1, 1, 1, 20, 0.0),    # one row
]


@pytest.mark.parametrize("seed,shape", list(enumerate(GRIDS)))
def test_singletons_match_the_optimum_and_certify(seed, shape):
    w, h, k, cap, n, occ = shape
    grid, kind, xy = random_grid(seed, w, h, k, cap, n, occ)
    code, a, prices, st = ffi.auction_singletons(grid, kind, xy)
    assert code == 0
    unmatched, optimum = grid_optimum(grid, kind, xy)
    assert st["unmatched"] == unmatched
    assert optimum <= st["total_base_cost"] <= optimum + n
    bad, first, base = ffi.auction_certificate(grid, kind, xy, a, prices.astype(np.uint32))
    assert bad == 0, first
    assert int(base.sum()) == st["total_base_cost"]


@pytest.mark.parametrize("scale", [2, 4, 8])
def test_scaled_costs_tighten_the_bound(scale):
    """With base costs times s (the reference's cost_scale) the result stays
    of maximum cardinality and within n / s of the optimum."""
    for seed, shape in enumerate(GRIDS[:4]):
        w, h, k, cap, n, occ = shape
        grid, kind, xy = random_grid(seed, w, h, k, cap, n, occ)
        code, a, prices, st = ffi.auction_singletons(grid, kind, xy, cost_scale=scale)
        assert code == 0
        unmatched, optimum = grid_optimum(grid, kind, xy)
        assert st["unmatched"] == unmatched
        assert optimum <= st["total_base_cost"] <= optimum + n / scale
        bad, first, _ = ffi.auction_certificate(grid, kind, xy, a, prices.astype(np.uint32), cost_scale=scale)
        assert bad == 0, first
    for nb, no, max_cost, costs in list(exhaustive_families())[:12]:
        unmatched, optimum = brute_force(costs)
        got = np.array([ffi.auction_explicit(domains_of(c), no, max_cost, scale)[1] for c in costs])
        got = got.reshape(len(costs), nb)
        q_unmatched, q_cost = quality(costs, got)
        assert np.array_equal(q_unmatched, unmatched) and np.all(q_cost <= optimum + nb / scale)


@pytest.mark.parametrize("scale", [1, 8])
def test_parallel_rounds_keep_the_guarantees(scale):
    """The restatement of the GPU's parallel rounds: maximum cardinality,
    cost within n / s of the optimum and a clean certificate, like the
    one-at-a-time auction."""
    for seed, shape in enumerate(GRIDS):
        w, h, k, cap, n, occ = shape
        grid, kind, xy = random_grid(seed, w, h, k, cap, n, occ)
        code, a, prices, st = ffi.auction_singletons(grid, kind, xy, cost_scale=scale, jacobi=True)
        assert code == 0 and st["rounds"] >= 1
        unmatched, optimum = grid_optimum(grid, kind, xy)
        assert st["unmatched"] == unmatched
        assert optimum <= st["total_base_cost"] <= optimum + n / scale
        bad, first, _ = ffi.auction_certificate(grid, kind, xy, a, prices.astype(np.uint32), cost_scale=scale)
        assert bad == 0, first
    for nb, no, max_cost, costs in exhaustive_families():
        unmatched, optimum = brute_force(costs[:512])
        got = np.array([ffi.auction_explicit(domains_of(c), no, max_cost, scale, jacobi=True)[1]
                        for c in costs[:512]]).reshape(-1, nb)
        q_unmatched, q_cost = quality(costs[:512], got)
        assert np.array_equal(q_unmatched, unmatched) and np.all(q_cost <= optimum + nb / scale)
    code, a, _, st = ffi.auction_explicit(KNOWN_ANSWERS[0][1], 3, 100, 1, jacobi=True)
    assert code == 0 and list(a) == KNOWN_ANSWERS[0][4]


def test_certificate_catches_planted_mistakes():
    grid, kind, xy = random_grid(7, 14, 12, 1, 1, 120, 0.0)
    code, a, prices, _ = ffi.auction_singletons(grid, kind, xy)
    assert code == 0
    p = prices.astype(np.uint32)
    held = set(int(o) for o in a if o >= 0)
    free = [o for o in range(grid.num_objects) if o not in held]
    # two bidders on one BEL
    twice = a.copy()
    twice[1] = twice[0]
    assert ffi.auction_certificate(grid, kind, xy, twice, p)[0] > 0
    # an unheld BEL with a price
    priced = p.copy()
    priced[free[0]] = 1
    assert ffi.auction_certificate(grid, kind, xy, a, priced)[0] > 0
    # a bidder moved to the free BEL farthest from its target
    where = grid.bel_tiles()
    far = max(free, key=lambda o: abs(where[o, 1] - int(xy[0, 0])) + abs(where[o, 2] - int(xy[0, 1])))
    moved = a.copy()
    moved[0] = far
    assert ffi.auction_certificate(grid, kind, xy, moved, p)[0] > 0


def test_singleton_edge_cases():
    grid = legalize.site_grid(np.ones((1, 4, 4), dtype=np.int64))
    # no bidders
    code, a, _, st = ffi.auction_singletons(grid, np.zeros(0, np.uint32), np.zeros((0, 2), np.uint32))
    assert code == 0 and len(a) == 0 and st["bids"] == 0
    # every BEL occupied: all unmatched
    full = legalize.site_grid(np.ones((1, 4, 4), dtype=np.int64), occupied=np.ones(16, np.uint8))
    code, a, _, st = ffi.auction_singletons(full, np.zeros(3, np.uint32), np.zeros((3, 2), np.uint32))
    assert code == 0 and list(a) == [-1, -1, -1] and st["unmatched"] == 3
    # one free BEL in the far corner: the walk reaches the last ring
    occ = np.ones(16, np.uint8)
    occ[15] = 0
    corner = legalize.site_grid(np.ones((1, 4, 4), dtype=np.int64), occupied=occ)
    code, a, _, st = ffi.auction_singletons(corner, np.zeros(1, np.uint32), np.zeros((1, 2), np.uint32))
    assert code == 0 and list(a) == [15] and st["total_base_cost"] == 6
    # a kind with no BELs: unmatched
    two = legalize.site_grid(np.stack([np.ones((4, 4)), np.zeros((4, 4))]).astype(np.int64))
    code, a, _, st = ffi.auction_singletons(two, np.array([1, 0], np.uint32), np.array([[0, 0], [3, 3]], np.uint32))
    assert code == 0 and a[0] == -1 and a[1] == 15


def test_singleton_malformed_inputs():
    grid = legalize.site_grid(np.ones((1, 3, 3), dtype=np.int64))
    bad_target = ffi.auction_singletons(grid, np.zeros(1, np.uint32), np.array([[3, 0]], np.uint32))
    assert bad_target[0] == AUCTION["INVALID_ARGUMENT"]
    bad_kind = ffi.auction_singletons(grid, np.array([1], np.uint32), np.array([[0, 0]], np.uint32))
    assert bad_kind[0] == AUCTION["INVALID_ARGUMENT"]
    twice = legalize.SiteGrid(3, 3, 1, grid.tile_ptr, np.array([0, 1, 2, 3, 4, 5, 6, 7, 7], np.uint32), 9)
    assert ffi.auction_singletons(twice, np.zeros(1, np.uint32), np.zeros((1, 2), np.uint32))[0] == \
        AUCTION["AUCTION_DUPLICATE_OBJECT"]
    outside = legalize.SiteGrid(3, 3, 1, grid.tile_ptr, np.arange(9, dtype=np.uint32), 8)
    assert ffi.auction_singletons(outside, np.zeros(1, np.uint32), np.zeros((1, 2), np.uint32))[0] == \
        AUCTION["AUCTION_OBJECT_RANGE"]


def test_site_grid_layout():
    cap = np.array([[[1, 0, 2], [0, 3, 1]], [[0, 1, 0], [2, 0, 0]]])   # [kind, y, x]
    g = legalize.site_grid(cap)
    assert (g.width, g.height, g.num_kinds, g.num_objects) == (3, 2, 2, 10)
    assert list(g.tile_ptr) == [0, 1, 1, 3, 3, 6, 7, 7, 8, 8, 10, 10, 10]
    where = g.bel_tiles()
    assert where[0].tolist() == [0, 0, 0]
    assert where[3].tolist() == [0, 1, 1] and where[5].tolist() == [0, 1, 1]
    assert where[7].tolist() == [1, 1, 0]
    assert where[9].tolist() == [1, 0, 1]


def test_fixed_occupancy_mask():
    cap = np.array([[[1, 2], [0, 3]], [[1, 1], [1, 1]]])   # [field, y, x]
    g = legalize.site_grid(cap)
    # field 0: tile (1,0) holds BELs 1-2, tile (1,1) BELs 3-5; field 1: BELs 6-9
    occ = legalize.fixed_occupancy_mask(g, [[0, 1, 1], [0, 1, 1], [1, 0, 0], [0, 1, 0]])
    assert np.nonzero(occ)[0].tolist() == [1, 3, 4, 6]
    assert not legalize.fixed_occupancy_mask(g, np.zeros((0, 3))).any()
    with pytest.raises(abi.TexoGpError) as e:
        legalize.fixed_occupancy_mask(g, [[0, 0, 1], [0, 0, 1]])   # tile (0,1) of field 0 has no BEL
    assert e.value.code == abi.CODE["FIXED_CAPACITY_EXHAUSTED"]
    with pytest.raises(abi.TexoGpError):
        legalize.fixed_occupancy_mask(g, [[0, 2, 0]])

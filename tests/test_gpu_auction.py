"""The GPU capacity auction (texo_gp_auction_explicit / _singletons) against
the reference's own auction tests (crates/texo-pnr/src/legalization/
auction.rs:341-505), the exact optimum of small grid problems, the oracle's
one-bidder-at-a-time auction and the epsilon-optimality certificate, up to
the 42k-cell placement's own targets."""
import numpy as np
import pytest

from auction_cases import (KNOWN_ANSWERS, brute_force, exhaustive_families, grid_optimum, quality, random_grid,
                           sixty_six_domains)
from oracle import ffi
from texo_gb300 import abi, legalize

pytestmark = pytest.mark.gpu


def expected_scale(grid, kind):
    """The automatic scale: 4 unless some kind has more bidders than free
    BELs, or a kind with bidders more than two BELs a tile on average."""
    where = grid.bel_tiles()
    free = np.ones(grid.num_objects, bool) if grid.occupied is None else grid.occupied == 0
    tiles = grid.width * grid.height
    counts = np.diff(np.asarray(grid.tile_ptr, dtype=np.int64))
    for q in range(grid.num_kinds):
        nq = (np.asarray(kind) == q).sum()
        if nq > (free & (where[:, 0] == q)).sum():
            return 1
        c = counts[q * tiles:(q + 1) * tiles]
        if nq and c.sum() > 2 * np.count_nonzero(c):
            return 1
    return 4


def _raises(code, fn, *args):
    with pytest.raises(abi.TexoGpError) as e:
        fn(*args)
    assert e.value.code == abi.CODE[code]


@pytest.mark.parametrize("scale", [1, 0])
@pytest.mark.parametrize("name,domains,objects,max_cost,expected", KNOWN_ANSWERS, ids=[k[0] for k in KNOWN_ANSWERS])
def test_known_answers(name, domains, objects, max_cost, expected, scale):
    r = legalize.assign_implicitly(domains, objects, max_cost, cost_scale=scale)
    assert r.as_options() == expected
    assert r.stats["unmatched"] == 0 and r.stats["kernel_launches"] == 1
    assert r.stats["cost_scale"] == 1   # explicit domains: the reference's scale unless asked


def test_sixty_six_and_deficiency_and_range():
    a = legalize.assign_implicitly(sixty_six_domains(), 66, 0)
    b = legalize.assign_implicitly(sixty_six_domains(), 66, 0)
    assert np.array_equal(a.assignment, b.assignment) and np.array_equal(a.prices, b.prices)
    assert a.stats["unmatched"] == 0 and a.assignment[65] == 65
    d = legalize.assign_implicitly([[(0, 0)], [(0, 0)]], 1, 0)
    assert (d.assignment >= 0).sum() == 1 and d.stats["unmatched"] == 1
    _raises("AUCTION_RANGE", legalize.assign_implicitly, [[]], 0, 2 ** 64 - 1)
    # the device keeps prices in 32 bits: n (max + 1) + max + 2 must stay below 2^32
    _raises("AUCTION_RANGE", legalize.assign_implicitly, [[(0, 0)]] * 3, 1, 2 ** 31)
    assert legalize.assign_implicitly([[]], 0, 0).as_options() == [None]
    assert legalize.assign_implicitly([], 0, 0).as_options() == []


def test_malformed_domains_match_the_oracle():
    for domains, m, mx, code in [([[(3, 0)]], 2, 0, "AUCTION_OBJECT_RANGE"),
                                 ([[(0, 5)]], 1, 4, "AUCTION_COST_RANGE"),
                                 ([[(0, 0), (1, 0), (0, 1)]], 2, 1, "AUCTION_DUPLICATE_OBJECT")]:
        assert ffi.auction_explicit(domains, m, mx)[0] == abi.CODE[code]
        _raises(code, legalize.assign_implicitly, domains, m, mx)


@pytest.mark.parametrize("scale", [1, 2])
def test_exhaustive_small_graphs_in_one_launch_each_family(scale):
    """Every case of the reference's exhaustive families, as disjoint
    components of one auction per chunk of 2048 cases: each component keeps
    the maximum cardinality and the cost bound (its bidders' ε-slackness
    holds component by component). The dummy cost grows with the bidders of
    the whole launch, and so do the price wars of the components with more
    bidders than objects: hence the chunks."""
    total = 0
    for nb, no, max_cost, all_costs in exhaustive_families():
        for start in range(0, len(all_costs), 2048):
            costs = all_costs[start:start + 2048]
            cases = len(costs)
            unmatched, optimum = brute_force(costs)
            domains = []
            for i in range(cases):
                for b in range(nb):
                    domains.append([(i * no + o, int(c)) for o, c in enumerate(costs[i, b]) if c >= 0])
            r = legalize.assign_implicitly(domains, cases * no, max_cost, cost_scale=scale)
            s = r.stats["cost_scale"]
            assert s == scale
            a = r.assignment.reshape(cases, nb).astype(np.int64)
            local = np.where(a >= 0, a - np.arange(cases)[:, None] * no, -1)
            assert np.all((a < 0) | ((local >= 0) & (local < max(no, 1)))), "an object of another case"
            q_unmatched, q_cost = quality(costs, local)
            assert np.array_equal(q_unmatched, unmatched), (nb, no)
            assert np.all(q_cost <= optimum + nb / s), (nb, no)
            total += cases
    assert total == 91205


GRIDS = [   # (width, height, kinds, max BELs a tile, bidders, occupied fraction)
    (12, 10, 1, 1, 100, 0.0),
    (16, 16, 2, 2, 300, 0.1),
    (20, 8, 3, 3, 250, 0.2),
    (9, 9, 1, 1, 120, 0.3),
    (1, 1, 1, 3, 5, 0.0),
    (25, 1, 1, 1, 20, 0.0),
    (40, 40, 1, 1, 1500, 0.0),
]


@pytest.mark.parametrize("scale", [1, 0])
@pytest.mark.parametrize("seed,shape", list(enumerate(GRIDS)))
def test_singletons_against_optimum_oracle_and_certificate(seed, shape, scale):
    w, h, k, cap, n, occ = shape
    grid, kind, xy = random_grid(seed, w, h, k, cap, n, occ)
    r = legalize.auction_singletons(grid, kind, xy, cost_scale=scale)
    s = r.stats["cost_scale"]
    assert s == (scale or expected_scale(grid, kind))
    unmatched, optimum = grid_optimum(grid, kind, xy)
    assert r.stats["unmatched"] == unmatched
    assert optimum <= r.stats["total_base_cost"] <= optimum + n / s
    bad, first, base = ffi.auction_certificate(grid, kind, xy, r.assignment, r.prices, cost_scale=s)
    assert bad == 0, first
    assert int(base.sum()) == r.stats["total_base_cost"]
    code, oa, _, ost = ffi.auction_singletons(grid, kind, xy, cost_scale=s)
    assert code == 0 and ost["unmatched"] == r.stats["unmatched"]
    assert abs(ost["total_base_cost"] - r.stats["total_base_cost"]) <= n / s
    again = legalize.auction_singletons(grid, kind, xy, cost_scale=scale)
    assert np.array_equal(again.assignment, r.assignment) and np.array_equal(again.prices, r.prices)
    assert again.stats["rounds"] == r.stats["rounds"] and again.stats["bids"] == r.stats["bids"]


@pytest.mark.parametrize("scale", [1, 8])
@pytest.mark.parametrize("seed,shape", list(enumerate(GRIDS)))
def test_singletons_bit_exact_against_the_parallel_restatement(seed, shape, scale):
    """The oracle's restatement of the GPU's parallel rounds (the same ring
    walk and bid rule, every active bidder bidding at the round's prices)
    gives the same assignment, prices, rounds and bids bit for bit."""
    w, h, k, cap, n, occ = shape
    grid, kind, xy = random_grid(seed, w, h, k, cap, n, occ)
    r = legalize.auction_singletons(grid, kind, xy, cost_scale=scale)
    code, a, prices, st = ffi.auction_singletons(grid, kind, xy, cost_scale=scale, jacobi=True)
    assert code == 0
    assert np.array_equal(r.assignment, a)
    assert np.array_equal(r.prices.astype(np.uint64), prices)
    assert (r.stats["rounds"], r.stats["bids"]) == (st["rounds"], st["bids"])
    assert (r.stats["unmatched"], r.stats["total_base_cost"]) == (st["unmatched"], st["total_base_cost"])


def test_explicit_bit_exact_against_the_parallel_restatement():
    for nb, no, max_cost, all_costs in exhaustive_families():
        costs = all_costs[:2048]
        domains = [[(i * no + o, int(c)) for o, c in enumerate(costs[i, b]) if c >= 0]
                   for i in range(len(costs)) for b in range(nb)]
        for scale in (1, 2):
            r = legalize.assign_implicitly(domains, len(costs) * no, max_cost, cost_scale=scale)
            code, a, prices, st = ffi.auction_explicit(domains, len(costs) * no, max_cost, scale, jacobi=True)
            assert code == 0
            assert np.array_equal(r.assignment, a) and np.array_equal(r.prices.astype(np.uint64), prices)
            assert (r.stats["rounds"], r.stats["bids"]) == (st["rounds"], st["bids"])


def test_singleton_edge_cases():
    ones = np.ones((1, 4, 4), dtype=np.int64)
    grid = legalize.site_grid(ones)
    r = legalize.auction_singletons(grid, np.zeros(0, np.uint32), np.zeros((0, 2), np.uint32))
    assert len(r.assignment) == 0
    full = legalize.site_grid(ones, occupied=np.ones(16, np.uint8))
    r = legalize.auction_singletons(full, np.zeros(3, np.uint32), np.zeros((3, 2), np.uint32))
    assert r.as_options() == [None, None, None] and r.stats["unmatched"] == 3
    occ = np.ones(16, np.uint8)
    occ[15] = 0
    corner = legalize.site_grid(ones, occupied=occ)
    r = legalize.auction_singletons(corner, np.zeros(1, np.uint32), np.zeros((1, 2), np.uint32))
    assert r.as_options() == [15] and r.stats["total_base_cost"] == 6
    two = legalize.site_grid(np.stack([np.ones((4, 4)), np.zeros((4, 4))]).astype(np.int64))
    r = legalize.auction_singletons(two, np.array([1, 0], np.uint32), np.array([[0, 0], [3, 3]], np.uint32))
    assert r.as_options() == [None, 15]
    _raises("INVALID_ARGUMENT", legalize.auction_singletons, grid, np.zeros(1, np.uint32),
            np.array([[4, 0]], np.uint32))
    twice = legalize.SiteGrid(4, 4, 1, grid.tile_ptr, np.r_[np.arange(15), 14].astype(np.uint32), 16)
    _raises("AUCTION_DUPLICATE_OBJECT", legalize.auction_singletons, twice, np.zeros(1, np.uint32),
            np.zeros((1, 2), np.uint32))


def test_singletons_on_the_42k_placement():
    """The 42k-cell placement's rounded targets bid for the 210 x 210 LUT
    sites: everyone is placed, the certificate holds, and the matched cost
    is within the bidder count of the oracle's one-at-a-time auction."""
    from texo_gb300 import problem as P
    from texo_gb300.placer import Placer, default_params
    prob = P.synthetic(210, 42000, 365, 50000, 12.0, 0)
    params = default_params(bins_x=256, bins_y=256, target_density=0.9, gamma_base=4.0, max_iterations=1000,
                            best_effort=1, engine=abi.ENGINE_DEVICE, dct_mode=abi.DCT_FP32)
    with Placer(prob, params) as g:
        targets, _, stats = g.run(allow_nonconverged=True)
    movable = np.nonzero(np.any(prob.lower_xy != prob.upper_xy, axis=1))[0]
    n = len(movable)
    assert n == 42000
    grid = legalize.site_grid(prob.capacity[0].reshape(1, prob.height, prob.width))
    kind = np.zeros(n, np.uint32)
    xy = np.ascontiguousarray(targets[movable])
    code, _, _, ost = ffi.auction_singletons(grid, kind, xy)   # the reference's setting, one bidder at a time
    assert code == 0 and ost["unmatched"] == 0
    for scale in (1, 0):
        r = legalize.auction_singletons(grid, kind, xy, cost_scale=scale)
        s = r.stats["cost_scale"]
        assert r.stats["unmatched"] == 0
        assert len(set(r.assignment.tolist())) == n
        bad, first, base = ffi.auction_certificate(grid, kind, xy, r.assignment, r.prices, cost_scale=s)
        assert bad == 0, first
        assert int(base.sum()) == r.stats["total_base_cost"]
        assert abs(ost["total_base_cost"] - r.stats["total_base_cost"]) <= n
        # bit for bit the oracle's restatement of the parallel rounds
        code, ja, jp, jst = ffi.auction_singletons(grid, kind, xy, cost_scale=s, jacobi=True)
        assert code == 0 and np.array_equal(r.assignment, ja) and np.array_equal(r.prices.astype(np.uint64), jp)
        assert (r.stats["rounds"], r.stats["bids"]) == (jst["rounds"], jst["bids"])
    # the default (scaled) result moves the units less than the reference's setting does
    assert r.stats["cost_scale"] == 4 and r.stats["total_base_cost"] <= ost["total_base_cost"]


def test_project_singletons_on_a_problem_with_fixed_bels():
    """From a placement problem and its targets to one BEL per unit: fixed
    units' BELs are never handed out, every movable single-cell unit of the
    48 x 48 workload gets a distinct LUT site, certified."""
    from texo_gb300 import problem as P
    from texo_gb300.placer import Placer, default_params
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 0)
    with Placer(prob, default_params(best_effort=1, max_iterations=1000, engine=abi.ENGINE_DEVICE)) as g:
        targets, _, _ = g.run(allow_nonconverged=True)
    bel, r, multi = legalize.project_singletons(prob, targets)
    movable = np.any(prob.lower_xy != prob.upper_xy, axis=1)
    assert len(multi) == 0 and r.stats["unmatched"] == 0
    assert np.all(bel[movable] >= 0) and np.all(bel[~movable] == -1)
    assert len(set(bel[movable].tolist())) == int(movable.sum())
    # the same problem with some LUT sites held by fixed units
    rng = np.random.default_rng(3)
    taken = rng.choice(48 * 48, 200, replace=False)
    fixed = np.stack([np.zeros(200, np.int64), taken % 48, taken // 48], axis=1)
    prob.fixed_occupancy = np.ascontiguousarray(fixed.astype(np.uint32))
    bel2, r2, _ = legalize.project_singletons(prob, targets)
    assert r2.stats["unmatched"] == 0
    assert not set(bel2[movable].tolist()) & set(taken.tolist())   # BEL id = site index for one BEL a site


def test_singletons_bit_exact_at_one_million_cells():
    """Full size: the 1M-cell workload's placement targets (host engine) bid
    for the 1024 x 1024 sites; at the automatic scale (2: the largest whose
    prices fit 32 bits) and at the reference's, the GPU's assignment, prices,
    rounds and bids equal the parallel restatement's, the certificate holds,
    and the matched cost is within n / s of the one-at-a-time auction's."""
    from texo_gb300 import problem as P
    from texo_gb300.placer import Placer, default_params
    prob = P.synthetic(1024, 1000000, 4096, 1200000, 24.0, 0)
    params = default_params(bins_x=1024, bins_y=1024, target_density=0.9, gamma_base=4.0, max_iterations=1000,
                            best_effort=1, engine=abi.ENGINE_HOST, dct_mode=abi.DCT_FP32)
    with Placer(prob, params) as g:
        targets, _, _ = g.run(allow_nonconverged=True)
    bel, r, multi = legalize.project_singletons(prob, targets)
    assert len(multi) == 0 and r.stats["unmatched"] == 0 and r.stats["cost_scale"] == 2
    movable = np.nonzero(np.any(prob.lower_xy != prob.upper_xy, axis=1))[0]
    grid = legalize.site_grid(prob.capacity[0].reshape(1, prob.height, prob.width))
    kind = np.zeros(len(movable), np.uint32)
    xy = np.ascontiguousarray(targets[movable])
    for scale in (2, 1):
        g = r if scale == 2 else legalize.auction_singletons(grid, kind, xy, cost_scale=1)
        code, a, prices, st = ffi.auction_singletons(grid, kind, xy, cost_scale=scale, jacobi=True)
        assert code == 0
        assert np.array_equal(g.assignment, a) and np.array_equal(g.prices.astype(np.uint64), prices)
        assert (g.stats["rounds"], g.stats["bids"]) == (st["rounds"], st["bids"])
        bad, first, _ = ffi.auction_certificate(grid, kind, xy, g.assignment, g.prices, cost_scale=scale)
        assert bad == 0, first
        code, _, _, fifo = ffi.auction_singletons(grid, kind, xy, cost_scale=scale)
        assert code == 0 and fifo["unmatched"] == 0
        assert abs(fifo["total_base_cost"] - g.stats["total_base_cost"]) <= len(movable) / scale


def test_kinds_sharing_bels_bit_exact_against_the_parallel_restatement():
    """Kinds may list the same BEL (the distinct candidate tables of
    SingleCell units): one price per BEL, bidders of both kinds compete; the
    automatic scale falls back to 1."""
    rng = np.random.default_rng(11)
    w, h = 10, 10
    tiles = w * h
    # kind 0: every BEL; kind 1: the BELs of the left half; kind 2: a random third
    lists = [list(range(tiles)), [t for t in range(tiles) if t % w < w // 2],
             sorted(rng.choice(tiles, tiles // 3, replace=False).tolist())]
    ptr = [0]
    obj = []
    for q in range(3):
        members = set(lists[q])
        for t in range(tiles):
            if t in members:
                obj.append(t)
            ptr.append(len(obj))
    grid = legalize.SiteGrid(w, h, 3, np.array(ptr, np.uint32), np.array(obj, np.uint32), tiles)
    n = 60
    kind = rng.integers(0, 3, n).astype(np.uint32)
    xy = np.stack([rng.integers(0, w, n), rng.integers(0, h, n)], 1).astype(np.uint32)
    for scale in (1, 0):
        r = legalize.auction_singletons(grid, kind, xy, cost_scale=scale)
        s = r.stats["cost_scale"]
        assert s == 1
        code, a, prices, st = ffi.auction_singletons(grid, kind, xy, cost_scale=s, jacobi=True)
        assert code == 0 and np.array_equal(r.assignment, a)
        assert np.array_equal(r.prices.astype(np.uint64), prices)
        got = r.assignment[r.assignment >= 0]
        assert len(set(got.tolist())) == len(got)
        for b in range(n):
            if r.assignment[b] >= 0:
                assert int(r.assignment[b]) in set(lists[kind[b]])

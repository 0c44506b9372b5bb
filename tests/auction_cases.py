"""Auction test cases shared by the CPU (oracle) and GPU tests.

- `exhaustive_families()`: the two exhaustive small-graph families of
  `implicit_auction_has_exact_cardinality_and_bounded_cost_on_small_graphs`
  (crates/texo-pnr/src/legalization/auction.rs:465-505), as dense cost
  arrays [cases, bidders, objects] with -1 for an absent edge.
- `brute_force(costs)`: the lexicographic optimum (fewest unmatched, then
  least base cost) of every case, as `brute_force_quality` (auction.rs:
  302-338) defines it, vectorised over the cases.
- `random_grid(...)`: a seeded BEL grid with several kinds, capacities and
  occupied BELs, and bidders with clustered targets.
- `grid_optimum(...)`: the same lexicographic optimum of a grid problem by
  the Hungarian method (scipy), each bidder's private dummy as an extra column.
"""
import itertools

import numpy as np

from texo_gb300 import legalize

# the reference's known-answer cases (auction.rs:358-444): (domains, objects, max cost, expected)
KNOWN_ANSWERS = [
    ("flexible_bidder_moves_instead_of_spilling_constrained_bidder",
     [[(0, 0), (1, 1), (2, 100)], [(0, 0), (2, 100)]], 3, 100, [1, 0]),
    ("restricted_graph_uses_real_solution_instead_of_false_no_bel",
     [[(0, 0), (1, 1)], [(0, 0)]], 2, 1, [1, 0]),
    ("private_dummy_gap_does_not_hide_a_perfect_matching",
     [[(1, 0), (2, 0)], [(0, 0), (1, 0)], [(0, 0)]], 3, 0, [2, 1, 0]),
]


def sixty_six_domains():
    """candidate_after_legacy_sixty_four_limit_remains_visible (auction.rs:398-415)."""
    d = [[(o, 0)] for o in range(65)]
    d.append([(o, 0) for o in range(66)])
    return d


def _family_one():
    for bidders in range(1, 4):
        for objects in range(0, 4):
            edges = bidders * objects
            codes = np.arange(3 ** edges, dtype=np.int64)
            c = np.empty((len(codes), bidders, objects), dtype=np.int64)
            for e in range(edges):   # bidder-major, object-minor digits, least significant first
                c[:, e // objects, e % objects] = codes % 3 - 1
                codes //= 3
            yield bidders, objects, 1, c


def _family_two():
    for objects in range(0, 5):
        edges = 4 * objects
        masks = np.arange(1 << edges, dtype=np.int64)
        c = np.full((len(masks), 4, objects), -1, dtype=np.int64)
        for b in range(4):
            for o in range(objects):
                bit = (masks >> (b * objects + o)) & 1
                c[:, b, o] = np.where(bit == 1, (b + o) & 1, -1)
        yield 4, objects, 1, c


def exhaustive_families():
    """(bidders, objects, max_base_cost, costs [cases, bidders, objects]) groups."""
    yield from _family_one()
    yield from _family_two()


def domains_of(costs):
    """One case's cost matrix as the reference's Vec<Vec<(object, cost)>>."""
    return [[(o, int(c)) for o, c in enumerate(row) if c >= 0] for row in costs]


def brute_force(costs):
    """(unmatched, base cost) of the lexicographic optimum of every case."""
    cases, nb, no = costs.shape
    options = [tuple(p) for p in itertools.product(range(-1, no), repeat=nb)
               if len([x for x in p if x >= 0]) == len({x for x in p if x >= 0})]
    inj = np.array(options, dtype=np.int64).reshape(len(options), nb)
    big = 10 ** 6
    padded = np.concatenate([costs, np.zeros((cases, nb, 1), dtype=np.int64)], axis=2)   # column no = dummy
    col = np.where(inj < 0, no, inj)                                                     # [J, nb]
    picked = padded[:, np.arange(nb)[None, :], col]                                      # [cases, J, nb]
    infeasible = ((picked < 0) & (inj[None] >= 0)).any(axis=2)   # uses an absent edge
    total = np.maximum(picked, 0).sum(axis=2)
    unmatched = (inj < 0).sum(axis=1)
    key = np.where(infeasible, np.iinfo(np.int64).max, unmatched[None, :] * big + total)
    best = key.argmin(axis=1)
    return unmatched[best], total[np.arange(cases), best]


def quality(costs, assignment):
    """(unmatched, base cost) of assignments [cases, bidders] (-1 = dummy);
    raises if an assignment uses an absent edge or an object twice."""
    cases, nb, no = costs.shape
    a = np.asarray(assignment, dtype=np.int64).reshape(cases, nb)
    unmatched = (a < 0).sum(axis=1)
    if no == 0:
        if np.any(a >= 0):
            raise AssertionError("an assignment to an object that does not exist")
        return unmatched, np.zeros(cases, dtype=np.int64)
    c = np.where(a >= 0, costs[np.arange(cases)[:, None], np.arange(nb)[None, :], np.clip(a, 0, no - 1)], 0)
    if np.any((a >= 0) & (c < 0)):
        raise AssertionError("an assignment uses an edge outside the bidder's domain")
    for i in range(nb):
        for j in range(i + 1, nb):
            if np.any((a[:, i] >= 0) & (a[:, i] == a[:, j])):
                raise AssertionError("an object assigned twice")
    return unmatched, c.sum(axis=1)


def random_grid(seed, width, height, kinds=1, cap_max=1, bidders=100, occupied=0.0, clusters=3, spread=2.0):
    rng = np.random.default_rng(seed)
    cap = rng.integers(0 if cap_max > 1 else 1, cap_max + 1, size=(kinds, height, width))
    m = int(cap.sum())
    occ = (rng.random(m) < occupied).astype(np.uint8) if occupied > 0 else None
    grid = legalize.site_grid(cap, occupied=occ)
    kind = rng.integers(0, kinds, bidders).astype(np.uint32)
    centres = np.stack([rng.integers(0, width, clusters), rng.integers(0, height, clusters)], axis=1)
    pick = rng.integers(0, clusters, bidders)
    xy = np.rint(centres[pick] + rng.normal(0, spread, (bidders, 2)))
    xy[:, 0] = np.clip(xy[:, 0], 0, width - 1)
    xy[:, 1] = np.clip(xy[:, 1], 0, height - 1)
    return grid, kind, xy.astype(np.uint32)


def grid_costs(grid, kind, targets):
    """Dense base costs [bidders, BELs], -1 where a BEL is not a candidate."""
    where = grid.bel_tiles()
    t = np.asarray(targets, dtype=np.int64).reshape(-1, 2)
    d = np.abs(where[None, :, 1] - t[:, None, 0]) + np.abs(where[None, :, 2] - t[:, None, 1])
    ok = where[None, :, 0] == np.asarray(kind, dtype=np.int64)[:, None]
    if grid.occupied is not None:
        ok &= grid.occupied[None, :] == 0
    return np.where(ok, d, -1)


def grid_optimum(grid, kind, targets):
    """(unmatched, base cost) of the lexicographic optimum (Hungarian method)."""
    from scipy.optimize import linear_sum_assignment
    c = grid_costs(grid, kind, targets)
    n, m = c.shape
    max_cost = grid.width - 1 + grid.height - 1
    dummy = n * max_cost + n + 1
    forbid = float(dummy) * (n + 2)
    full = np.full((n, m + n), forbid)
    full[:, :m] = np.where(c >= 0, c, forbid)
    full[np.arange(n), m + np.arange(n)] = dummy
    r, col = linear_sum_assignment(full)
    unmatched = int((col >= m).sum())
    cost = int(sum(c[i, j] for i, j in zip(r, col) if j < m))
    return unmatched, cost

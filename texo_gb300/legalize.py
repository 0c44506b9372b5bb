"""Host mirror of the legalizer's capacity auction (crates/texo-pnr/src/legalization).

`project` (legalization/mod.rs:322-389) turns the rounded global-placement
targets into BEL choices: fixed units first, then auctions of shared-row
families and of single-BEL units, then a transactional repair. This module
exposes the auction, which runs on the GPU through include/texo_gp.h:

- `assign_implicitly(domains, object_count, max_base_cost)`: the auction
  (auction.rs:131-247) over explicit candidate lists, the form the
  reference's own tests drive it with;
- `auction_singletons(grid, bidder_kind, targets)`: the single-BEL auction
  of `project` (`auction_singletons`, mod.rs:657-677), candidates found by
  Manhattan ring walks around each unit's target tile;
- `SiteGrid` / `site_grid`: the BEL layout those walks read;
- `project_singletons(problem, targets)`: the single-cell part of `project`
  for a placement problem: fixed units' BELs occupied, singleton bidders,
  the auction, one BEL per unit;
- `project` / `project_native`: `project` up to its repair (fixed units,
  shared-row families, singletons; texo_gp_project);
- `repair`: the transactional repair (`repair_relaxed`, repair.rs) with
  occupancy, pin-wire and shared-resource legality (texo_gp_repair, host
  code), and `project_and_repair`, the whole `project`.

The GPU bids all unassigned bidders at once each round; the result carries
the reference's guarantees (exact maximum cardinality, total base cost at
most the bidder count above the least one of that cardinality) and is
deterministic, but where several assignments meet them it may differ from
the reference's one-bidder-at-a-time order. By default the base costs are
scaled (the reference's own `cost_scale`, fixed there at 1), which tightens
the cost bound to n / scale.
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi


@dataclass
class AuctionResult:
    """`AuctionResult` (auction.rs:36-42): per bidder its object, or -1 for
    the bidder's private dummy; the final prices (the epsilon-optimality
    certificate); the work done (`AuctionStats`, auction.rs:28-34, plus the
    rounds, the matched base cost and the device time)."""
    assignment: np.ndarray
    prices: np.ndarray
    stats: dict

    def as_options(self):
        """The assignment as the reference's Vec<Option<usize>>."""
        return [None if a < 0 else int(a) for a in self.assignment]


def _stats(st):
    return {"cost_scale": st.cost_scale, "bids": st.bids, "candidates_examined": st.candidates_examined,
            "unmatched": st.unmatched, "rounds": st.rounds, "tail_rounds": st.tail_rounds,
            "total_base_cost": st.total_base_cost, "elapsed_ms": st.elapsed_ms,
            "kernel_launches": st.kernel_launches}


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def assign_implicitly(domains, object_count, max_base_cost, cost_scale=0, device=0):
    """`assign_implicitly` with `explicit_best_two` (auction.rs:253-272):
    `domains[b]` is bidder b's list of (object, base cost); `cost_scale` 1 is
    the reference's setting, 0 the largest of 4, 2, 1 that fits (explicit
    domains: 1). Raises
    TexoGpError with AUCTION_RANGE (ArithmeticOverflow), AUCTION_OBJECT_RANGE,
    AUCTION_COST_RANGE or AUCTION_DUPLICATE_OBJECT like the reference's
    AuctionError."""
    n = len(domains)
    ptr = np.zeros(n + 1, dtype=np.uint32)
    ptr[1:] = np.cumsum([len(d) for d in domains]) if n else []
    obj = _u32([o for d in domains for o, _ in d]) if ptr[-1] else np.zeros(1, np.uint32)
    cost = np.ascontiguousarray([c for d in domains for _, c in d] if ptr[-1] else [0], dtype=np.uint64)
    assignment = np.full(max(n, 1), -1, dtype=np.int32)
    prices = np.zeros(max(object_count, 1), dtype=np.uint32)
    st = abi.AuctionStats()
    lib = abi.load()
    abi.check(lib.texo_gp_auction_explicit(device, n, object_count, max_base_cost, cost_scale,
                                           abi.ptr(ptr, C.c_uint32),
                                           abi.ptr(obj, C.c_uint32), abi.ptr(cost, C.c_uint64),
                                           abi.ptr(assignment, C.c_int32), abi.ptr(prices, C.c_uint32),
                                           C.byref(st)),
              "texo_gp_auction_explicit")
    return AuctionResult(assignment[:n].copy(), prices[:object_count].copy(), _stats(st))


@dataclass
class SiteGrid:
    """BELs by (kind, tile): the BELs of kind q at tile t = y * width + x are
    tile_object[tile_ptr[q * width * height + t] : tile_ptr[... + t + 1]];
    `occupied` (or None) marks BELs held by fixed units or earlier cohorts."""
    width: int
    height: int
    num_kinds: int
    tile_ptr: np.ndarray
    tile_object: np.ndarray
    num_objects: int
    occupied: np.ndarray = None

    def bel_tiles(self):
        """(kind, x, y) of every BEL id (-1 where an id is not on the grid)."""
        where = np.full((self.num_objects, 3), -1, dtype=np.int64)
        counts = np.diff(self.tile_ptr.astype(np.int64))
        slot = np.repeat(np.arange(len(counts)), counts)
        tiles = self.width * self.height
        where[self.tile_object, 0] = slot // tiles
        where[self.tile_object, 1] = (slot % tiles) % self.width
        where[self.tile_object, 2] = (slot % tiles) // self.width
        return where


def site_grid(capacity, occupied=None):
    """A SiteGrid from per-kind BEL counts `capacity` [K, H, W]: BEL ids run
    kind-major, then row-major over tiles, then over the slots of a tile."""
    cap = np.asarray(capacity, dtype=np.int64)
    if cap.ndim == 2:
        cap = cap[None]
    k, h, w = cap.shape
    ptr = np.zeros(k * h * w + 1, dtype=np.uint32)
    ptr[1:] = np.cumsum(cap.reshape(-1))
    m = int(ptr[-1])
    occ = None if occupied is None else np.ascontiguousarray(occupied, dtype=np.uint8)
    return SiteGrid(w, h, k, ptr, np.arange(m, dtype=np.uint32), m, occ)


def auction_singletons(grid, bidder_kind, targets, cost_scale=0, device=0):
    """The single-BEL auction of `project` on the GPU: bidder b (a unit of
    kind bidder_kind[b] with rounded target targets[b] = (x, y), as
    `rounded_targets_from_coordinates` gives them) takes one unoccupied BEL
    of its kind at base cost |x - tx| + |y - ty|. `cost_scale` as in
    `assign_implicitly`: the total base cost is at most n / scale above the
    optimum of the maximum cardinality."""
    kind = _u32(bidder_kind).reshape(-1)
    txy = _u32(targets).reshape(-1)
    n = kind.shape[0]
    if txy.shape[0] != 2 * n:
        raise ValueError("targets must hold one (x, y) per bidder")
    assignment = np.full(max(n, 1), -1, dtype=np.int32)
    prices = np.zeros(max(grid.num_objects, 1), dtype=np.uint32)
    tobj = grid.tile_object if len(grid.tile_object) else np.zeros(1, np.uint32)
    occ = None if grid.occupied is None else np.ascontiguousarray(grid.occupied, dtype=np.uint8)
    st = abi.AuctionStats()
    lib = abi.load()
    abi.check(lib.texo_gp_auction_singletons(device, grid.width, grid.height, grid.num_kinds,
                                             abi.ptr(_u32(grid.tile_ptr), C.c_uint32), abi.ptr(_u32(tobj), C.c_uint32),
                                             grid.num_objects, None if occ is None else abi.ptr(occ, C.c_uint8), n,
                                             abi.ptr(kind if n else np.zeros(1, np.uint32), C.c_uint32),
                                             abi.ptr(txy if n else np.zeros(2, np.uint32), C.c_uint32),
                                             cost_scale, abi.ptr(assignment, C.c_int32), abi.ptr(prices, C.c_uint32),
                                             C.byref(st)),
              "texo_gp_auction_singletons")
    return AuctionResult(assignment[:n].copy(), prices[:grid.num_objects].copy(), _stats(st))


def fixed_occupancy_mask(grid, fixed_occupancy):
    """The BELs held by fixed units (`install_fixed_units`, legalization/mod.rs:
    391-430) as an occupied mask: each (field, x, y) entry of a problem's
    `fixed_occupancy` takes the first free BEL of that field at that tile.
    Raises TexoGpError (FIXED_CAPACITY_EXHAUSTED, the reference's
    ElectrostaticError) when a tile has more fixed entries than BELs."""
    occ = np.zeros(grid.num_objects, dtype=np.uint8)
    fo = np.asarray(fixed_occupancy, dtype=np.int64).reshape(-1, 3)
    if len(fo) == 0:
        return occ
    tiles = grid.width * grid.height
    if np.any(fo[:, 0] >= grid.num_kinds) or np.any(fo[:, 1] >= grid.width) or np.any(fo[:, 2] >= grid.height):
        raise abi.TexoGpError(abi.CODE["POINT_OUTSIDE_GRID"], "fixed_occupancy_mask")
    slot = fo[:, 0] * tiles + fo[:, 2] * grid.width + fo[:, 1]
    order = np.argsort(slot, kind="stable")
    s = slot[order]
    first = np.r_[0, np.nonzero(np.diff(s))[0] + 1]
    rank = np.arange(len(s)) - np.repeat(first, np.diff(np.r_[first, len(s)]))   # k-th entry of its slot
    ptr = np.asarray(grid.tile_ptr, dtype=np.int64)
    if np.any(ptr[s] + rank >= ptr[s + 1]):
        raise abi.TexoGpError(abi.CODE["FIXED_CAPACITY_EXHAUSTED"], "fixed_occupancy_mask")
    occ[np.asarray(grid.tile_object, dtype=np.int64)[ptr[s] + rank]] = 1
    return occ


def project_singletons(problem, targets, cost_scale=0, device=0):
    """The single-cell part of `project` (legalization/mod.rs:322-389) for a
    placement problem and its rounded targets [U, 2] (what `place` returns):
    the BELs of each density field by tile from the problem's capacity grid,
    those of fixed units occupied, every movable unit with one density member
    a bidder of its member's field at its target (`classify_units`,
    mod.rs:432-471), and the
    single-BEL auction on the GPU. Returns (BEL id per unit: -1 for fixed
    units, unmatched ones and the units this path leaves out; the auction
    result; the movable multi-member units, which the reference places by its
    shared-row auctions, not built here)."""
    k = len(problem.fields)
    cap = np.asarray(problem.capacity, dtype=np.int64).reshape(k, problem.height, problem.width)
    grid = site_grid(cap)
    grid.occupied = fixed_occupancy_mask(grid, problem.fixed_occupancy)
    ptr = np.asarray(problem.member_ptr, dtype=np.int64)
    members = np.diff(ptr)
    movable = np.any(problem.lower_xy != problem.upper_xy, axis=1)
    bidders = np.nonzero(movable & (members == 1))[0]
    kind = np.asarray(problem.member_field, dtype=np.uint32)[ptr[bidders]]
    xy = np.ascontiguousarray(np.asarray(targets, dtype=np.uint32).reshape(-1, 2)[bidders])
    result = auction_singletons(grid, kind, xy, cost_scale=cost_scale, device=device)
    bel = np.full(problem.num_units, -1, dtype=np.int64)
    bel[bidders] = result.assignment
    return bel, result, np.nonzero(movable & (members > 1))[0]


# ---- project: fixed units, shared-row families and singletons ------------

@dataclass
class Unit:
    """A placement unit (`PlacementUnit`): its cells and its choices, one BEL
    per cell each. `shared` False is the reference's SingleCell choice table
    (one cell, candidates in ascending BEL order), True a Shared table of
    assignment rows; None picks Shared for multi-cell units. Units whose
    `choices` are the same list object form one family, as units sharing an
    Arc'd table do in the reference (`cache_key`, lib.rs:3756-3761)."""
    cells: list
    choices: list
    shared: bool = None

    def is_shared(self):
        return len(self.cells) > 1 if self.shared is None else bool(self.shared)


class ProjectionError(ValueError):
    """PnrError::InvalidPlacement from `project` (the reason in the message)."""


@dataclass
class Projection:
    """What `project` leaves for its repair: per unit the preferred choice
    (-1 where none was found), per BEL whether it is taken, and the cohort
    statistics (`ProjectionStats`, legalization/mod.rs)."""
    preferred: np.ndarray
    occupied: np.ndarray
    stats: dict

    def bels(self, units):
        """BEL of every cell (-1 for cells of units without a choice)."""
        n = 1 + max((c for u in units for c in u.cells), default=-1)
        out = np.full(n, -1, dtype=np.int64)
        for u, unit in enumerate(units):
            if self.preferred[u] >= 0:
                out[unit.cells] = unit.choices[int(self.preferred[u])]
        return out


def ring_coordinates(center, offset, extent):
    """`ring_coordinates` (lib.rs:6814-6821): center - offset, then
    center + offset (once for offset 0), inside [0, extent)."""
    out = []
    if center >= offset:
        out.append(center - offset)
    if offset != 0:
        out.append(center + offset)
    return [v for v in out if v < extent]


def _by_point(bel_xy, width, height, choices):
    """`SpatialChoiceIndex` (lib.rs:3774-3787): choice indices by the tile of
    the choice's first BEL, ascending within a tile."""
    first = np.fromiter((a[0] for a in choices), dtype=np.int64, count=len(choices))
    tile = bel_xy[first, 1] * width + bel_xy[first, 0]
    order = np.argsort(tile, kind="stable")
    ends = np.searchsorted(tile[order], np.arange(1, width * height + 1))
    return [v.tolist() for v in np.split(order, ends[:-1])]


def _nearest_direct_choice(unit, by_point, bel_xy, target, occupied, width, height):
    """`nearest_direct_choice` (legalization/mod.rs:533-575): the least
    (point, choice) with every BEL free on the first Manhattan ring around
    the target that has one."""
    tx, ty = int(target[0]), int(target[1])
    for radius in range(0, width - 1 + height - 1 + 1):
        best = None
        for dy in range(radius + 1):
            dx = radius - dy
            for y in ring_coordinates(ty, dy, height):
                for x in ring_coordinates(tx, dx, width):
                    for c in by_point[y * width + x]:
                        if not occupied[unit.choices[c]].any() and (best is None or ((x, y), c) < best):
                            best = ((x, y), c)
        if best is not None:
            return best[1]
    return None


def _rows_disjoint(choices):
    seen = set()
    for a in choices:
        for b in a:
            if b in seen:
                return False
            seen.add(b)
    return True


def _object_grid(width, height, num_kinds, kind_by_point, num_objects, occupied):
    """A SiteGrid whose objects of kind q at tile t are kind_by_point[q][t]."""
    lists = [v for q in range(num_kinds) for v in kind_by_point[q]]
    ptr = np.zeros(len(lists) + 1, np.uint32)
    ptr[1:] = np.cumsum([len(v) for v in lists])
    obj = np.fromiter((o for v in lists for o in v), dtype=np.uint32, count=int(ptr[-1]))
    return SiteGrid(width, height, num_kinds, ptr, obj, num_objects, np.ascontiguousarray(occupied, dtype=np.uint8))


def gpu_auction(grid, bidder_kind, targets, cost_scale):
    """The object auction of `project` on the GPU: (assignment, stats)."""
    r = auction_singletons(grid, bidder_kind, targets, cost_scale=cost_scale)
    return r.assignment, r.stats


def project(width, height, bel_xy, units, targets, cost_scale=0, auction=None):
    """`project` (legalization/mod.rs:322-389) up to its repair: the units'
    choices from their rounded targets [U, 2], occupancy being the only
    legality rule (BELs whose pin-wire or shared-resource rules fail are the
    caller's to mark by leaving them out of the choices).

    1. `install_fixed_units` (:391-430): one-choice units take their BELs; two
       on one BEL is an error.
    2. `classify_units` (:432-471): Shared tables form families (units by
       first cell); a family whose rows are pairwise BEL-disjoint is auctioned,
       the others' units are seeded; SingleCell units are singletons.
    3. `seed_overlapping_units` (:473-531): by (choices, -cells, first cell),
       each takes the nearest free row (`nearest_direct_choice`).
    4. `auction_disjoint_families` (:577-655): families in scarcity order
       (rows x other family's size, then larger units, then first cell), each
       an auction whose objects are its free rows at the ring distance of the
       row's first BEL.
    5. `auction_singletons` (:657-677): one auction over every singleton,
       objects the BELs of each distinct candidate table.

    `bel_xy` [B, 2]: BEL tiles. By default the whole composition runs in
    native code (`texo_gp_project`, auctions on the GPU); `auction(grid, kinds,
    targets, cost_scale) -> (assignment, stats)` runs these steps here in
    Python with the given auction instead (a checker passes the oracle's).
    Unmatched units keep -1; `repair` (texo_gp_repair) then places them by
    the reference's transactional search, and `project_and_repair` runs
    both steps."""
    if auction is None:
        return project_native(width, height, bel_xy, units, targets, cost_scale)
    bel_xy = np.asarray(bel_xy, dtype=np.int64).reshape(-1, 2)
    B = bel_xy.shape[0]
    U = len(units)
    tg = np.asarray(targets, dtype=np.int64).reshape(-1, 2)
    if tg.shape[0] != U:
        raise ValueError("one target per unit")
    occupied = np.zeros(B, dtype=bool)
    preferred = np.full(U, -1, dtype=np.int64)
    stats = {"fixed_units": 0, "overlapping_shared_families": 0, "overlapping_shared_units": 0,
             "disjoint_shared_families": 0, "disjoint_shared_units": 0, "singleton_units": 0,
             "relaxed_unmatched_units": 0, "bids": 0, "candidates_examined": 0}
    for u, unit in enumerate(units):
        if len(unit.choices) != 1:
            continue
        a = np.asarray(unit.choices[0], dtype=np.int64)
        if occupied[a].any():
            raise ProjectionError("fixed analytical placement assignments conflict")
        occupied[a] = True
        preferred[u] = 0
        stats["fixed_units"] += 1
    families, singletons = {}, []
    for u, unit in enumerate(units):
        if len(unit.choices) == 1:
            continue
        if unit.is_shared():
            families.setdefault(id(unit.choices), []).append(u)
        else:
            singletons.append(u)
    overlapping, disjoint = [], []
    for fam in families.values():
        fam.sort(key=lambda u: units[u].cells[0])
        if _rows_disjoint(units[fam[0]].choices):
            stats["disjoint_shared_families"] += 1
            stats["disjoint_shared_units"] += len(fam)
            disjoint.append(fam)
        else:
            stats["overlapping_shared_families"] += 1
            stats["overlapping_shared_units"] += len(fam)
            overlapping += fam
    singletons.sort(key=lambda u: units[u].cells[0])
    stats["singleton_units"] = len(singletons)
    # 3. overlapping families: nearest free row, one unit at a time
    overlapping.sort(key=lambda u: (len(units[u].choices), -len(units[u].cells), units[u].cells[0]))
    index_cache = {}
    for u in overlapping:
        unit = units[u]
        key = id(unit.choices)
        if key not in index_cache:
            index_cache[key] = _by_point(bel_xy, width, height, unit.choices)
        c = _nearest_direct_choice(unit, index_cache[key], bel_xy, tg[u], occupied, width, height)
        if c is None:
            continue
        preferred[u] = c
        occupied[np.asarray(unit.choices[c], dtype=np.int64)] = True
    # 4. disjoint families, scarcest first
    import functools

    def scarcity(a, b):
        ua, ub = units[a[0]], units[b[0]]
        la, lb = len(ua.choices) * len(b), len(ub.choices) * len(a)
        if la != lb:
            return -1 if la < lb else 1
        if len(ua.cells) != len(ub.cells):
            return -1 if len(ua.cells) > len(ub.cells) else 1
        return -1 if ua.cells[0] < ub.cells[0] else (1 if ua.cells[0] > ub.cells[0] else 0)
    disjoint.sort(key=functools.cmp_to_key(scarcity))

    def record(bidders, assignment, to_choice):
        for u, obj in zip(bidders, assignment):
            if obj < 0:
                stats["relaxed_unmatched_units"] += 1
                continue
            c = to_choice(u, int(obj))
            a = np.asarray(units[u].choices[c], dtype=np.int64)
            if occupied[a].any():
                raise ProjectionError("capacity auction returned an occupied assignment")
            preferred[u] = c
            occupied[a] = True

    def add_stats(st):
        stats["bids"] += int(st.get("bids", 0))
        stats["candidates_examined"] += int(st.get("candidates_examined", 0))

    for fam in disjoint:
        rows = units[fam[0]].choices
        free = np.array([not occupied[np.asarray(a, dtype=np.int64)].any() for a in rows], dtype=np.uint8)
        grid = _object_grid(width, height, 1, [_by_point(bel_xy, width, height, rows)], len(rows), 1 - free)
        asg, st = auction(grid, np.zeros(len(fam), np.uint32), tg[fam].astype(np.uint32), cost_scale)
        add_stats(st)
        record(fam, asg, lambda u, obj: obj)
    # 5. singletons: one auction, a kind per distinct candidate table
    if singletons:
        kind_of, tables = {}, []
        for u in singletons:
            key = id(units[u].choices)
            if key not in kind_of:
                kind_of[key] = len(tables)
                tables.append(units[u].choices)
        kb = []
        for t in tables:
            first = np.fromiter((a[0] for a in t), dtype=np.int64, count=len(t))
            kb.append([sorted(first[v].tolist()) for v in _by_point(bel_xy, width, height, t)])
        grid = _object_grid(width, height, len(tables), kb, B, occupied.astype(np.uint8))
        kinds = np.array([kind_of[id(units[u].choices)] for u in singletons], np.uint32)
        asg, st = auction(grid, kinds, tg[singletons].astype(np.uint32), cost_scale)
        add_stats(st)
        pos = {}

        def to_choice(u, bel):
            key = id(units[u].choices)
            if key not in pos:
                pos[key] = {int(a[0]): i for i, a in enumerate(units[u].choices)}
            if bel not in pos[key]:
                raise ProjectionError("auction returned a noncandidate BEL")
            return pos[key][bel]
        record(singletons, asg, to_choice)
    return Projection(preferred, occupied, stats)


def _native_tables(units):
    """The units' choice tables for the C ABI (units sharing a `choices` list
    share one table): (table array, count, table of every unit, the row
    arrays the tables point into)."""
    table_of, shared_of, tables, keep = {}, [], [], []
    index = []
    for unit in units:
        key = id(unit.choices)
        t = table_of.get(key)
        shared = unit.is_shared()
        if t is None:
            t = table_of[key] = len(shared_of)
            shared_of.append(shared)
            rows = np.ascontiguousarray(np.asarray(unit.choices, dtype=np.uint32).reshape(len(unit.choices), -1))
            keep.append(rows)
            ct = abi.ChoiceTable()
            ct.num_choices, ct.width = rows.shape
            ct.bels = abi.ptr(rows, C.c_uint32)
            ct.shared = 1 if shared else 0
            tables.append(ct)
        elif shared_of[t] != shared:
            raise ValueError("units sharing a choice table must agree on Shared / SingleCell")
        index.append(t)
    unit_table = np.zeros(max(len(units), 1), np.uint32)
    unit_table[:len(index)] = index
    arr = (abi.ChoiceTable * max(len(tables), 1))(*tables)
    return arr, len(tables), unit_table, keep


def project_native(width, height, bel_xy, units, targets, cost_scale=0, device=0):
    """`project` through texo_gp_project: the same steps as `project` with an
    auction callback, in native code with the GPU auctions. Units sharing a
    `choices` list share one choice table."""
    xy = np.ascontiguousarray(np.asarray(bel_xy, dtype=np.uint32).reshape(-1, 2))
    tg = np.ascontiguousarray(np.asarray(targets, dtype=np.uint32).reshape(-1, 2))
    U = len(units)
    if tg.shape[0] != U:
        raise ValueError("one target per unit")
    arr, ntables, unit_table, keep = _native_tables(units)
    first = np.zeros(max(U, 1), np.uint32)
    for u, unit in enumerate(units):
        first[u] = unit.cells[0]
    out = np.full(max(U, 1), -1, np.int32)
    st = abi.ProjectionStats()
    lib = abi.load()
    code = lib.texo_gp_project(device, width, height, xy.shape[0], abi.ptr(xy, C.c_uint32), ntables, arr, U,
                               abi.ptr(unit_table, C.c_uint32), abi.ptr(first, C.c_uint32),
                               abi.ptr(tg if U else np.zeros(2, np.uint32), C.c_uint32), cost_scale,
                               abi.ptr(out, C.c_int32), C.byref(st))
    if code == abi.CODE["PROJECTION_CONFLICT"]:
        raise ProjectionError(lib.texo_gp_last_error().decode())
    abi.check(code, "texo_gp_project")
    stats = {f: getattr(st, f) for f, _ in abi.ProjectionStats._fields_ if f != "reserved"}
    return Projection(out[:U].astype(np.int64), None, stats)


def spatial_choices_within(by_point, center, max_distance, width, height):
    """`spatial_choices_within` (lib.rs:3789-3811): the choices anchored at
    every tile up to Manhattan distance `max_distance` of `center`, ring by
    ring in the ring-walk order."""
    max_radius = int(min(max_distance, width + height))
    out = []
    cx, cy = int(center[0]), int(center[1])
    for radius in range(max_radius + 1):
        for dy in range(radius + 1):
            dx = radius - dy
            for y in ring_coordinates(cy, dy, height):
                for x in ring_coordinates(cx, dx, width):
                    out.extend(by_point[y * width + x])
    return out


def project_anchored(width, height, bel_xy, units, targets, incumbent):
    """`project_anchored_targets` (lib.rs:4157-4231): a timing iteration's
    targets projected from the legal incumbent (`incumbent`: the BEL of every
    cell). Every unit starts on its incumbent BELs; units in order of
    decreasing distance from their incumbent origin to their target (then
    index) with more than one choice and a nonzero distance are lifted and
    take the first free choice strictly closer to the target (the choices
    within distance - 1 in ring order), else their incumbent again.
    Occupancy is the only legality rule. Returns the BEL of every cell."""
    bel_xy = np.asarray(bel_xy, dtype=np.int64).reshape(-1, 2)
    placed = np.asarray(incumbent, dtype=np.int64).copy()
    occupied = np.zeros(bel_xy.shape[0], dtype=bool)
    tg = np.asarray(targets, dtype=np.int64).reshape(-1, 2)
    for unit in units:
        occupied[placed[unit.cells]] = True

    def dist(u):
        ox, oy = bel_xy[placed[units[u].cells[0]]]
        return abs(int(ox) - int(tg[u][0])) + abs(int(oy) - int(tg[u][1]))
    order = sorted(range(len(units)), key=lambda u: (-dist(u), u))
    index_cache = {}
    for u in order:
        unit = units[u]
        if len(unit.choices) == 1:
            continue
        old = placed[unit.cells].copy()
        ox, oy = bel_xy[old[0]]
        distance = abs(int(ox) - int(tg[u][0])) + abs(int(oy) - int(tg[u][1]))
        if distance == 0:
            continue
        occupied[old] = False
        key = id(unit.choices)
        if key not in index_cache:
            index_cache[key] = _by_point(bel_xy, width, height, unit.choices)
        chosen = old
        for c in spatial_choices_within(index_cache[key], tg[u], distance - 1, width, height):
            a = np.asarray(unit.choices[c], dtype=np.int64)
            if not occupied[a].any():
                chosen = a
                break
        placed[unit.cells] = chosen
        occupied[chosen] = True
    return placed


class NoBelError(RuntimeError):
    """PnrError::NoBel { cell } from the repair: no legal completion exists."""

    def __init__(self, cell, message):
        super().__init__(message)
        self.cell = cell


@dataclass
class Legality:
    """Legality beyond BEL occupancy for the repair (texo_gp_legality):
    `wire_capacity[w]` distinct nets a wire admits; `cell_pins`: cell ->
    [(pin key, net)] of its connected pins; `bel_pins`: BEL -> {pin key:
    wire}; `rules`: [(cell -> value, BEL -> resource)], a (rule, resource)
    holding one value."""
    wire_capacity: list = None
    cell_pins: dict = None
    bel_pins: dict = None
    rules: list = None


def _legality_struct(leg):
    L = abi.Legality()
    keep = []

    def arr(values, dtype):
        a = np.ascontiguousarray(np.asarray(values, dtype=dtype).reshape(-1))
        if a.size == 0:
            a = np.zeros(1, dtype)
        keep.append(a)
        return abi.ptr(a, C.c_uint64 if dtype == np.uint64 else C.c_uint32)

    cap = list(leg.wire_capacity or [])
    L.num_wires = len(cap)
    L.wire_capacity = arr(cap, np.uint32)
    cp = [(c, k, n) for c, pins in sorted((leg.cell_pins or {}).items()) for k, n in pins]
    L.num_cell_pins = len(cp)
    L.cell_pin_cell = arr([e[0] for e in cp], np.uint32)
    L.cell_pin_key = arr([e[1] for e in cp], np.uint32)
    L.cell_pin_net = arr([e[2] for e in cp], np.uint32)
    bp = [(b, k, w) for b, pins in sorted((leg.bel_pins or {}).items()) for k, w in sorted(pins.items())]
    L.num_bel_pins = len(bp)
    L.bel_pin_bel = arr([e[0] for e in bp], np.uint32)
    L.bel_pin_key = arr([e[1] for e in bp], np.uint32)
    L.bel_pin_wire = arr([e[2] for e in bp], np.uint32)
    rules = list(leg.rules or [])
    L.num_rules = len(rules)
    cv = [(r, c, v) for r, (cells, _) in enumerate(rules) for c, v in sorted(cells.items())]
    br = [(r, b, x) for r, (_, bels) in enumerate(rules) for b, x in sorted(bels.items())]
    L.num_cell_values = len(cv)
    L.cell_value_rule = arr([e[0] for e in cv], np.uint32)
    L.cell_value_cell = arr([e[1] for e in cv], np.uint32)
    L.cell_value = arr([e[2] for e in cv], np.uint64)
    L.num_bel_resources = len(br)
    L.bel_resource_rule = arr([e[0] for e in br], np.uint32)
    L.bel_resource_bel = arr([e[1] for e in br], np.uint32)
    L.bel_resource = arr([e[2] for e in br], np.uint64)
    return L, keep


def repair(width, height, bel_xy, units, targets, preferred, fixed, legality=None, num_cells=None):
    """`repair_relaxed` (legalization/repair.rs:60-151) through
    texo_gp_repair: the relaxed proposal `preferred` (a row per unit, -1
    unmatched; rows may conflict) made legal by transactional search. `fixed`
    marks units never evicted. Returns (BEL per cell, -1 for cells of no
    unit; the search counters `RepairStats`). Raises ProjectionError for the
    reference's invalid-placement cases and NoBelError when no legal
    completion exists."""
    U = len(units)
    xy = np.ascontiguousarray(np.asarray(bel_xy, dtype=np.uint32).reshape(-1, 2))
    tg = np.ascontiguousarray(np.asarray(targets, dtype=np.uint32).reshape(-1, 2))
    pref = np.ascontiguousarray(np.asarray(preferred, dtype=np.int32).reshape(-1))
    fx = np.ascontiguousarray(np.asarray(fixed, dtype=np.uint8).reshape(-1))
    if tg.shape[0] != U or pref.size != U or fx.size != U:
        raise ProjectionError("transactional repair input lengths do not match placement units")
    if num_cells is None:
        num_cells = 1 + max((c for u in units for c in u.cells), default=-1)
    arr, ntables, unit_table, keep = _native_tables(units)
    ptr = np.zeros(U + 1, np.uint32)
    ptr[1:] = np.cumsum([len(u.cells) for u in units]) if U else []
    cells = np.ascontiguousarray(np.asarray([c for u in units for c in u.cells] or [0], dtype=np.uint32))
    out = np.full(max(num_cells, 1), -1, np.int32)
    st = abi.RepairStats()
    L, keep_l = (None, []) if legality is None else _legality_struct(legality)
    lib = abi.load()
    code = lib.texo_gp_repair(width, height, xy.shape[0], abi.ptr(xy, C.c_uint32), ntables, arr, U,
                              abi.ptr(unit_table, C.c_uint32), abi.ptr(ptr, C.c_uint32), abi.ptr(cells, C.c_uint32),
                              num_cells, abi.ptr(tg if U else np.zeros(2, np.uint32), C.c_uint32),
                              abi.ptr(pref if U else np.zeros(1, np.int32), C.c_int32),
                              abi.ptr(fx if U else np.zeros(1, np.uint8), C.c_uint8),
                              C.byref(L) if L is not None else None, abi.ptr(out, C.c_int32), C.byref(st))
    if code == abi.CODE["PROJECTION_CONFLICT"]:
        raise ProjectionError(lib.texo_gp_last_error().decode())
    if code == abi.CODE["NO_BEL"]:
        raise NoBelError(st.failed_cell, lib.texo_gp_last_error().decode())
    abi.check(code, "texo_gp_repair")
    stats = {f: getattr(st, f) for f, _ in abi.RepairStats._fields_ if f not in ("reserved", "failed_cell")}
    return out[:num_cells].astype(np.int64), stats


def project_and_repair(width, height, bel_xy, units, targets, legality=None, cost_scale=0, device=0):
    """The whole `project` (legalization/mod.rs:322-389): the relaxed
    projection (texo_gp_project, GPU auctions) and its transactional repair
    (texo_gp_repair), fixed units being those with one choice. Returns (BEL
    per cell, projection statistics, repair statistics)."""
    pj = project_native(width, height, bel_xy, units, targets, cost_scale, device)
    fixed = [len(u.choices) == 1 for u in units]
    placed, rs = repair(width, height, bel_xy, units, targets, pj.preferred, fixed, legality)
    return placed, pj.stats, rs

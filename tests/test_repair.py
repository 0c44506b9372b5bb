"""The transactional repair of `project` (legalization/repair.rs): the
reference's own repair tests (repair.rs:1319-1929) on the oracle's
restatement and through texo_gp_repair (host code in the C-ABI library),
and the native search against the restatement on seeded instances with BEL,
pin-wire and shared-resource conflicts: the same placement, the same search
counters, the same errors."""
import numpy as np
import pytest

from oracle import repair_oracle as R
from texo_gb300 import legalize as L


def line_bels(n, y=0):
    return [(i, y) for i in range(n)]


def both(width, height, bel_xy, units, targets, preferred, fixed, leg=None, num_cells=None):
    """Runs the oracle and the native repair; returns both results."""
    o = R.repair(width, height, bel_xy, units, targets, preferred, fixed,
                 None if leg is None else R.Legality(**leg), num_cells)
    n = L.repair(width, height, bel_xy, units, targets, [(-1 if p is None else p) for p in preferred], fixed,
                 None if leg is None else L.Legality(**leg), num_cells)
    return o, n


def same(o, n):
    assert list(o[0]) == list(n[0])
    for k, v in o[1].items():
        assert n[1][k] == v, k


def test_cursor_order_is_preferred_first_then_ring_by_ring():
    # repair.rs:1319-1345
    bel_xy = [(2, 1), (0, 1), (1, 2), (1, 1), (1, 0)]
    choices = [[b] for b in range(5)]
    idx = R.by_point(bel_xy, 3, choices)
    assert list(R.cursor(idx, 3, 3, (1, 1), 0)) == [0, 3, 1, 4, 2]


def test_twelve_thousand_unit_augmenting_chain():
    # repair.rs:1347-1408: unit 0 may take only BEL 0, unit u BEL u-1 or u
    n = 12000
    bel_xy = [(0, 0)] * n
    units = [L.Unit([0], [[0]], False)] + [L.Unit([u], [[u - 1], [u]], False) for u in range(1, n)]
    pref = [None] + [0] * (n - 1)
    placed, st = L.repair(1, 1, bel_xy, units, [(0, 0)] * n, [-1] + [0] * (n - 1), [False] * n)
    assert list(placed) == list(range(n))
    assert st["direct_fast_fallbacks"] == 1 and st["augmenting_roots"] == 1 and st["augmenting_fallbacks"] == 0
    assert st["states_visited"] >= n
    # the restatement on a shorter chain gives the same placement and counters
    m = 300
    o, nn = both(1, 1, bel_xy[:m], units[:m], [(0, 0)] * m, pref[:m], [False] * m)
    same(o, nn)
    assert list(o[0]) == list(range(m))


def test_deep_single_combination():
    # repair.rs:1410-1419
    c = R.combinations(12000, 12000)
    assert len(c) == 1 and len(c[0]) == 12000 and c[0][0] == 0 and c[0][-1] == 11999
    assert R.combinations(4, 2) == [[0, 1], [0, 2], [0, 3], [1, 2], [1, 3], [2, 3]]
    assert R.combinations(2, 3) == [] and R.combinations(3, 0) == [[]]


def test_multi_blocker_candidate_falls_back_to_the_exact_search():
    # repair.rs:1421-1477
    units = [L.Unit([0, 1], [[0, 1]], True), L.Unit([2], [[0], [2]], False), L.Unit([3], [[1], [3]], False)]
    o, n = both(4, 1, line_bels(4), units, [(0, 0)] * 3, [None, 0, 0], [False] * 3)
    same(o, n)
    assert list(n[0]) == [0, 1, 2, 3]
    st = n[1]
    assert st["direct_fast_fallbacks"] == 1 and st["augmenting_fallbacks"] == 1 and st["states_visited"] >= 3


def test_partial_direct_fast_path_rolls_back_before_augmenting():
    # repair.rs:1479-1540
    domains = [[[3]], [[0], [1]], [[0], [2]], [[1]]]
    units = [L.Unit([c], d, False) for c, d in enumerate(domains)]
    o, n = both(1, 1, [(0, 0)] * 4, units, [(0, 0)] * 4, [None, None, 0, 0], [False, False, False, True])
    same(o, n)
    assert list(n[0]) == [3, 0, 2, 1]
    st = n[1]
    assert st["direct_fast_moves"] == 1 and st["direct_fast_fallbacks"] == 1
    assert st["augmenting_roots"] == 2 and st["augmenting_fallbacks"] == 0


def test_far_spill_displaces_a_clean_owner():
    # repair.rs:1542-1572
    units = [L.Unit([0], [[0], [1]]), L.Unit([1], [[0], [64]]), L.Unit([2], [[1]])]
    o, n = both(65, 1, line_bels(65), units, [(0, 0)] * 3, [None, 0, 0], [False, False, True])
    same(o, n)
    assert list(n[0]) == [0, 64, 1]


def test_overlapping_bundle_rows_are_repaired_atomically():
    # repair.rs:1574-1613
    rows = [[0, 1], [1, 2], [2, 3]]
    units = [L.Unit([0, 1], rows), L.Unit([2, 3], rows)]
    o, n = both(4, 1, line_bels(4), units, [(0, 0), (1, 0)], [0, 1], [False, False])
    same(o, n)
    assert sorted(n[0]) == [0, 1, 2, 3]
    for u in units:
        assert list(n[0][u.cells]) in rows


SHARED = {"rules": [({0: 0, 1: 1}, {0: 0, 1: 0, 2: 1, 3: 1})]}


def test_incompatible_shared_values_move_to_different_resources():
    # repair.rs:1615-1645
    units = [L.Unit([0], [[0], [2]]), L.Unit([1], [[1], [3]])]
    o, n = both(4, 1, line_bels(4), units, [(0, 0)] * 2, [0, 0], [False, False], SHARED)
    same(o, n)
    assert n[0][0] // 2 != n[0][1] // 2
    assert n[1]["initial_pending"] == 1


def test_unavoidable_shared_value_conflict_is_no_bel():
    # repair.rs:1722-1753
    units = [L.Unit([0], [[0], [1]]), L.Unit([1], [[2], [3]])]
    leg = {"rules": [({0: 0, 1: 1}, {b: 0 for b in range(4)})]}
    with pytest.raises(R.NoBel):
        R.repair(4, 1, line_bels(4), units, [(0, 0)] * 2, [0, 0], [False, False], R.Legality(**leg))
    with pytest.raises(L.NoBelError):
        L.repair(4, 1, line_bels(4), units, [(0, 0)] * 2, [0, 0], [False, False], L.Legality(**leg))


# pin keys of the reference's pin names
P, Q, A, AI, C_, CI, D, DI = range(8)


def test_initial_pending_keeps_the_fixed_net_class():
    # repair.rs:1647-1720: one wire of capacity 2, three net classes
    leg = R.Legality(wire_capacity=[2],
                     cell_pins={0: [(P, 0)], 1: [(P, 0)], 2: [(P, 1), (Q, 1)], 3: [(P, 2), (Q, 2)]},
                     bel_pins={0: {P: 0}, 1: {P: 0}, 2: {P: 0, Q: 0}, 3: {P: 0, Q: 0}})
    units = [L.Unit([c], [[c]]) for c in range(4)]
    assert R.initial_pending(units, [0] * 4, [True, False, False, False], leg, 4) == {3}


def test_pin_class_remains_until_its_last_owner_is_blocked_and_rollback_is_exact():
    # repair.rs:1755-1849
    leg = R.Legality(wire_capacity=[1, 1, 1],
                     cell_pins={0: [(P, 0)], 1: [(P, 0)], 2: [(P, 1), (Q, 1)]},
                     bel_pins={0: {P: 0}, 1: {P: 0}, 2: {P: 0, Q: 0}, 3: {P: 1}, 4: {P: 2}})
    bel_xy = [(0, 0), (0, 0), (0, 0), (1, 0), (2, 0)]
    units = [L.Unit([0], [[0], [3]]), L.Unit([1], [[1], [4]]), L.Unit([2], [[2]])]
    pref, fixed = [0, 0, None], [False] * 3
    s = R.State(units, pref, fixed, leg, 3, 5)
    s.raw_install(0, 0)
    s.raw_install(1, 0)
    idx = {id(u.choices): R.by_point(bel_xy, 3, u.choices) for u in units}
    search = R.Search(s, idx, 3, 1, [(0, 0)] * 3, {"max_blocker_branches": 0})
    assert search.pin_branches(2, 0, {0}) == [frozenset({0, 1})]
    before = s.key()
    assert before == ()
    mark = len(s.journal)
    s.remove_branch(0)
    s.remove_branch(1)
    s.install_branch(2, 0)
    assert s.key() != ()
    s.rollback(mark)
    assert s.key() == before and s.choice == [0, 0, None]
    # the whole repair: the candidate takes the shared wire, the net-a pair moves
    o, n = both(3, 1, bel_xy, units, [(0, 0)] * 3, pref, fixed,
                {"wire_capacity": leg.wire_capacity, "cell_pins": leg.cell_pins, "bel_pins": leg.bel_pins})
    same(o, n)
    assert list(n[0]) == [3, 4, 2]


def test_candidate_distinct_nets_share_the_wire_capacity():
    # repair.rs:1851-1928
    leg = R.Legality(wire_capacity=[2],
                     cell_pins={0: [(A, 0), (AI, 0)], 1: [(C_, 1), (CI, 1)], 2: [(D, 2), (DI, 2)]},
                     bel_pins={0: {A: 0, AI: 0}, 1: {C_: 0, CI: 0}, 2: {D: 0, DI: 0}})
    units = [L.Unit([0], [[0]]), L.Unit([1, 2], [[1, 2]])]
    s = R.State(units, [0, None], [False, False], leg, 3, 3)
    s.raw_install(0, 0)
    idx = {id(u.choices): R.by_point([(0, 0)] * 3, 1, u.choices) for u in units}
    search = R.Search(s, idx, 1, 1, [(0, 0)] * 2, {"max_blocker_branches": 0})
    assert search.pin_branches(1, 0, set()) == [frozenset({0})]


def test_invalid_inputs_are_the_reference_errors():
    units = [L.Unit([0], [[0]]), L.Unit([1], [[0]])]
    for impl in ("oracle", "native"):
        run = (lambda *a: R.repair(*a)) if impl == "oracle" else (lambda *a: L.repair(*a))
        err = R.ProjectionError if impl == "oracle" else L.ProjectionError
        with pytest.raises(err, match="multiple fixed units"):
            run(1, 1, [(0, 0)], units, [(0, 0)] * 2, [0, 0], [True, True])
        with pytest.raises(err, match="unmatched fixed unit"):
            run(1, 1, [(0, 0)], units, [(0, 0)] * 2, [0, -1 if impl == "native" else None], [True, True])
        with pytest.raises(err, match="out-of-range assignment"):
            run(1, 1, [(0, 0)], units, [(0, 0)] * 2, [0, 5], [False, False])
    # a candidate BEL without the pin the cell needs
    leg = {"wire_capacity": [1], "cell_pins": {0: [(P, 0)]}, "bel_pins": {0: {P: 0}}}
    with pytest.raises(Exception, match="bound physical pin"):
        L.repair(2, 1, line_bels(2), [L.Unit([0], [[1], [0]])], [(1, 0)], [-1], [False], L.Legality(**leg))
    with pytest.raises(R.ProjectionError, match="bound physical pin"):
        R.repair(2, 1, line_bels(2), [L.Unit([0], [[1], [0]])], [(1, 0)], [None], [False], R.Legality(**leg))


def random_case(rng):
    """A small grid with SingleCell and Shared tables, a relaxed proposal
    with conflicts and unmatched units, some fixed units, pin wires and a
    shared-resource rule."""
    W, H = int(rng.integers(2, 5)), int(rng.integers(1, 4))
    B = int(rng.integers(6, 14))
    bel_xy = [(int(rng.integers(0, W)), int(rng.integers(0, H))) for _ in range(B)]
    tables = []
    for _ in range(int(rng.integers(1, 4))):
        k = int(rng.integers(1, min(5, B) + 1))
        tables.append(([[int(b)] for b in sorted(rng.choice(B, k, replace=False))], False))
    for _ in range(int(rng.integers(0, 2))):
        rows = [list(map(int, rng.choice(B, 2, replace=False))) for _ in range(int(rng.integers(1, 4)))]
        tables.append((rows, True))
    units, cell = [], 0
    for _ in range(int(rng.integers(2, 7))):
        rows, shared = tables[int(rng.integers(0, len(tables)))]
        w = len(rows[0])
        units.append(L.Unit(list(range(cell, cell + w)), rows, shared))
        cell += w
    U = len(units)
    pref = [int(rng.integers(0, len(u.choices))) if rng.random() < 0.75 else None for u in units]
    fixed = [False] * U
    taken = set()
    for u in range(U):   # a few fixed units on distinct BELs
        if pref[u] is not None and rng.random() < 0.2 and not taken & set(units[u].choices[pref[u]]):
            fixed[u] = True
            taken |= set(units[u].choices[pref[u]])
    targets = [(int(rng.integers(0, W)), int(rng.integers(0, H))) for _ in range(U)]
    nwires = int(rng.integers(1, 4))
    cell_pins = {c: [(0, int(rng.integers(0, 3)))] for c in range(cell) if rng.random() < 0.5}
    bel_pins = {b: {0: int(rng.integers(0, nwires))} for b in range(B)}
    rule = ({c: int(rng.integers(0, 2)) for c in range(cell) if rng.random() < 0.5},
            {b: int(rng.integers(0, 3)) for b in range(B)})
    leg = {"wire_capacity": [int(rng.integers(1, 3)) for _ in range(nwires)], "cell_pins": cell_pins,
           "bel_pins": bel_pins, "rules": [rule]}
    return W, H, bel_xy, units, targets, pref, fixed, leg, cell


def test_native_equals_the_restatement_on_seeded_instances():
    rng = np.random.default_rng(2026)
    outcomes = {"placed": 0, "no_bel": 0, "invalid": 0}
    for _ in range(400):
        W, H, bel_xy, units, targets, pref, fixed, leg, ncells = random_case(rng)
        for lg in (None, leg):
            try:
                o = R.repair(W, H, bel_xy, units, targets, pref, fixed,
                             None if lg is None else R.Legality(**lg), ncells)
            except R.NoBel as e:
                with pytest.raises(L.NoBelError) as ei:
                    L.repair(W, H, bel_xy, units, targets, [(-1 if p is None else p) for p in pref], fixed,
                             None if lg is None else L.Legality(**lg), ncells)
                assert ei.value.cell == e.cell
                outcomes["no_bel"] += 1
                continue
            except R.ProjectionError as e:
                with pytest.raises(L.ProjectionError, match=str(e)):
                    L.repair(W, H, bel_xy, units, targets, [(-1 if p is None else p) for p in pref], fixed,
                             None if lg is None else L.Legality(**lg), ncells)
                outcomes["invalid"] += 1
                continue
            n = L.repair(W, H, bel_xy, units, targets, [(-1 if p is None else p) for p in pref], fixed,
                         None if lg is None else L.Legality(**lg), ncells)
            same(o, n)
            outcomes["placed"] += 1
            # legal: no BEL twice, each unit on one of its rows, fixed units kept
            placed = np.asarray(n[0])
            assert len(set(placed[placed >= 0].tolist())) == int((placed >= 0).sum())
            for u, unit in enumerate(units):
                row = list(placed[unit.cells])
                assert row in [list(r) for r in unit.choices]
                if fixed[u]:
                    assert row == list(unit.choices[pref[u]])
    assert outcomes["placed"] > 100 and outcomes["no_bel"] > 10 and outcomes["invalid"] >= 1, outcomes


def test_fabric_projection_repaired_like_the_restatement():
    """The relaxed projection of the ECP5-like fabric case (the oracle's
    auctions) with a third of the units' choices replaced by a neighbour's
    (BEL conflicts) and every tenth unit unmatched: native repair equals the
    restatement, every cell on a BEL of its unit's rows, no BEL twice."""
    from test_project import fabric_case, oracle_auction
    arch, units, targets = fabric_case(0)
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    pj = L.project(arch.width, arch.height, bel_xy, units, targets, cost_scale=1, auction=oracle_auction(False))
    pref = [int(p) for p in pj.preferred]
    rng = np.random.default_rng(7)
    for u in range(len(units)):
        if len(units[u].choices) == 1:
            continue
        if u % 10 == 0:
            pref[u] = -1
        elif rng.random() < 0.33:
            pref[u] = int(rng.integers(0, len(units[u].choices)))
    fixed = [len(u.choices) == 1 for u in units]
    o = R.repair(arch.width, arch.height, bel_xy, units, targets, [None if p < 0 else p for p in pref], fixed)
    n = L.repair(arch.width, arch.height, bel_xy, units, targets, pref, fixed)
    same(o, n)
    placed = np.asarray(n[0])
    assert np.all(placed >= 0) and len(np.unique(placed)) == len(placed)
    for unit in units:
        assert list(placed[unit.cells]) in [list(r) for r in unit.choices]
    assert n[1]["initial_pending"] > 0


def test_fabric_control_sets_repaired_like_the_restatement():
    """ECP5 register control sets (`constrain_ff_control_sets`) as the
    repair's shared-resource rules on the 16^2 fabric: the occupancy-only
    projection puts registers of different clocks, resets or enables
    together; the repair separates them. Native equals the restatement, and
    every tile's registers share one clock and one LSR value, every slice's
    one CE value."""
    from test_project import fabric_case, oracle_auction
    from texo_gb300 import ecp5
    arch, units, targets = fabric_case(0)
    kinds = [None] * (1 + max(c for u in units for c in u.cells))
    for u in units:
        for c, b in zip(u.cells, u.choices[0]):
            kinds[c] = arch.bel_kind[b]
    sets = ecp5.synthetic_control_sets(kinds, seed=3)
    rules = ecp5.ff_control_set_rules(arch, sets)
    assert len(rules) == 3 and len(sets) > 300
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    pj = L.project(arch.width, arch.height, bel_xy, units, targets, cost_scale=1, auction=oracle_auction(False))
    fixed = [len(u.choices) == 1 for u in units]
    pref = [int(p) for p in pj.preferred]
    o = R.repair(arch.width, arch.height, bel_xy, units, targets, pref, fixed, R.Legality(rules=rules))
    n = L.repair(arch.width, arch.height, bel_xy, units, targets, pref, fixed, L.Legality(rules=rules))
    same(o, n)
    assert n[1]["initial_pending"] > 0
    placed = np.asarray(n[0])
    assert np.all(placed >= 0) and len(np.unique(placed)) == len(placed)
    for r, (cell_values, bel_res) in enumerate(rules):
        seen = {}
        for c, v in cell_values.items():
            res = bel_res[int(placed[c])]
            assert seen.setdefault(res, v) == v, (r, c)

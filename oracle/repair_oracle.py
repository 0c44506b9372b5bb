"""CPU restatement of the transactional repair of `project`
(crates/texo-pnr/src/legalization/repair.rs), pure Python for small cases.

Test infrastructure only: the parity tests compare texo_gp_repair (native
code) with this restatement, and both with the known answers of the
reference's own repair tests (repair.rs:1319-1929).

Inputs mirror the reference's: placement units (cells, choice rows), the
BEL tiles, the rounded targets, the relaxed preferred choice of every unit
(None / -1 = unmatched; conflicting choices allowed), the fixed flags, and
the legality model beyond BEL occupancy (`Legality`):
- pin wires: a connected cell pin (key, net) placed on a BEL takes the BEL
  pin wire of that key; a wire admits `capacity` distinct nets
  (`visit_assignment_pin_resources`, lib.rs:6989-7005; `candidate_pin_wire`);
- shared resources: under rule r a cell carries a value and a BEL belongs to
  a resource; one resource holds one value (`visit_assignment_shared_resources`,
  lib.rs:6972-6987).
"""
from dataclasses import dataclass, field

UNPLACED = -1


class ProjectionError(ValueError):
    """PnrError::InvalidPlacement raised by the repair (reason in the message)."""


class NoBel(Exception):
    """PnrError::NoBel { cell }: the search exhausted every state."""

    def __init__(self, cell):
        super().__init__(f"no BEL for cell {cell}")
        self.cell = cell


@dataclass
class Legality:
    wire_capacity: list = field(default_factory=list)
    cell_pins: dict = field(default_factory=dict)    # cell -> [(key, net)]
    bel_pins: dict = field(default_factory=dict)     # bel -> {key: wire}
    rules: list = field(default_factory=list)        # [(cell_values {cell: v}, bel_resources {bel: r})]


def footprint(leg, cells, row):
    """`assignment_footprint` (repair.rs:161-188): sorted distinct pin-wire
    claims (wire, net) and shared claims ((rule, resource), value)."""
    pins, shared = set(), set()
    if leg is None:
        return [], []
    for cell, bel in zip(cells, row):
        for key, net in leg.cell_pins.get(cell, ()):
            wires = leg.bel_pins.get(bel, {})
            if key not in wires:
                raise ProjectionError("placement candidate lacks a bound physical pin")
            pins.add((wires[key], net))
        for r, (cell_values, bel_resources) in enumerate(leg.rules):
            if cell in cell_values and bel in bel_resources:
                shared.add(((r, bel_resources[bel]), cell_values[cell]))
    return sorted(pins), sorted(shared)


def by_point(bel_xy, width, choices):
    """`SpatialChoiceIndex::new` (lib.rs:3778-3787): choices by the tile of
    their first BEL, in choice order."""
    idx = {}
    for c, row in enumerate(choices):
        x, y = bel_xy[row[0]]
        idx.setdefault(int(y) * width + int(x), []).append(c)
    return idx


def cursor(index, width, height, target, preferred):
    """`ChoiceCursor` (repair.rs:641-790): the preferred choice, then every
    other choice ring by Manhattan ring around the target; within a ring x
    ascending, below before above, a point's choices in index order."""
    if preferred is not None:
        yield preferred
    tx, ty = int(target[0]), int(target[1])
    max_r = (width - 1) + (height - 1)
    for r in range(max_r + 1):
        for x in range(max(tx - r, 0), min(tx + r, width - 1) + 1):
            dx = abs(x - tx)
            if dx > r:
                continue
            dy = r - dx
            ys = []
            if ty >= dy and ty - dy < height:
                ys.append(ty - dy)
            if dy != 0 and ty + dy < height:
                ys.append(ty + dy)
            for y in ys:
                for c in index.get(y * width + x, ()):
                    if c != preferred:
                        yield c


class State:
    """`RepairState` (repair.rs:418-590): a legal partial placement with
    owners of BELs, pin-wire nets and shared values, journalled."""

    def __init__(self, units, preferred, fixed, leg, num_cells, num_bels):
        self.units, self.preferred, self.fixed, self.leg = units, preferred, fixed, leg
        self.choice = [None] * len(units)
        self.unplaced = len(units)
        self.dev = {u: UNPLACED for u, p in enumerate(preferred) if p is not None}
        self.placed = [None] * num_cells
        self.bel_owner = [None] * num_bels
        self.pin_owner = {}      # wire -> {net: set(units)}
        self.shared_owner = {}   # resource -> {value: set(units)}
        self.journal = []
        self._fp = {}

    def fp(self, u, c):
        k = (u, c)
        if k not in self._fp:
            self._fp[k] = footprint(self.leg, self.units[u].cells, self.units[u].choices[c])
        return self._fp[k]

    def record(self, u, c):
        if c == self.preferred[u]:
            self.dev.pop(u, None)
        else:
            self.dev[u] = UNPLACED if c is None else c

    def can_install(self, u, c):
        row = self.units[u].choices[c]
        if any(self.bel_owner[b] is not None for b in row):
            return False
        pins, shared = self.fp(u, c)
        i = 0
        while i < len(pins):
            w = pins[i][0]
            j = i
            nets = self.pin_owner.get(w, {})
            new = 0
            while j < len(pins) and pins[j][0] == w:
                new += pins[j][1] not in nets
                j += 1
            if len(nets) + new > self.leg.wire_capacity[w]:
                return False
            i = j
        i = 0
        while i < len(shared):
            res = shared[i][0]
            j = i
            vals = self.shared_owner.get(res, {})
            new = 0
            while j < len(shared) and shared[j][0] == res:
                new += shared[j][1] not in vals
                j += 1
            if len(vals) + new > 1:
                return False
            i = j
        return True

    def raw_install(self, u, c):
        row = self.units[u].choices[c]
        pins, shared = self.fp(u, c)
        for b in row:
            self.bel_owner[b] = u
        for w, n in pins:
            self.pin_owner.setdefault(w, {}).setdefault(n, set()).add(u)
        for res, v in shared:
            self.shared_owner.setdefault(res, {}).setdefault(v, set()).add(u)
        for cell, b in zip(self.units[u].cells, row):
            self.placed[cell] = b
        self.choice[u] = c
        self.unplaced -= 1
        self.record(u, c)

    def raw_remove(self, u, c):
        row = self.units[u].choices[c]
        pins, shared = self.fp(u, c)
        for b in row:
            self.bel_owner[b] = None
        for w, n in pins:
            s = self.pin_owner[w][n]
            s.discard(u)
            if not s:
                del self.pin_owner[w][n]
                if not self.pin_owner[w]:
                    del self.pin_owner[w]
        for res, v in shared:
            s = self.shared_owner[res][v]
            s.discard(u)
            if not s:
                del self.shared_owner[res][v]
                if not self.shared_owner[res]:
                    del self.shared_owner[res]
        for cell in self.units[u].cells:
            self.placed[cell] = None
        self.choice[u] = None
        self.unplaced += 1
        self.record(u, None)

    def remove_branch(self, u):
        c = self.choice[u]
        self.raw_remove(u, c)
        self.journal.append(("rm", u, c))

    def install_branch(self, u, c):
        self.raw_install(u, c)
        self.journal.append(("in", u, c))

    def rollback(self, mark):
        while len(self.journal) > mark:
            op, u, c = self.journal.pop()
            if op == "in":
                self.raw_remove(u, c)
            else:
                self.raw_install(u, c)

    def next_unplaced(self):
        best = None
        for u, c in enumerate(self.choice):
            if c is None:
                k = (len(self.units[u].choices), -len(self.units[u].cells), self.units[u].cells[0])
                if best is None or k < best[0]:
                    best = (k, u)
        return None if best is None else best[1]

    def key(self):
        return tuple(sorted(self.dev.items()))


def combinations(n, k):
    """`enumerate_combinations` (repair.rs:1232-1257): k-subsets of range(n)
    in lexicographic order."""
    if k > n:
        return []
    if k == 0:
        return [[]]
    out, cur = [], list(range(k))
    while True:
        out.append(cur[:])
        piv = next((i for i in reversed(range(k)) if cur[i] < n - k + i), None)
        if piv is None:
            return out
        cur[piv] += 1
        for i in range(piv + 1, k):
            cur[i] = cur[i - 1] + 1


class Search:
    """`RepairSearch` (repair.rs:592-1230)."""

    def __init__(self, state, index, width, height, targets, stats):
        self.s, self.index, self.W, self.H, self.targets = state, index, width, height, targets
        self.visiting, self.failed, self.st = set(), set(), stats

    def cur(self, u):
        unit = self.s.units[u]
        return cursor(self.index[id(unit.choices)], self.W, self.H, self.targets[u], self.s.preferred[u])

    def frame_seen(self):
        self.st["states_visited"] += 1
        self.st["max_unplaced"] = max(self.st["max_unplaced"], self.s.unplaced)

    def mandatory(self, u, c):
        """`mandatory_blockers` (repair.rs:1119-1167)."""
        s = self.s
        blockers = set()
        for b in s.units[u].choices[c]:
            o = s.bel_owner[b]
            if o is not None:
                if s.fixed[o]:
                    return None
                blockers.add(o)
        shared = s.fp(u, c)[1]
        i = 0
        while i < len(shared):
            res = shared[i][0]
            j = i
            vals = set()
            while j < len(shared) and shared[j][0] == res:
                vals.add(shared[j][1])
                j += 1
            if len(vals) > 1:
                return None
            v = shared[i][1]
            for known, owners in s.shared_owner.get(res, {}).items():
                if known == v:
                    continue
                for o in owners:
                    if s.fixed[o]:
                        return None
                    blockers.add(o)
            i = j
        return blockers

    def pin_branches(self, u, c, mandatory):
        """`pin_blocker_branches` (repair.rs:1169-1230): every distinct-net
        eviction set per touched wire; branches sorted, deduplicated."""
        s = self.s
        by_wire = {}
        for w, n in s.fp(u, c)[0]:
            by_wire.setdefault(w, set()).add(n)
        branches = [frozenset(mandatory)]
        for w in sorted(by_wire):
            cand = by_wire[w]
            cap = s.leg.wire_capacity[w]
            if len(cand) > cap:
                return []
            nxt = []
            for bl in branches:
                eff = []
                for net, owners in s.pin_owner.get(w, {}).items():
                    rem = [o for o in owners if o not in bl]
                    if rem:
                        eff.append((net, rem))
                distinct = len({n for n, _ in eff} | cand)
                need = max(distinct - cap, 0)
                if need == 0:
                    nxt.append(bl)
                    continue
                removable = [(n, o) for n, o in eff if n not in cand and all(not s.fixed[x] for x in o)]
                if len(removable) < need:
                    continue
                for comb in combinations(len(removable), need):
                    nb = set(bl)
                    for k in comb:
                        nb.update(removable[k][1])
                    nxt.append(frozenset(nb))
            branches = sorted(set(nxt), key=lambda b: sorted(b))
            if not branches:
                break
        return branches

    def direct(self):
        """`try_direct_empty_fast_path` (repair.rs:853-886)."""
        s, st = self.s, self.st
        mark = len(s.journal)
        while (u := s.next_unplaced()) is not None:
            done = False
            for c in self.cur(u):
                st["direct_fast_choices"] += 1
                st["choices_examined"] += 1
                if s.can_install(u, c):
                    s.install_branch(u, c)
                    st["direct_fast_moves"] += 1
                    done = True
                    break
            if not done:
                s.rollback(mark)
                st["direct_fast_fallbacks"] += 1
                return False
        del s.journal[mark:]
        return True

    def single_blocker(self):
        """`try_single_blocker_fast_path` (repair.rs:888-917)."""
        s, st = self.s, self.st
        mark = len(s.journal)
        while (root := s.next_unplaced()) is not None:
            st["augmenting_roots"] += 1
            if self.augment(root):
                continue
            s.rollback(mark)
            st["augmenting_fallbacks"] += 1
            return False
        del s.journal[mark:]
        return True

    def augment(self, root):
        """`augment_one` (repair.rs:919-996): an alternating path in which
        every step evicts at most one unit; explicit frames."""
        s, st = self.s, self.st
        root_mark = len(s.journal)
        seen_units, seen_assign = {root}, set()
        self.frame_seen()
        stack = [[root, self.cur(root), None]]
        while stack:
            fr = stack.pop()
            if fr[2] is not None:
                s.rollback(fr[2])
                fr[2] = None
            c = next(fr[1], None)
            if c is None:
                continue
            u = fr[0]
            if (u, c) in seen_assign:
                stack.append(fr)
                continue
            seen_assign.add((u, c))
            st["choices_examined"] += 1
            mand = self.mandatory(u, c)
            if mand is None:
                stack.append(fr)
                continue
            br = self.pin_branches(u, c, mand)
            st["max_blocker_branches"] = max(st["max_blocker_branches"], len(br))
            if len(br) != 1 or len(br[0]) > 1:
                stack.append(fr)
                continue
            blocker = next(iter(br[0]), None)
            if blocker is not None and blocker in seen_units:
                stack.append(fr)
                continue
            mark = len(s.journal)
            if blocker is not None:
                s.remove_branch(blocker)
                st["units_evicted"] += 1
            if not s.can_install(u, c):
                s.rollback(mark)
                stack.append(fr)
                continue
            s.install_branch(u, c)
            if blocker is None:
                return True
            seen_units.add(blocker)
            self.frame_seen()
            fr[2] = mark
            stack.append(fr)
            stack.append([blocker, self.cur(blocker), None])
        s.rollback(root_mark)
        return False

    def begin(self):
        s = self.s
        u = s.next_unplaced()
        if u is None:
            return None
        key = s.key()
        if key in self.failed or key in self.visiting:
            return None
        self.visiting.add(key)
        self.frame_seen()
        # unit, key, cursor, current choice, branches, next branch, resume mark
        return {"u": u, "key": key, "cur": self.cur(u), "choice": None, "br": [], "nb": 0, "mark": None}

    def attempt(self, fr):
        st = self.st
        while True:
            if fr["nb"] < len(fr["br"]):
                b = fr["br"][fr["nb"]]
                fr["nb"] += 1
                return fr["choice"], b
            c = next(fr["cur"], None)
            if c is None:
                return None
            st["choices_examined"] += 1
            mand = self.mandatory(fr["u"], c)
            if mand is None:
                continue
            br = self.pin_branches(fr["u"], c, mand)
            st["max_blocker_branches"] = max(st["max_blocker_branches"], len(br))
            fr["choice"], fr["br"], fr["nb"] = c, br, 0

    def exact(self):
        """`solve_exact_iterative` (repair.rs:1050-1117): depth-first over
        legal partial placements, every blocker set of every choice, states
        memoised by their deviation from the proposal."""
        s, st = self.s, self.st
        root = self.begin()
        if root is None:
            return s.next_unplaced() is None
        stack = [root]
        while stack:
            fr = stack.pop()
            if fr["mark"] is not None:
                s.rollback(fr["mark"])
                fr["mark"] = None
            a = self.attempt(fr)
            if a is None:
                self.visiting.discard(fr["key"])
                self.failed.add(fr["key"])
                if not stack:
                    return False
                continue
            c, blockers = a
            mark = len(s.journal)
            for b in sorted(blockers):
                if s.choice[b] is not None:
                    s.remove_branch(b)
                    st["units_evicted"] += 1
            if s.can_install(fr["u"], c):
                s.install_branch(fr["u"], c)
                if s.next_unplaced() is None:
                    self.visiting.clear()
                    return True
                child = self.begin()
                if child is not None:
                    fr["mark"] = mark
                    stack.append(fr)
                    stack.append(child)
                    continue
            s.rollback(mark)
            stack.append(fr)
        return False

    def solve(self):
        if self.s.next_unplaced() is None:
            return True
        return self.direct() or self.single_blocker() or self.exact()


def initial_pending(units, preferred, fixed, leg, num_bels):
    """`initial_pending_units` (repair.rs:325-414): unmatched units, and of
    every conflict all owners but one survivor (a fixed owner, else the
    scarcest unit; the most popular shared value; the first `capacity` net
    classes of a wire, fixed ones first, then larger classes, then net)."""
    bel_owners = [[] for _ in range(num_bels)]
    pins, shared = {}, {}
    pending = set()
    for u, c in enumerate(preferred):
        if c is None:
            pending.add(u)
            continue
        row = units[u].choices[c]
        fp = footprint(leg, units[u].cells, row)
        for b in row:
            bel_owners[b].append(u)
        for w, n in fp[0]:
            pins.setdefault(w, {}).setdefault(n, set()).add(u)
        for res, v in fp[1]:
            shared.setdefault(res, {}).setdefault(v, set()).add(u)
    for owners in bel_owners:
        if len(owners) < 2:
            continue
        fx = [u for u in owners if fixed[u]]
        if len(fx) > 1:
            raise ProjectionError("multiple fixed units occupy one BEL during repair")
        keep = fx[0] if fx else min(owners, key=lambda u: (len(units[u].choices), -len(units[u].cells), u))
        pending.update(u for u in owners if u != keep)
    for res, values in shared.items():
        if len(values) < 2:
            continue
        fv = [v for v, o in values.items() if any(fixed[u] for u in o)]
        if len(fv) > 1:
            raise ProjectionError("fixed units require incompatible shared-resource values")
        keep = fv[0] if fv else min(values.items(), key=lambda kv: (-len(kv[1]), kv[0]))[0]
        for v, o in values.items():
            if v != keep:
                pending.update(o)
    for w, nets in pins.items():
        cap = leg.wire_capacity[w]
        if len(nets) <= cap:
            continue
        ranked = sorted(nets.items(), key=lambda kv: (not any(fixed[u] for u in kv[1]), -len(kv[1]), kv[0]))
        if sum(1 for _, o in ranked if any(fixed[u] for u in o)) > cap:
            raise ProjectionError("fixed units exceed a placement pin-wire capacity")
        for _, o in ranked[cap:]:
            pending.update(o)
    return pending


def repair(width, height, bel_xy, units, targets, preferred, fixed, legality=None, num_cells=None):
    """`repair_relaxed` (repair.rs:60-151): returns (placed BEL per cell,
    statistics). Raises ProjectionError on invalid input, NoBel(cell) when no
    legal completion exists."""
    U = len(units)
    pref = [None if (p is None or p < 0) else int(p) for p in preferred]
    fixed = [bool(f) for f in fixed]
    if len(pref) != U or len(fixed) != U or len(targets) != U:
        raise ProjectionError("transactional repair input lengths do not match placement units")
    for u, c in enumerate(pref):
        if c is not None and c >= len(units[u].choices):
            raise ProjectionError("transactional repair received an out-of-range assignment")
        if fixed[u] and c is None:
            raise ProjectionError("transactional repair received an unmatched fixed unit")
    leg = legality or Legality()
    bel_xy = [(int(x), int(y)) for x, y in bel_xy]
    num_bels = len(bel_xy)
    if num_cells is None:
        num_cells = 1 + max((c for u in units for c in u.cells), default=-1)
    pending = initial_pending(units, pref, fixed, leg, num_bels)
    st = {"initial_pending": len(pending), "direct_fast_choices": 0, "direct_fast_moves": 0,
          "direct_fast_fallbacks": 0, "augmenting_roots": 0, "augmenting_fallbacks": 0, "states_visited": 0,
          "failed_states": 0, "max_unplaced": len(pending), "max_blocker_branches": 0, "units_evicted": 0,
          "choices_examined": 0}
    state = State(units, pref, fixed, leg, num_cells, num_bels)
    order = [u for u in range(U) if fixed[u]] + [u for u in range(U) if not fixed[u]]
    for u in order:
        c = pref[u]
        if c is None or u in pending:
            continue
        if not state.can_install(u, c):
            raise ProjectionError("relaxed-conflict removal did not leave a legal repair base")
        state.raw_install(u, c)
    first = state.next_unplaced()
    index = {}
    for unit in units:
        if id(unit.choices) not in index:
            index[id(unit.choices)] = by_point(bel_xy, width, unit.choices)
    search = Search(state, index, width, height, [tuple(t) for t in targets], st)
    if not search.solve():
        u = first if first is not None else 0
        raise NoBel(units[u].cells[0])
    st["failed_states"] = len(search.failed)
    return [(-1 if b is None else b) for b in state.placed], st

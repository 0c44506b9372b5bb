"""ECP5 device adapter: from a Project Trellis architecture snapshot to this
library's placement problem.

Host-side data conversion on the path's input side (no GPU work):

* `read_architecture` reads the reference's schema-7 device JSON the way
  `expand` does (crates/texo-target-ecp5/src/lib.rs:4491-4590): the header
  checks of `validate_header` (:4767-4813, timing left out), wires numbered
  location by location, BELs numbered location by location in each location
  type's order (so BEL ids are the reference's), pin and pip wires resolved
  from (dx, dy, index) references (`resolve_wire`, :4887-4909), and each BEL's
  resource kind by type (`resource_kind`, :4948-4958).
* The reference's placement-choice generators over that device: LUT-FF pairs
  (`lut_ff_assignments`, :3868-3893), physical carry pairs and carry chains
  (`physical_carry_pairs`, :2768-2804; `carry_chain_assignments` with
  `fixed_carry_successors`, :2961-3043), distributed-RAM slots
  (`distributed_ram_assignments`, :2806-2843) and wide-LUT clusters
  (`wide_lut_assignments`, :2845-2907).
* `placement_problem` builds the `texo_gp_problem` that `eplace::place`
  (crates/texo-pnr/src/eplace.rs:242-300) forms from placement units: a
  density member for every exchangeable BEL (LUT, register, memory) of a
  unit's first assignment at its offset from the unit origin, fixed
  occupancy for one-choice units, one density field per member kind in
  ascending kind order with the device's BEL count per tile as capacity, the
  unit bounds of `choice_bounds` (eplace.rs:1470-1481), and the hypergraph of
  `AnalyticalHypergraph::new` (analytical_placement.rs:116-168: nets without
  sinks and nets driven by clock cells left out, sink weights above 1 as
  timed arcs).
"""
import json
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .legalize import Unit  # noqa: F401  (placement units are shared with the legalizer)
from .problem import Problem

SCHEMA_VERSION = 7

# resource_kind (lib.rs:4948-4958): BEL type -> (kind, LUT inputs)
_BEL_KIND = {
    "TRELLIS_COMB": (abi.KIND_LUT, 4),
    "TRELLIS_FF": (abi.KIND_REGISTER, 0),
    "DP16KD": (abi.KIND_MEMORY, 0),
    "MULT18X18D": (abi.KIND_DSP, 0),
    "DCCA": (abi.KIND_CLOCK, 0),
    "PIO": (abi.KIND_IO, 0),
    "TRELLIS_IO": (abi.KIND_IO, 0),
}
LUT4 = (abi.KIND_LUT, 4)
REGISTER = (abi.KIND_REGISTER, 0)
EXCHANGEABLE = (abi.KIND_LUT, abi.KIND_REGISTER, abi.KIND_MEMORY)   # density_kind_is_exchangeable


def resource_kind(bel_type):
    return _BEL_KIND.get(bel_type, (abi.KIND_LOGIC, 0))


def kind_order(kind):
    """ResourceKind's derived order: the variant, then the LUT input count."""
    return (int(kind[0]), int(kind[1]))


class ArchitectureError(ValueError):
    """ImportError of the reference's importer; `reason` names the variant."""

    def __init__(self, reason, detail=""):
        self.reason = reason
        super().__init__(reason + (": " + detail if detail else ""))


@dataclass
class Architecture:
    name: str
    width: int
    height: int
    bel_name: list
    bel_type: list
    bel_z: np.ndarray
    bel_x: np.ndarray
    bel_y: np.ndarray
    bel_kind: list
    bel_pins: list                  # per BEL: [(pin name, wire id)] in record order
    num_wires: int
    pip_from: np.ndarray
    pip_to: np.ndarray
    pip_fixed: np.ndarray
    _downhill: list = field(default=None, repr=False)

    @property
    def num_bels(self):
        return len(self.bel_name)

    def bels_of_kind(self, kind):
        return [b for b in range(self.num_bels) if self.bel_kind[b] == tuple(kind)]

    def find_bel_pin(self, bel, name):
        """The wire of the BEL's first pin called `name`, or None."""
        for pin, wire in self.bel_pins[bel]:
            if pin == name:
                return wire
        return None

    def routing_neighbors(self, wire):
        """(downhill wire, fixed) of every pip leaving `wire`."""
        if self._downhill is None:
            self._downhill = [[] for _ in range(self.num_wires)]
            for f, t, fx in zip(self.pip_from.tolist(), self.pip_to.tolist(), self.pip_fixed.tolist()):
                self._downhill[f].append((t, bool(fx)))
        return self._downhill[wire]

    def point(self, bel):
        return int(self.bel_x[bel]), int(self.bel_y[bel])


def _validate_header(d):
    if d.get("schema_version") != SCHEMA_VERSION:
        raise ArchitectureError("UnsupportedSchema", str(d.get("schema_version")))
    if d.get("family") != "ECP5":
        raise ArchitectureError("WrongFamily", str(d.get("family")))
    prov = d.get("provenance", {})
    if not prov.get("project_trellis_revision") or not prov.get("database_revision"):
        raise ArchitectureError("MissingProvenance")
    if not prov.get("split_slice_mode", False):
        raise ArchitectureError("SplitSliceRequired")
    W, H = int(d["width"]), int(d["height"])
    for loc in d["locations"]:
        if loc["location_type"] >= len(d["location_types"]):
            raise ArchitectureError("UnknownLocationType", str(loc["location_type"]))
        if loc["x"] >= W or loc["y"] >= H:
            raise ArchitectureError("LocationOutsideDevice", "(%d, %d)" % (loc["x"], loc["y"]))
        g = loc.get("global")
        if g is not None:
            spine = g.get("spine")
            if g["tap_column"] >= W or (spine is not None and (spine["x"] >= W or spine["y"] >= H)):
                raise ArchitectureError("InvalidGlobalTopology", "(%d, %d)" % (loc["x"], loc["y"]))
    if len(d["locations"]) != W * H:
        raise ArchitectureError("IncompleteLocationGrid", "%d of %d" % (len(d["locations"]), W * H))


def read_architecture(source):
    """Reads an architecture snapshot (a path, JSON text or bytes, or the
    decoded dict) into an Architecture; raises ArchitectureError."""
    if isinstance(source, dict):
        d = source
    elif isinstance(source, (bytes, bytearray)):
        d = json.loads(source.decode())
    elif isinstance(source, str) and source.lstrip().startswith("{"):
        d = json.loads(source)
    else:
        with open(source) as f:
            d = json.load(f)
    _validate_header(d)
    W, H = int(d["width"]), int(d["height"])
    locations = {}
    for loc in d["locations"]:   # indexed_locations (:4871-4885)
        key = (loc["x"], loc["y"])
        if key in locations:
            raise ArchitectureError("DuplicateLocation", "(%d, %d)" % key)
        locations[key] = loc["location_type"]
    types = d["location_types"]
    wires = {}
    for loc in d["locations"]:
        for index in range(len(types[loc["location_type"]]["wires"])):
            wires[(loc["x"], loc["y"], index)] = len(wires)

    def resolve(loc, ref):
        x, y = loc["x"] + ref["dx"], loc["y"] + ref["dy"]
        if x < 0 or y < 0 or x >= W or y >= H or (x, y) not in locations:
            raise ArchitectureError("RelativeReferenceOutsideDevice")
        w = wires.get((x, y, ref["index"]))
        if w is None:
            raise ArchitectureError("UnknownWireReference", "(%d, %d, %d)" % (x, y, ref["index"]))
        return w

    names, btypes, zs, xs, ys, kinds, pins = [], [], [], [], [], [], []
    for loc in d["locations"]:
        for bel in types[loc["location_type"]]["bels"]:
            names.append("X%d/Y%d/%s" % (loc["x"], loc["y"], bel["name"]))
            btypes.append(bel["bel_type"])
            zs.append(int(bel["z"]))
            xs.append(loc["x"])
            ys.append(loc["y"])
            kinds.append(resource_kind(bel["bel_type"]))
            pins.append([(p["name"], resolve(loc, p["wire"])) for p in bel["pins"]])
    pf, pt, px = [], [], []
    for loc in d["locations"]:
        for pip in types[loc["location_type"]]["pips"]:
            pf.append(resolve(loc, pip["from"]))
            pt.append(resolve(loc, pip["to"]))
            px.append(bool(pip["fixed"]))
    return Architecture(str(d["device"]), W, H, names, btypes, np.array(zs, np.int64), np.array(xs, np.int64),
                        np.array(ys, np.int64), kinds, pins, len(wires), np.array(pf, np.int64),
                        np.array(pt, np.int64), np.array(px, bool))


# ---- placement-choice generators -----------------------------------------

def _comb_by_slot(arch):
    """TRELLIS_COMB BELs by (x, y, z), in the reference's BTreeMap order."""
    slots = {}
    for b in arch.bels_of_kind(LUT4):
        if arch.bel_type[b] == "TRELLIS_COMB":
            slots[(*arch.point(b), int(arch.bel_z[b]))] = b
    return dict(sorted(slots.items()))


def lut_ff_assignments(arch):
    """[LUT, FF] where a TRELLIS_FF sits at the LUT's z + 1 on its tile."""
    ff = {}
    for b in arch.bels_of_kind(REGISTER):
        if arch.bel_type[b] == "TRELLIS_FF":
            ff[(*arch.point(b), int(arch.bel_z[b]))] = b
    out = []
    for b in arch.bels_of_kind(LUT4):
        if arch.bel_type[b] != "TRELLIS_COMB":
            continue
        f = ff.get((*arch.point(b), int(arch.bel_z[b]) + 1))
        if f is not None:
            out.append([b, f])
    return out


def physical_carry_pairs(arch):
    """[first, second] COMBs at z = 0 mod 8 and z + 4 of one tile whose first
    FCO wire is the second's FCI wire (both with FCI and FCO pins)."""
    slots = _comb_by_slot(arch)
    out = []
    for (x, y, z), first in slots.items():
        if z % 8 != 0:
            continue
        second = slots.get((x, y, z + 4))
        if second is None:
            continue
        fco = arch.find_bel_pin(first, "FCO")
        if fco is None or arch.find_bel_pin(first, "FCI") is None:
            continue
        fci2 = arch.find_bel_pin(second, "FCI")
        if fci2 is None or arch.find_bel_pin(second, "FCO") is None:
            continue
        if fco == fci2:
            out.append([first, second])
    return out


def _fixed_carry_successors(arch, start, pairs_by_fci):
    queue, visited, succ = deque([start]), {start}, set()
    while queue:
        w = queue.popleft()
        if w in pairs_by_fci:
            succ.update(pairs_by_fci[w])
            if w != start:
                continue
        for nxt, fixed in arch.routing_neighbors(w):
            if fixed and nxt not in visited:
                visited.add(nxt)
                queue.append(nxt)
    return sorted(succ)


def carry_chain_assignments(arch, pair_count):
    """Chains of `pair_count` physical carry pairs, each pair's second FCO
    reaching the next pair's first FCI through fixed pips (or the same wire),
    starting only at pairs whose first COMB has z = 0; flattened BEL lists."""
    pairs = physical_carry_pairs(arch)
    if pair_count == 0:
        return []
    by_fci = {}
    fco = []
    for i, (a, b) in enumerate(pairs):
        by_fci.setdefault(arch.find_bel_pin(a, "FCI"), []).append(i)
        fco.append(arch.find_bel_pin(b, "FCO"))
    succ = [_fixed_carry_successors(arch, w, by_fci) for w in fco]
    seqs = [[i] for i, p in enumerate(pairs) if arch.bel_z[p[0]] == 0]
    for _ in range(1, pair_count):
        seqs = [s + [n] for s in seqs for n in succ[s[-1]] if n not in s]
    return [[b for i in s for b in pairs[i]] for s in seqs]


def distributed_ram_assignments(arch):
    """Six COMBs at z, z + 4, ..., z + 20 (z = 0 mod 32) and the TRELLIS_RAMW
    at z + 18 of the same tile."""
    comb, ramw = {}, {}
    for b in range(arch.num_bels):
        key = (*arch.point(b), int(arch.bel_z[b]))
        if arch.bel_type[b] == "TRELLIS_COMB":
            comb[key] = b
        elif arch.bel_type[b] == "TRELLIS_RAMW":
            ramw[key] = b
    out = []
    for (x, y, z), first in sorted(comb.items()):
        if z % 32 != 0:
            continue
        rest = [comb.get((x, y, z + o)) for o in (4, 8, 12, 16, 20)]
        if any(r is None for r in rest):
            continue
        w = ramw.get((x, y, z + 18))
        if w is None:
            continue
        out.append([first] + rest + [w])
    return out


_WIDE_ROOT = ("A", "B", "C", "D", "F", "F1", "M", "OFX")
_WIDE_MUX = ("A", "B", "C", "D", "F", "FXA", "FXB", "M", "OFX")
_WIDE_LEAF = ("A", "B", "C", "D", "F")
_WIDE_PINS = {2: (8, (_WIDE_ROOT, _WIDE_LEAF)),
              4: (16, (_WIDE_ROOT, _WIDE_MUX, _WIDE_ROOT, _WIDE_LEAF)),
              8: (32, (_WIDE_ROOT, _WIDE_MUX, _WIDE_ROOT, _WIDE_MUX, _WIDE_ROOT, _WIDE_MUX, _WIDE_ROOT,
                       _WIDE_LEAF))}


def wide_lut_assignments(arch, cluster_size):
    """Clusters of 2, 4 or 8 COMBs at z, z + 4, ... (z aligned to 4 x size)
    whose BELs carry the pins the wide-function muxes need."""
    if cluster_size not in _WIDE_PINS:
        return []
    align, required = _WIDE_PINS[cluster_size]
    slots = _comb_by_slot(arch)
    out = []
    for (x, y, z) in slots:
        if z % align != 0:
            continue
        bels = [slots.get((x, y, z + 4 * i)) for i in range(cluster_size)]
        if any(b is None for b in bels):
            continue
        if all(all(arch.find_bel_pin(b, p) is not None for p in pins) for b, pins in zip(bels, required)):
            out.append(bels)
    return out


# ---- placement problem ----------------------------------------------------

def single_cell_choices(arch, kind):
    """The SingleCell choices of a cell of `kind`: every BEL of that kind."""
    return [[b] for b in arch.bels_of_kind(kind)]


def placement_problem(arch, num_cells, units, nets, cell_kind=None, initial_xy=None, sink_weights=None):
    """The texo_gp problem of `units` (Unit list covering cells 0..num_cells-1)
    on `arch`. `nets`: [(driver cell, [sink cells])] in design order;
    `cell_kind` (optional, per cell): nets driven by a clock cell are left
    out; `initial_xy` [U, 2] (default: the device centre); `sink_weights`:
    {(net index, sink ordinal): weight}, a weight w > 1 adds a timed arc of
    extra weight w - 1. Returns (Problem, info dict with the field kinds and
    the units that carry density members)."""
    W, H = arch.width, arch.height
    U = len(units)
    unit_of = np.full(num_cells, -1, np.int64)
    cell_off = np.zeros((num_cells, 2))
    cell_fixed = np.zeros(num_cells, np.uint8)
    cell_fixed_xy = np.zeros((num_cells, 2))
    fixed_occ = []
    members = []          # (unit, kind, offset x, offset y, cell)
    density = np.zeros(U, bool)
    lower = np.zeros((U, 2))
    upper = np.zeros((U, 2))
    init = np.zeros((U, 2))
    centre = (float(W // 2), float(H // 2))
    bounds_of = {}      # choice_bounds per choice table
    checked = set()     # (choice table, cells) shapes already validated
    for u, unit in enumerate(units):
        shape = (id(unit.choices), len(unit.cells))
        if shape not in checked:
            if not unit.choices or any(len(a) != len(unit.cells) for a in unit.choices):
                raise ValueError("unit %d: every choice assigns one BEL per cell" % u)
            checked.add(shape)
        first = unit.choices[0]
        ox, oy = arch.point(first[0])
        for c, b in zip(unit.cells, first):
            if unit_of[c] >= 0:
                raise ValueError("cell %d is in two units" % c)
            unit_of[c] = u
            px, py = arch.point(b)
            cell_off[c] = (px - ox, py - oy)
            if len(unit.choices) == 1:
                cell_fixed[c] = 1
                cell_fixed_xy[c] = (px, py)
        key = id(unit.choices)
        if key not in bounds_of:
            first_bel = np.array([a[0] for a in unit.choices], np.int64)
            xs, ys = arch.bel_x[first_bel], arch.bel_y[first_bel]
            bounds_of[key] = ((int(xs.min()), int(ys.min())), (int(xs.max()), int(ys.max())))
        lo, hi = bounds_of[key]
        p0 = centre if initial_xy is None else tuple(np.asarray(initial_xy, dtype=np.float64)[u])
        if len(unit.choices) == 1:
            for b in first:
                if arch.bel_kind[b][0] in EXCHANGEABLE:
                    fixed_occ.append((arch.bel_kind[b], *arch.point(b)))
            lower[u] = upper[u] = init[u] = (ox, oy)
            continue
        mem = [(u, arch.bel_kind[b], arch.point(b)[0] - ox, arch.point(b)[1] - oy, c)
               for c, b in zip(unit.cells, first) if arch.bel_kind[b][0] in EXCHANGEABLE]
        if not mem:
            # no exchangeable member: the unit keeps its coordinate in the
            # continuous solve (not one of eplace's movable units)
            lower[u] = upper[u] = init[u] = p0
            continue
        density[u] = True
        members += mem
        lower[u], upper[u] = lo, hi
        init[u] = np.clip(p0, lo, hi)
    if np.any(unit_of < 0):
        raise ValueError("cell %d is in no unit" % int(np.nonzero(unit_of < 0)[0][0]))
    kinds = sorted({m[1] for m in members}, key=kind_order)
    field_of = {k: i for i, k in enumerate(kinds)}
    cap = np.zeros((len(kinds), W * H), np.uint32)
    for b in range(arch.num_bels):
        f = field_of.get(arch.bel_kind[b])
        if f is not None:
            x, y = arch.point(b)
            cap[f, y * W + x] += 1
    occ = [(field_of[k], x, y) for (k, x, y) in fixed_occ if k in field_of]
    member_ptr = np.zeros(U + 1, np.int64)
    for m in members:
        member_ptr[m[0] + 1] += 1
    member_ptr = np.cumsum(member_ptr)
    net_ptr, pin_cell, arcs = [0], [], []
    for e, (drv, sinks) in enumerate(nets):
        if not sinks:
            continue
        if cell_kind is not None and tuple(cell_kind[drv])[0] == abi.KIND_CLOCK:
            continue
        pin_cell.append(drv)
        for k, s in enumerate(sinks):
            pin_cell.append(s)
            w = 1 if sink_weights is None else int(sink_weights.get((e, k), 1))
            if w > 1:
                arcs.append((drv, s, w - 1))
        net_ptr.append(len(pin_cell))
    prob = Problem(
        width=W, height=H, fields=kinds, capacity=cap, initial_xy=init, lower_xy=lower, upper_xy=upper,
        member_ptr=member_ptr, member_field=[field_of[m[1]] for m in members],
        member_offset_xy=[(m[2], m[3]) for m in members], member_charge=np.ones(len(members)),
        member_cell=[m[4] for m in members], cell_unit=unit_of, cell_offset_xy=cell_off, cell_fixed=cell_fixed,
        cell_fixed_xy=cell_fixed_xy, net_ptr=net_ptr, pin_cell=pin_cell,
        arc_driver_cell=[a[0] for a in arcs], arc_sink_cell=[a[1] for a in arcs],
        arc_extra_weight=np.array([a[2] for a in arcs], np.uint64),
        fixed_occupancy=np.array(occ, np.uint32).reshape(-1, 3) if occ else None)
    return prob, {"fields": kinds, "density_units": np.nonzero(density)[0]}


# ---- a seeded ECP5-like device snapshot ------------------------------------

def synthetic_architecture(width, height, io_per_edge_tile=2):
    """A schema-7 snapshot of an ECP5-like fabric for workloads the reference
    fixture is too small for: interior PLC tiles with four slices of two
    TRELLIS_COMB (z = 8s, 8s + 4) and two TRELLIS_FF (LUT z + 1), a
    TRELLIS_RAMW at z 18, carry wiring K0.FCO = K1.FCI within a slice and
    K1.FCO = the next slice's K0.FCI within a tile, the last slice's FCO
    reaching the next tile's first FCI (x + 1) through a fixed pip; the
    wide-function pins (F1, M, OFX on K0; FXA, FXB, M, OFX on K1); and PIO
    tiles around the edge. Returns the decoded dict (read_architecture takes
    it)."""
    wires = []

    def wire(name):
        wires.append({"name": name})
        return len(wires) - 1
    rel = lambda i, dx=0, dy=0: {"dx": dx, "dy": dy, "index": i}   # noqa: E731
    bels, pips = [], []
    fci0 = wire("FCI_IN")
    carry_in = fci0
    for s in range(4):
        comb = []
        for k in range(2):
            z = 8 * s + 4 * k
            p = {n: wire("%s%d_SLICE%s" % (n, k, "ABCD"[s])) for n in ("A", "B", "C", "D", "F", "M", "OFX")}
            pins = [{"name": n, "direction": "input", "wire": rel(p[n])} for n in ("A", "B", "C", "D", "M")]
            pins += [{"name": "F", "direction": "output", "wire": rel(p["F"])},
                     {"name": "OFX", "direction": "output", "wire": rel(p["OFX"])}]
            comb.append((z, pins, p))
        # K0 F1 is K1's F; K1's FXA / FXB are wide-function inputs
        comb[0][1].append({"name": "F1", "direction": "input", "wire": rel(comb[1][2]["F"])})
        for n in ("FXA", "FXB"):
            comb[1][1].append({"name": n, "direction": "input", "wire": rel(wire(n + "_SLICE" + "ABCD"[s]))})
        mid = wire("FCO0_SLICE" + "ABCD"[s])
        out = wire("FCO1_SLICE" + "ABCD"[s])
        comb[0][1].extend([{"name": "FCI", "direction": "input", "wire": rel(carry_in)},
                           {"name": "FCO", "direction": "output", "wire": rel(mid)}])
        comb[1][1].extend([{"name": "FCI", "direction": "input", "wire": rel(mid)},
                           {"name": "FCO", "direction": "output", "wire": rel(out)}])
        carry_in = out
        for k in range(2):
            z, pins, _ = comb[k]
            bels.append({"name": "SLICE%s.K%d" % ("ABCD"[s], k), "bel_type": "TRELLIS_COMB", "z": z, "pins": pins})
            ffp = [{"name": n, "direction": "input", "wire": rel(wire("%s%d_SLICE%s" % (n, k, "ABCD"[s])))}
                   for n in ("DI", "CLK", "LSR", "CE")]
            ffp.append({"name": "Q", "direction": "output", "wire": rel(wire("Q%d_SLICE%s" % (k, "ABCD"[s])))})
            bels.append({"name": "SLICE%s.FF%d" % ("ABCD"[s], k), "bel_type": "TRELLIS_FF", "z": z + 1,
                         "pins": ffp})
    bels.append({"name": "RAMW", "bel_type": "TRELLIS_RAMW", "z": 18,
                 "pins": [{"name": "WCK", "direction": "input", "wire": rel(wire("WCK_RAMW"))}]})
    plc_out = carry_in
    plc = {"wires": wires, "bels": bels, "pips": []}
    # the fixed carry pip to the next PLC tile (x + 1); the last column has none
    plc_edge = {"wires": list(wires), "bels": bels, "pips": []}
    plc["pips"].append({"from": rel(plc_out), "to": rel(fci0, dx=1), "fixed": True, "tile_type": "PLC2",
                        "timing_class": "default", "lutperm_flags": 0})
    io_wires = []
    io_bels = []
    for i in range(io_per_edge_tile):
        base = len(io_wires)
        io_wires += [{"name": "%s_PIO%d" % (n, i)} for n in ("I", "T", "O")]
        io_bels.append({"name": "PIO%d" % i, "bel_type": "PIO", "z": i, "pins": [
            {"name": "I", "direction": "input", "wire": rel(base)},
            {"name": "T", "direction": "input", "wire": rel(base + 1)},
            {"name": "O", "direction": "output", "wire": rel(base + 2)}]})
    io = {"wires": io_wires, "bels": io_bels, "pips": []}
    locations = []
    for y in range(height):
        for x in range(width):
            edge = x == 0 or y == 0 or x == width - 1 or y == height - 1
            t = 2 if edge else (0 if x + 1 < width - 1 else 1)
            locations.append({"x": x, "y": y, "location_type": t,
                              "global": {"quadrant": "ul", "tap_direction": "left", "tap_column": 0,
                                         "spine": {"x": 0, "y": 0}}})
    return {"schema_version": SCHEMA_VERSION,
            "provenance": {"project_trellis_revision": "synthetic", "database_revision": "synthetic",
                           "include_lutperm_pips": False, "split_slice_mode": True},
            "family": "ECP5", "device": "synthetic-%dx%d" % (width, height), "width": width, "height": height,
            "location_types": [plc, plc_edge, io], "locations": locations}


def ff_control_set_rules(arch, control_sets):
    """The shared-resource rules of ECP5 register control sets
    (`constrain_ff_control_sets`, texo-target-ecp5/src/lib.rs:1184-1200),
    for the repair's legality (`legalize.Legality(rules=...)`):
    `control_sets` [(cell, slice CE value, tile clock value, tile LSR value)]
    (`FfControlSet`, :803-812; values are opaque identifiers of the control
    net, polarity and mode). Three rules, each (cell -> value, BEL ->
    resource) over the TRELLIS_FF BELs in BEL order, resource ids numbered by
    first appearance:
    - the slice CE mux (`constrain_ff_slice_ce_muxes`, :1074-1108): one
      resource per (tile, z >> 3), the two registers of a slice;
    - the tile clock (`constrain_ff_clock_muxes`, :1110-1144) and the tile
      LSR (`constrain_ff_lsr_muxes`, :1146-1181): one resource per tile, its
      eight registers.
    No control sets: no rules."""
    sets = list(control_sets)
    if not sets:
        return []
    ffs = [b for b in arch.bels_of_kind(REGISTER) if arch.bel_type[b] == "TRELLIS_FF"]
    rules = []
    for column, key in ((1, lambda b: (*arch.point(b), int(arch.bel_z[b]) >> 3)),
                        (2, lambda b: arch.point(b)), (3, lambda b: arch.point(b))):
        ids, bel_res = {}, {}
        for b in ffs:
            bel_res[b] = ids.setdefault(key(b), len(ids))
        rules.append(({int(e[0]): int(e[column]) for e in sets}, bel_res))
    return rules


def synthetic_control_sets(kinds, seed=0, clocks=2, resets=2, enables=3):
    """Seeded control sets for every register cell of a synthetic design:
    [(cell, slice CE, tile clock, tile LSR)] drawn from `enables`, `clocks`
    and `resets` distinct values."""
    rng = np.random.default_rng(seed)
    regs = [c for c, k in enumerate(kinds) if tuple(k) == tuple(REGISTER)]
    return [(c, int(rng.integers(0, enables)), int(rng.integers(0, clocks)), int(rng.integers(0, resets)))
            for c in regs]


def synthetic_design(arch, seed=0, luts=0, ffs=0, lut_ff_pairs=0, carry=(), io=0, nets_per_unit=1.2,
                     sigma=4.0, max_fanout=8):
    """A seeded netlist for `arch` as placement units: `luts` and `ffs`
    single cells (SingleCell over every BEL of their kind), `lut_ff_pairs`
    LUT-FF pairs (one shared table of `lut_ff_assignments` rows), carry chains
    given as (count, pairs) entries (one shared table of
    `carry_chain_assignments(arch, pairs)` rows per entry), and `io` cells
    fixed on PIO BELs spread along the edge. Nets: a driver unit and 1 to
    `max_fanout` sinks drawn with Gaussian locality (`sigma`) over a square
    index grid of the units, driver and sinks on random cells of their units.
    Returns (num_cells, units, cell kinds, nets)."""
    from .legalize import Unit
    rng = np.random.default_rng(seed)
    units, kinds = [], []
    lut_table = single_cell_choices(arch, LUT4)
    ff_table = single_cell_choices(arch, REGISTER)
    ncell = 0

    def add(cells_kinds, choices, shared=None):
        nonlocal ncell
        cells = list(range(ncell, ncell + len(cells_kinds)))
        ncell += len(cells_kinds)
        kinds.extend(cells_kinds)
        units.append(Unit(cells, choices, shared))
    for _ in range(luts):
        add([LUT4], lut_table, False)
    for _ in range(ffs):
        add([REGISTER], ff_table, False)
    if lut_ff_pairs:
        rows = lut_ff_assignments(arch)
        for _ in range(lut_ff_pairs):
            add([LUT4, REGISTER], rows, True)
    for count, pairs in carry:
        rows = carry_chain_assignments(arch, pairs)
        for _ in range(count):
            add([LUT4] * (2 * pairs), rows, True)
    pio = [b for b in range(arch.num_bels) if arch.bel_type[b] == "PIO"]
    if io > len(pio):
        raise ValueError("more IO cells than PIO BELs")
    for b in np.linspace(0, len(pio) - 1, io).astype(np.int64) if io else []:
        add([(abi.KIND_IO, 0)], [[pio[int(b)]]], False)
    n = len(units)
    side = int(np.ceil(np.sqrt(n)))
    order = rng.permutation(n)
    slot = np.empty(n, np.int64)
    slot[order] = np.arange(n)
    at = {int(s): u for u, s in enumerate(slot)}
    nets = []
    for _ in range(int(nets_per_unit * n)):
        d = int(rng.integers(n))
        k = int(rng.integers(1, max_fanout + 1))
        sx, sy = slot[d] % side, slot[d] // side
        sinks = []
        for _ in range(k):
            for _ in range(8):
                x = int(np.clip(np.rint(sx + rng.normal(0, sigma)), 0, side - 1))
                y = int(np.clip(np.rint(sy + rng.normal(0, sigma)), 0, side - 1))
                u = at.get(y * side + x)
                if u is not None and u != d:
                    sinks.append(u)
                    break
        if not sinks:
            continue
        pick = lambda u: units[u].cells[int(rng.integers(len(units[u].cells)))]   # noqa: E731
        nets.append((pick(d), [pick(u) for u in sinks]))
    return ncell, units, kinds, nets

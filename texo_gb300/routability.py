"""Host mirror of elfPlace's instance-area arithmetic (crates/texo-pnr/src/instance_area.rs).

The routability step of `eplace::place` (`propose_area_adjustment`,
eplace.rs:627-740) turns the routing demand map (`texo_gp_routing_demand`
on the GPU, `placer.routing_demand` here) into larger member areas and
smaller filler areas, conserving each resource kind's total charge. These
wrappers call the library's host functions, which follow the reference's
FP64 operation order bit for bit.

A resource kind is an integer key that sorts like the reference's
ResourceKind (for example kind << 8 | lut_inputs with the kind codes of
`abi`); per-kind results come back in ascending key order.
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi


@dataclass
class InstanceAreaAdjustment:
    """`InstanceAreaAdjustment` (instance_area.rs:47-53)."""
    member_areas: np.ndarray
    filler_areas: np.ndarray
    resource_scales: dict
    requires_optimizer_reset: bool


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1))


def _u32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32).reshape(-1))


def adjust_instance_areas(member_kind, current_area, routability_area, pin_area, filler_kind, filler_area,
                          clustering_area=None):
    """`adjust_instance_areas` (instance_area.rs:157-253), elfPlace equations
    (23)-(26). Raises TexoGpError with INSTANCE_AREA_MEMBER / _FILLER (its
    `index` attribute names the entry), _POSTCONDITION or _OVERFLOW like the
    reference's InstanceAreaError."""
    kind = _u32(member_kind)
    n = kind.shape[0]
    cur, rout, pin = _f64(current_area), _f64(routability_area), _f64(pin_area)
    clus = np.zeros(n) if clustering_area is None else _f64(clustering_area)
    fk, fa = _u32(filler_kind), _f64(filler_area)
    nf = fk.shape[0]
    if not (len(cur) == len(rout) == len(pin) == len(clus) == n and len(fa) == nf):
        raise ValueError("member and filler arrays must have matching lengths")
    out_m = np.zeros(max(n, 1))
    out_f = np.zeros(max(nf, 1))
    reset = C.c_int32()
    cap = max(n + nf, 1)
    count = C.c_uint32()
    skind = np.zeros(cap, dtype=np.uint32)
    sval = np.zeros(cap)
    err = C.c_uint64()
    keep = [np.zeros(1, np.uint32) if n == 0 else kind, np.zeros(1) if n == 0 else cur,
            np.zeros(1) if n == 0 else rout, np.zeros(1) if n == 0 else pin, np.zeros(1) if n == 0 else clus,
            np.zeros(1, np.uint32) if nf == 0 else fk, np.zeros(1) if nf == 0 else fa]
    code = abi.load().texo_gp_adjust_instance_areas(
        n, abi.ptr(keep[0], C.c_uint32), abi.ptr(keep[1], C.c_double), abi.ptr(keep[2], C.c_double),
        abi.ptr(keep[3], C.c_double), abi.ptr(keep[4], C.c_double), nf, abi.ptr(keep[5], C.c_uint32),
        abi.ptr(keep[6], C.c_double), abi.ptr(out_m, C.c_double), abi.ptr(out_f, C.c_double), C.byref(reset),
        cap, C.byref(count), abi.ptr(skind, C.c_uint32), abi.ptr(sval, C.c_double), C.byref(err))
    if code:
        e = abi.TexoGpError(code, "texo_gp_adjust_instance_areas")
        e.index = err.value
        raise e
    scales = {int(skind[i]): float(sval[i]) for i in range(count.value)}
    return InstanceAreaAdjustment(out_m[:n].copy(), out_f[:nf].copy(), scales, bool(reset.value))


def routability_optimized_area(current_area, horizontal_utilization, vertical_utilization):
    """`routability_optimized_area` (instance_area.rs:64-84), elfPlace eq. (29)."""
    out = C.c_double()
    abi.check(abi.load().texo_gp_routability_optimized_area(current_area, horizontal_utilization,
                                                            vertical_utilization, C.byref(out)),
              "texo_gp_routability_optimized_area")
    return out.value


def routability_optimized_area_from_bin(current_area, horizontal_demand, horizontal_capacity, vertical_demand,
                                        vertical_capacity):
    """`routability_optimized_area_from_bin` (instance_area.rs:91-127)."""
    out = C.c_double()
    abi.check(abi.load().texo_gp_routability_optimized_area_from_bin(current_area, horizontal_demand,
                                                                     horizontal_capacity, vertical_demand,
                                                                     vertical_capacity, C.byref(out)),
              "texo_gp_routability_optimized_area_from_bin")
    return out.value


def pin_optimized_area(pin_count, unit_area_pin_capacity, local_pin_utilization):
    """`pin_optimized_area` (instance_area.rs:130-148), elfPlace eq. (30)."""
    out = C.c_double()
    abi.check(abi.load().texo_gp_pin_optimized_area(pin_count, unit_area_pin_capacity, local_pin_utilization,
                                                    C.byref(out)),
              "texo_gp_pin_optimized_area")
    return out.value


def register_clustering_areas(xy, clock_lsr, ce, movable_instance_count, device=0):
    """`clustering_areas` (register_clustering.rs:17-80) on the GPU: the area
    elfPlace's register clustering asks for each register at xy [R, 2] with
    control set clock_lsr [R, 2] and clock enable ce [R]. Returns (areas,
    device ms). Raises TexoGpError (INVALID_NORMALIZATION) where the
    reference returns None."""
    p = np.ascontiguousarray(np.asarray(xy, dtype=np.float64).reshape(-1))
    cl = np.ascontiguousarray(np.asarray(clock_lsr, dtype=np.uint64).reshape(-1))
    c = np.ascontiguousarray(np.asarray(ce, dtype=np.uint64).reshape(-1))
    n = c.shape[0]
    if p.shape[0] != 2 * n or cl.shape[0] != 2 * n:
        raise ValueError("xy and clock_lsr need two entries per register")
    out = np.zeros(max(n, 1))
    ms = C.c_double()
    abi.check(abi.load().texo_gp_register_clustering_areas(
        device, n, abi.ptr(p if n else np.zeros(2), C.c_double),
        abi.ptr(cl if n else np.zeros(2, np.uint64), C.c_uint64),
        abi.ptr(c if n else np.zeros(1, np.uint64), C.c_uint64), movable_instance_count, abi.ptr(out, C.c_double),
        C.byref(ms)), "texo_gp_register_clustering_areas")
    return out[:n].copy(), ms.value


SQRT_2 = 1.4142135623730951


def kind_key(field):
    """The order-preserving key of a density field (kind, lut_inputs)."""
    kind, lut = field
    return int(kind) << 8 | int(lut)


def routability_adjusted_member_area(kind, current_area, horizontal_utilization, vertical_utilization):
    """`routability_adjusted_member_area` (eplace.rs:741-758): eq. (29) for
    LUT and register members; every other kind keeps its area (a hard block
    inflated in its own field reserves none of the congested slice routing)."""
    area = routability_optimized_area(current_area, horizontal_utilization, vertical_utilization)
    return area if int(kind) in (abi.KIND_LUT, abi.KIND_REGISTER) else float(current_area)


def _rounded(value, extent):
    # rounded_coordinate (lib.rs:4566-4568): round half away from zero (value
    # - trunc(value) is exact, so no addition of 0.5 can round up), clamp to
    # the grid; NaN goes to 0 like Rust's saturating cast
    value = np.asarray(value, dtype=np.float64)
    t = np.trunc(value)
    r = t + np.where(np.abs(value - t) >= 0.5, np.sign(value), 0.0)
    r = np.where(np.isnan(r), 0.0, r)
    return np.clip(r, 0, extent - 1).astype(np.int64)


def _utilization(demand, capacity, x, y):
    # ContinuousRoutingDemand::utilization (eplace.rs:822-853)
    d = demand[y, x]
    c = capacity[y, x].astype(np.float64)
    u = np.where(c == 0, np.where(d == 0.0, 0.0, SQRT_2), d / np.where(c == 0, 1.0, c))
    if not np.all(np.isfinite(u) & (u >= 0.0)):
        raise abi.TexoGpError(abi.CODE["INVALID_NORMALIZATION"], "propose_area_adjustment")
    return u


def propose_area_adjustment(problem, coordinates, capacity_h, capacity_v, filler_field, filler_charge,
                            member_charge=None, register_controls=None, device=0, demand=None, clustering=None):
    """`propose_area_adjustment` (eplace.rs:627-740) for one placement state:
    the nets' bounding boxes at the unit origins `coordinates[:2U]`, their
    RUDY demand on the routing-capacity grid (`capacity_h` / `capacity_v`,
    [H, W] channel capacities) on the GPU, every movable member's
    utilization at its rounded position, capped at sqrt(2), elfPlace eq. (29)
    for LUT and register members (others keep their area), the register
    clustering areas on the GPU (`register_controls`: cell -> (clock, lsr,
    ce), for the register members), and `adjust_instance_areas` against the
    fillers (`filler_field`, `filler_charge`, as `Placer.fillers()` gives
    them). `member_charge` overrides the problem's member charges (after an
    earlier round). `demand(W, H, boxes) -> (h, v)` and `clustering(xy,
    clock_lsr, ce, count) -> areas` replace the GPU RUDY map and clustering
    areas (a checker passes its own). Returns (InstanceAreaAdjustment,
    metrics dict)."""
    from .placer import net_bounding_boxes, routing_demand
    if demand is None:
        def demand(w, h, boxes):
            hd, vd, _ = routing_demand(w, h, boxes, device=device)
            return hd, vd
    if clustering is None:
        def clustering(xy, clock_lsr, ce, count):
            return register_clustering_areas(xy, clock_lsr, ce, count, device=device)[0]
    cap_h = np.asarray(capacity_h, dtype=np.uint32)
    cap_v = np.asarray(capacity_v, dtype=np.uint32)
    if cap_h.ndim != 2 or cap_h.shape != cap_v.shape or cap_h.size == 0:
        raise abi.TexoGpError(abi.CODE["INVALID_NORMALIZATION"], "propose_area_adjustment")
    H, W = cap_h.shape
    U = problem.num_units
    pos = np.asarray(coordinates, dtype=np.float64)[: 2 * U].reshape(-1, 2)
    h_dem, v_dem = demand(W, H, net_bounding_boxes(problem, pos))
    ptr = np.asarray(problem.member_ptr, dtype=np.int64)
    movable = np.any(problem.lower_xy != problem.upper_xy, axis=1)
    members = np.concatenate([np.arange(ptr[u], ptr[u + 1]) for u in np.nonzero(movable)[0]] or [np.zeros(0, int)])
    unit_of = np.repeat(np.arange(U), np.diff(ptr))[members]
    off = np.asarray(problem.member_offset_xy, dtype=np.float64).reshape(-1, 2)[members]
    charge = np.asarray(problem.member_charge if member_charge is None else member_charge, dtype=np.float64)[members]
    fields = [tuple(f) for f in problem.fields]
    field = np.asarray(problem.member_field, dtype=np.int64)[members]
    keys = np.array([kind_key(fields[f]) for f in field], dtype=np.uint32)
    x = _rounded(pos[unit_of, 0] + off[:, 0], W)
    y = _rounded(pos[unit_of, 1] + off[:, 1], H)
    hu = _utilization(h_dem, cap_h, x, y)
    vu = _utilization(v_dem, cap_v, x, y)
    routing = np.array([routability_adjusted_member_area(fields[f][0], c, min(a, SQRT_2), min(b, SQRT_2))
                        for f, c, a, b in zip(field, charge, hu, vu)])
    clus_area = np.zeros(len(members))
    if register_controls:
        cells = np.asarray(problem.member_cell, dtype=np.int64)[members]
        is_reg = np.array([fields[f][0] == abi.KIND_REGISTER for f in field], dtype=bool)
        regs = np.nonzero(is_reg)[0]
        if len(regs):
            missing = [int(c) for c in cells[regs] if int(c) not in register_controls]
            if missing:   # clustering_areas returns None (register_clustering.rs:33)
                raise abi.TexoGpError(abi.CODE["INVALID_NORMALIZATION"],
                                      "propose_area_adjustment: register cell %d has no control set" % missing[0])
            ctl = np.array([register_controls[int(c)] for c in cells[regs]], dtype=np.uint64).reshape(-1, 3)
            cell_unit = np.asarray(problem.cell_unit, dtype=np.int64)
            count = int(np.sum(movable[cell_unit]))   # cells of movable units (movable_instance_count)
            areas = clustering(pos[unit_of[regs]] + off[regs], ctl[:, :2], ctl[:, 2], count)
            clus_area[regs] = areas
    fk = np.array([kind_key(fields[int(f)]) for f in np.asarray(filler_field).reshape(-1)], dtype=np.uint32)
    fq = np.asarray(filler_charge, dtype=np.float64).reshape(-1)
    adj = adjust_instance_areas(keys, charge, routing, np.zeros(len(members)), fk, fq, clus_area)
    before, increase = {}, {}
    for k, c, a in zip(keys.tolist(), charge, adj.member_areas):
        before[k] = before.get(k, 0.0) + c
        increase[k] = increase.get(k, 0.0) + (a - c)
    # totals in ascending kind order, like the reference's BTreeMap sums
    total_before = sum(before[k] for k in sorted(before))
    total_increase = sum(increase[k] for k in sorted(increase))
    rel = total_increase / total_before if total_before else float("nan")
    rel_max = max([increase[k] / before[k] if before[k] else float("nan") for k in sorted(before)], default=0.0)
    if not (np.isfinite(rel) and np.isfinite(rel_max)):   # the reference's InvalidNormalization
        raise abi.TexoGpError(abi.CODE["INVALID_NORMALIZATION"], "propose_area_adjustment")
    metrics = {"maximum_horizontal_utilization": float(np.max(hu, initial=0.0)),
               "maximum_vertical_utilization": float(np.max(vu, initial=0.0)),
               "members_inflated": int(np.sum(adj.member_areas - charge > 0.0)),
               "total_relative_increase": rel, "maximum_relative_increase": rel_max,
               "members": members}
    return adj, metrics


def area_round_limit(problem):
    """`area_adjustment_round_limit` (eplace.rs:584-626): every round that
    installs area raises the total by at least 1 %, and the area can only
    grow into the free capacity of the member kinds, so rounds beyond
    ceil(log_1.01(available / initial)) + 1 mean a malformed loop."""
    ptr = np.asarray(problem.member_ptr, dtype=np.int64)
    movable = np.any(problem.lower_xy != problem.upper_xy, axis=1)
    mem = np.concatenate([np.arange(ptr[u], ptr[u + 1]) for u in np.nonzero(movable)[0]] or [np.zeros(0, int)])
    initial = float(np.sum(np.asarray(problem.member_charge, dtype=np.float64)[mem]))
    fields = sorted(set(int(f) for f in np.asarray(problem.member_field)[mem]))
    fixed = np.asarray(problem.fixed_occupancy, dtype=np.int64).reshape(-1, 3)
    available = 0.0
    for f in fields:
        available += float(int(np.sum(problem.capacity[f], dtype=np.int64)) - int(np.sum(fixed[:, 0] == f)))
    if not (np.isfinite(initial) and initial > 0.0 and available >= initial):
        raise abi.TexoGpError(abi.CODE["INVALID_NORMALIZATION"], "area_round_limit")
    threshold, rounds = initial, 0
    while threshold < available:
        threshold *= 1.01
        rounds += 1
    return rounds + 1


class DeviceRounds:
    """The rounds of place_routable on this library's GPU engines (the
    params' engine: host-driven stages or the persistent kernel)."""

    def __init__(self, problem, params):
        from .placer import Placer
        self.g = Placer(problem, params)
        self.demand = None
        self.clustering = None

    def fillers(self):
        return self.g.fillers()

    def round(self, stop, reset, scales, completed, coordinates):
        # the handle keeps the previous round's final coordinates itself
        t, c, _, res = self.g.optimize_round(stop, reset, scales, completed)
        return res["status"], t, c, res

    def set_charges(self, member_charge, filler_charge):
        self.g.set_charges(member_charge, filler_charge)

    def close(self):
        self.g.close()


def place_routable(problem, params, capacity_h, capacity_v, register_controls=None, rounds=None):
    """eplace::place with a routing-capacity map (eplace.rs:320-420): density
    rounds that stop at AreaAdjustmentReady (LUT and register overflow at
    15 %), each followed by `propose_area_adjustment` (RUDY utilization,
    elfPlace eq. 29, register clustering, the charge-conserving instance
    areas); an adjustment that grows any kind is installed (member and filler
    charges) and the next round restarts the optimizer with the elfPlace
    eq. (27)-(28) multipliers and the first round's density scales; once the
    installed increase is below 1 % (or nothing grew) a last round runs to
    the final targets. `rounds` runs the rounds (default: DeviceRounds, this
    library's engine named by `params`). Returns (targets [U, 2], coordinates,
    info)."""
    backend = rounds or DeviceRounds(problem, params)
    K = len(problem.fields)
    limit = area_round_limit(problem)
    member_charge = np.array(problem.member_charge, dtype=np.float64)
    filler_field, filler_charge = backend.fillers()
    filler_charge = np.array(filler_charge, dtype=np.float64)
    completed, area_round, previous, scales, reset = 0, 0, None, None, False
    coords = None
    info = {"rounds": [], "area_rounds": 0}
    try:
        while True:
            stop = 0 if (previous is not None and previous < 0.01) else 1
            status, targets, coords, res = backend.round(stop, reset, scales, completed, coords)
            if status not in (0, abi.CODE["DID_NOT_CONVERGE"]):
                raise abi.TexoGpError(status, "place_routable")
            if scales is None:
                scales = np.array(res["density_scales"][:K])
            entry = {"stop": "final" if stop == 0 else "area_ready",
                     "iterations": int(res["completed_iterations"] - completed), "exhausted": res["exhausted"]}
            info["rounds"].append(entry)
            completed = int(res["completed_iterations"])
            if stop == 0 or res["exhausted"]:
                if status == abi.CODE["DID_NOT_CONVERGE"]:
                    raise abi.TexoGpError(status, "place_routable")
                info["iterations"] = completed
                info["member_charge"] = member_charge
                info["filler_charge"] = filler_charge
                return targets, coords, info
            adj, metrics = propose_area_adjustment(problem, coords, capacity_h, capacity_v, filler_field,
                                                   filler_charge, member_charge=member_charge,
                                                   register_controls=register_controls, demand=backend.demand,
                                                   clustering=backend.clustering)
            entry["relative_increase"] = float(metrics["total_relative_increase"])
            entry["members_inflated"] = int(metrics["members_inflated"])
            if not adj.requires_optimizer_reset:
                previous, reset = 0.0, True
                continue
            if area_round >= limit:
                raise abi.TexoGpError(abi.CODE["INVALID_NORMALIZATION"], "place_routable: area round limit")
            member_charge[metrics["members"]] = adj.member_areas
            filler_charge = np.array(adj.filler_areas, dtype=np.float64)
            backend.set_charges(member_charge, filler_charge)
            previous, reset = float(metrics["total_relative_increase"]), True
            area_round += 1
            info["area_rounds"] = area_round
    finally:
        if rounds is None:
            backend.close()

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
        device, n, abi.ptr(p if n else np.zeros(2), C.c_double), abi.ptr(cl if n else np.zeros(2, np.uint64), C.c_uint64),
        abi.ptr(c if n else np.zeros(1, np.uint64), C.c_uint64), movable_instance_count, abi.ptr(out, C.c_double),
        C.byref(ms)), "texo_gp_register_clustering_areas")
    return out[:n].copy(), ms.value

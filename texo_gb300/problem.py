"""Flattened `eplace::place` problem (the texo_gp_problem C struct) in numpy.

`Problem` owns contiguous numpy arrays for every field of texo_gp_problem and
builds the ctypes view on demand. Builders cover the reference's own test
fixtures (tiny hand-built devices) and wrap the library's seeded synthetic
ECP5-like generator for benchmark-scale netlists.
"""
import ctypes as C

import numpy as np

from . import abi


def _u32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint32))


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


class Problem:
    """Holds the arrays of one placement problem.

    width, height  : tile grid
    fields         : list of (kind, lut_inputs) in ResourceKind order
    capacity       : uint32 [K, H*W]
    units          : initial_xy/lower_xy/upper_xy float64 [U, 2]
    members        : member_ptr [U+1], member_field, member_offset_xy [M, 2],
                     member_charge, member_cell
    cells          : cell_unit, cell_offset_xy [C, 2], cell_fixed (uint8), cell_fixed_xy
    nets           : net_ptr [E+1], pin_cell [P]
    timed arcs     : arc_driver_cell, arc_sink_cell, arc_extra_weight (uint64)
    """

    def __init__(self, width, height, fields, capacity, initial_xy, lower_xy, upper_xy,
                 member_ptr, member_field, member_offset_xy, member_charge, member_cell,
                 cell_unit, cell_offset_xy, cell_fixed, cell_fixed_xy, net_ptr, pin_cell,
                 arc_driver_cell=(), arc_sink_cell=(), arc_extra_weight=(),
                 fixed_occupancy=None, _owner=None):
        self.width = int(width)
        self.height = int(height)
        self.fields = [(int(k), int(l)) for (k, l) in fields]
        self.capacity = _u32(capacity).reshape(len(self.fields), self.width * self.height)
        self.initial_xy = _f64(initial_xy).reshape(-1, 2)
        self.lower_xy = _f64(lower_xy).reshape(-1, 2)
        self.upper_xy = _f64(upper_xy).reshape(-1, 2)
        self.member_ptr = _u32(member_ptr)
        self.member_field = _u32(member_field)
        self.member_offset_xy = _f64(member_offset_xy).reshape(-1, 2)
        self.member_charge = _f64(member_charge)
        self.member_cell = _u32(member_cell)
        self.cell_unit = _u32(cell_unit)
        self.cell_offset_xy = _f64(cell_offset_xy).reshape(-1, 2)
        self.cell_fixed = np.ascontiguousarray(np.asarray(cell_fixed, dtype=np.uint8))
        self.cell_fixed_xy = _f64(cell_fixed_xy).reshape(-1, 2)
        self.net_ptr = _u32(net_ptr)
        self.pin_cell = _u32(pin_cell)
        self.arc_driver_cell = _u32(arc_driver_cell)
        self.arc_sink_cell = _u32(arc_sink_cell)
        self.arc_extra_weight = np.ascontiguousarray(np.asarray(arc_extra_weight, dtype=np.uint64))
        fo = np.zeros((0, 3), dtype=np.uint32) if fixed_occupancy is None else _u32(fixed_occupancy).reshape(-1, 3)
        self.fixed_occupancy = np.ascontiguousarray(fo)
        self._fields_c = (abi.Field * max(1, len(self.fields)))(*[abi.Field(k, l) for k, l in self.fields])
        self._owner = _owner   # keeps a synthetic generator handle alive

    @property
    def num_units(self):
        return self.initial_xy.shape[0]

    @property
    def num_cells(self):
        return self.cell_unit.shape[0]

    @property
    def num_nets(self):
        return self.net_ptr.shape[0] - 1

    @property
    def num_pins(self):
        return int(self.net_ptr[-1]) if self.net_ptr.size else 0

    def c_struct(self):
        p = abi.ProblemC()
        p.width, p.height = self.width, self.height
        p.num_fields = len(self.fields)
        p.fields = C.cast(self._fields_c, C.POINTER(abi.Field))
        p.capacity = abi.ptr(self.capacity, C.c_uint32)
        p.num_fixed_occupancy = self.fixed_occupancy.shape[0]
        p.fixed_occupancy = abi.ptr(self.fixed_occupancy, C.c_uint32)
        p.num_units = self.num_units
        p.initial_xy = abi.ptr(self.initial_xy, C.c_double)
        p.lower_xy = abi.ptr(self.lower_xy, C.c_double)
        p.upper_xy = abi.ptr(self.upper_xy, C.c_double)
        p.member_ptr = abi.ptr(self.member_ptr, C.c_uint32)
        p.member_field = abi.ptr(self.member_field, C.c_uint32)
        p.member_offset_xy = abi.ptr(self.member_offset_xy, C.c_double)
        p.member_charge = abi.ptr(self.member_charge, C.c_double)
        p.member_cell = abi.ptr(self.member_cell, C.c_uint32)
        p.num_cells = self.num_cells
        p.cell_unit = abi.ptr(self.cell_unit, C.c_uint32)
        p.cell_offset_xy = abi.ptr(self.cell_offset_xy, C.c_double)
        p.cell_fixed = abi.ptr(self.cell_fixed, C.c_uint8)
        p.cell_fixed_xy = abi.ptr(self.cell_fixed_xy, C.c_double)
        p.num_nets = self.num_nets
        p.net_ptr = abi.ptr(self.net_ptr, C.c_uint32)
        p.pin_cell = abi.ptr(self.pin_cell, C.c_uint32)
        p.num_timed_arcs = self.arc_driver_cell.shape[0]
        p.arc_driver_cell = abi.ptr(self.arc_driver_cell, C.c_uint32)
        p.arc_sink_cell = abi.ptr(self.arc_sink_cell, C.c_uint32)
        p.arc_extra_weight = abi.ptr(self.arc_extra_weight, C.c_uint64)
        self._c = p
        return p

    @staticmethod
    def from_c(pc, owner=None):
        """Copies a texo_gp_problem produced by the library into numpy arrays."""
        W, H, K = pc.width, pc.height, pc.num_fields
        U, Cn, E, A = pc.num_units, pc.num_cells, pc.num_nets, pc.num_timed_arcs

        def arr(p, n, dt):
            if n == 0:
                return np.zeros(0, dtype=dt)
            return np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True)
        fields = [(pc.fields[i].kind, pc.fields[i].lut_inputs) for i in range(K)]
        member_ptr = arr(pc.member_ptr, U + 1, np.uint32)
        M = int(member_ptr[-1])
        net_ptr = arr(pc.net_ptr, E + 1, np.uint32)
        P = int(net_ptr[-1])
        return Problem(
            W, H, fields, arr(pc.capacity, K * W * H, np.uint32),
            arr(pc.initial_xy, 2 * U, np.float64), arr(pc.lower_xy, 2 * U, np.float64),
            arr(pc.upper_xy, 2 * U, np.float64), member_ptr, arr(pc.member_field, M, np.uint32),
            arr(pc.member_offset_xy, 2 * M, np.float64), arr(pc.member_charge, M, np.float64),
            arr(pc.member_cell, M, np.uint32), arr(pc.cell_unit, Cn, np.uint32),
            arr(pc.cell_offset_xy, 2 * Cn, np.float64), arr(pc.cell_fixed, Cn, np.uint8),
            arr(pc.cell_fixed_xy, 2 * Cn, np.float64), net_ptr, arr(pc.pin_cell, P, np.uint32),
            arr(pc.arc_driver_cell, A, np.uint32), arr(pc.arc_sink_cell, A, np.uint32),
            arr(pc.arc_extra_weight, A, np.uint64),
            arr(pc.fixed_occupancy, 3 * pc.num_fixed_occupancy, np.uint32), _owner=owner)


def density_problem(width, height, fields, capacity, units, nets=(), fixed_occupancy=None,
                    bounds=None):
    """A density-only problem from reference-test style units.

    units: list of (origin_x, origin_y, [(field_index, dx, dy, charge), ...]).
    Every member is its own cell; nets (lists of cell ids, driver first) are
    optional. Bounds default to the whole tile grid.
    """
    U = len(units)
    initial, member_ptr, mf, mo, mq, mc = [], [0], [], [], [], []
    cell_unit, cell_off = [], []
    for u, (ox, oy, members) in enumerate(units):
        initial.append((ox, oy))
        for (f, dx, dy, q) in members:
            mf.append(f)
            mo.append((dx, dy))
            mq.append(q)
            mc.append(len(cell_unit))
            cell_unit.append(u)
            cell_off.append((dx, dy))
        member_ptr.append(len(mf))
    if bounds is None:
        lower = [(0.0, 0.0)] * U
        upper = [(float(width - 1), float(height - 1))] * U
    else:
        lower, upper = bounds
    Cn = len(cell_unit)
    net_ptr, pins = [0], []
    for net in nets:
        pins.extend(net)
        net_ptr.append(len(pins))
    return Problem(width, height, fields, capacity, initial, lower, upper, member_ptr, mf,
                   np.array(mo, dtype=np.float64).reshape(-1, 2), mq, mc, cell_unit,
                   np.array(cell_off, dtype=np.float64).reshape(-1, 2), np.zeros(Cn, np.uint8),
                   np.zeros((Cn, 2)), net_ptr, pins, fixed_occupancy=fixed_occupancy)


def synthetic(side, cells, io, nets, sigma, seed, p_local=0.8, jitter=1.0, lib=None):
    """The seeded ECP5-like netlist generator of the C library (host code)."""
    lib = lib or abi.load()
    spec = abi.SynthSpec(side, cells, io, nets, float(sigma), float(p_local), float(jitter), int(seed))
    h = C.c_void_p()
    pc = C.POINTER(abi.ProblemC)()
    abi.check(lib.texo_gp_synth_create(C.byref(spec), C.byref(h), C.byref(pc)), "texo_gp_synth_create")
    try:
        return Problem.from_c(pc.contents)
    finally:
        lib.texo_gp_synth_destroy(h)


# Benchmark workloads, sized as the reference's synthetic ECP5-like configs.
WORKLOADS = {
    # side, cells, io, nets, sigma, bins, target density, gamma base (bin widths)
    "ecp5-2k": dict(side=48, cells=2000, io=96, nets=2400, sigma=6.0, bins=64, td=1.0, gamma=4.0),
    "lfe5u-85-42k": dict(side=210, cells=42000, io=365, nets=50000, sigma=12.0, bins=256, td=0.9, gamma=4.0),
    "stress-1m": dict(side=1024, cells=1000000, io=4096, nets=1200000, sigma=24.0, bins=1024, td=0.9, gamma=4.0),
}

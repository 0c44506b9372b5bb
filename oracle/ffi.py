"""ctypes binding of the parity oracle (TEST INFRASTRUCTURE ONLY).

Loaded by the test suite, the smoke check and the benchmark's CPU-baseline
leg; never by the product package.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from texo_gb300 import abi  # noqa: E402  (data-format structs only)
from oracle import build as _build  # noqa: E402

c_f64p = C.POINTER(C.c_double)
c_u32p = C.POINTER(C.c_uint32)
c_u64p = C.POINTER(C.c_uint64)
c_i64p = C.POINTER(C.c_int64)


class FieldResult(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("lut_inputs", C.c_uint32),
                ("available_capacity", C.c_uint64), ("real_charge", C.c_uint64),
                ("real_area", C.c_double), ("filler_charge", C.c_double), ("energy", C.c_double),
                ("normalized_overflow", C.c_double), ("net_charge", C.c_double),
                ("force_l1", C.c_double)]


class RunStats(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("evaluations", C.c_uint64),
                ("line_search_trials", C.c_uint64), ("num_fields", C.c_uint32),
                ("overflow", C.c_double * abi.MAX_FIELDS), ("gamma", C.c_double),
                ("objective", C.c_double), ("converged", C.c_uint32), ("exhausted", C.c_uint32),
                ("inner_status", C.c_int32), ("hpwl", C.c_double)]


class NState(C.Structure):
    _fields_ = [("coordinates", c_f64p), ("previous", c_f64p), ("n", C.c_uint64),
                ("momentum", C.c_double), ("has_lipschitz", C.c_int32), ("lipschitz", C.c_double)]


class StepOut(C.Structure):
    _fields_ = [("stationary", C.c_int32), ("objective", C.c_double), ("stationarity", C.c_double),
                ("coordinate_change", C.c_double), ("trials", C.c_uint64), ("payload", C.c_int64),
                ("inner", C.c_int32), ("error_index", C.c_uint64), ("expected", C.c_uint64),
                ("actual", C.c_uint64)]


EVAL_CB = C.CFUNCTYPE(C.c_int32, C.c_void_p, c_f64p, C.c_uint64, c_f64p, c_f64p, c_u64p,
                      C.POINTER(C.c_int64))

_lib = None


class OrcRound(C.Structure):
    _fields_ = [("stop", C.c_int32), ("reset_multipliers", C.c_int32), ("density_scales", C.POINTER(C.c_double)),
                ("completed_iterations", C.c_uint64)]


class OrcRoundResult(C.Structure):
    _fields_ = [("completed_iterations", C.c_uint64), ("exhausted", C.c_uint32),
                ("density_scales", C.c_double * 4)]


class PcgStats(C.Structure):
    _fields_ = [("iterations", C.c_uint64), ("restarts", C.c_uint64), ("stop", C.c_int32),
                ("converged", C.c_int32), ("initial_residual_squared", C.c_double),
                ("target_squared", C.c_double), ("final_residual_squared", C.c_double)]


def solve_quadratic(diagonal, ptr, index, weight, rhs, solution=None):
    """solve_quadratic (lib.rs:4586-4752) restated in FP64: returns (x, stats, converged)."""
    n = len(diagonal)
    d = np.ascontiguousarray(diagonal, dtype=np.float64)
    p = np.ascontiguousarray(ptr, dtype=np.uint32)
    i = np.ascontiguousarray(index, dtype=np.uint32)
    w = np.ascontiguousarray(weight, dtype=np.float64)
    b = np.ascontiguousarray(rhs, dtype=np.float64)
    x = np.zeros(n) if solution is None else np.array(solution, dtype=np.float64, copy=True)
    st = PcgStats()
    code = lib().orc_solve_quadratic(n, P(d), P(p, C.c_uint32), P(i, C.c_uint32), P(w), P(b), P(x), C.byref(st))
    return x, st, code == 0


def routing_demand(width, height, boxes):
    """continuous_routing_demand (eplace.rs:856-937) in FP64: (h, v, ok)."""
    b = np.ascontiguousarray(boxes, dtype=np.float64).reshape(-1, 4)
    h = np.zeros(width * height)
    v = np.zeros(width * height)
    code = lib().orc_routing_demand(width, height, b.shape[0], P(b), P(h), P(v))
    return h.reshape(height, width), v.reshape(height, width), code == 0


class AuctionStats(C.Structure):
    _fields_ = [("bids", C.c_uint64), ("examined", C.c_uint64), ("unmatched", C.c_uint64),
                ("total_base_cost", C.c_uint64)]


def _stats(st, rounds=None):
    out = {"bids": st.bids, "candidates_examined": st.examined, "unmatched": st.unmatched,
           "total_base_cost": st.total_base_cost}
    if rounds is not None:
        out["rounds"] = rounds
    return out


def auction_explicit(domains, object_count, max_base_cost, cost_scale=1, jacobi=False):
    """assign_implicitly with explicit_best_two (auction.rs:131-272), one
    bidder at a time (or, with jacobi=True, all active bidders each round as
    the GPU bids), base costs times `cost_scale` (1 in the reference):
    (code, assignment with -1 for the dummy, prices, stats)."""
    n = len(domains)
    ptr = np.zeros(n + 1, dtype=np.uint32)
    if n:
        ptr[1:] = np.cumsum([len(d) for d in domains])
    obj = np.ascontiguousarray([o for d in domains for o, _ in d] or [0], dtype=np.uint32)
    cost = np.ascontiguousarray([c for d in domains for _, c in d] or [0], dtype=np.uint64)
    a = np.full(max(n, 1), -1, dtype=np.int32)
    pr = np.zeros(max(object_count, 1), dtype=np.uint64)
    st = AuctionStats()
    rounds = C.c_uint64()
    code = lib().orc_auction_explicit(n, object_count, max_base_cost, cost_scale, P(ptr, C.c_uint32),
                                      P(obj, C.c_uint32), P(cost, C.c_uint64), P(a, C.c_int32), P(pr, C.c_uint64),
                                      C.byref(st), C.byref(rounds) if jacobi else None)
    return code, a[:n], pr[:object_count], _stats(st, rounds.value if jacobi else None)


def _grid_args(grid):
    tobj = grid.tile_object if len(grid.tile_object) else np.zeros(1, np.uint32)
    occ = None if grid.occupied is None else np.ascontiguousarray(grid.occupied, dtype=np.uint8)
    return (grid.width, grid.height, grid.num_kinds,
            P(np.ascontiguousarray(grid.tile_ptr, dtype=np.uint32), C.c_uint32),
            P(np.ascontiguousarray(tobj, dtype=np.uint32), C.c_uint32), grid.num_objects,
            None if occ is None else P(occ, C.c_uint8))


def auction_singletons(grid, bidder_kind, targets, cost_scale=1, jacobi=False):
    """auction_singletons with the ring walk (legalization/mod.rs:657-1021),
    one bidder at a time (or, with jacobi=True, in the GPU's parallel
    rounds), base costs times `cost_scale` (1 in the reference):
    (code, assignment, prices, stats)."""
    kind = np.ascontiguousarray(bidder_kind, dtype=np.uint32).reshape(-1)
    txy = np.ascontiguousarray(targets, dtype=np.uint32).reshape(-1)
    n = kind.shape[0]
    a = np.full(max(n, 1), -1, dtype=np.int32)
    pr = np.zeros(max(grid.num_objects, 1), dtype=np.uint64)
    st = AuctionStats()
    rounds = C.c_uint64()
    code = lib().orc_auction_singletons(*_grid_args(grid), n, P(kind if n else np.zeros(1, np.uint32), C.c_uint32),
                                        P(txy if n else np.zeros(2, np.uint32), C.c_uint32), cost_scale,
                                        P(a, C.c_int32), P(pr, C.c_uint64), C.byref(st),
                                        C.byref(rounds) if jacobi else None)
    return code, a[:n], pr[:grid.num_objects], _stats(st, rounds.value if jacobi else None)


def auction_certificate(grid, bidder_kind, targets, assignment, prices, dual=False, cost_scale=1):
    """Epsilon-complementary-slackness check of a singleton result: (number
    of violations, first failing index or None, per-bidder base costs), plus
    with dual=True the assignment dual at these prices (a lower bound on the
    least total cost, dummies at n * max_base_cost + n + 1)."""
    kind = np.ascontiguousarray(bidder_kind, dtype=np.uint32).reshape(-1)
    txy = np.ascontiguousarray(targets, dtype=np.uint32).reshape(-1)
    n = kind.shape[0]
    a = np.ascontiguousarray(assignment, dtype=np.int32)
    pr = np.ascontiguousarray(prices, dtype=np.uint32)
    base = np.zeros(max(n, 1), dtype=np.uint64)
    first = C.c_uint64()
    bound = C.c_int64()
    bad = lib().orc_auction_check_singletons(*_grid_args(grid), n, P(kind, C.c_uint32), P(txy, C.c_uint32),
                                             cost_scale, P(a, C.c_int32),
                                             P(pr if len(pr) else np.zeros(1, np.uint32), C.c_uint32),
                                             P(base, C.c_uint64), C.byref(first), C.byref(bound))
    out = (bad, (None if first.value == 2**64 - 1 else first.value), base[:n])
    return out + (bound.value,) if dual else out


def register_clustering_areas(xy, clock_lsr, ce, movable_instance_count):
    """clustering_areas (register_clustering.rs:17-80) in FP64: (code, areas)."""
    p = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1)
    cl = np.ascontiguousarray(clock_lsr, dtype=np.uint64).reshape(-1)
    c = np.ascontiguousarray(ce, dtype=np.uint64).reshape(-1)
    n = c.shape[0]
    out = np.zeros(max(n, 1))
    code = lib().orc_register_clustering_areas(n, P(p), P(cl, C.c_uint64), P(c, C.c_uint64),
                                               movable_instance_count, P(out))
    return code, out[:n]


def soft_division_ceiling(value, divisor):
    return lib().orc_soft_division_ceiling(value, divisor)


def multiply_quadratic(diagonal, ptr, index, weight, values):
    n = len(diagonal)
    out = np.zeros(n)
    lib().orc_multiply_quadratic(n, P(np.ascontiguousarray(diagonal, dtype=np.float64)),
                                 P(np.ascontiguousarray(ptr, dtype=np.uint32), C.c_uint32),
                                 P(np.ascontiguousarray(index, dtype=np.uint32), C.c_uint32),
                                 P(np.ascontiguousarray(weight, dtype=np.float64)),
                                 P(np.ascontiguousarray(values, dtype=np.float64)), P(out))
    return out


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        sig = {
            "orc_bspline_axis": (None, [C.c_uint64, C.c_double, c_u64p, c_f64p, c_f64p]),
            "orc_deposit": (None, [c_f64p, C.c_uint64, C.c_uint64, C.c_double, C.c_double, C.c_double]),
            "orc_sample": (None, [c_f64p, C.c_uint64, C.c_uint64, C.c_double, C.c_double, c_f64p]),
            "orc_deposit_bilinear": (None, [c_f64p, C.c_uint64, C.c_uint64, C.c_double, C.c_double, C.c_double]),
            "orc_sample_bilinear": (None, [c_f64p, C.c_uint64, C.c_uint64, C.c_double, C.c_double, c_f64p]),
            "orc_poisson": (C.c_int32, [C.c_uint32, C.c_uint32, c_f64p, c_f64p, c_f64p, C.c_int32]),
            "orc_dct_basis": (None, [C.c_uint32, c_f64p]),
            "orc_create": (C.c_int32, [C.POINTER(abi.ProblemC), C.POINTER(abi.Params), C.POINTER(C.c_void_p), c_u64p]),
            "orc_destroy": (None, [C.c_void_p]),
            "orc_sizes": (None, [C.c_void_p, c_u64p, c_u64p, c_u64p, c_u32p, c_u32p, c_u32p]),
            "orc_initial": (None, [C.c_void_p, c_f64p, c_f64p, c_f64p]),
            "orc_fillers": (None, [C.c_void_p, c_u32p, c_f64p, c_f64p]),
            "orc_set_filler_charge": (None, [C.c_void_p, C.c_uint64, C.c_double]),
            "orc_capacity": (None, [C.c_void_p, C.c_uint32, c_u32p]),
            "orc_evaluate": (C.c_int32, [C.c_void_p, c_f64p, C.c_double, C.c_int32, c_f64p,
                                         C.POINTER(FieldResult), c_f64p, c_f64p, c_f64p, c_f64p, c_u64p]),
            "orc_scatter_fixed": (C.c_int32, [C.c_void_p, c_f64p, c_i64p, c_i64p, c_i64p, c_u64p]),
            "orc_place": (C.c_int32, [C.c_void_p, C.c_int32, C.c_uint32, c_u32p, c_f64p, C.POINTER(RunStats)]),
            "orc_hpwl": (C.c_int32, [C.c_void_p, c_f64p, c_f64p]),
            "orc_trace": (C.c_uint32, [C.c_void_p, C.POINTER(abi.Iteration), C.c_uint32]),
            "orc_set_charges": (C.c_int32, [C.c_void_p, c_f64p, c_f64p]),
            "orc_place_round": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(OrcRound), c_f64p, c_u32p, c_f64p,
                                            C.POINTER(RunStats), C.POINTER(OrcRoundResult)]),
            "orc_wirelength_preconditioner": (None, [C.c_void_p, c_f64p]),
            "orc_cell_incidence_weights": (None, [C.c_void_p, c_f64p]),
            "orc_nesterov_step": (C.c_int32, [C.POINTER(NState), c_f64p, C.c_uint64, c_f64p, C.c_uint64,
                                              c_f64p, C.c_uint64, EVAL_CB, C.c_void_p, C.POINTER(StepOut)]),
            "orc_nesterov_init": (None, [C.POINTER(NState), c_f64p, c_f64p, C.c_uint64, c_f64p, C.c_uint64]),
            "orc_box_metric_kkt": (C.c_double, [c_f64p, c_f64p, c_f64p, c_f64p, c_f64p, C.c_uint64]),
            "orc_augmented": (None, [C.c_double, C.c_double, C.c_double, C.c_double, c_f64p, c_f64p]),
            "orc_multiplier_growth": (C.c_int32, [C.c_double, C.c_double, C.c_double, c_f64p]),
            "orc_area_adjusted_multiplier_step": (C.c_int32, [c_f64p, C.c_uint64, C.c_double, c_f64p]),
            "orc_field_gamma": (C.c_int32, [C.c_double, C.c_double, C.c_double, c_f64p]),
            "orc_weighted_gamma_mean": (C.c_int32, [c_f64p, c_f64p, C.c_uint64, C.c_double, c_f64p]),
            "orc_overflow_target": (C.c_double, [C.c_uint32]),
            "orc_area_adjustment_ready": (C.c_int32, [C.c_uint32, c_u32p, c_f64p]),
            "orc_area_adjusted_multipliers": (C.c_int32, [C.c_uint32, c_f64p, c_f64p, c_f64p, C.c_double, c_f64p,
                                                          C.c_uint64, c_f64p]),
            "orc_checkpoint_better": (C.c_int32, [C.c_double, C.c_double, C.c_double, C.c_double]),
            "orc_validate_units": (C.c_int32, [c_u32p, C.c_uint64, c_u64p]),
            "orc_routing_demand": (C.c_int32, [C.c_uint32, C.c_uint32, C.c_uint64, c_f64p, c_f64p, c_f64p]),
            "orc_solve_quadratic": (C.c_int32, [C.c_uint64, c_f64p, c_u32p, c_u32p, c_f64p, c_f64p, c_f64p,
                                                C.POINTER(PcgStats)]),
            "orc_multiply_quadratic": (None, [C.c_uint64, c_f64p, c_u32p, c_u32p, c_f64p, c_f64p, c_f64p]),
            "orc_register_clustering_areas": (C.c_int32, [C.c_uint64, c_f64p, c_u64p, c_u64p, C.c_uint64, c_f64p]),
            "orc_soft_division_ceiling": (C.c_double, [C.c_double, C.c_double]),
            "orc_auction_explicit": (C.c_int32, [C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, c_u32p, c_u32p,
                                                 c_u64p, C.POINTER(C.c_int32), c_u64p, C.POINTER(AuctionStats),
                                                 c_u64p]),
            "orc_auction_singletons": (C.c_int32, [C.c_uint32, C.c_uint32, C.c_uint32, c_u32p, c_u32p, C.c_uint32,
                                                   C.POINTER(C.c_uint8), C.c_uint32, c_u32p, c_u32p, C.c_uint32,
                                                   C.POINTER(C.c_int32), c_u64p, C.POINTER(AuctionStats), c_u64p]),
            "orc_auction_check_singletons": (C.c_int64, [C.c_uint32, C.c_uint32, C.c_uint32, c_u32p, c_u32p,
                                                         C.c_uint32, C.POINTER(C.c_uint8), C.c_uint32, c_u32p,
                                                         c_u32p, C.c_uint32, C.POINTER(C.c_int32), c_u32p, c_u64p,
                                                         c_u64p,
                                                         c_i64p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def P(a, t=C.c_double):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


# ---- stencil and Poisson ---------------------------------------------------
def bspline_axis(length, coordinate):
    idx = np.zeros(3, np.uint64)
    w = np.zeros(3)
    d = np.zeros(3)
    lib().orc_bspline_axis(length, coordinate, P(idx, C.c_uint64), P(w), P(d))
    return idx, w, d


def deposit(density, width, height, x, y, charge):
    lib().orc_deposit(P(density), width, height, x, y, charge)


def sample(potential, width, height, x, y):
    out = np.zeros(3)
    lib().orc_sample(P(potential), width, height, x, y, P(out))
    return out


def deposit_bilinear(density, width, height, x, y, charge):
    lib().orc_deposit_bilinear(P(density), width, height, x, y, charge)


def sample_bilinear(potential, width, height, x, y):
    out = np.zeros(3)
    lib().orc_sample_bilinear(P(potential), width, height, x, y, P(out))
    return out


def poisson(width, height, density, matrix=False):
    d = np.ascontiguousarray(np.asarray(density, dtype=np.float64))
    pot = np.zeros(width * height)
    e = C.c_double()
    st = lib().orc_poisson(width, height, P(d), P(pot), C.byref(e), 1 if matrix else 0)
    if st:
        raise abi.TexoGpError(st, "orc_poisson")
    return pot, e.value


def dct_basis(n):
    b = np.zeros(n * n)
    lib().orc_dct_basis(n, P(b))
    return b.reshape(n, n)


# ---- problem-level oracle ---------------------------------------------------
class Oracle:
    """FP64 restatement of the reference on one problem."""

    def __init__(self, problem, params=None):
        self.problem = problem
        self.params = params or abi.default_params_py()
        self._pc = problem.c_struct()
        h = C.c_void_p()
        err = C.c_uint64()
        st = lib().orc_create(C.byref(self._pc), C.byref(self.params), C.byref(h), C.byref(err))
        if st:
            self.h = None
            raise abi.TexoGpError(st, "orc_create", "index %d" % err.value)
        self.h = h
        u, f, n = C.c_uint64(), C.c_uint64(), C.c_uint64()
        bx, by, k = C.c_uint32(), C.c_uint32(), C.c_uint32()
        lib().orc_sizes(h, C.byref(u), C.byref(f), C.byref(n), C.byref(bx), C.byref(by), C.byref(k))
        self.units, self.num_fillers, self.n = u.value, f.value, n.value
        self.bins_x, self.bins_y, self.num_fields = bx.value, by.value, k.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    @property
    def bins(self):
        return self.bins_x * self.bins_y

    def initial(self):
        c, lo, hi = np.zeros(self.n), np.zeros(self.n), np.zeros(self.n)
        lib().orc_initial(self.h, P(c), P(lo), P(hi))
        return c, lo, hi

    def fillers(self):
        f = np.zeros(self.num_fillers, np.uint32)
        q = np.zeros(self.num_fillers)
        xy = np.zeros(2 * self.num_fillers)
        lib().orc_fillers(self.h, P(f, C.c_uint32), P(q), P(xy))
        return f, q, xy.reshape(-1, 2)

    def set_filler_charge(self, i, q):
        lib().orc_set_filler_charge(self.h, i, q)

    def capacity(self, field):
        out = np.zeros(self.problem.width * self.problem.height, np.uint32)
        lib().orc_capacity(self.h, field, P(out, C.c_uint32))
        return out

    def evaluate(self, coords, gamma, threads=1, arrays=True):
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        K, n, B = self.num_fields, self.n, self.bins
        fr = (FieldResult * max(1, K))()
        wa = C.c_double()
        err = C.c_uint64()
        wag = np.zeros(2 * self.units) if arrays else None
        fg = np.zeros(K * n) if arrays else None
        dens = np.zeros(K * B) if arrays else None
        pot = np.zeros(K * B) if arrays else None
        st = lib().orc_evaluate(self.h, P(coords), gamma, threads, C.byref(wa), fr, P(wag), P(fg),
                                P(dens), P(pot), C.byref(err))
        if st:
            raise abi.TexoGpError(st, "orc_evaluate", "index %d" % err.value)
        out = {"wirelength": wa.value, "fields": [fr[i] for i in range(K)]}
        if arrays:
            out.update(wa_gradient=wag, field_gradient=fg.reshape(K, n),
                       density=dens.reshape(K, B), potential=pot.reshape(K, B))
        return out

    def scatter_fixed(self, coords):
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        K, B = self.num_fields, self.bins
        phys = np.zeros(K * B, np.int64)
        fill = np.zeros(K * B, np.int64)
        ov = np.zeros(max(1, K), np.int64)
        cnt = np.zeros(max(1, K), np.uint64)
        lib().orc_scatter_fixed(self.h, P(coords), P(phys, C.c_int64), P(fill, C.c_int64),
                                P(ov, C.c_int64), P(cnt, C.c_uint64))
        return phys.reshape(K, B), fill.reshape(K, B), ov[:K], cnt[:K]

    def place(self, threads=1, max_iterations=0):
        t = np.zeros(2 * self.units, np.uint32)
        c = np.zeros(self.n)
        s = RunStats()
        st = lib().orc_place(self.h, threads, max_iterations, P(t, C.c_uint32), P(c), C.byref(s))
        return st, t.reshape(-1, 2), c, s

    def hpwl(self, coords):
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        out = C.c_double()
        lib().orc_hpwl(self.h, P(coords), C.byref(out))
        return out.value

    def set_charges(self, member_charge=None, filler_charge=None):
        m = None if member_charge is None else np.ascontiguousarray(member_charge, dtype=np.float64)
        q = None if filler_charge is None else np.ascontiguousarray(filler_charge, dtype=np.float64)
        lib().orc_set_charges(self.h, P(m), P(q))

    def place_round(self, stop, reset_multipliers, density_scales=None, completed_iterations=0, coordinates=None,
                    threads=1):
        """One round of eplace::place's area loop (optimize_density_once) from
        `coordinates` (None: the initial ones): (status, targets, coords, stats, result)."""
        r = OrcRound()
        r.stop = int(stop)
        r.reset_multipliers = 1 if reset_multipliers else 0
        sc = None
        if density_scales is not None:
            sc = np.ascontiguousarray(density_scales, dtype=np.float64)
            r.density_scales = P(sc)
        r.completed_iterations = int(completed_iterations)
        cin = None if coordinates is None else np.ascontiguousarray(coordinates, dtype=np.float64)
        t = np.zeros(2 * self.units, np.uint32)
        c = np.zeros(self.n)
        s = RunStats()
        res = OrcRoundResult()
        st = lib().orc_place_round(self.h, threads, C.byref(r), P(cin), P(t, C.c_uint32), P(c), C.byref(s),
                                   C.byref(res))
        out = {"completed_iterations": res.completed_iterations, "exhausted": bool(res.exhausted),
               "density_scales": [res.density_scales[f] for f in range(self.num_fields)]}
        return st, t.reshape(-1, 2), c, s, out

    def trace(self):
        """Controller records of the last place() (texo_gp_iteration each)."""
        n = lib().orc_trace(self.h, None, 0)
        buf = (abi.Iteration * max(1, n))()
        lib().orc_trace(self.h, buf, n)
        return [buf[i] for i in range(n)]

    def wirelength_preconditioner(self):
        out = np.zeros(self.units)
        lib().orc_wirelength_preconditioner(self.h, P(out))
        return out

    def cell_incidence_weights(self):
        out = np.zeros(self.problem.num_cells)
        lib().orc_cell_incidence_weights(self.h, P(out))
        return out


# ---- Nesterov step with a Python evaluator ----------------------------------
class NesterovState:
    def __init__(self, coordinates, previous=None, momentum=1.0, lipschitz=None):
        self.x = np.array(coordinates, dtype=np.float64)
        self.prev = np.array(self.x if previous is None else previous, dtype=np.float64)
        self.momentum = float(momentum)
        self.lipschitz = lipschitz

    @staticmethod
    def new(initial, lower, upper):
        initial = np.array(initial, dtype=np.float64)
        lower = np.array(lower, dtype=np.float64)
        upper = np.array(upper, dtype=np.float64)
        s = NesterovState(initial)
        ns = s._c()
        lib().orc_nesterov_init(C.byref(ns), P(initial), P(lower), lower.size, P(upper), upper.size)
        s._read(ns)
        return s

    def _c(self):
        ns = NState()
        ns.coordinates = P(self.x)
        ns.previous = P(self.prev)
        ns.n = self.x.size
        ns.momentum = self.momentum
        ns.has_lipschitz = 0 if self.lipschitz is None else 1
        ns.lipschitz = 0.0 if self.lipschitz is None else float(self.lipschitz)
        return ns

    def _read(self, ns):
        self.momentum = ns.momentum
        self.lipschitz = ns.lipschitz if ns.has_lipschitz else None

    def key(self):
        return (self.x.tobytes(), self.prev.tobytes(), self.momentum, self.lipschitz)


def nesterov_step(state, lower, upper, metric, evaluate):
    """evaluate(coords) -> (value, gradient, payload) or raises/returns an int error."""
    lower = np.ascontiguousarray(lower, dtype=np.float64)
    upper = np.ascontiguousarray(upper, dtype=np.float64)
    metric = np.ascontiguousarray(metric, dtype=np.float64)

    def cb(user, coords, n, value, grad, glen, payload):
        c = np.ctypeslib.as_array(coords, shape=(n,)).copy() if n else np.zeros(0)
        r = evaluate(c)
        if isinstance(r, int):
            return r
        v, g, pl = r
        g = np.asarray(g, dtype=np.float64)
        value[0] = v
        for i in range(min(g.size, n + 64)):
            grad[i] = g[i]
        glen[0] = g.size
        payload[0] = int(pl)
        return 0
    ccb = EVAL_CB(cb)
    ns = state._c()
    out = StepOut()
    st = lib().orc_nesterov_step(C.byref(ns), P(lower), lower.size, P(upper), upper.size, P(metric),
                                 metric.size, ccb, None, C.byref(out))
    if st == 0:
        state._read(ns)
    return st, out


def box_metric_kkt(gradient, coordinates, lower, upper, metric):
    a = [np.ascontiguousarray(v, dtype=np.float64) for v in (gradient, coordinates, lower, upper, metric)]
    return lib().orc_box_metric_kkt(P(a[0]), P(a[1]), P(a[2]), P(a[3]), P(a[4]), a[0].size)

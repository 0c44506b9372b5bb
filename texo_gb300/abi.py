"""ctypes mirror of include/texo_gp.h (the C ABI of the placement engine).

The structures here are byte-for-byte the C declarations; `load()` opens the
in-tree CUDA library built by `texo_gb300.build`. There is no CPU fallback:
if the library is missing, `load()` raises.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libtexo_gp.so")

# texo_gp_status (include/texo_gp.h), one per reference error variant.
STATUS = {
    0: "OK",
    1: "EMPTY_GRID", 2: "GRID_TOO_LARGE", 3: "DENSITY_LENGTH", 4: "NONFINITE_DENSITY",
    5: "EMPTY_UNIT", 6: "NONFINITE_UNIT_COORDINATE", 7: "INVALID_MEMBER_CHARGE",
    8: "POINT_OUTSIDE_GRID", 9: "FIXED_CAPACITY_EXHAUSTED", 10: "INSUFFICIENT_CAPACITY",
    11: "INSUFFICIENT_AREA", 12: "NONFINITE_FILLER", 13: "NEGATIVE_FILLER_CHARGE",
    14: "UNEXPECTED_FILLER_KIND", 15: "FILLER_CHARGE_MISMATCH",
    32: "INVALID_BOUNDS", 33: "INVALID_METRIC_LENGTH", 34: "NONPOSITIVE_METRIC",
    35: "INVALID_INITIAL_COORDINATE", 36: "INVALID_MOMENTUM_PARAMETER",
    37: "INVALID_LIPSCHITZ_ESTIMATE", 38: "INVALID_OBJECTIVE", 39: "INVALID_GRADIENT_LENGTH",
    40: "NONFINITE_GRADIENT", 41: "LINE_SEARCH_OVERFLOW", 42: "ITERATION_OVERFLOW",
    43: "EVALUATION",
    64: "DENSITY_FIELD_CHANGED", 65: "INVALID_NORMALIZATION", 66: "DID_NOT_CONVERGE",
    96: "INVALID_ARGUMENT", 97: "CUDA", 98: "OUT_OF_MEMORY", 99: "DEVICE_TIMEOUT",
    100: "FIXED_POINT_RANGE", 101: "UNSUPPORTED", 102: "BUSY",
    110: "PCG_NOT_CONVERGED",
    111: "AUCTION_RANGE", 112: "AUCTION_OBJECT_RANGE", 113: "AUCTION_COST_RANGE",
    114: "AUCTION_DUPLICATE_OBJECT",
    115: "INSTANCE_AREA_MEMBER", 116: "INSTANCE_AREA_FILLER", 117: "INSTANCE_AREA_POSTCONDITION",
    118: "INSTANCE_AREA_OVERFLOW",
    119: "PROJECTION_CONFLICT",
    120: "NO_BEL",
}
CODE = {v: k for k, v in STATUS.items()}

KIND_LOGIC, KIND_LUT, KIND_REGISTER, KIND_MEMORY, KIND_CLOCK, KIND_IO, KIND_CONSTANT, KIND_DSP = range(8)
DCT_FP32, DCT_TENSOR, DCT_FP32_GEMM = 0, 1, 2
DCT_BF16X3 = DCT_TENSOR   # earlier name of the tensor-core mode
ENGINE_HOST, ENGINE_DEVICE = 0, 1
SCATTER_AUTO, SCATTER_DIRECT, SCATTER_TILED = 0, 1, 2
MAX_FIELDS = 4

c_u32p = C.POINTER(C.c_uint32)
c_u64p = C.POINTER(C.c_uint64)
c_i64p = C.POINTER(C.c_int64)
c_f64p = C.POINTER(C.c_double)
c_u8p = C.POINTER(C.c_uint8)


class TexoGpError(RuntimeError):
    def __init__(self, code, where="", detail=""):
        self.code = int(code)
        self.name = STATUS.get(self.code, "UNKNOWN_%d" % self.code)
        msg = "%s failed: %s" % (where, self.name) if where else self.name
        if detail:
            msg += " (" + detail + ")"
        super().__init__(msg)


class Field(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("lut_inputs", C.c_uint32)]


class ProblemC(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32),
        ("num_fields", C.c_uint32), ("fields", C.POINTER(Field)),
        ("capacity", c_u32p),
        ("num_fixed_occupancy", C.c_uint32), ("fixed_occupancy", c_u32p),
        ("num_units", C.c_uint32),
        ("initial_xy", c_f64p), ("lower_xy", c_f64p), ("upper_xy", c_f64p),
        ("member_ptr", c_u32p), ("member_field", c_u32p), ("member_offset_xy", c_f64p),
        ("member_charge", c_f64p), ("member_cell", c_u32p),
        ("num_cells", C.c_uint32), ("cell_unit", c_u32p), ("cell_offset_xy", c_f64p),
        ("cell_fixed", c_u8p), ("cell_fixed_xy", c_f64p),
        ("num_nets", C.c_uint32), ("net_ptr", c_u32p), ("pin_cell", c_u32p),
        ("num_timed_arcs", C.c_uint32), ("arc_driver_cell", c_u32p), ("arc_sink_cell", c_u32p),
        ("arc_extra_weight", c_u64p),
    ]


class Params(C.Structure):
    _fields_ = [
        ("gamma_base", C.c_double), ("max_iterations", C.c_uint32), ("beta", C.c_double),
        ("initial_density_weight", C.c_double), ("alpha_low", C.c_double),
        ("alpha_high", C.c_double), ("overflow_target_override", C.c_double),
        ("bins_x", C.c_uint32), ("bins_y", C.c_uint32), ("target_density", C.c_double),
        ("best_effort", C.c_int32), ("dct_mode", C.c_int32), ("engine", C.c_int32),
        ("device", C.c_int32), ("objective_margin_ulps", C.c_double),
        ("autotune", C.c_int32), ("scatter_mode", C.c_int32), ("reserved", C.c_uint32 * 6),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("status", C.c_int32), ("iterations", C.c_uint32), ("evaluations", C.c_uint64),
        ("line_search_trials", C.c_uint64), ("num_fields", C.c_uint32),
        ("overflow", C.c_double * MAX_FIELDS), ("energy", C.c_double * MAX_FIELDS),
        ("gamma", C.c_double), ("objective", C.c_double), ("hpwl", C.c_double),
        ("error_index", C.c_uint64), ("error_field", C.c_uint32), ("converged", C.c_uint32),
        ("elapsed_ms", C.c_double), ("kernel_launches", C.c_uint64),
        ("density_evaluations", C.c_uint64),
    ]


class Iteration(C.Structure):
    """texo_gp_iteration: one eplace iteration as the controller saw it."""
    _fields_ = [("iteration", C.c_uint32), ("trials", C.c_uint32), ("gamma", C.c_double),
                ("objective", C.c_double), ("lipschitz", C.c_double), ("momentum", C.c_double),
                ("lambda_", C.c_double * 4), ("energy_scale", C.c_double * 4), ("overflow", C.c_double * 4)]


class Round(C.Structure):
    """texo_gp_round: one round of the area-adjustment loop."""
    _fields_ = [("stop", C.c_int32), ("reset_multipliers", C.c_int32), ("density_scales", C.POINTER(C.c_double)),
                ("completed_iterations", C.c_uint64), ("reserved", C.c_uint32 * 4)]


class RoundResult(C.Structure):
    _fields_ = [("completed_iterations", C.c_uint64), ("exhausted", C.c_uint32), ("reserved", C.c_uint32),
                ("density_scales", C.c_double * 4)]


class RoutingCapacity(C.Structure):
    """texo_gp_routing_capacity: RoutingCapacityMap's channel capacities."""
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("horizontal", C.POINTER(C.c_uint32)),
                ("vertical", C.POINTER(C.c_uint32))]


class RegisterControl(C.Structure):
    """texo_gp_register_control: RegisterControlSet (cell, clock_lsr, ce)."""
    _fields_ = [("cell", C.c_uint32), ("reserved", C.c_uint32), ("clock_lsr", C.c_uint64 * 2), ("ce", C.c_uint64)]


class RoutableReport(C.Structure):
    _fields_ = [("rounds", C.c_uint32), ("area_rounds", C.c_uint32), ("iterations", C.c_uint64),
                ("last_relative_increase", C.c_double), ("last_maximum_relative_increase", C.c_double),
                ("max_horizontal_utilization", C.c_double), ("max_vertical_utilization", C.c_double),
                ("last_members_inflated", C.c_uint64), ("reserved", C.c_uint32 * 8)]


class ChoiceTable(C.Structure):
    """texo_gp_choice_table: a unit's choice rows."""
    _fields_ = [("num_choices", C.c_uint32), ("width", C.c_uint32), ("bels", C.POINTER(C.c_uint32)),
                ("shared", C.c_int32), ("reserved", C.c_uint32)]


class ProjectionStats(C.Structure):
    _fields_ = [("fixed_units", C.c_uint64), ("overlapping_shared_families", C.c_uint64),
                ("overlapping_shared_units", C.c_uint64), ("disjoint_shared_families", C.c_uint64),
                ("disjoint_shared_units", C.c_uint64), ("singleton_units", C.c_uint64),
                ("relaxed_unmatched_units", C.c_uint64), ("bids", C.c_uint64), ("candidates_examined", C.c_uint64),
                ("auctions", C.c_uint64), ("elapsed_ms", C.c_double), ("reserved", C.c_uint32 * 8)]


class Legality(C.Structure):
    """texo_gp_legality: pin wires and shared resources of the repair."""
    _fields_ = [("num_wires", C.c_uint32), ("wire_capacity", C.POINTER(C.c_uint32)),
                ("num_cell_pins", C.c_uint32), ("cell_pin_cell", C.POINTER(C.c_uint32)),
                ("cell_pin_key", C.POINTER(C.c_uint32)), ("cell_pin_net", C.POINTER(C.c_uint32)),
                ("num_bel_pins", C.c_uint32), ("bel_pin_bel", C.POINTER(C.c_uint32)),
                ("bel_pin_key", C.POINTER(C.c_uint32)), ("bel_pin_wire", C.POINTER(C.c_uint32)),
                ("num_rules", C.c_uint32), ("num_cell_values", C.c_uint32),
                ("cell_value_rule", C.POINTER(C.c_uint32)), ("cell_value_cell", C.POINTER(C.c_uint32)),
                ("cell_value", C.POINTER(C.c_uint64)), ("num_bel_resources", C.c_uint32),
                ("bel_resource_rule", C.POINTER(C.c_uint32)), ("bel_resource_bel", C.POINTER(C.c_uint32)),
                ("bel_resource", C.POINTER(C.c_uint64))]


class RepairStats(C.Structure):
    _fields_ = [("initial_pending", C.c_uint64), ("direct_fast_choices", C.c_uint64),
                ("direct_fast_moves", C.c_uint64), ("direct_fast_fallbacks", C.c_uint64),
                ("augmenting_roots", C.c_uint64), ("augmenting_fallbacks", C.c_uint64),
                ("states_visited", C.c_uint64), ("failed_states", C.c_uint64), ("max_unplaced", C.c_uint64),
                ("max_blocker_branches", C.c_uint64), ("units_evicted", C.c_uint64),
                ("choices_examined", C.c_uint64), ("elapsed_ms", C.c_double), ("failed_cell", C.c_uint32),
                ("reserved", C.c_uint32 * 7)]


class FieldEval(C.Structure):
    _fields_ = [
        ("energy", C.c_double), ("normalized_overflow", C.c_double), ("net_charge", C.c_double),
        ("force_l1", C.c_double), ("real_area", C.c_double), ("filler_charge", C.c_double),
        ("overflow_fixed", C.c_int64), ("overflow_bins", C.c_uint64),
    ]


class Eval(C.Structure):
    _fields_ = [("wirelength", C.c_double), ("num_fields", C.c_uint32),
                ("fields", FieldEval * MAX_FIELDS)]


class PcgStats(C.Structure):
    _fields_ = [("status", C.c_int32), ("iterations", C.c_uint32), ("restarts", C.c_uint32), ("stop", C.c_int32),
                ("initial_residual_squared", C.c_double), ("target_squared", C.c_double),
                ("final_residual_squared", C.c_double), ("elapsed_ms", C.c_double),
                ("kernel_launches", C.c_uint64)]


class AuctionStats(C.Structure):
    _fields_ = [("status", C.c_int32), ("rounds", C.c_uint32), ("cost_scale", C.c_uint32),
                ("tail_rounds", C.c_uint32), ("bids", C.c_uint64),
                ("candidates_examined", C.c_uint64), ("unmatched", C.c_uint64),
                ("total_base_cost", C.c_uint64), ("elapsed_ms", C.c_double), ("kernel_launches", C.c_uint64)]


class ServerOptions(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_resident", C.c_uint32), ("chunk_iterations", C.c_uint32),
                ("admission_threads", C.c_uint32), ("reserved", C.c_uint32 * 5)]


class JobResult(C.Structure):
    _fields_ = [("job_id", C.c_uint64), ("status", C.c_int32), ("units", C.c_uint32), ("stats", Stats),
                ("submit_ms", C.c_double), ("admit_ms", C.c_double), ("finish_ms", C.c_double)]


class SynthSpec(C.Structure):
    _fields_ = [("side", C.c_uint32), ("cells", C.c_uint32), ("io", C.c_uint32),
                ("nets", C.c_uint32), ("sigma", C.c_double), ("p_local", C.c_double),
                ("jitter", C.c_double), ("seed", C.c_uint64)]


def default_params_py():
    """The reference constants (eplace.rs:125-134), without loading the library."""
    p = Params()
    p.gamma_base = 8.0
    p.max_iterations = 3000
    p.beta = 2000.0
    p.initial_density_weight = 1.0e-4
    p.alpha_low = 1.05
    p.alpha_high = 1.06
    p.overflow_target_override = -1.0
    p.bins_x = 0
    p.bins_y = 0
    p.target_density = 1.0
    p.best_effort = 0
    p.dct_mode = DCT_FP32
    p.engine = ENGINE_HOST
    p.device = 0
    p.objective_margin_ulps = 64.0
    p.autotune = 0
    return p


# Every symbol include/texo_gp.h declares, with its ctypes signature.
_P = C.c_void_p
SIGNATURES = {
    "texo_gp_abi_version": (C.c_uint32, []),
    "texo_gp_default_params": (None, [C.POINTER(Params)]),
    "texo_gp_status_name": (C.c_char_p, [C.c_int32]),
    "texo_gp_last_error": (C.c_char_p, []),
    "texo_gp_place": (C.c_int32, [C.POINTER(ProblemC), C.POINTER(Params), c_u32p, c_f64p, C.POINTER(Stats)]),
    "texo_gp_create": (C.c_int32, [C.POINTER(ProblemC), C.POINTER(Params), C.POINTER(_P)]),
    "texo_gp_destroy": (C.c_int32, [_P]),
    "texo_gp_sizes": (C.c_int32, [_P, c_u64p, c_u64p, c_u64p, c_u32p, c_u32p, c_u32p]),
    "texo_gp_initial": (C.c_int32, [_P, c_f64p, c_f64p, c_f64p]),
    "texo_gp_fillers": (C.c_int32, [_P, c_u32p, c_f64p]),
    "texo_gp_evaluate": (C.c_int32, [_P, c_f64p, C.c_double, C.POINTER(Eval), c_f64p, c_f64p, c_f64p, c_f64p]),
    "texo_gp_scatter": (C.c_int32, [_P, c_f64p, c_i64p, c_i64p]),
    "texo_gp_poisson": (C.c_int32, [_P, c_f64p, c_f64p, c_f64p]),
    "texo_gp_scatter_static": (C.c_int32, [_P, c_f64p, c_i64p, c_i64p]),
    "texo_gp_run": (C.c_int32, [_P, C.c_uint32, c_u32p, c_f64p, C.POINTER(Stats)]),
    "texo_gp_dct_form": (C.c_int32, [_P, C.POINTER(C.c_int32)]),
    "texo_gp_reset": (C.c_int32, [_P]),
    "texo_gp_optimize_round": (C.c_int32, [_P, C.POINTER(Round), c_u32p, c_f64p, C.POINTER(Stats),
                                           C.POINTER(RoundResult)]),
    "texo_gp_set_charges": (C.c_int32, [_P, c_f64p, c_f64p]),
    "texo_gp_project": (C.c_int32, [C.c_int32, C.c_uint32, C.c_uint32, C.c_uint32, c_u32p, C.c_uint32,
                                    C.POINTER(ChoiceTable), C.c_uint32, c_u32p, c_u32p, c_u32p, C.c_uint32,
                                    C.POINTER(C.c_int32), C.POINTER(ProjectionStats)]),
    "texo_gp_repair": (C.c_int32, [C.c_uint32, C.c_uint32, C.c_uint32, c_u32p, C.c_uint32, C.POINTER(ChoiceTable),
                                   C.c_uint32, c_u32p, c_u32p, c_u32p, C.c_uint32, c_u32p, C.POINTER(C.c_int32),
                                   c_u8p, C.POINTER(Legality), C.POINTER(C.c_int32), C.POINTER(RepairStats)]),
    "texo_gp_place_routable": (C.c_int32, [C.POINTER(ProblemC), C.POINTER(Params), C.POINTER(RoutingCapacity),
                                           C.c_uint64, C.POINTER(RegisterControl), c_u32p, c_f64p,
                                           C.POINTER(Stats), C.POINTER(RoutableReport)]),
    "texo_gp_hpwl": (C.c_int32, [_P, c_f64p, c_f64p]),
    "texo_gp_trace": (C.c_int32, [_P, C.POINTER(Iteration), C.c_uint32, c_u32p]),
    "texo_gp_stage_times": (C.c_int32, [_P, C.c_uint32, c_f64p, C.c_uint32, c_u32p]),
    "texo_gp_stage_name": (C.c_char_p, [C.c_uint32]),
    "texo_gp_device_profile": (C.c_int32, [_P, c_f64p]),
    "texo_gp_synth_create": (C.c_int32, [C.POINTER(SynthSpec), C.POINTER(_P), C.POINTER(C.POINTER(ProblemC))]),
    "texo_gp_synth_destroy": (C.c_int32, [_P]),
    "texo_gp_batch_create": (C.c_int32, [C.POINTER(Params), C.c_uint64, C.c_uint32, C.POINTER(_P)]),
    "texo_gp_batch_destroy": (C.c_int32, [_P]),
    "texo_gp_batch_admit": (C.c_int32, [_P, C.POINTER(ProblemC), C.POINTER(Params), C.c_uint64, c_u32p]),
    "texo_gp_batch_advance": (C.c_int32, [_P, C.c_uint32]),
    "texo_gp_batch_retire": (C.c_int32, [_P, c_u64p, c_u32p, C.c_uint64, C.POINTER(Stats)]),
    "texo_gp_batch_counts": (C.c_int32, [_P, c_u32p, c_u32p, c_u64p]),
    "texo_gp_batch_graphs": (C.c_int32, [_P, c_u64p, c_u64p]),
    "texo_gp_server_create": (C.c_int32, [C.POINTER(Params), C.POINTER(ServerOptions), C.POINTER(_P)]),
    "texo_gp_server_destroy": (C.c_int32, [_P]),
    "texo_gp_server_submit": (C.c_int32, [_P, C.POINTER(ProblemC), C.POINTER(Params), C.c_uint64]),
    "texo_gp_server_poll": (C.c_int32, [_P, C.c_int32, C.POINTER(JobResult), c_u32p, C.c_uint64]),
    "texo_gp_server_counts": (C.c_int32, [_P, c_u32p, c_u32p, c_u32p, c_u64p]),
    "texo_gp_server_clock_ms": (C.c_double, [_P]),
    "texo_gp_selftest_waits": (C.c_int32, [C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "texo_gp_routing_demand": (C.c_int32, [C.c_int32, C.c_uint32, C.c_uint32, C.c_uint64, C.POINTER(C.c_double),
                                           C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "texo_gp_quadratic_solve": (C.c_int32, [C.c_int32, C.c_uint32, C.POINTER(C.c_double), C.POINTER(C.c_uint32),
                                            C.POINTER(C.c_uint32), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                            C.POINTER(C.c_double), C.POINTER(PcgStats)]),
    "texo_gp_adjust_instance_areas": (C.c_int32, [C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_double),
                                                  C.POINTER(C.c_double), C.POINTER(C.c_double),
                                                  C.POINTER(C.c_double), C.c_uint64, C.POINTER(C.c_uint32),
                                                  C.POINTER(C.c_double), C.POINTER(C.c_double),
                                                  C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_uint32,
                                                  C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                                  C.POINTER(C.c_double), C.POINTER(C.c_uint64)]),
    "texo_gp_routability_optimized_area": (C.c_int32, [C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double)]),
    "texo_gp_routability_optimized_area_from_bin": (C.c_int32, [C.c_double, C.c_double, C.c_uint64, C.c_double,
                                                                C.c_uint64, C.POINTER(C.c_double)]),
    "texo_gp_pin_optimized_area": (C.c_int32, [C.c_uint64, C.c_double, C.c_double, C.POINTER(C.c_double)]),
    "texo_gp_register_clustering_areas": (C.c_int32, [C.c_int32, C.c_uint64, C.POINTER(C.c_double),
                                                      C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_uint64,
                                                      C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "texo_gp_auction_explicit": (C.c_int32, [C.c_int32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32,
                                             C.POINTER(C.c_uint32),
                                             C.POINTER(C.c_uint32), C.POINTER(C.c_uint64), C.POINTER(C.c_int32),
                                             C.POINTER(C.c_uint32), C.POINTER(AuctionStats)]),
    "texo_gp_auction_singletons": (C.c_int32, [C.c_int32, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32),
                                               C.POINTER(C.c_uint32), C.c_uint32, C.POINTER(C.c_uint8), C.c_uint32,
                                               C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_uint32,
                                               C.POINTER(C.c_int32), C.POINTER(C.c_uint32), C.POINTER(AuctionStats)]),
}

_lib = None


def load(path=None):
    """Opens the in-tree engine library (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("texo_gp CUDA library not built: %s (run texo_gb300.build.build())" % p)
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(code, where=""):
    if code != 0:
        detail = ""
        if code in (CODE["CUDA"], CODE["INVALID_ARGUMENT"]) and _lib is not None:
            detail = (_lib.texo_gp_last_error() or b"").decode()
        raise TexoGpError(code, where, detail)
    return code


def ptr(arr, ctype):
    """ctypes pointer into a contiguous numpy array (None for None)."""
    if arr is None:
        return None
    return arr.ctypes.data_as(C.POINTER(ctype))

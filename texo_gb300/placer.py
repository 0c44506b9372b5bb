"""Python mirror of the reference's global-placement entry points.

`place(problem, params)` is `eplace::place` (crates/texo-pnr/src/eplace.rs:242-421):
it returns the rounded unit targets of the best checkpoint, or raises
`TexoGpError` carrying the reference error variant. `Placer` exposes the
device-resident handle underneath for per-stage parity checks
(`ContinuousProblem::evaluate`, eplace.rs:137-205), resumable runs and
stage timing. Every call goes through the C ABI of include/texo_gp.h; there
is no CPU path.
"""
import ctypes as C

import numpy as np

from . import abi


def default_params(**overrides):
    p = abi.Params()
    abi.load().texo_gp_default_params(C.byref(p))
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def _stats_dict(s):
    K = s.num_fields
    return dict(status=abi.STATUS.get(s.status, s.status), iterations=s.iterations,
                evaluations=s.evaluations, line_search_trials=s.line_search_trials,
                overflow=[s.overflow[i] for i in range(K)], energy=[s.energy[i] for i in range(K)],
                gamma=s.gamma, objective=s.objective, hpwl=s.hpwl, converged=bool(s.converged),
                elapsed_ms=s.elapsed_ms, kernel_launches=s.kernel_launches,
                density_evaluations=s.density_evaluations)


def place(problem, params=None, coordinates=False):
    """eplace::place through texo_gp_place: returns (targets [U,2] uint32,
    coordinates, stats dict). The continuous coordinates [2(U+F)] float64
    come back with coordinates=True; their length is known only once the
    fillers exist, so that form runs the same create / run / destroy
    through a Placer. Otherwise coordinates is None."""
    params = params or default_params()
    if coordinates:
        with Placer(problem, params) as h:
            targets, coords, stats = h.run()
        return targets, coords, stats
    lib = abi.load()
    pc = problem.c_struct()
    targets = np.zeros(2 * problem.num_units, np.uint32)
    st = abi.Stats()
    code = lib.texo_gp_place(C.byref(pc), C.byref(params), abi.ptr(targets, C.c_uint32), None, C.byref(st))
    abi.check(code, "texo_gp_place")
    return targets.reshape(-1, 2), None, _stats_dict(st)


def place_with_routing_capacity(problem, params, capacity_h, capacity_v, register_controls=None, coordinates=False):
    """eplace::place with routing_capacity / register_controls
    (eplace.rs:242-420) through texo_gp_place_routable: the area rounds, the
    proposals and their installation in one native call. capacity_h /
    capacity_v: [H, W] channel capacities; register_controls: cell ->
    (clock, lsr, ce). Returns (targets [U, 2], coordinates or None, stats,
    report dict)."""
    lib = abi.load()
    params = params or default_params()
    pc = problem.c_struct()
    ch = np.ascontiguousarray(capacity_h, dtype=np.uint32)
    cv = np.ascontiguousarray(capacity_v, dtype=np.uint32)
    if ch.ndim != 2 or ch.shape != cv.shape:
        raise ValueError("capacity maps must be [H, W] and of one shape")
    cap = abi.RoutingCapacity(ch.shape[1], ch.shape[0], abi.ptr(ch, C.c_uint32), abi.ptr(cv, C.c_uint32))
    items = sorted((register_controls or {}).items())
    ctl = (abi.RegisterControl * max(len(items), 1))()
    for k, (cell, (clock, lsr, ce)) in enumerate(items):
        ctl[k].cell = int(cell)
        ctl[k].clock_lsr[0] = int(clock)
        ctl[k].clock_lsr[1] = int(lsr)
        ctl[k].ce = int(ce)
    targets = np.zeros(2 * problem.num_units, np.uint32)
    coords = None
    if coordinates:
        with Placer(problem, params) as h:
            coords = np.zeros(h.n)
    st = abi.Stats()
    rep = abi.RoutableReport()
    code = lib.texo_gp_place_routable(C.byref(pc), C.byref(params), C.byref(cap), len(items), ctl,
                                      abi.ptr(targets, C.c_uint32),
                                      abi.ptr(coords, C.c_double) if coords is not None else None, C.byref(st),
                                      C.byref(rep))
    abi.check(code, "texo_gp_place_routable")
    report = {f: getattr(rep, f) for f, _ in abi.RoutableReport._fields_ if f != "reserved"}
    return targets.reshape(-1, 2), coords, _stats_dict(st), report


class Batch:
    """Many resident placements advanced together (texo_gp_batch)."""

    def __init__(self, params=None, hbm_budget=64 << 30, max_slots=256):
        self.lib = abi.load()
        self.params = params or default_params()
        h = C.c_void_p()
        abi.check(self.lib.texo_gp_batch_create(C.byref(self.params), hbm_budget, max_slots, C.byref(h)),
                  "texo_gp_batch_create")
        self.h = h
        self._units = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.texo_gp_batch_destroy(self.h)
            self.h = None

    __del__ = close

    def admit(self, problem, job_id, params=None):
        """Returns True when admitted, False when the batch is full (slots or HBM budget)."""
        pc = problem.c_struct()
        slot = C.c_uint32()
        pp = C.byref(params) if params is not None else None
        code = self.lib.texo_gp_batch_admit(self.h, C.byref(pc), pp, job_id, C.byref(slot))
        if code == abi.CODE["BUSY"]:
            return False
        abi.check(code, "texo_gp_batch_admit")
        self._units[job_id] = problem.num_units
        return True

    def advance(self, iterations):
        abi.check(self.lib.texo_gp_batch_advance(self.h, iterations), "texo_gp_batch_advance")

    def retire(self):
        """Pops one finished job: (job_id, targets [U,2], stats) or None."""
        cap = max(self._units.values()) * 2 if self._units else 0
        targets = np.zeros(max(cap, 2), np.uint32)
        jid = C.c_uint64()
        st = abi.Stats()
        code = self.lib.texo_gp_batch_retire(self.h, C.byref(jid), abi.ptr(targets, C.c_uint32), targets.size,
                                            C.byref(st))
        if code == abi.CODE["BUSY"]:
            return None
        if code in (abi.CODE["CUDA"], abi.CODE["INVALID_ARGUMENT"], abi.CODE["DEVICE_TIMEOUT"]):
            abi.check(code, "texo_gp_batch_retire")
        u = self._units.pop(jid.value)
        stats = _stats_dict(st)
        if code not in (0, abi.CODE["DID_NOT_CONVERGE"]):
            # the job failed with a placement error (a reference error variant)
            stats["status"] = abi.STATUS.get(code, code)
            return jid.value, None, stats
        return jid.value, targets[:2 * u].reshape(-1, 2).copy(), stats

    def graphs(self):
        """(captures, replays) of the batch advance's CUDA graph."""
        c, r = C.c_uint64(), C.c_uint64()
        abi.check(self.lib.texo_gp_batch_graphs(self.h, C.byref(c), C.byref(r)), "texo_gp_batch_graphs")
        return c.value, r.value

    def counts(self):
        r, f, b = C.c_uint32(), C.c_uint32(), C.c_uint64()
        abi.check(self.lib.texo_gp_batch_counts(self.h, C.byref(r), C.byref(f), C.byref(b)), "texo_gp_batch_counts")
        return r.value, f.value, b.value


def routing_demand(width, height, boxes, device=0):
    """`continuous_routing_demand` (eplace.rs:856-937) through
    texo_gp_routing_demand: (horizontal [H, W], vertical [H, W], device ms)."""
    lib = abi.load()
    b = np.ascontiguousarray(boxes, dtype=np.float64).reshape(-1, 4)
    h = np.zeros(width * height)
    v = np.zeros(width * height)
    ms = C.c_double()
    abi.check(lib.texo_gp_routing_demand(device, width, height, b.shape[0], abi.ptr(b, C.c_double),
                                         abi.ptr(h, C.c_double), abi.ptr(v, C.c_double), C.byref(ms)),
              "texo_gp_routing_demand")
    return h.reshape(height, width), v.reshape(height, width), ms.value


def net_bounding_boxes(problem, positions):
    """`external_baseline_net_bounding_boxes` (analytical_placement.rs:238-276)
    for unit origins `positions` [U, 2]: (min_x, max_x, min_y, max_y) of every
    net not wholly inside one unit, fixed cells at their coordinates."""
    net_ptr = np.asarray(problem.net_ptr, dtype=np.int64)
    pin_cell = np.asarray(problem.pin_cell, dtype=np.int64)
    cell_unit = np.asarray(problem.cell_unit, dtype=np.int64)
    fixed = np.asarray(problem.cell_fixed, dtype=bool)
    fixed_xy = np.asarray(problem.cell_fixed_xy, dtype=np.float64).reshape(-1, 2)
    off = np.asarray(problem.cell_offset_xy, dtype=np.float64).reshape(-1, 2)
    pos = np.asarray(positions, dtype=np.float64).reshape(-1, 2)
    cxy = np.where(fixed[:, None], fixed_xy, pos[cell_unit] + off)
    pin_xy = cxy[pin_cell]
    pin_unit = cell_unit[pin_cell]
    starts = net_ptr[:-1]
    lo = np.minimum.reduceat(pin_xy, starts, axis=0)
    hi = np.maximum.reduceat(pin_xy, starts, axis=0)
    umin = np.minimum.reduceat(pin_unit, starts)
    umax = np.maximum.reduceat(pin_unit, starts)
    keep = umin != umax
    return np.stack([lo[:, 0], hi[:, 0], lo[:, 1], hi[:, 1]], axis=1)[keep]


PCG_STOP = ("residual", "breakdown", "dimension")


def quadratic_solve(diagonal, adjacency_ptr, adjacency_index, adjacency_weight, rhs, solution=None,
                    device=0, allow_nonconverged=False):
    """`solve_quadratic` (lib.rs:4586-4752) through texo_gp_quadratic_solve:
    Jacobi-preconditioned CG for (D - W) x = b on the GPU, W given as CSR rows
    in the reference's adjacency order. Returns (x, stats dict)."""
    lib = abi.load()
    n = len(diagonal)
    d = np.ascontiguousarray(diagonal, dtype=np.float64)
    ptr = np.ascontiguousarray(adjacency_ptr, dtype=np.uint32)
    idx = np.ascontiguousarray(adjacency_index, dtype=np.uint32)
    w = np.ascontiguousarray(adjacency_weight, dtype=np.float64)
    b = np.ascontiguousarray(rhs, dtype=np.float64)
    x = np.zeros(n) if solution is None else np.array(solution, dtype=np.float64, copy=True)
    if ptr.size != n + 1 or b.size != n or x.size != n:
        raise ValueError("quadratic_solve: inconsistent sizes")
    st = abi.PcgStats()
    code = lib.texo_gp_quadratic_solve(device, n, abi.ptr(d, C.c_double), abi.ptr(ptr, C.c_uint32),
                                       abi.ptr(idx, C.c_uint32), abi.ptr(w, C.c_double), abi.ptr(b, C.c_double),
                                       abi.ptr(x, C.c_double), C.byref(st))
    if not (allow_nonconverged and code == abi.CODE["PCG_NOT_CONVERGED"]):
        abi.check(code, "texo_gp_quadratic_solve")
    return x, dict(status=abi.STATUS.get(st.status, st.status), iterations=st.iterations, restarts=st.restarts,
                   stop=PCG_STOP[st.stop] if 0 <= st.stop < 3 else st.stop,
                   initial_residual_squared=st.initial_residual_squared, target_squared=st.target_squared,
                   final_residual_squared=st.final_residual_squared, elapsed_ms=st.elapsed_ms,
                   kernel_launches=st.kernel_launches)


class Server:
    """The serving loop (texo_gp_server): submit requests at any time, poll
    finished jobs. Results are (job_id, targets [U,2] or None, info dict)."""

    def __init__(self, params=None, hbm_budget=0, max_resident=256, chunk_iterations=20, admission_threads=4):
        self.lib = abi.load()
        self.params = params or default_params()
        opt = abi.ServerOptions()
        opt.hbm_budget_bytes = hbm_budget
        opt.max_resident = max_resident
        opt.chunk_iterations = chunk_iterations
        opt.admission_threads = admission_threads
        h = C.c_void_p()
        abi.check(self.lib.texo_gp_server_create(C.byref(self.params), C.byref(opt), C.byref(h)),
                  "texo_gp_server_create")
        self.h = h
        self._units = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.texo_gp_server_destroy(self.h)
            self.h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, problem, job_id, params=None):
        pc = problem.c_struct()
        pp = C.byref(params) if params is not None else None
        abi.check(self.lib.texo_gp_server_submit(self.h, C.byref(pc), pp, job_id), "texo_gp_server_submit")
        self._units[job_id] = problem.num_units

    def clock_ms(self):
        return self.lib.texo_gp_server_clock_ms(self.h)

    def poll(self, wait_ms=-1):
        """One finished job or None (nothing finished within wait_ms)."""
        cap = 2 * max(self._units.values(), default=1)
        targets = np.zeros(cap, np.uint32)
        r = abi.JobResult()
        code = self.lib.texo_gp_server_poll(self.h, wait_ms, C.byref(r), abi.ptr(targets, C.c_uint32), targets.size)
        if code == abi.CODE["INVALID_ARGUMENT"] and 2 * r.units > targets.size:
            # a job submitted (by another thread) during the wait finished first
            targets = np.zeros(2 * r.units, np.uint32)
            code = self.lib.texo_gp_server_poll(self.h, 0, C.byref(r), abi.ptr(targets, C.c_uint32), targets.size)
        if code == abi.CODE["BUSY"]:
            return None
        abi.check(code, "texo_gp_server_poll")
        self._units.pop(r.job_id, None)
        info = _stats_dict(r.stats)
        info.update(status=abi.STATUS.get(r.status, r.status), submit_ms=r.submit_ms, admit_ms=r.admit_ms,
                    finish_ms=r.finish_ms)
        ok = r.status in (0, abi.CODE["DID_NOT_CONVERGE"])
        return r.job_id, (targets[:2 * r.units].reshape(-1, 2).copy() if ok else None), info

    def counts(self):
        q, r, f, b = C.c_uint32(), C.c_uint32(), C.c_uint32(), C.c_uint64()
        abi.check(self.lib.texo_gp_server_counts(self.h, C.byref(q), C.byref(r), C.byref(f), C.byref(b)),
                  "texo_gp_server_counts")
        return q.value, r.value, f.value, b.value


class Placer:
    """A device-resident placement instance (texo_gp_handle)."""

    def __init__(self, problem, params=None):
        self.lib = abi.load()
        self.problem = problem
        self.params = params or default_params()
        self._pc = problem.c_struct()
        h = C.c_void_p()
        abi.check(self.lib.texo_gp_create(C.byref(self._pc), C.byref(self.params), C.byref(h)),
                  "texo_gp_create")
        self.h = h
        u, f, n = C.c_uint64(), C.c_uint64(), C.c_uint64()
        bx, by, k = C.c_uint32(), C.c_uint32(), C.c_uint32()
        abi.check(self.lib.texo_gp_sizes(h, C.byref(u), C.byref(f), C.byref(n), C.byref(bx),
                                         C.byref(by), C.byref(k)), "texo_gp_sizes")
        self.units, self.num_fillers, self.n = u.value, f.value, n.value
        self.bins_x, self.bins_y, self.num_fields = bx.value, by.value, k.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.texo_gp_destroy(self.h)
            self.h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def bins(self):
        return self.bins_x * self.bins_y

    def initial(self):
        c, lo, hi = np.zeros(self.n), np.zeros(self.n), np.zeros(self.n)
        abi.check(self.lib.texo_gp_initial(self.h, abi.ptr(c, C.c_double), abi.ptr(lo, C.c_double),
                                           abi.ptr(hi, C.c_double)), "texo_gp_initial")
        return c, lo, hi

    def fillers(self):
        f = np.zeros(self.num_fillers, np.uint32)
        q = np.zeros(self.num_fillers)
        abi.check(self.lib.texo_gp_fillers(self.h, abi.ptr(f, C.c_uint32), abi.ptr(q, C.c_double)),
                  "texo_gp_fillers")
        return f, q

    def evaluate(self, coords, gamma, arrays=True):
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        K, n, B = self.num_fields, self.n, self.bins
        ev = abi.Eval()
        wag = np.zeros(2 * self.units) if arrays else None
        fg = np.zeros(K * n) if arrays else None
        dens = np.zeros(K * B) if arrays else None
        pot = np.zeros(K * B) if arrays else None
        abi.check(self.lib.texo_gp_evaluate(self.h, abi.ptr(coords, C.c_double), gamma, C.byref(ev),
                                            abi.ptr(wag, C.c_double), abi.ptr(fg, C.c_double),
                                            abi.ptr(dens, C.c_double), abi.ptr(pot, C.c_double)),
                  "texo_gp_evaluate")
        out = {"wirelength": ev.wirelength, "fields": [ev.fields[i] for i in range(K)]}
        if arrays:
            out.update(wa_gradient=wag, field_gradient=fg.reshape(K, n), density=dens.reshape(K, B),
                       potential=pot.reshape(K, B))
        return out

    def scatter(self, coords):
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        K, B = self.num_fields, self.bins
        phys = np.zeros(K * B, np.int64)
        fill = np.zeros(K * B, np.int64)
        abi.check(self.lib.texo_gp_scatter(self.h, abi.ptr(coords, C.c_double), abi.ptr(phys, C.c_int64),
                                           abi.ptr(fill, C.c_int64)), "texo_gp_scatter")
        return phys.reshape(K, B), fill.reshape(K, B)

    def poisson(self, density):
        d = np.ascontiguousarray(density, dtype=np.float64)
        pot = np.zeros(self.bins)
        e = C.c_double()
        abi.check(self.lib.texo_gp_poisson(self.h, abi.ptr(d, C.c_double), abi.ptr(pot, C.c_double),
                                           C.byref(e)), "texo_gp_poisson")
        return pot, e.value

    def run(self, max_iterations=0, allow_nonconverged=False):
        targets = np.zeros(2 * self.units, np.uint32)
        coords = np.zeros(self.n)
        st = abi.Stats()
        code = self.lib.texo_gp_run(self.h, max_iterations, abi.ptr(targets, C.c_uint32),
                                    abi.ptr(coords, C.c_double), C.byref(st))
        if not (allow_nonconverged and code == abi.CODE["DID_NOT_CONVERGE"]):
            abi.check(code, "texo_gp_run")
        return targets.reshape(-1, 2), coords, _stats_dict(st)

    def optimize_round(self, stop, reset_multipliers, density_scales=None, completed_iterations=0):
        """One round of eplace::place's area-adjustment loop from the current
        coordinates (texo_gp_optimize_round): returns (targets [U, 2],
        coordinates, stats, result dict)."""
        r = abi.Round()
        r.stop = int(stop)
        r.reset_multipliers = 1 if reset_multipliers else 0
        sc = None
        if density_scales is not None:
            sc = np.ascontiguousarray(density_scales, dtype=np.float64)
            r.density_scales = abi.ptr(sc, C.c_double)
        r.completed_iterations = int(completed_iterations)
        t = np.zeros(2 * self.units, np.uint32)
        c = np.zeros(self.n)
        s = abi.Stats()
        res = abi.RoundResult()
        code = self.lib.texo_gp_optimize_round(self.h, C.byref(r), abi.ptr(t, C.c_uint32), abi.ptr(c, C.c_double),
                                               C.byref(s), C.byref(res))
        if code not in (0, abi.CODE["DID_NOT_CONVERGE"]):
            abi.check(code, "texo_gp_optimize_round")
        out = {"completed_iterations": res.completed_iterations, "exhausted": bool(res.exhausted),
               "density_scales": [res.density_scales[f] for f in range(self.num_fields)], "status": code}
        return t.reshape(-1, 2), c, _stats_dict(s), out

    def set_charges(self, member_charge=None, filler_charge=None):
        """Installs an area adjustment (texo_gp_set_charges)."""
        m = None if member_charge is None else np.ascontiguousarray(member_charge, dtype=np.float64)
        f = None if filler_charge is None else np.ascontiguousarray(filler_charge, dtype=np.float64)
        abi.check(self.lib.texo_gp_set_charges(self.h, abi.ptr(m, C.c_double) if m is not None else None,
                                               abi.ptr(f, C.c_double) if f is not None else None),
                  "texo_gp_set_charges")

    def reset(self):
        abi.check(self.lib.texo_gp_reset(self.h), "texo_gp_reset")

    def hpwl(self, coords):
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        out = C.c_double()
        abi.check(self.lib.texo_gp_hpwl(self.h, abi.ptr(coords, C.c_double), C.byref(out)), "texo_gp_hpwl")
        return out.value

    def device_profile(self):
        """Phase times of the persistent engine (microseconds) and barrier counts."""
        out = np.zeros(10)
        abi.check(self.lib.texo_gp_device_profile(self.h, abi.ptr(out, C.c_double)), "texo_gp_device_profile")
        names = ["scatter_wa", "prep", "dct", "gather_combine", "precond_init", "extrapolate", "candidate",
                 "other", "barrier_wait", "barriers"]
        return dict(zip(names, out.tolist()))

    DCT_FORMS = ("gemm16", "gemm64", "tensor_core", "fft")

    def trace(self):
        """Host-engine controller records since create/reset (texo_gp_iteration each)."""
        n = C.c_uint32()
        abi.check(self.lib.texo_gp_trace(self.h, None, 0, C.byref(n)), "texo_gp_trace")
        buf = (abi.Iteration * max(1, n.value))()
        abi.check(self.lib.texo_gp_trace(self.h, buf, n.value, C.byref(n)), "texo_gp_trace")
        return [buf[i] for i in range(n.value)]

    def dct_form(self):
        """The DCT form this instance runs: 0 GEMM (16-bin tiles), 1 GEMM
        (64-bin tiles), 2 tensor cores (integer slices, exact accumulation), 3 FFT."""
        f = C.c_int32()
        abi.check(self.lib.texo_gp_dct_form(self.h, C.byref(f)), "texo_gp_dct_form")
        return int(f.value)

    def stage_times(self, reps=20):
        ms = np.zeros(64)
        cnt = C.c_uint32()
        abi.check(self.lib.texo_gp_stage_times(self.h, reps, abi.ptr(ms, C.c_double), 64, C.byref(cnt)),
                  "texo_gp_stage_times")
        return {self.lib.texo_gp_stage_name(i).decode(): float(ms[i]) for i in range(cnt.value)}

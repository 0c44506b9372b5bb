"""GPU parity on the cases the benchmark sizes do not cover, through the C ABI
against the FP64 oracle.

  * The smallest benchmark configuration verbatim: 2,000 cells + 96 IO on
    48 x 48 sites, 2,400 nets, a 64 x 64 bin grid, target density 1.0, WA
    gamma base 4 bin widths, 300 iterations or overflow <= 0.10.
  * A two-field (LUT + register) problem at the same scale with rigid
    two-member macros, fixed exchangeable occupancy and timed arcs
    (tests/rich_problems.py).
  * The reference's sink-local timing-overlay case
    (analytical_placement.rs:1106-1183) on the device.
  * The controller's scalars over the first iterations (gamma, lambda per
    field, E0, the Lipschitz estimate, trials, accepted objective).

Bounds: scatter grids, overflow sums and overflowed-bin counts bit-exact;
density, potential, field and WA gradients normwise within 1e-5 (max|a-b| /
max|b|); WA value, energies and force within 1e-5 relative; final HPWL within
1% at overflow <= target; controller scalars within the bounds stated on the
test.
"""
import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi, problem as P
from texo_gb300.placer import Placer, default_params

from rich_problems import rich_problem
from test_oracle_wirelength import wa_problem, wide_net

pytestmark = pytest.mark.gpu

TOL = 1e-5


def normwise(a, b):
    return float(np.max(np.abs(a - b))) / float(np.max(np.abs(b)))


def config0():
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 0)
    return prob, dict(bins_x=64, bins_y=64, target_density=1.0, gamma_base=4.0, max_iterations=300, best_effort=1)


def spread(o, seed):
    c, lo, hi = o.initial()
    c = lo + (hi - lo) * np.random.default_rng(seed).random(c.size)
    return c.astype(np.float32).astype(np.float64)


def check_evaluation(prob, kw, seed, gamma):
    prm = default_params(**kw)
    o = ffi.Oracle(prob, prm)
    c = spread(o, seed)
    with Placer(prob, prm) as g:
        phys, fill = g.scatter(c)
        d = g.evaluate(c, gamma)
    rp, rf, rov, rcnt = o.scatter_fixed(c)
    assert np.array_equal(phys, rp) and np.array_equal(fill, rf)
    r = o.evaluate(c, gamma)
    for f in range(len(prob.fields)):
        a, b = d["fields"][f], r["fields"][f]
        assert a.overflow_fixed == rov[f] and a.overflow_bins == rcnt[f]
        assert abs(a.energy - b.energy) <= TOL * abs(b.energy)
        assert abs(a.force_l1 - b.force_l1) <= TOL * b.force_l1
        # the device normalizes its bit-exact fixed-point overflow; the oracle
        # sums the FP64 density: they differ by the 2^-32 rounding of each of
        # the 9 taps a member deposits, over the real area (< 1e-8 absolute)
        assert abs(a.normalized_overflow - b.normalized_overflow) <= 1e-8
    assert normwise(d["density"], r["density"]) <= TOL
    assert normwise(d["potential"], r["potential"]) <= TOL
    assert normwise(d["field_gradient"], r["field_gradient"]) <= TOL
    assert normwise(d["wa_gradient"], r["wa_gradient"]) <= TOL
    assert abs(d["wirelength"] - r["wirelength"]) <= TOL * abs(r["wirelength"])


def check_placement(prob, kw, engine):
    prm = default_params(**kw)
    st, _, _, s_ref = ffi.Oracle(prob, prm).place(threads=5)
    assert st == 0 and s_ref.converged
    prm.engine = engine
    with Placer(prob, prm) as g:
        _, _, s = g.run()
    assert s["converged"]
    for f, (kind, _) in enumerate(prob.fields):
        assert s["overflow"][f] <= (0.20 if kind == abi.KIND_MEMORY else 0.10)
    assert abs(s["hpwl"] - s_ref.hpwl) <= 0.01 * s_ref.hpwl
    return s, s_ref


@pytest.mark.parametrize("seed,gamma", [(3, 4.0 * 48 / 64), (4, 1.5)])
def test_config0_verbatim_evaluation(seed, gamma):
    prob, kw = config0()
    check_evaluation(prob, kw, seed, gamma)


@pytest.mark.parametrize("engine", [abi.ENGINE_HOST, abi.ENGINE_DEVICE])
def test_config0_verbatim_placement(engine):
    prob, kw = config0()
    s, s_ref = check_placement(prob, kw, engine)
    assert s["iterations"] <= 300


@pytest.mark.parametrize("seed", [0, 1])
def test_rich_problem_scatter_and_evaluation(seed):
    # two fields, macros, fixed exchangeable occupancy (inside the scatter's
    # capacity background) and timed arcs (inside WA), at 2,000 cells
    prob = rich_problem(seed)
    assert len(prob.fields) == 2 and prob.fixed_occupancy.shape[0] > 0 and prob.arc_driver_cell.size > 0
    assert int(np.max(np.diff(prob.member_ptr))) == 2
    check_evaluation(prob, dict(best_effort=1), 10 + seed, 2.0)


def test_rich_problem_bins_differ_from_tiles():
    prob = rich_problem(2)
    check_evaluation(prob, dict(bins_x=64, bins_y=40, target_density=0.95, best_effort=1), 5, 1.7)


@pytest.mark.parametrize("engine", [abi.ENGINE_HOST, abi.ENGINE_DEVICE])
def test_rich_problem_placement(engine):
    check_placement(rich_problem(0), dict(best_effort=1, max_iterations=1000), engine)


def _wa(problem, positions, gamma):
    c = np.array(positions, np.float64).ravel()
    with Placer(problem, default_params()) as g:
        d = g.evaluate(c, gamma)
    w = d["wa_gradient"].reshape(-1, 2)
    o = ffi.Oracle(problem).evaluate(c, gamma)
    ow = o["wa_gradient"].reshape(-1, 2)
    assert abs(d["wirelength"] - o["wirelength"]) <= TOL * abs(o["wirelength"])
    assert normwise(w, ow) <= TOL
    return d["wirelength"], w[:, 0], w[:, 1]


@pytest.mark.parametrize("gamma", [0.25, 2.5])
def test_timing_overlay_is_sink_local_on_the_device(gamma):
    # analytical_placement.rs:1106-1183: a sink weight of 5 on arc (0, 1) adds
    # exactly 4x the two-pin net (0, 1) and leaves the other sink's gradient alone
    pos = [(0.0, 0.0), (2.0, 1.0), (-1.0, 3.0)]
    base = _wa(wide_net(2), pos, gamma)
    crit = _wa(wide_net(2, 5), pos, gamma)
    arc = _wa(wide_net(1), pos[:2], gamma)
    scale = abs(crit[0])
    assert abs((crit[0] - base[0]) - 4.0 * arc[0]) <= TOL * scale
    gs = max(np.max(np.abs(crit[1])), np.max(np.abs(crit[2])))
    for u in range(2):
        assert abs((crit[1][u] - base[1][u]) - 4.0 * arc[1][u]) <= TOL * gs
        assert abs((crit[2][u] - base[2][u]) - 4.0 * arc[2][u]) <= TOL * gs
    assert abs(crit[1][2] - base[1][2]) <= TOL * gs and abs(crit[2][2] - base[2][2]) <= TOL * gs


def test_timing_overlay_fixed_pins_and_offsets_on_the_device():
    # a macro with an offset member, a fixed sink and a weighted arc into the macro
    p = wa_problem(3, [0, 0, 1, 2], [[1, 2, 3], [3, 0]],
                   fixed=[None, None, (10.0, 5.0), None],
                   offsets=[(0.0, 0.0), (3.0, -2.0), (0.0, 0.0), (-1.0, 1.0)],
                   arcs=[(1, 3, 2), (3, 0, 1)])
    _wa(p, [(2.0, 4.0), (99.0, 99.0), (7.0, 8.0)], 0.75)


# Controller scalars of the first iterations, host engine against the oracle.
# The device evaluates in FP32 and compares line-search objectives with a
# margin widened to 64 * 2^-24 (1 + |a| + |b|); its trajectory drifts from the
# FP64 one by FP32 rounding, slowly (measured on GB300 over 20 iterations of
# both problems: gamma 3e-5, lambda 4e-7, E0 4e-8, objective 6e-7, Lipschitz
# 6e-8 relative, overflow 6e-6 absolute). Bounds over the first 20 iterations:
#   line-search trials equal in every iteration; gamma within 1e-4 relative;
#   lambda and the accepted objective within 1e-5 relative; E0 within 1e-6
#   relative; the Lipschitz estimate within 1e-5 relative; the momentum
#   within 1e-12 relative; per-field overflow within 1e-4 absolute.
TRACE_ITERATIONS = 20


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def check_trace(prob, kw):
    prm = default_params(**kw)
    o = ffi.Oracle(prob, prm)
    st, _, _, _ = o.place(threads=5, max_iterations=TRACE_ITERATIONS)
    assert st == 0
    ref = o.trace()
    with Placer(prob, prm) as g:
        g.run(TRACE_ITERATIONS, allow_nonconverged=True)
        got = g.trace()
    assert len(got) == len(ref) == TRACE_ITERATIONS
    K = len(prob.fields)
    for a, b in zip(got, ref):
        it = a.iteration
        assert it == b.iteration
        assert a.trials == b.trials, (it, "trials", a.trials, b.trials)
        assert rel(a.gamma, b.gamma) <= 1e-4, (it, "gamma")
        assert rel(a.objective, b.objective) <= 1e-5, (it, "objective")
        assert rel(a.lipschitz, b.lipschitz) <= 1e-5, (it, "lipschitz")
        assert rel(a.momentum, b.momentum) <= 1e-12, (it, "momentum")
        for f in range(K):
            assert rel(a.lambda_[f], b.lambda_[f]) <= 1e-5, (it, "lambda", f)
            assert rel(a.energy_scale[f], b.energy_scale[f]) <= 1e-6, (it, "E0", f)
            assert abs(a.overflow[f] - b.overflow[f]) <= 1e-4, (it, "overflow", f)


def test_controller_trace_matches_oracle_config0():
    prob, kw = config0()
    check_trace(prob, kw)


def test_controller_trace_matches_oracle_rich():
    check_trace(rich_problem(0), dict(best_effort=1))


def test_rich_problem_at_scale_scatter_and_evaluation():
    """The same features at 12,000 cells on a 128 x 128 fabric with two BELs
    of each kind a tile (two fields, macros, fixed exchangeable occupancy,
    timed arcs), on the tile grid and on a 256 x 256 bin grid."""
    prob = rich_problem(5, side=128, cells=12000, io=240, nets=14400, sigma=8.0, capacity=2)
    assert len(prob.fields) == 2 and prob.fixed_occupancy.shape[0] > 0 and prob.arc_driver_cell.size > 0
    check_evaluation(prob, dict(best_effort=1), 7, 2.0)
    check_evaluation(prob, dict(best_effort=1, bins_x=256, bins_y=256, target_density=0.9), 8, 4.0)


def test_ecp5_adapter_problem_evaluation():
    """A placement problem built by the ECP5 adapter (LUT-FF pairs, carry
    chains, units without density members, fixed IO) on a 24 x 24 fabric of
    8 LUT4 and 8 FF a tile: grids bit-exact, evaluation within 1e-5."""
    from texo_gb300 import ecp5
    arch = ecp5.read_architecture(ecp5.synthetic_architecture(24, 24))
    nc, units, kinds, nets = ecp5.synthetic_design(arch, 4, luts=1200, ffs=600, lut_ff_pairs=400,
                                                   carry=((30, 4), (10, 6)), io=40)
    prob, _ = ecp5.placement_problem(arch, nc, units, nets, cell_kind=kinds, sink_weights={(0, 0): 3, (5, 1): 2})
    check_evaluation(prob, dict(best_effort=1), 9, 1.0)

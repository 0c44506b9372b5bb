"""GPU parity: the CUDA engine against the FP64 oracle on identical inputs.

Tolerances (stated per quantity):
  * density scatter grids, overflow sums and overflowed-bin counts: bit-exact
    against the oracle's fixed-point restatement of the device arithmetic;
  * density, potential, field gradient and WA gradient at identical
    coordinates: normwise relative error max|a-b| / max|b| <= 1e-5 against FP64;
  * WA value and field energies: relative error <= 1e-5;
  * final HPWL of a full placement: within 1% of the oracle's.
"""
import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi, problem as P
from texo_gb300.placer import Placer, default_params

pytestmark = pytest.mark.gpu

TOL = 1e-5


def normwise(a, b):
    scale = float(np.max(np.abs(b)))
    if scale == 0.0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - b))) / scale


def params(**kw):
    p = default_params()
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def mixed_problem():
    cap = np.zeros((2, 12), np.uint32)
    cap[0, 0:4] = 1
    cap[1, 4:8] = 1
    units = [(1.25, 0.25, [(0, 0.0, 0.0, 1.0), (1, 0.5, 0.5, 1.0)]),
             (2.5, 0.75, [(0, 0.0, 0.0, 1.25)]),
             (0.3, 1.1, [(1, 0.0, 0.0, 1.0)])]
    return P.density_problem(4, 3, [(abi.KIND_LUT, 4), (abi.KIND_REGISTER, 0)], cap, units,
                             nets=[[0, 2], [1, 3, 2]])


CASES = {
    "mixed-4x3": (mixed_problem, {}),
    "ecp5-2k-tiles": (lambda: P.synthetic(48, 2000, 96, 2400, 6.0, 0), {}),
    "ecp5-2k-bins64-td0.9": (lambda: P.synthetic(48, 2000, 96, 2400, 6.0, 0),
                             dict(bins_x=64, bins_y=64, target_density=0.9, gamma_base=4.0)),
    "prime-side-127": (lambda: P.synthetic(127, 9000, 120, 10000, 6.0, 7), {}),
}


def positions(o, kind, seed=0):
    """Identical inputs for both sides: the device holds FP32 coordinates, so
    the coordinates are made FP32-representable before the oracle sees them."""
    c, lo, hi = o.initial()
    if kind != "initial":
        rng = np.random.default_rng(seed)
        c = lo + (hi - lo) * rng.random(c.size)
    return c.astype(np.float32).astype(np.float64)


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    make, kw = CASES[request.param]
    prob = make()
    prm = params(**kw)
    return request.param, prob, prm, ffi.Oracle(prob, prm), Placer(prob, prm)


@pytest.mark.parametrize("where", ["initial", "spread"])
def test_scatter_is_bit_exact(case, where):
    _, prob, prm, o, g = case
    c = positions(o, where)
    phys, fill = g.scatter(c)
    rp, rf, rov, rcnt = o.scatter_fixed(c)
    assert np.array_equal(phys, rp)
    assert np.array_equal(fill, rf)
    ev = g.evaluate(c, 8.0, arrays=False)
    for f in range(o.num_fields):
        assert ev["fields"][f].overflow_fixed == rov[f]
        assert ev["fields"][f].overflow_bins == rcnt[f]


@pytest.mark.parametrize("where", ["initial", "spread"])
def test_evaluation_matches_fp64(case, where):
    name, prob, prm, o, g = case
    c = positions(o, where, seed=1)
    gamma = 8.0 if where == "initial" else 2.5
    r = o.evaluate(c, gamma)
    d = g.evaluate(c, gamma)
    assert normwise(d["density"], r["density"]) <= TOL
    assert normwise(d["potential"], r["potential"]) <= TOL
    assert normwise(d["field_gradient"], r["field_gradient"]) <= TOL
    assert normwise(d["wa_gradient"], r["wa_gradient"]) <= TOL
    assert abs(d["wirelength"] - r["wirelength"]) <= TOL * abs(r["wirelength"])
    for f in range(o.num_fields):
        a, b = d["fields"][f], r["fields"][f]
        assert abs(a.energy - b.energy) <= TOL * max(abs(b.energy), 1e-30)
        assert abs(a.normalized_overflow - b.normalized_overflow) <= TOL * max(b.normalized_overflow, 1e-12)
        assert abs(a.force_l1 - b.force_l1) <= TOL * max(b.force_l1, 1e-30)


def test_evaluation_is_deterministic(case):
    _, prob, prm, o, g = case
    c = positions(o, "spread", seed=2)
    a = g.evaluate(c, 3.0)
    b = g.evaluate(c, 3.0)
    for k in ("density", "potential", "field_gradient", "wa_gradient"):
        assert np.array_equal(a[k], b[k])
    assert a["wirelength"] == b["wirelength"]


def test_poisson_prime_grid_matches_matrix_oracle():
    prob = P.synthetic(127, 9000, 120, 10000, 6.0, 7)
    g = Placer(prob, params(bins_x=127, bins_y=96))
    i = np.arange(127 * 96)
    d = ((i * 31 + 7) % 101) - 50.0 + ((i * 13 + 5) % 17) / 17.0
    pot, e = g.poisson(d)
    ref, er = ffi.poisson(127, 96, d, matrix=True)
    assert normwise(pot, ref) <= TOL
    assert abs(e - er) <= TOL * abs(er)
    pot0, e0 = g.poisson(np.full(127 * 96, 3.25))
    assert np.max(np.abs(pot0)) <= 1e-6 and abs(e0) <= 1e-6


def test_placement_matches_oracle_hpwl():
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 0)
    prm = params(best_effort=1, max_iterations=400)
    st, t_ref, c_ref, s_ref = ffi.Oracle(prob, prm).place()
    assert st == 0 and s_ref.converged
    g = Placer(prob, prm)
    targets, coords, s = g.run()
    assert s["converged"] and s["overflow"][0] <= 0.10
    assert abs(s["hpwl"] - s_ref.hpwl) <= 0.01 * s_ref.hpwl
    # bit-for-bit repeatable
    g.reset()
    t2, c2, s2 = g.run()
    assert np.array_equal(targets, t2) and np.array_equal(coords, c2)
    assert 0 <= targets.min() and targets[:, 0].max() <= 47


def test_typed_errors_through_the_abi():
    cap = np.zeros((3, 12), np.uint32)
    cap[0, 0:4] = 1
    cap[1, 4:8] = 1
    p = P.density_problem(4, 3, [(abi.KIND_LUT, 4), (abi.KIND_REGISTER, 0), (abi.KIND_MEMORY, 0)], cap,
                          [(0.0, 0.0, [(2, 0, 0, 1.0)])])
    with pytest.raises(abi.TexoGpError) as e:
        Placer(p)
    assert e.value.name == "INSUFFICIENT_CAPACITY"
    q = P.density_problem(4, 3, [(abi.KIND_LUT, 4)], cap[:1], [(0.0, 0.0, [(0, 0, 0, 1.0)])],
                          fixed_occupancy=[[0, 0, 0], [0, 0, 0]])
    with pytest.raises(abi.TexoGpError) as e:
        Placer(q)
    assert e.value.name == "FIXED_CAPACITY_EXHAUSTED"


def test_device_engine_placement_matches_oracle_and_repeats():
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 0)
    prm = params(best_effort=1, max_iterations=400)
    st, _, _, s_ref = ffi.Oracle(prob, prm).place()
    assert st == 0 and s_ref.converged
    prm_dev = params(best_effort=1, max_iterations=400, engine=abi.ENGINE_DEVICE)
    g = Placer(prob, prm_dev)
    targets, coords, s = g.run()
    assert s["converged"] and s["overflow"][0] <= 0.10
    assert s["kernel_launches"] == 1
    assert abs(s["hpwl"] - s_ref.hpwl) <= 0.01 * s_ref.hpwl
    g.reset()
    t2, c2, s2 = g.run()
    assert np.array_equal(targets, t2) and np.array_equal(coords, c2)
    assert s2["iterations"] == s["iterations"]


def test_device_engine_is_resumable():
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 3)
    prm = params(best_effort=1, max_iterations=400, engine=abi.ENGINE_DEVICE)
    a = Placer(prob, prm)
    _, ca, sa = a.run(15)
    b = Placer(prob, prm)
    for _ in range(3):
        _, cb, sb = b.run(5)
    assert sa["iterations"] == sb["iterations"] == 15
    assert np.array_equal(ca, cb)


def test_device_engine_single_iteration_steps_replay_the_same_graph():
    """One-iteration steps replay the captured step graph (state in, kernel,
    state out); twenty of them end where one twenty-iteration call does."""
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 5)
    prm = params(best_effort=1, max_iterations=400, engine=abi.ENGINE_DEVICE)
    a = Placer(prob, prm)
    ta, ca, sa = a.run(20)
    b = Placer(prob, prm)
    for _ in range(20):
        tb, cb, sb = b.run(1)
        assert sb["kernel_launches"] == 1 and sb["elapsed_ms"] > 0.0
    assert sa["iterations"] == sb["iterations"] == 20
    assert np.array_equal(ca, cb) and np.array_equal(ta, tb)


@pytest.mark.parametrize("engine", [abi.ENGINE_HOST, abi.ENGINE_DEVICE])
def test_density_evaluations_are_counted(engine):
    """Every iteration re-evaluates its origin with the density side reused
    (eplace's closure changes with gamma and the multipliers), so the
    evaluations that rebuild the density side are strictly fewer than all
    evaluations and more than the iterations."""
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 0)
    with Placer(prob, params(best_effort=1, max_iterations=30, engine=engine)) as g:
        _, _, s = g.run(allow_nonconverged=True)
    assert s["iterations"] < s["density_evaluations"] < s["evaluations"]


def test_place_entry_matches_a_handle_run():
    """texo_gp_place (no coordinates asked) and create / run / destroy give
    the same targets and statistics."""
    from texo_gb300.placer import place
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 4)
    prm = params(best_effort=1, max_iterations=400, engine=abi.ENGINE_DEVICE)
    t1, c1, s1 = place(prob, prm)
    t2, c2, s2 = place(prob, prm, coordinates=True)
    assert c1 is None and c2.ndim == 1 and c2.size >= 2 * prob.num_units
    assert np.array_equal(t1, t2)
    assert s1["iterations"] == s2["iterations"] and s1["hpwl"] == s2["hpwl"]


def test_device_engine_on_a_1024_bin_grid_repeats_and_tracks_the_host_engine():
    """The persistent kernel's FFT passes at 1024 points (one vector per
    group, 1024-slot data): two device runs agree bit for bit, and after 10
    iterations the device and host engines (different reduction orders) agree
    on HPWL and overflow to 1e-3."""
    prob = P.synthetic(110, 10000, 96, 12000, 6.0, 2)
    kw = dict(bins_x=1024, bins_y=1024, best_effort=1, max_iterations=400, target_density=0.9, gamma_base=4.0)
    with Placer(prob, params(engine=abi.ENGINE_DEVICE, **kw)) as g:
        t1, c1, s1 = g.run(10)
        g.reset()
        t2, c2, s2 = g.run(10)
    assert np.array_equal(c1, c2) and s1["iterations"] == 10
    with Placer(prob, params(engine=abi.ENGINE_HOST, **kw)) as h:
        _, ch, sh = h.run(10)
    assert abs(s1["hpwl"] - sh["hpwl"]) <= 1e-3 * sh["hpwl"]
    assert abs(s1["overflow"][0] - sh["overflow"][0]) <= 1e-3

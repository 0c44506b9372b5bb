"""texo_gp_quadratic_solve (the GPU `solve_quadratic`, crates/texo-pnr/src/
lib.rs:4586-4752) against the FP64 oracle restatement.

Row products and vector updates are the reference's operations in its order;
the dot products fold in a fixed tree, so iterates agree with the oracle to
rounding: the same stop label, iteration counts within 2, residual target
met, solutions within 1e-8 relative; results repeat bit for bit."""
import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi, problem as P
from texo_gb300 import seed
from texo_gb300.placer import quadratic_solve

pytestmark = pytest.mark.gpu


def test_reference_known_answer_on_the_gpu():
    """lib.rs:14384-14439: the 24-decade diagonal system reaches a relative
    residual below 1e-12."""
    n = 128
    d = np.array([10.0 ** (-12.0 + 24.0 * i / (n - 1)) for i in range(n)])
    x, st = quadratic_solve(d, np.zeros(n + 1, np.uint32), np.zeros(0, np.uint32), np.zeros(0), np.ones(n))
    res = 1.0 - d * x
    assert st["stop"] == "residual" and st["kernel_launches"] == 1
    assert np.sqrt(float(res @ res) / n) < 1e-12


@pytest.mark.parametrize("side,cells,nets,seed_no", [(48, 2000, 2400, 0), (48, 2000, 2400, 3), (110, 10000, 12000, 1)])
def test_gpu_pcg_matches_the_oracle_on_seed_systems(side, cells, nets, seed_no):
    prob = P.synthetic(side, cells, 96, nets, 6.0, seed_no)
    pos = np.asarray(prob.initial_xy).reshape(-1, 2)
    for axis in (0, 1):
        d, ptr, idx, w, rhs, anch = seed.axis_system(prob, pos, axis)
        d, ptr, idx, w, rhs, _ = seed.finalize_gauges(d, ptr, idx, w, rhs, anch)
        x0 = pos[:, axis].copy()
        xr, sr, ok = ffi.solve_quadratic(d, ptr, idx, w, rhs, x0)
        assert ok
        xg, sg = quadratic_solve(d, ptr, idx, w, rhs, x0)
        assert sg["stop"] == "residual"
        assert sg["final_residual_squared"] <= sg["target_squared"]
        assert abs(sg["iterations"] - sr.iterations) <= 2
        assert abs(sg["initial_residual_squared"] - sr.initial_residual_squared) <= 1e-12 * sr.initial_residual_squared
        assert np.max(np.abs(xg - xr)) <= 1e-8 * np.max(np.abs(xr))
        xg2, _ = quadratic_solve(d, ptr, idx, w, rhs, x0)
        assert np.array_equal(xg, xg2)


def test_breakdown_is_reported_like_the_reference():
    d = np.array([1.0, 1.0])
    ptr = np.array([0, 1, 2], np.uint32)
    idx = np.array([1, 0], np.uint32)
    w = np.array([3.0, 3.0])
    x, st = quadratic_solve(d, ptr, idx, w, np.array([1.0, 1.0]), allow_nonconverged=True)
    _, sr, ok = ffi.solve_quadratic(d, ptr, idx, w, np.array([1.0, 1.0]))
    assert not ok and st["status"] == "PCG_NOT_CONVERGED" and st["stop"] == "breakdown" and sr.stop == 1
    with pytest.raises(abi.TexoGpError) as e:
        quadratic_solve(d, ptr, idx, w, np.array([1.0, 1.0]))
    assert e.value.name == "PCG_NOT_CONVERGED"


@pytest.mark.parametrize("case", ["diag", "index"])
def test_invalid_systems_are_rejected(case):
    d = np.array([1.0, 2.0])
    ptr = np.array([0, 1, 2], np.uint32)
    idx = np.array([1, 0], np.uint32)
    w = np.array([0.5, 0.5])
    if case == "diag":
        d[1] = 0.0
    else:
        idx[0] = 7
    with pytest.raises(abi.TexoGpError) as e:
        quadratic_solve(d, ptr, idx, w, np.ones(2))
    assert e.value.name == "INVALID_ARGUMENT"


def test_seed_axis_solve_matches_the_oracle_path():
    """solve_axis (gauges, GPU solve, recentring) against the same steps with
    the oracle's solve."""
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 2)
    pos = np.asarray(prob.initial_xy).reshape(-1, 2)
    xg, st = seed.solve_axis(prob, pos, 0, center=24)
    d, ptr, idx, w, rhs, anch = seed.axis_system(prob, pos, 0)
    d, ptr, idx, w, rhs, floating = seed.finalize_gauges(d, ptr, idx, w, rhs, anch)
    x0 = pos[:, 0].copy()
    for comp in floating:
        x0[comp] -= x0[comp[0]]
    xr, _, ok = ffi.solve_quadratic(d, ptr, idx, w, rhs, x0)
    for comp in floating:
        xr[comp] += 24.0 - xr[comp].sum() / len(comp)
    assert ok and st["stop"] == "residual"
    assert np.max(np.abs(xg - xr)) <= 1e-8 * np.max(np.abs(xr))


def test_seed_solve_at_the_42k_workload():
    """The 42k workload's own seed systems (42,365 unknowns an axis) on the
    GPU against the oracle's FP64 solve."""
    prob = P.synthetic(210, 42000, 365, 50000, 12.0, 0)
    pos = np.asarray(prob.initial_xy).reshape(-1, 2)
    for axis in (0, 1):
        d, ptr, idx, w, rhs, anch = seed.axis_system(prob, pos, axis)
        d, ptr, idx, w, rhs, _ = seed.finalize_gauges(d, ptr, idx, w, rhs, anch)
        x0 = pos[:, axis].copy()
        xr, sr, ok = ffi.solve_quadratic(d, ptr, idx, w, rhs, x0)
        assert ok
        xg, sg = quadratic_solve(d, ptr, idx, w, rhs, x0)
        assert sg["stop"] == "residual" and sg["final_residual_squared"] <= sg["target_squared"]
        assert abs(sg["iterations"] - sr.iterations) <= 2
        assert np.max(np.abs(xg - xr)) <= 1e-8 * np.max(np.abs(xr))


def test_seed_with_macros_and_timed_arcs_matches_the_oracle_path():
    """The seed of a problem with two-member macros (offsets), fixed units and
    timed arcs: solve_axis on the GPU against the same steps with the oracle's
    solve, and the reference's own macro case (lib.rs:14975-15003)."""
    from rich_problems import rich_problem
    from test_seed_macros import macro_offsets_case, oracle_solver
    prob = rich_problem(1)
    pos = np.asarray(prob.initial_xy).reshape(-1, 2)
    for axis, center in ((0, prob.width // 2), (1, prob.height // 2)):
        xg, st = seed.solve_axis(prob, pos, axis, center)
        xr, _ = seed.solve_axis(prob, pos, axis, center, solver=oracle_solver)
        assert st["stop"] == "residual"
        assert np.max(np.abs(xg - xr)) <= 1e-8 * np.max(np.abs(xr)), axis
    prob = macro_offsets_case()
    x, _ = seed.solve_axis(prob, np.array([[4.0, 0.0], [4.0, 0.0]]), 0, 4)
    assert np.allclose(x, [2.5, 5.5], atol=1e-12, rtol=0)

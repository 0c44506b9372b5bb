"""The oracle's restatement of `solve_quadratic` (crates/texo-pnr/src/lib.rs:
4586-4790) against the reference's own test and against direct solves."""
import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import problem as P
from texo_gb300 import seed


def reference_diagonal(n=128):
    return np.array([10.0 ** (-12.0 + 24.0 * i / (n - 1)) for i in range(n)])


def test_jacobi_pcg_is_not_truncated_at_the_legacy_hundred_iteration_budget():
    """lib.rs:14384-14439: raw CG stopped at 100 steps leaves a relative
    residual above 1e-4 on this 24-decade diagonal system; the Jacobi PCG
    reaches below 1e-12."""
    n = 128
    d = reference_diagonal(n)
    rhs = np.ones(n)
    # the legacy raw-CG budget, restated from the test
    x = np.zeros(n)
    r = rhs.copy()
    p = r.copy()
    init = float(r @ r)
    rr = init
    for _ in range(100):
        q = p * d
        dq = float(p @ q)
        if dq <= np.finfo(float).eps:
            break
        a = rr / dq
        x += a * p
        r -= a * q
        nxt = float(r @ r)
        p = r + (nxt / rr) * p
        rr = nxt
    legacy = np.sqrt(rr / init)
    xs, st, ok = ffi.solve_quadratic(d, np.zeros(n + 1, np.uint32), np.zeros(0, np.uint32), np.zeros(0), rhs)
    res = 1.0 - d * xs
    assert legacy > 1e-4
    assert ok and np.sqrt(float(res @ res) / init) < 1e-12


def b2b_system(seed_no=0, cells=2000, side=48, nets=2400):
    prob = P.synthetic(side, cells, 96, nets, 6.0, seed_no)
    pos = np.asarray(prob.initial_xy).reshape(-1, 2)
    d, ptr, idx, w, rhs, anch = seed.axis_system(prob, pos, 0)
    d, ptr, idx, w, rhs, floating = seed.finalize_gauges(d, ptr, idx, w, rhs, anch)
    return prob, pos, d, ptr, idx, w, rhs, floating


def test_multiply_quadratic_matches_the_csr_product():
    _, pos, d, ptr, idx, w, _, _ = b2b_system()
    from scipy.sparse import csr_matrix, diags
    v = np.random.default_rng(3).standard_normal(len(d))
    A = diags(d) - csr_matrix((w, idx, ptr), shape=(len(d), len(d)))
    got = ffi.multiply_quadratic(d, ptr, idx, w, v)
    assert np.max(np.abs(got - A @ v)) <= 1e-12 * np.max(np.abs(A @ v))


@pytest.mark.parametrize("seed_no", [0, 1])
def test_pcg_on_bound_to_bound_systems_meets_its_residual_target(seed_no):
    """The seed's systems (bound-to-bound edges at the initial positions,
    fixed IO anchored, floating components gauged) are SPD: PCG stops at
    |r| <= 1e-4 |r0| and lands next to the direct solution."""
    _, pos, d, ptr, idx, w, rhs, floating = b2b_system(seed_no)
    from scipy.sparse import csr_matrix, diags
    from scipy.sparse.linalg import spsolve
    x, st, ok = ffi.solve_quadratic(d, ptr, idx, w, rhs, pos[:, 0].copy())
    assert ok and st.stop == 0
    assert st.final_residual_squared <= st.target_squared
    A = diags(d) - csr_matrix((w, idx, ptr), shape=(len(d), len(d)))
    xd = spsolve(A.tocsc(), rhs)
    assert np.max(np.abs(x - xd)) <= 1e-3 * np.max(np.abs(xd))


def test_pcg_reports_breakdown_on_an_indefinite_system():
    """A negative curvature direction stops the recurrence as a breakdown and
    the solve reports it (finish_quadratic_solve's "breakdown" label)."""
    d = np.array([1.0, 1.0])
    ptr = np.array([0, 1, 2], np.uint32)
    idx = np.array([1, 0], np.uint32)
    w = np.array([3.0, 3.0])   # D - W = [[1, -3], [-3, 1]]: curvature -2 along (1, 1)
    x, st, ok = ffi.solve_quadratic(d, ptr, idx, w, np.array([1.0, 1.0]))
    assert not ok and st.stop == 1


def test_gauges_fix_one_unit_per_floating_component():
    _, _, d, ptr, idx, w, rhs, floating = b2b_system()
    for comp in floating:
        g = comp[0]
        assert d[g] == 1.0 and rhs[g] == 0.0 and ptr[g + 1] == ptr[g]
        assert not np.any(idx == g)

"""Pins the oracle's density model and Poisson solve against the reference's
own known-answer tests (crates/texo-pnr/src/electrostatic_placement.rs:1064-1844),
ported one by one, plus an independent scipy DCT cross-check."""
import functools
import math
import operator

import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi
from texo_gb300.problem import density_problem

LUT = (abi.KIND_LUT, 4)
REG = (abi.KIND_REGISTER, 0)
MEM = (abi.KIND_MEMORY, 0)


def fold_sum(values):
    """Sequential left fold, as Rust's Iterator::sum."""
    return functools.reduce(operator.add, list(values), -0.0)


def assert_close(actual, expected, tol):
    assert abs(actual - expected) <= tol, (actual, expected, tol)


def neumann_laplacian(w, h, v):
    r = np.zeros(w * h)
    for y in range(h):
        for x in range(w):
            i = y * w + x
            d = 0.0
            if x != 0:
                r[i] -= v[i - 1]
                d += 1
            if x + 1 != w:
                r[i] -= v[i + 1]
                d += 1
            if y != 0:
                r[i] -= v[i - w]
                d += 1
            if y + 1 != h:
                r[i] -= v[i + w]
                d += 1
            r[i] += d * v[i]
    return r


# electrostatic_placement.rs:1114-1120
def test_constant_density_is_only_the_removed_dc_mode():
    pot, e = ffi.poisson(7, 5, np.full(35, 3.25))
    assert_close(e, 0.0, 1e-24)
    assert np.all(pot == 0.0)


# :1122-1135
def test_spectral_solution_matches_the_direct_neumann_operator():
    d = np.array([((i * 17 + 3) % 23) - 11.0 for i in range(35)])
    mean = fold_sum(d) / 35.0
    pot, _ = ffi.poisson(7, 5, d)
    rec = neumann_laplacian(7, 5, pot)
    for a, b in zip(rec, d - mean):
        assert_close(a, b, 2e-12)


# :1137-1154
def test_manufactured_cosine_is_one_laplacian_eigenmode():
    f = 3.0
    d = np.array([math.cos(math.pi * f * (c + 0.5) / 11.0) for c in range(11)])
    ev = 4.0 * math.sin(math.pi * f / 22.0) ** 2
    pot, _ = ffi.poisson(11, 1, d)
    for a, rho in zip(pot, d):
        assert_close(a, rho / ev, 2e-13)


# :1156-1162
def test_cloud_in_cell_deposit_preserves_charge():
    d = np.zeros(30)
    ffi.deposit_bilinear(d, 6, 5, 2.25, 3.5, 7.0)
    ffi.deposit_bilinear(d, 6, 5, 5.0, 0.0, 11.0)
    assert_close(fold_sum(d), 18.0, 1e-14)


# :1164-1184
def test_interpolated_potential_gradient_matches_energy_finite_difference():
    def energy(x, y):
        d = np.full(117, -2.0 / 117.0)
        ffi.deposit_bilinear(d, 13, 9, x, y, 2.0)
        return ffi.poisson(13, 9, d)[1]
    x, y = 4.25, 5.375
    d = np.full(117, -2.0 / 117.0)
    ffi.deposit_bilinear(d, 13, 9, x, y, 2.0)
    pot, _ = ffi.poisson(13, 9, d)
    _, gx, gy = ffi.sample_bilinear(pot, 13, 9, x, y)
    eps = 1e-6
    assert_close(2 * gx, (energy(x + eps, y) - energy(x - eps, y)) / (2 * eps), 2e-8)
    assert_close(2 * gy, (energy(x, y + eps) - energy(x, y - eps)) / (2 * eps), 2e-8)


# :1186-1201
def test_quadratic_bspline_preserves_charge_and_has_zero_derivative_sum():
    for c in [0.0, 0.25, 1.0, 1.5, 3.75, 5.0]:
        _, w, dw = ffi.bspline_axis(6, c)
        assert_close(fold_sum(w), 1.0, 1e-15)
        assert_close(fold_sum(dw), 0.0, 1e-15)
    d = np.zeros(30)
    ffi.deposit(d, 6, 5, 2.25, 3.5, 7.0)
    ffi.deposit(d, 6, 5, 5.0, 0.0, 11.0)
    assert_close(fold_sum(d), 18.0, 1e-14)


def test_bspline_axis_folds_out_of_range_taps_onto_the_edge():
    idx, w, _ = ffi.bspline_axis(6, 0.0)
    assert list(idx) == [0, 0, 1]
    idx, w, _ = ffi.bspline_axis(6, 5.0)
    assert list(idx) == [4, 5, 5]
    idx, w, _ = ffi.bspline_axis(6, -3.0)       # clamped to 0
    assert list(idx) == [0, 0, 1]
    idx, w, _ = ffi.bspline_axis(6, 2.5)        # floor(3.0) = 3
    assert list(idx) == [2, 3, 4]
    assert w[0] == 0.5 and w[1] == 0.5 and w[2] == 0.0


# :1203-1223
@pytest.mark.parametrize("x,y", [(4.0, 5.0), (4.5, 5.5)])
def test_quadratic_bspline_energy_gradient_is_smooth_at_stencil_knots(x, y):
    def energy(px, py):
        d = np.full(117, -2.0 / 117.0)
        ffi.deposit(d, 13, 9, px, py, 2.0)
        return ffi.poisson(13, 9, d)[1]
    d = np.full(117, -2.0 / 117.0)
    ffi.deposit(d, 13, 9, x, y, 2.0)
    pot, _ = ffi.poisson(13, 9, d)
    _, gx, gy = ffi.sample(pot, 13, 9, x, y)
    eps = 1e-6
    assert_close(2 * gx, (energy(x + eps, y) - energy(x - eps, y)) / (2 * eps), 2e-8)
    assert_close(2 * gy, (energy(x, y + eps) - energy(x, y - eps)) / (2 * eps), 2e-8)


def prime_density(fine):
    i = np.arange(12192)
    d = ((i * 31 + 7) % 101) - 50.0
    if fine:
        d = d + ((i * 13 + 5) % 17) / 17.0
    return d


# :1225-1237
def test_prime_width_architecture_grid_is_supported_and_repeatable():
    d = prime_density(False)
    p1, e1 = ffi.poisson(127, 96, d)
    p2, e2 = ffi.poisson(127, 96, d)
    assert np.array_equal(p1, p2) and e1 == e2
    assert math.isfinite(e1) and e1 > 0


# :1239-1264 — the pin of the fast DCT against the orthonormal matrix form.
def test_fast_prime_grid_solver_matches_orthonormal_matrix_oracle():
    d = prime_density(True)
    fast, ef = ffi.poisson(127, 96, d)
    ref, er = ffi.poisson(127, 96, d, matrix=True)
    scale = max(1.0, float(np.max(np.abs(ref))))
    assert np.max(np.abs(fast - ref)) <= 2e-11 * scale
    assert_close(ef, er, 2e-12 * max(abs(er), 1.0))


def test_dct_basis_matches_scipy_orthonormal_dct():
    scipy_fft = pytest.importorskip("scipy.fft")
    for n in (1, 2, 7, 64, 127):
        b = ffi.dct_basis(n)
        ref = scipy_fft.dct(np.eye(n), type=2, norm="ortho", axis=0)
        assert np.max(np.abs(b - ref)) < 1e-13


def test_poisson_matches_scipy_spectral_solve():
    scipy_fft = pytest.importorskip("scipy.fft")
    rng = np.random.default_rng(3)
    w, h = 48, 37
    d = rng.standard_normal(w * h)
    pot, e = ffi.poisson(w, h, d)
    c = (d - d.mean()).reshape(h, w)
    X = scipy_fft.dctn(c, type=2, norm="ortho")
    ky = np.arange(h)[:, None]
    kx = np.arange(w)[None, :]
    lam = 4 * np.sin(np.pi * kx / (2 * w)) ** 2 + 4 * np.sin(np.pi * ky / (2 * h)) ** 2
    lam[0, 0] = 1.0
    Y = X / lam
    Y[0, 0] = 0.0
    ref = scipy_fft.idctn(Y, type=2, norm="ortho").ravel()
    assert np.max(np.abs(pot - ref)) <= 1e-12 * np.max(np.abs(ref))
    assert_close(e, 0.5 * float(np.dot(c.ravel(), ref)), 1e-10 * abs(e))


# ---- density model on the reference's 4x3 mixed device (:1303-1314) ------
def mixed_capacity():
    cap = np.zeros((2, 12), np.uint32)
    cap[0, 0:4] = 1     # LUT BELs on row 0
    cap[1, 4:8] = 1     # FF BELs on row 1
    return cap


def mixed(units, fixed_occupancy=None):
    return density_problem(4, 3, [LUT, REG], mixed_capacity(), units, fixed_occupancy=fixed_occupancy)


def evaluate_initial(problem):
    o = ffi.Oracle(problem)
    c, _, _ = o.initial()
    return o, c, o.evaluate(c, 8.0)


# :1316-1347
def test_fixed_occupancy_is_subtracted_from_its_exact_kind_and_point():
    units = [(1.0, 0.0, [(0, 0, 0, 1.0)]), (1.0, 1.0, [(1, 0, 0, 1.0)])]
    o = ffi.Oracle(mixed(units, fixed_occupancy=[[0, 0, 0]]))
    assert o.capacity(0)[0] == 0
    assert o.capacity(1)[4] == 1
    with pytest.raises(abi.TexoGpError) as e:
        ffi.Oracle(mixed(units, fixed_occupancy=[[0, 0, 0], [0, 0, 0]]))
    assert e.value.name == "FIXED_CAPACITY_EXHAUSTED"


# :1349-1388
def test_lut_and_register_fields_are_separate_for_one_atomic_unit():
    units = [(1.25, 0.25, [(0, 0.0, 0.0, 1.0), (1, 0.5, 0.5, 1.0)])]
    o, c, r = evaluate_initial(mixed(units))
    r2 = o.evaluate(c, 8.0)
    assert [f.kind for f in r["fields"]] == [abi.KIND_LUT, abi.KIND_REGISTER]
    assert all(f.real_charge == 1 for f in r["fields"])
    assert all(f.filler_charge == 3.0 for f in r["fields"])
    assert all(math.isfinite(f.energy) for f in r["fields"])
    assert np.array_equal(r["density"], r2["density"])
    assert np.array_equal(r["field_gradient"], r2["field_gradient"])


# :1390-1428
def test_model_gradient_matches_total_energy_finite_difference():
    def unit(x):
        return [(x, 0.4, [(0, 0.0, 0.0, 1.0), (1, 0.3, 0.4, 1.0)])]
    o = ffi.Oracle(mixed(unit(1.2)))
    c, _, _ = o.initial()

    def energy(x):
        cc = c.copy()
        cc[0] = x
        return fold_sum(f.energy for f in o.evaluate(cc, 8.0)["fields"])
    r = o.evaluate(c, 8.0)
    eps = 1e-6
    fd = (energy(1.2 + eps) - energy(1.2 - eps)) / (2 * eps)
    assert_close(fold_sum(r["field_gradient"][:, 0]), fd, 2e-8)


# :1430-1452
def test_capacity_background_and_real_deposit_preserve_charge():
    units = [(x + 0.25, 0.5, [(0, 0, 0, 1.0)]) for x in range(3)]
    o, c, r = evaluate_initial(mixed(units))
    r2 = o.evaluate(c, 8.0)
    assert np.array_equal(r["density"], r2["density"])
    f = r["fields"][0]
    assert_close(fold_sum(r["density"][0]), 0.0, 1e-14)
    assert_close(f.net_charge, 0.0, 1e-14)
    assert f.filler_charge == 1.0
    assert f.normalized_overflow <= 1.0


# :1454-1484
def test_physical_overflow_is_independent_of_filler_coordinates():
    o, c, base = evaluate_initial(mixed([(0.0, 0.0, [(0, 0, 0, 1.0)])]))
    moved = c.copy()
    for i in range(o.num_fillers):
        moved[2 * (o.units + i)] = 0.0 if i % 2 == 0 else 3.0
        moved[2 * (o.units + i) + 1] = 2.0
    r = o.evaluate(moved, 8.0)
    assert base["fields"][0].normalized_overflow == r["fields"][0].normalized_overflow
    assert base["fields"][0].energy != r["fields"][0].energy


# :1486-1509
def test_separating_overlapping_physical_cells_reduces_overflow():
    o = ffi.Oracle(mixed([(0.0, 0.0, [(0, 0, 0, 1.0)]), (0.0, 0.0, [(0, 0, 0, 1.0)])]))
    c, _, _ = o.initial()
    overlapping = o.evaluate(c, 8.0)
    c[2] = 1.0
    separated = o.evaluate(c, 8.0)
    assert separated["fields"][0].normalized_overflow < overlapping["fields"][0].normalized_overflow


# :1511-1532
def test_four_lut_carry_like_macro_is_one_rigid_variable():
    units = [(0.25, 0.0, [(0, float(k), 0.0, 1.0) for k in range(4)])]
    o, c, r = evaluate_initial(mixed(units))
    assert len(r["fields"]) == 1
    assert r["fields"][0].real_charge == 4
    assert r["fields"][0].filler_charge == 0.0
    assert_close(fold_sum(r["density"][0]), 0.0, 1e-14)


# :1534-1601
def test_adjusted_carry_macro_and_register_share_one_origin_across_density_fields():
    cap = np.ones((2, 8), np.uint32)

    def problem(x):
        members = [(0, float(k), 0.0, 1.0 + 0.1 * k) for k in range(4)] + [(1, 2.0, 0.0, 1.5)]
        return density_problem(8, 1, [LUT, REG], cap, [(x, 0.0, members)])
    o = ffi.Oracle(problem(2.0))
    c, _, _ = o.initial()
    r = o.evaluate(c, 8.0)
    assert [(f.kind, f.real_charge) for f in r["fields"]] == [(abi.KIND_LUT, 4), (abi.KIND_REGISTER, 1)]
    assert_close(r["fields"][0].filler_charge, 3.4, 1e-14)
    assert_close(r["fields"][1].filler_charge, 6.5, 1e-14)

    def total(x):
        cc = c.copy()
        cc[0] = x
        return fold_sum(f.energy for f in o.evaluate(cc, 8.0)["fields"])
    eps = 1e-6
    fd = (total(2.0 + eps) - total(2.0 - eps)) / (2 * eps)
    assert_close(fold_sum(r["field_gradient"][:, 0]), fd, 2e-8)


# :1664-1684
def test_legal_site_charges_exactly_cancel_the_smoothed_capacity():
    units = [(0.0, 0.0, [(0, float(k), 0.0, 1.0) for k in range(4)])]
    o, c, r = evaluate_initial(mixed(units))
    f = r["fields"][0]
    assert f.filler_charge == 0.0
    assert np.all(r["density"][0] == 0.0)
    assert f.energy == 0.0
    assert f.normalized_overflow == 0.0


# :1686-1724
def test_initial_fillers_are_capacity_proportional_and_kind_separated():
    units = [(1.0, 0.5, [(0, 0, 0, 1.0), (1, 0, 0, 1.0)])]
    o = ffi.Oracle(mixed(units))
    kinds, charges, _ = o.fillers()
    assert len(kinds) == 8
    for f in (0, 1):
        q = charges[kinds == f]
        assert len(q) == 4
        assert np.all(np.abs(q - 0.75) <= np.finfo(float).eps)
        assert fold_sum(q) == 3.0
    c, _, _ = o.initial()
    r = o.evaluate(c, 8.0)
    assert all(f.net_charge == 0.0 for f in r["fields"])


# :1726-1749
def test_adjusted_physical_area_consumes_only_filler_charge():
    o, c, r = evaluate_initial(mixed([(1.25, 0.0, [(0, 0, 0, 1.75)])]))
    _, q, _ = o.fillers()
    assert_close(fold_sum(q), 2.25, 1e-15)
    f = r["fields"][0]
    assert f.real_area == 1.75
    assert f.filler_charge == 2.25
    assert_close(f.net_charge, 0.0, 1e-14)


# :1751-1786
def test_filler_gradient_matches_energy_finite_difference():
    o = ffi.Oracle(mixed([(2.25, 0.5, [(0, 0, 0, 1.0)])]))
    kinds, _, xy = o.fillers()
    idx = int(np.nonzero((kinds == 0) & (xy[:, 0] == 1.0))[0][0])
    c, _, _ = o.initial()
    base = 2 * (o.units + idx)

    def energy(x):
        cc = c.copy()
        cc[base] = x
        return o.evaluate(cc, 8.0)["fields"][0].energy
    r = o.evaluate(c, 8.0)
    eps = 1e-6
    fd = (energy(1.0 + eps) - energy(1.0 - eps)) / (2 * eps)
    assert_close(r["field_gradient"][0][base], fd, 2e-8)


# :1788-1843
def test_capacity_shortage_and_malformed_units_are_typed_errors():
    cap = np.zeros((3, 12), np.uint32)
    cap[:2] = mixed_capacity()
    p = density_problem(4, 3, [LUT, REG, MEM], cap, [(0.0, 0.0, [(2, 0, 0, 1.0)])])
    with pytest.raises(abi.TexoGpError) as e:
        ffi.Oracle(p)
    assert e.value.name == "INSUFFICIENT_CAPACITY"
    ptr = np.array([0, 0], np.uint32)
    err = np.zeros(1, np.uint64)
    assert ffi.lib().orc_validate_units(ffi.P(ptr, ffi.C.c_uint32), 1, ffi.P(err, ffi.C.c_uint64)) == abi.CODE["EMPTY_UNIT"]
    real = mixed([(0.0, 0.0, [(0, 0, 0, 1.0)])])
    o = ffi.Oracle(real)
    c, _, _ = o.initial()
    o.set_filler_charge(0, -1.0)
    with pytest.raises(abi.TexoGpError) as e:
        o.evaluate(c, 8.0)
    assert e.value.name == "NEGATIVE_FILLER_CHARGE"
    o2 = ffi.Oracle(real)
    _, q, _ = o2.fillers()
    o2.set_filler_charge(0, q[0] + 1.0)
    with pytest.raises(abi.TexoGpError) as e:
        o2.evaluate(c, 8.0)
    assert e.value.name == "FILLER_CHARGE_MISMATCH"


def test_fixed_point_scatter_restatement_matches_fp64_density():
    """The device's int64 2^-32 scatter restated on the CPU agrees with the
    FP64 reference deposit to FP32 tap precision."""
    units = [(0.3 + 0.7 * k, 0.2 + 0.1 * k, [(0, 0, 0, 1.0)]) for k in range(3)]
    o = ffi.Oracle(mixed(units))
    c, _, _ = o.initial()
    r = o.evaluate(c, 8.0)
    phys, fill, ov, cnt = o.scatter_fixed(c)
    dens = (phys + fill).astype(np.float64) / 2.0 ** 32
    assert np.max(np.abs(dens - r["density"])) < 1e-6
    ref_over = np.maximum(phys, 0).sum()
    assert ov[0] == ref_over and cnt[0] == int((phys[0] > 0).sum())

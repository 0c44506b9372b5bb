"""The instance-area arithmetic (texo_gp_adjust_instance_areas and the area
formulas, host code behind the C ABI) against the reference's own tests,
crates/texo-pnr/src/instance_area.rs:427-662, ported one for one. Host logic
only: runs without a GPU."""
import struct

import numpy as np
import pytest

from texo_gb300 import abi
from texo_gb300 import routability as R

LUT4 = abi.KIND_LUT << 8 | 4          # keys sorting like ResourceKind: Lut(4) < Register
REG = abi.KIND_REGISTER << 8


def adjust(members, fillers):
    """members: (kind, current, routability, pin); fillers: (kind, current)."""
    m = np.array([x[1:] for x in members], dtype=np.float64).reshape(-1, 3)
    return R.adjust_instance_areas([x[0] for x in members], m[:, 0], m[:, 1], m[:, 2],
                                   [f[0] for f in fillers], [f[1] for f in fillers])


def totals(members, member_areas, fillers, filler_areas):
    t = {}
    for x, a in zip(members, member_areas):
        t[x[0]] = t.get(x[0], 0.0) + a
    for f, a in zip(fillers, filler_areas):
        t[f[0]] = t.get(f[0], 0.0) + a
    return t


def close(a, b):
    assert abs(a - b) < 1.0e-9, (a, b)


def test_fractional_charge_is_conserved_per_resource():
    members = [(LUT4, 0.75, 1.50, 0.50), (LUT4, 1.25, 1.50, 2.00), (REG, 0.50, 0.75, 0.50)]
    fillers = [(LUT4, 0.30), (LUT4, 0.70), (REG, 0.75)]
    before = totals(members, [x[1] for x in members], fillers, [f[1] for f in fillers])
    r = adjust(members, fillers)
    after = totals(members, r.member_areas, fillers, r.filler_areas)
    assert sorted(before) == sorted(after)
    for k, v in before.items():
        close(after[k], v)
    assert r.requires_optimizer_reset


def test_resource_scaling_never_exceeds_capacity_or_borrows_other_fillers():
    for lut_quarters in range(0, 9):
        for requested_quarters in range(0, 17):
            lut_filler = lut_quarters / 4.0
            requested = 1.0 + requested_quarters / 4.0
            r = adjust([(LUT4, 1.0, requested, 0.0), (REG, 1.0, 5.0, 0.0)], [(LUT4, lut_filler), (REG, 10.0)])
            assert r.member_areas[0] <= 1.0 + lut_filler + 1.0e-12
            assert r.member_areas[0] <= requested + 1.0e-12
            assert r.filler_areas[0] >= 0.0
            close(r.member_areas[0] + r.filler_areas[0], 1.0 + lut_filler)


def test_varied_fractional_inputs_preserve_charge_and_only_shrink_fillers():
    for first_eighths in range(0, 17):
        for second_eighths in range(0, 17):
            for requested_eighths in range(0, 33):
                first, second = first_eighths / 8.0, second_eighths / 8.0
                requested = 0.625 + requested_eighths / 8.0
                r = adjust([(LUT4, 0.625, requested, 0.0)], [(LUT4, first), (LUT4, second)])
                assert r.member_areas[0] >= 0.625
                assert r.filler_areas[0] <= first and r.filler_areas[1] <= second
                close(r.member_areas[0] + r.filler_areas[0] + r.filler_areas[1], 0.625 + first + second)


def test_physical_members_never_deflate():
    members = [(LUT4, 1.25, 0.0, 0.5), (REG, 0.5, 0.1, 0.0)]
    r = adjust(members, [(LUT4, 2.0)])
    assert all(a >= x[1] for x, a in zip(members, r.member_areas))
    assert not r.requires_optimizer_reset


def test_heterogeneous_macro_has_one_origin_and_distinct_member_forces():
    r = adjust([(LUT4, 0.75, 1.50, 0.0), (REG, 0.50, 0.50, 1.25)], [(LUT4, 2.0), (REG, 2.0)])
    a0, a1 = r.member_areas
    assert abs(a0 - a1) > 1.0e-9

    def energy(x, y):
        lut = 0.5 * (x + 0.25) ** 2 + 1.5 * (y - 0.50) ** 2
        ff = 2.0 * (x - 0.75) ** 2 + 0.25 * (y + 0.25) ** 2
        return a0 * lut + a1 * ff

    x, y, eps = 1.3, 2.1, 1.0e-6
    ax = a0 * (x + 0.25) + a1 * 4.0 * (x - 0.75)
    ay = a0 * 3.0 * (y - 0.50) + a1 * 0.5 * (y + 0.25)
    assert abs(ax - (energy(x + eps, y) - energy(x - eps, y)) / (2 * eps)) < 1.0e-8
    assert abs(ay - (energy(x, y + eps) - energy(x, y - eps)) / (2 * eps)) < 1.0e-8


def test_zero_congestion_is_identity_and_does_not_request_reset():
    current = 1.25
    routing = R.routability_optimized_area(current, 0.0, 0.0)
    pin = R.pin_optimized_area(0, 4.0, 0.0)
    r = adjust([(LUT4, current, routing, pin)], [(LUT4, 3.75)])
    assert list(r.member_areas) == [current] and list(r.filler_areas) == [3.75]
    assert not r.requires_optimizer_reset


def bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def test_full_scale_installs_the_requested_bits_without_a_fake_followup_reset():
    current = 1.0
    requested = struct.unpack("<d", struct.pack("<Q", bits(current) + 1))[0]
    first = adjust([(REG, current, requested, 0.0)], [(REG, 1.0)])
    assert bits(first.member_areas[0]) == bits(requested)
    assert first.requires_optimizer_reset
    second = adjust([(REG, first.member_areas[0], requested, 0.0)], [(REG, 1.0)])
    assert bits(second.member_areas[0]) == bits(requested)
    assert bits(second.filler_areas[0]) == bits(1.0)
    assert not second.requires_optimizer_reset


def test_rudy_bin_uses_architecture_capacity_and_caps_blocked_direction_inflation():
    close(R.routability_optimized_area_from_bin(1.25, 0.0, 0, 0.0, 0), 0.0)
    close(R.routability_optimized_area_from_bin(1.25, 0.25, 0, 0.0, 0), 2.5)
    wide = 2 ** 32 - 1 + 17
    close(R.routability_optimized_area_from_bin(1.25, float(2 ** 32 - 1) + 17.0, wide, 0.0, 0), 1.25)


def test_adjustment_is_deterministic():
    members = [(REG, 0.5, 1.25, 0.0), (LUT4, 0.75, 0.0, 2.0), (REG, 1.0, 1.125, 1.25)]
    fillers = [(REG, 0.125), (LUT4, 0.25), (REG, 0.875)]
    first = adjust(members, fillers)
    for _ in range(100):
        again = adjust(members, fillers)
        assert np.array_equal(again.member_areas, first.member_areas)
        assert np.array_equal(again.filler_areas, first.filler_areas)
        assert again.resource_scales == first.resource_scales
        assert again.requires_optimizer_reset == first.requires_optimizer_reset
    assert list(first.resource_scales) == [LUT4, REG]   # ascending kind order


def test_invalid_inputs_name_the_entry():
    with pytest.raises(abi.TexoGpError) as e:
        adjust([(LUT4, 1.0, 1.0, 0.0), (LUT4, 1.0, -1.0, 0.0)], [(LUT4, 1.0)])
    assert e.value.code == abi.CODE["INSTANCE_AREA_MEMBER"] and e.value.index == 1
    with pytest.raises(abi.TexoGpError) as e:
        adjust([(LUT4, 1.0, 1.0, 0.0)], [(LUT4, 1.0), (LUT4, float("nan"))])
    assert e.value.code == abi.CODE["INSTANCE_AREA_FILLER"] and e.value.index == 1
    with pytest.raises(abi.TexoGpError) as e:
        R.routability_optimized_area(-1.0, 0.0, 0.0)
    assert e.value.code == abi.CODE["INSTANCE_AREA_OVERFLOW"]
    with pytest.raises(abi.TexoGpError):
        R.pin_optimized_area(2 ** 32, 1.0, 1.0)


# eplace.rs:1778-1797
def test_rudy_inflates_exchangeable_slice_area_but_not_hard_memory_charge():
    congested = 2.0 ** 0.5
    f = R.routability_adjusted_member_area
    assert abs(f(abi.KIND_LUT, 1.0, congested, 0.0) - 2.0) <= np.finfo(float).eps
    assert abs(f(abi.KIND_REGISTER, 1.0, 0.0, congested) - 2.0) <= np.finfo(float).eps
    assert f(abi.KIND_MEMORY, 1.0, congested, congested) == 1.0

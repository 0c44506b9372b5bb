"""The ECP5 device adapter on the reference's own device fixture
(tests/golden/minimal_ecp5.json, derived from crates/texo-target-ecp5/
fixtures/minimal-ecp5.json by tests/golden/make_ecp5_fixture.py).

The fixture is a 2 x 1 device: location 0 holds SLICEA.K0/K1 (COMB z 0 / 4,
FCO of K0 on K1's FCI, K1's FCO on location 1's K0 FCI), SLICEB.K0/K1 (z 8 /
12, no carry pins), a PIO, one FF at z 1, an EBR and a DCCA; location 1 holds
one slice (K0/K1 chained), an FF, an EBR and two PIOs. The expected BEL ids,
carry pairs and chains, LUT-FF pairs and wide-LUT clusters below follow by
hand from the reference's rules (lib.rs:2768-2907, 2961-3043, 3868-3893)
applied to that fixture.
"""
import copy
import json
import os

import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi, ecp5

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "minimal_ecp5.json")


@pytest.fixture(scope="module")
def raw():
    with open(FIXTURE) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def arch(raw):
    return ecp5.read_architecture(raw)


def test_bels_in_location_then_record_order(arch):
    assert (arch.width, arch.height, arch.num_bels) == (2, 1, 14)
    assert arch.bel_name[:4] == ["X0/Y0/SLICEA.K0", "X0/Y0/SLICEA.K1", "X0/Y0/SLICEB.K0", "X0/Y0/SLICEB.K1"]
    assert arch.bel_name[8] == "X1/Y0/SLICEA.K0"
    assert arch.bels_of_kind(ecp5.LUT4) == [0, 1, 2, 3, 8, 9]
    assert arch.bels_of_kind(ecp5.REGISTER) == [5, 10]
    assert arch.bels_of_kind((abi.KIND_MEMORY, 0)) == [6, 11]
    assert arch.bels_of_kind((abi.KIND_IO, 0)) == [4, 12, 13]
    assert arch.bels_of_kind((abi.KIND_CLOCK, 0)) == [7]
    # FCO of location 0's K1 resolves to location 1's wire 19, K0's FCI there
    assert arch.find_bel_pin(1, "FCO") == arch.find_bel_pin(8, "FCI")
    assert arch.num_wires == 36 + 27 and len(arch.pip_from) == 14


def test_choice_generators(arch):
    assert ecp5.physical_carry_pairs(arch) == [[0, 1], [8, 9]]
    assert ecp5.carry_chain_assignments(arch, 1) == [[0, 1], [8, 9]]
    assert ecp5.carry_chain_assignments(arch, 2) == [[0, 1, 8, 9]]
    assert ecp5.carry_chain_assignments(arch, 3) == []
    assert ecp5.carry_chain_assignments(arch, 0) == []
    assert ecp5.lut_ff_assignments(arch) == [[0, 5], [8, 10]]
    assert ecp5.wide_lut_assignments(arch, 2) == [[0, 1], [2, 3], [8, 9]]
    assert ecp5.wide_lut_assignments(arch, 4) == [[0, 1, 2, 3]]
    assert ecp5.wide_lut_assignments(arch, 8) == []
    assert ecp5.wide_lut_assignments(arch, 3) == []
    assert ecp5.distributed_ram_assignments(arch) == []


@pytest.mark.parametrize("edit,reason", [
    (lambda d: d.update(schema_version=6), "UnsupportedSchema"),
    (lambda d: d.update(family="ICE40"), "WrongFamily"),
    (lambda d: d["provenance"].update(database_revision=""), "MissingProvenance"),
    (lambda d: d["provenance"].update(split_slice_mode=False), "SplitSliceRequired"),
    (lambda d: d["locations"].pop(), "IncompleteLocationGrid"),
    (lambda d: d["locations"][1].update(x=0), "DuplicateLocation"),
    (lambda d: d["locations"][1].update(location_type=5), "UnknownLocationType"),
    (lambda d: d["locations"][1].update(x=7), "LocationOutsideDevice"),
    (lambda d: d["location_types"][1]["pips"][5]["to"].update(dx=-2), "RelativeReferenceOutsideDevice"),
    (lambda d: d["location_types"][0]["bels"][0]["pins"][0]["wire"].update(index=99), "UnknownWireReference"),
])
def test_import_errors(raw, edit, reason):
    d = copy.deepcopy(raw)
    edit(d)
    with pytest.raises(ecp5.ArchitectureError) as e:
        ecp5.read_architecture(d)
    assert e.value.reason == reason


def fixture_design(arch):
    """Cells: 0-1 a one-pair carry chain, 2-3 a LUT-FF pair, 4 a lone LUT,
    5 an IO fixed on PIOA, 6 a clock buffer fixed on DCCA0 driving the FF."""
    luts = ecp5.single_cell_choices(arch, ecp5.LUT4)
    units = [
        ecp5.Unit([0, 1], ecp5.carry_chain_assignments(arch, 1)),
        ecp5.Unit([2, 3], ecp5.lut_ff_assignments(arch)),
        ecp5.Unit([4], luts),
        ecp5.Unit([5], [[4]]),
        ecp5.Unit([6], [[7]]),
    ]
    kinds = [ecp5.LUT4, ecp5.LUT4, ecp5.LUT4, ecp5.REGISTER, ecp5.LUT4, (abi.KIND_IO, 0), (abi.KIND_CLOCK, 0)]
    nets = [(5, [0, 4]), (1, [2]), (2, [3]), (3, [5]), (6, [3]), (4, [])]
    return units, kinds, nets


def test_placement_problem_on_the_fixture(arch):
    units, kinds, nets = fixture_design(arch)
    prob, info = ecp5.placement_problem(arch, 7, units, nets, cell_kind=kinds, sink_weights={(1, 0): 3})
    assert prob.fields == [ecp5.LUT4, ecp5.REGISTER]
    assert np.array_equal(prob.capacity, [[4, 2], [1, 1]])
    # one-choice units: fixed cells and, for exchangeable kinds, fixed occupancy
    assert prob.fixed_occupancy.shape == (0, 3)       # PIO and DCCA are not density kinds
    assert list(info["density_units"]) == [0, 1, 2]
    assert np.array_equal(prob.lower_xy[:3], [[0, 0], [0, 0], [0, 0]])
    assert np.array_equal(prob.upper_xy[:3], [[1, 0], [1, 0], [1, 0]])
    assert np.array_equal(prob.lower_xy[3], prob.upper_xy[3]) and prob.cell_fixed[5] == 1
    assert list(prob.member_ptr) == [0, 2, 4, 5, 5, 5]
    assert list(prob.member_field) == [0, 0, 0, 1, 0]
    # the clock-driven net and the sinkless net are left out; the weight-3
    # sink is a timed arc of extra weight 2
    assert list(prob.net_ptr) == [0, 3, 5, 7, 9]
    assert list(prob.arc_driver_cell) == [1] and list(prob.arc_sink_cell) == [2]
    assert list(prob.arc_extra_weight) == [2]
    # the oracle accepts the problem and evaluates it
    o = ffi.Oracle(prob, abi.default_params_py())
    c, lo, hi = o.initial()
    ev = o.evaluate(c, 2.0)
    assert np.isfinite(ev["wirelength"]) and ev["wirelength"] > 0 and len(ev["fields"]) == 2


def test_units_must_cover_every_cell(arch):
    units, kinds, nets = fixture_design(arch)
    with pytest.raises(ValueError):
        ecp5.placement_problem(arch, 8, units, nets)
    bad = units[:2] + [ecp5.Unit([4], [[0, 1]])] + units[3:]
    with pytest.raises(ValueError):
        ecp5.placement_problem(arch, 7, bad, nets)


# eplace.rs:1905-1914 (only_interchangeable_ecp5_resource_classes_get_density_fields)
def test_only_interchangeable_resource_classes_get_density_fields():
    ex = ecp5.EXCHANGEABLE
    assert abi.KIND_LUT in ex and abi.KIND_REGISTER in ex and abi.KIND_MEMORY in ex
    for k in (abi.KIND_CLOCK, abi.KIND_LOGIC, abi.KIND_IO, abi.KIND_CONSTANT):
        assert k not in ex

"""The register-clustering oracle against the reference's own tests,
crates/texo-pnr/src/register_clustering.rs:114-190, ported one for one.
CPU only."""
import struct

import numpy as np

from oracle import ffi
from texo_gb300 import abi


def bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def test_soft_ceiling_linearizes_only_the_start_of_each_step():
    for (v, d), want in [((2.0, 2.0), 1.0), ((2.5, 2.0), 1.5), ((3.5, 2.0), 2.0), ((8.0, 4.0), 2.0)]:
        assert bits(ffi.soft_division_ceiling(v, d)) == bits(want)


def test_ce_partition_changes_charge_but_other_tile_controls_do_not():
    xy = np.full((4, 2), 10.0)
    clock_lsr = [[1, 2], [1, 2], [1, 2], [9, 2]]
    code, areas = ffi.register_clustering_areas(xy, clock_lsr, [3, 3, 4, 3], 4)
    assert code == 0
    assert bits(areas[0]) == bits(areas[1])
    code, compatible = ffi.register_clustering_areas(xy, clock_lsr, [3, 3, 3, 3], 4)
    assert code == 0
    assert bits(areas[0]) != bits(compatible[0])
    assert bits(areas[3]) == bits(compatible[3])


def test_rigid_members_are_not_duplicated_by_the_charge_estimator():
    code, areas = ffi.register_clustering_areas([[3.25, 4.5]], [[1, 2]], [3], 2)
    assert code == 0 and len(areas) == 1
    assert abs(areas[0] - 8.0) < 1.0e-12


def test_other_control_sets_are_excluded_from_a_registers_expectation():
    """The reference's fixed-control test: control records of cells that are
    not movable registers do not enter the expectation. With per-register
    controls, the same statement is that registers of another control set do
    not change a register's area."""
    code, alone = ffi.register_clustering_areas([[2.0, 3.0]], [[4, 5]], [6], 2)
    code2, with_other = ffi.register_clustering_areas([[2.0, 3.0], [2.0, 3.0]], [[4, 5], [4, 9]], [6, 7], 2)
    assert code == 0 and code2 == 0
    assert bits(alone[0]) == bits(with_other[0])


def test_empty_and_invalid():
    assert ffi.register_clustering_areas(np.zeros((0, 2)), np.zeros((0, 2)), [], 5)[0] == 0
    code, areas = ffi.register_clustering_areas([[1.0, 1.0]], [[1, 1]], [1], 0)
    assert code == 0 and areas[0] == 0.0
    assert ffi.register_clustering_areas([[1.0, 1.0]], [[1, 1]], [1], 2 ** 32)[0] == abi.CODE["INVALID_NORMALIZATION"]
    assert ffi.register_clustering_areas([[np.nan, 1.0]], [[1, 1]], [1], 3)[0] == abi.CODE["INVALID_NORMALIZATION"]

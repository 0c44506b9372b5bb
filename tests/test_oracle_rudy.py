"""The oracle's restatement of `continuous_routing_demand`
(crates/texo-pnr/src/eplace.rs:856-937) against the reference's own test."""
import numpy as np

from oracle import ffi


def test_overlap_weighted_continuous_rudy_conserves_directional_hpwl():
    """eplace.rs:1687-1695: the two boxes spread 3.5 horizontal and 9.5
    vertical demand (their directional HPWL), all entries non-negative."""
    boxes = [(1.25, 4.75, 2.50, 5.00), (0.0, 0.0, 0.0, 7.0)]
    h, v, ok = ffi.routing_demand(10, 10, boxes)
    assert ok
    assert abs(h.sum() - 3.5) <= 1e-12 and abs(v.sum() - 9.5) <= 1e-12
    assert (h >= 0).all() and (v >= 0).all()


def test_unordered_or_nonfinite_boxes_are_rejected():
    assert not ffi.routing_demand(4, 4, [(2.0, 1.0, 0.0, 1.0)])[2]
    assert not ffi.routing_demand(4, 4, [(0.0, np.inf, 0.0, 1.0)])[2]


def test_boxes_partly_outside_the_grid_deposit_only_inside():
    h, v, ok = ffi.routing_demand(4, 4, [(-3.0, 1.0, 2.0, 6.0)])
    assert ok
    area = 5.0 * 5.0
    # the widened box [-3.5, 1.5] x [1.5, 6.5] covers x tiles 0..1 and y
    # tiles 2..3 of the grid fully: 2 x 2 tiles of density dx / area each
    assert abs(h.sum() - 4.0 / area * 2.0 * 2.0) <= 1e-12
    assert h[2, 0] == h[3, 1] == 4.0 / area and h[:2].sum() == 0.0

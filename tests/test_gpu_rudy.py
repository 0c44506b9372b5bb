"""texo_gp_routing_demand (the GPU `continuous_routing_demand`,
crates/texo-pnr/src/eplace.rs:856-937) against the FP64 oracle: the
fixed-point map is within 2^-41 per box and tile of the FP64 sums (tested:
1e-10 absolute on the reference's own case, 1e-9 normwise relative on
placement-scale maps), deterministic, and rejects bad boxes alike."""
import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi, problem as P
from texo_gb300.placer import net_bounding_boxes, routing_demand

pytestmark = pytest.mark.gpu


def test_reference_known_answer_on_the_gpu():
    boxes = [(1.25, 4.75, 2.50, 5.00), (0.0, 0.0, 0.0, 7.0)]
    h, v, _ = routing_demand(10, 10, boxes)
    hr, vr, ok = ffi.routing_demand(10, 10, boxes)
    assert ok
    assert abs(h.sum() - 3.5) <= 1e-10 and abs(v.sum() - 9.5) <= 1e-10
    assert (h >= 0).all() and (v >= 0).all()
    assert np.max(np.abs(h - hr)) <= 1e-11 and np.max(np.abs(v - vr)) <= 1e-11


@pytest.mark.parametrize("side,cells,nets,seed_no", [(48, 2000, 2400, 0), (110, 10000, 12000, 5)])
def test_gpu_demand_matches_the_oracle_on_placement_boxes(side, cells, nets, seed_no):
    prob = P.synthetic(side, cells, 96, nets, 6.0, seed_no)
    rng = np.random.default_rng(seed_no)
    pos = rng.uniform(0, side - 1, size=(prob.num_units, 2))
    boxes = net_bounding_boxes(prob, pos)
    h, v, _ = routing_demand(side, side, boxes)
    hr, vr, ok = ffi.routing_demand(side, side, boxes)
    assert ok
    assert np.max(np.abs(h - hr)) <= 1e-9 * np.max(hr)
    assert np.max(np.abs(v - vr)) <= 1e-9 * np.max(vr)
    # conservation: each box spreads dx (dy) over the grid when it lies inside
    h2, v2, _ = routing_demand(side, side, boxes)
    assert np.array_equal(h, h2) and np.array_equal(v, v2)


def test_bad_boxes_are_rejected():
    with pytest.raises(abi.TexoGpError) as e:
        routing_demand(4, 4, [(2.0, 1.0, 0.0, 1.0)])
    assert e.value.name == "INVALID_NORMALIZATION"


@pytest.mark.parametrize("side,cells,io,nets,sigma", [(210, 42000, 365, 50000, 12.0),
                                                     (1024, 1000000, 4096, 1200000, 24.0)])
def test_full_size_demand(side, cells, io, nets, sigma):
    """The workloads' own sizes: the 42k workload's 50,000 boxes against the
    oracle in full; the 1M workload's 1.2 M boxes deterministic on the GPU
    and, on a 20,000-box sample, equal to the oracle."""
    prob = P.synthetic(side, cells, io, nets, sigma, 0)
    pos = np.random.default_rng(1).uniform(0, side - 1, size=(prob.num_units, 2))
    boxes = net_bounding_boxes(prob, pos)
    h, v, _ = routing_demand(side, side, boxes)
    h2, v2, _ = routing_demand(side, side, boxes)
    assert np.array_equal(h, h2) and np.array_equal(v, v2)
    sample = boxes if len(boxes) <= 60000 else boxes[:20000]
    hs, vs, _ = routing_demand(side, side, sample)
    hr, vr, ok = ffi.routing_demand(side, side, sample)
    assert ok
    assert np.max(np.abs(hs - hr)) <= 1e-9 * np.max(hr)
    assert np.max(np.abs(vs - vr)) <= 1e-9 * np.max(vr)

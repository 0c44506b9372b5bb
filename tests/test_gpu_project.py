"""`project` with the GPU auctions on the adapter's ECP5-like fabric: the
same choices as with the oracle's parallel-round auctions (the GPU matches
that restatement bit for bit), and the whole path from the device snapshot
(adapter -> placement -> projection) on the GPU."""
import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi, ecp5, legalize as L
from texo_gb300.placer import default_params, place

from test_project import fabric_case, oracle_auction

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed,scale", [(0, 1), (1, 1), (0, 4)])
def test_gpu_projection_equals_the_parallel_restatement(seed, scale):
    arch, units, targets = fabric_case(seed)
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    g = L.project(arch.width, arch.height, bel_xy, units, targets, cost_scale=scale)
    o = L.project(arch.width, arch.height, bel_xy, units, targets, cost_scale=scale, auction=oracle_auction(True))
    assert np.array_equal(g.preferred, o.preferred)
    assert g.stats["bids"] == o.stats["bids"]
    assert np.all(g.preferred >= 0)


def test_device_snapshot_to_legal_choices_on_the_gpu():
    arch = ecp5.read_architecture(ecp5.synthetic_architecture(24, 24))
    nc, units, kinds, nets = ecp5.synthetic_design(arch, 3, luts=1200, ffs=600, lut_ff_pairs=400,
                                                   carry=((30, 4), (10, 6)), io=40)
    prob, _ = ecp5.placement_problem(arch, nc, units, nets, cell_kind=kinds)
    targets, _, st = place(prob, default_params(best_effort=1))
    prm = abi.default_params_py()
    prm.best_effort = 1
    _, _, _, rs = ffi.Oracle(prob, prm).place(threads=4)
    assert st["converged"] and abs(st["hpwl"] - rs.hpwl) <= 0.01 * rs.hpwl
    bel_xy = np.stack([arch.bel_x, arch.bel_y], 1)
    pj = L.project(arch.width, arch.height, bel_xy, units, targets)
    bels = pj.bels(units)
    assert np.all(pj.preferred >= 0) and np.all(bels >= 0)
    assert len(np.unique(bels)) == len(bels)
    for u, unit in enumerate(units):
        assert list(bels[unit.cells]) == list(unit.choices[pj.preferred[u]])

"""The GPU register-clustering areas (texo_gp_register_clustering_areas)
against the oracle's restatement of `clustering_areas`
(crates/texo-pnr/src/register_clustering.rs:17-97) and the reference's own
test cases. erf differs between the device and the C library, so areas agree
to 1e-12 relative, not bit for bit."""
import numpy as np
import pytest

from oracle import ffi
from texo_gb300 import abi
from texo_gb300 import routability as R

pytestmark = pytest.mark.gpu


def random_registers(seed, n, side, sets, enables):
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0, side, (max(1, n // 50), 2))
    xy = centres[rng.integers(0, len(centres), n)] + rng.normal(0, 1.5, (n, 2))
    clock_lsr = np.stack([rng.integers(0, sets, n), rng.integers(0, 2, n)], axis=1).astype(np.uint64)
    ce = rng.integers(0, enables, n).astype(np.uint64) * np.uint64(1 << 40)   # keys above 2^32
    return xy, clock_lsr, ce


@pytest.mark.parametrize("seed,n,side,sets,enables,count", [
    (0, 300, 12.0, 2, 3, 300), (1, 2000, 40.0, 4, 8, 5000), (2, 1500, 20.0, 1, 1, 1500), (3, 50, 2.0, 1, 5, 60)])
def test_matches_the_oracle(seed, n, side, sets, enables, count):
    xy, clock_lsr, ce = random_registers(seed, n, side, sets, enables)
    got, _ = R.register_clustering_areas(xy, clock_lsr, ce, count)
    code, want = ffi.register_clustering_areas(xy, clock_lsr, ce, count)
    assert code == 0
    assert np.max(np.abs(got - want) / np.abs(want)) <= 1.0e-12
    again, _ = R.register_clustering_areas(xy, clock_lsr, ce, count)
    assert np.array_equal(again, got)


def test_reference_cases_on_the_device():
    xy = np.full((4, 2), 10.0)
    clock_lsr = [[1, 2], [1, 2], [1, 2], [9, 2]]
    a, _ = R.register_clustering_areas(xy, clock_lsr, [3, 3, 4, 3], 4)
    b, _ = R.register_clustering_areas(xy, clock_lsr, [3, 3, 3, 3], 4)
    assert a[0] == a[1] and a[0] != b[0] and a[3] == b[3]
    one, _ = R.register_clustering_areas([[3.25, 4.5]], [[1, 2]], [3], 2)
    assert abs(one[0] - 8.0) < 1.0e-12
    empty, _ = R.register_clustering_areas(np.zeros((0, 2)), np.zeros((0, 2)), [], 5)
    assert len(empty) == 0
    zero, _ = R.register_clustering_areas([[1.0, 1.0]], [[1, 1]], [1], 0)
    assert zero[0] == 0.0
    for args in (([[1.0, 1.0]], [[1, 1]], [1], 2 ** 32), ([[np.nan, 1.0]], [[1, 1]], [1], 3)):
        with pytest.raises(abi.TexoGpError) as e:
            R.register_clustering_areas(*args)
        assert e.value.code == abi.CODE["INVALID_NORMALIZATION"]


def test_propose_area_adjustment_matches_a_restatement():
    """`propose_area_adjustment` (eplace.rs:627-740) composed from the GPU
    RUDY map and clustering areas against the same step restated with the
    oracle's FP64 RUDY and clustering and plain loops, on the 48 x 48
    workload's placement with half its members turned into registers, a
    routing-capacity map with a blocked band, and register control sets."""
    import types

    from texo_gb300 import problem as P
    from texo_gb300.placer import Placer, default_params, net_bounding_boxes
    prob = P.synthetic(48, 2000, 96, 2400, 6.0, 0)
    with Placer(prob, default_params(best_effort=1, max_iterations=1000, engine=abi.ENGINE_DEVICE)) as g:
        _, coords, _ = g.run(allow_nonconverged=True)
    view = types.SimpleNamespace(**{k: getattr(prob, k) for k in (
        "num_units", "member_ptr", "lower_xy", "upper_xy", "member_offset_xy", "member_charge", "member_cell",
        "cell_unit", "cell_offset_xy", "cell_fixed", "cell_fixed_xy", "net_ptr", "pin_cell")})
    view.fields = [(abi.KIND_LUT, 4), (abi.KIND_REGISTER, 0)]
    view.member_field = (np.arange(len(prob.member_field)) % 2).astype(np.uint32)
    cap_h = np.full((48, 48), 3, np.uint32)
    cap_v = np.full((48, 48), 4, np.uint32)
    cap_h[20:24, :] = 0                                   # a blocked band: demand there is a hotspot
    controls = {int(c): (int(c) % 3, 0, int(c) % 5) for c in prob.member_cell}
    fillers = ([0, 1], [300.0, 250.0])
    adj, m = R.propose_area_adjustment(view, coords, cap_h, cap_v, *fillers, register_controls=controls)

    # the restatement
    U = prob.num_units
    pos = coords[: 2 * U].reshape(-1, 2)
    h, v, ok = ffi.routing_demand(48, 48, net_bounding_boxes(view, pos))
    assert ok
    ptr = prob.member_ptr
    movable = np.any(prob.lower_xy != prob.upper_xy, axis=1)
    members = [i for u in range(U) if movable[u] for i in range(ptr[u], ptr[u + 1])]
    unit_of = {i: u for u in range(U) for i in range(ptr[u], ptr[u + 1])}

    def rnd(v_, n):
        return int(min(max(np.floor(v_ + 0.5), 0), n - 1))

    def util(dem, cap, x, y):
        return (0.0 if dem[y, x] == 0.0 else np.sqrt(2.0)) if cap[y, x] == 0 else dem[y, x] / float(cap[y, x])

    want_route, keys, cur, regs = [], [], [], []
    for i in members:
        u = unit_of[i]
        x = rnd(pos[u, 0] + prob.member_offset_xy[i][0], 48)
        y = rnd(pos[u, 1] + prob.member_offset_xy[i][1], 48)
        hu, vu = min(util(h, cap_h, x, y), np.sqrt(2.0)), min(util(v, cap_v, x, y), np.sqrt(2.0))
        q = float(prob.member_charge[i])
        want_route.append(q * min(max(hu, vu) ** 2, 2.0))
        keys.append(R.kind_key(view.fields[view.member_field[i]]))
        cur.append(q)
        if view.member_field[i] == 1:
            regs.append(i)
    rxy = np.array([pos[unit_of[i]] + prob.member_offset_xy[i] for i in regs])
    rctl = np.array([controls[int(prob.member_cell[i])] for i in regs], dtype=np.uint64)
    code, rarea = ffi.register_clustering_areas(rxy, rctl[:, :2], rctl[:, 2], int(np.sum(movable[prob.cell_unit])))
    assert code == 0
    clus = np.zeros(len(members))
    clus[[members.index(i) for i in regs]] = rarea
    want = R.adjust_instance_areas(keys, cur, want_route, np.zeros(len(members)),
                                   [R.kind_key(view.fields[f]) for f in fillers[0]], fillers[1], clus)
    assert np.max(np.abs(adj.member_areas - want.member_areas) / want.member_areas) <= 1e-9
    assert np.max(np.abs(adj.filler_areas - want.filler_areas) / np.maximum(want.filler_areas, 1.0)) <= 1e-9
    assert adj.requires_optimizer_reset == want.requires_optimizer_reset
    assert m["members_inflated"] > 0 and m["maximum_horizontal_utilization"] >= np.sqrt(2.0) - 1e-12


def test_full_size_register_set():
    """The 42k workload's size: 42,000 registers at the placement's movable
    positions in 8 control sets x 16 clock enables; control set 0 (about
    5,000 registers, the oracle's every pair) equal to the GPU's full-set
    areas within 1e-12, the whole set deterministic."""
    from texo_gb300 import problem as P
    from texo_gb300.placer import Placer, default_params
    prob = P.synthetic(210, 42000, 365, 50000, 12.0, 0)
    params = default_params(bins_x=256, bins_y=256, target_density=0.9, gamma_base=4.0, max_iterations=1000,
                            best_effort=1, engine=abi.ENGINE_DEVICE, dct_mode=abi.DCT_FP32)
    with Placer(prob, params) as g:
        _, coords, _ = g.run(allow_nonconverged=True)
    movable = np.nonzero(np.any(prob.lower_xy != prob.upper_xy, axis=1))[0]
    xy = coords[: 2 * prob.num_units].reshape(-1, 2)[movable]
    rng = np.random.default_rng(7)
    n = len(movable)
    clock_lsr = np.stack([rng.integers(0, 8, n), np.zeros(n, np.int64)], axis=1).astype(np.uint64)
    ce = rng.integers(0, 16, n).astype(np.uint64)
    areas, _ = R.register_clustering_areas(xy, clock_lsr, ce, 2 * n)
    again, _ = R.register_clustering_areas(xy, clock_lsr, ce, 2 * n)
    assert np.array_equal(areas, again)
    sample = np.nonzero(clock_lsr[:, 0] == 0)[0]
    code, ref = ffi.register_clustering_areas(xy[sample], clock_lsr[sample], ce[sample], 2 * n)
    assert code == 0
    assert np.max(np.abs(areas[sample] - ref) / ref) <= 1e-12

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

"""Host logic of the served form (no GPU): the size lanes' layout of world slots, body pools and
servers, and the Poisson load it is driven with."""
import numpy as np
import pytest

from physkit_gb300.serve import lane_layout, poisson_load


@pytest.mark.parametrize("lanes", [2, 3, 4])
@pytest.mark.parametrize("servers", [1, 3, 6])
def test_lane_layout_covers_every_size_within_the_pool(lanes, servers):
    lay = lane_layout(lanes, max_worlds=1024, max_bodies=1_500_000, nmax=4096, lane_servers=servers)
    bounds = [b for b, _, _, _ in lay]
    assert bounds == sorted(bounds) and bounds[-1] == 4096 and len(lay) == lanes
    # slots and bodies stay within the pool (each lane keeps a floor of 16 slots and 4 worlds)
    assert sum(w for _, w, _, _ in lay) <= 1024 + 16 * lanes
    assert sum(b for _, _, b, _ in lay) <= 1_500_000 + 4 * 4096 * lanes
    for b, w, pool, r in lay:
        assert w >= 16 and pool >= 4 * b
        assert r == (servers if b > 1024 else 1)  # only the large-world lanes are replicated
        assert pool // r >= 2 * b                  # a server's share still holds two of its largest worlds


def test_lane_shares_follow_the_log_uniform_size_law():
    lay = lane_layout(4, max_worlds=1 << 20, max_bodies=1 << 30, nmax=4096)
    w = np.array([x[1] for x in lay], float)
    b = np.array([x[2] for x in lay], float)
    # worlds: log-width of each lane's size range; bodies: linear width
    np.testing.assert_allclose(w / w.sum(), [np.log(256 / 16), np.log(4), np.log(2), np.log(2)] / np.log(256), rtol=1e-4)
    np.testing.assert_allclose(b / b.sum(), np.array([240, 768, 1024, 2048]) / 4080, rtol=1e-4)


def test_poisson_load_rate_sizes_and_opens():
    t, kind, sizes, lifes, pick, _ = poisson_load(5000.0, 2.0, nmin=16, nmax=4096, seed=3)
    assert abs(len(t) / 2.0 - 5000.0) < 5 * np.sqrt(5000.0 * 2.0) / 2.0
    assert np.all(np.diff(t) >= 0) and t.min() >= 0 and t.max() <= 2.0
    assert sizes.min() >= 16 and sizes.max() <= 4096 and lifes.min() >= 60 and lifes.max() <= 600
    assert 0.0 < kind.mean() < 0.02  # about one request in 331 opens a world

"""Host logic of the segmented panel walk: the segment count per launch and the
bounds, which must start at depth-1 entries of the DFS pre-order tape."""
import numpy as np
import pytest

from smolyax_gb300.spectral import segment_bounds, segment_count


def _tape_levels(rng, n):
    """Levels of a random DFS pre-order walk (first entry at depth 1; a step
    goes at most one level deeper)."""
    lv = [1]
    while len(lv) < n:
        lv.append(int(rng.integers(1, min(lv[-1] + 1, 8) + 1)))
    return np.array(lv)


@pytest.mark.parametrize("seed", range(5))
def test_segment_bounds_start_at_depth_one(seed):
    rng = np.random.default_rng(seed)
    lv = _tape_levels(rng, int(rng.integers(300, 30000)))
    K = lv.size
    lvl1 = np.nonzero(lv == 1)[0]
    for want in (2, 3, 7, 32):
        b = segment_bounds(lvl1, K, want)
        assert b[0] == 0 and b[-1] == K and np.all(np.diff(b) > 0)
        assert set(b[:-1].tolist()) <= set(lvl1.tolist())
        assert len(b) - 1 <= want


def test_segment_count():
    # a launch that fills the GPU on its own keeps one segment
    assert segment_count(20009, 205, 152 * 12 * 128, 152) == 1
    # a small chunk is split up to the limits
    assert segment_count(20009, 205, 11904, 152) == 20
    assert segment_count(20009, 205, 128, 152) == 32
    assert segment_count(300, 205, 128, 152) == 1  # short tapes are not split
    assert segment_count(20009, 3, 128, 152) == 3  # nor beyond their depth-1 entries


def test_vjp_segment_count_and_bounds():
    """Tape segments of the gradient walk: one per 4096 tape entries, at most
    32 and at most the number of depth-1 entries; the bounds start at depth-1
    entries and cover the tape (the same bounds as the panel's)."""
    from smolyax_gb300.spectral import segment_bounds, vjp_segment_count

    assert vjp_segment_count(5000, 300) == 1
    assert vjp_segment_count(8192, 300) == 2
    assert vjp_segment_count(63932, 400) == 15
    assert vjp_segment_count(10**6, 400) == 32
    assert vjp_segment_count(63932, 5) == 5
    assert vjp_segment_count(0, 0) == 1
    lvl1 = np.array([0, 10, 4000, 4100, 9000, 12000, 15000])
    b = segment_bounds(lvl1, 16000, vjp_segment_count(16000, lvl1.size))
    assert b[0] == 0 and b[-1] == 16000 and np.all(np.diff(b) > 0)
    assert set(b[:-1].tolist()) <= set(lvl1.tolist())

"""Host logic of the batched pipeline's ray layout (no GPU): targets grouped
by the sample capacity of the training kernel that holds them, rays laid out
contiguously in that order, one launch group per capacity."""
import numpy as np
import pytest

from sailor_gb300.batch import capacity_layout, sample_capacity


def test_sample_capacity():
    assert [sample_capacity(s) for s in (1, 32, 33, 64, 65, 96, 128)] == [32, 32, 64, 64, 128, 128, 128]


@pytest.mark.parametrize("seed", range(6))
def test_capacity_layout(seed):
    rng = np.random.default_rng(seed)
    T = int(rng.integers(1, 20))
    targets = [(int(rng.integers(0, 4)), int(rng.integers(0, 5000)), int(rng.choice([8, 32, 48, 64, 96, 128])))
               for _ in range(T)]
    order, rb, slices, groups = capacity_layout(targets)
    # order: by capacity, the given order within a capacity (stable)
    assert sorted(order) == list(range(T))
    caps = [sample_capacity(targets[t][2]) for t in order]
    assert caps == sorted(caps)
    for a, b in zip(order, order[1:]):
        if caps[order.index(a)] == caps[order.index(b)]:
            assert a < b
    # rays: contiguous, in layout order, covering [0, R)
    assert rb.dtype == np.int64 and rb[0] == 0 and rb[-1] == sum(n for _, n, _ in targets)
    for i, t in enumerate(order):
        assert slices[t] == (rb[i], rb[i + 1]) and rb[i + 1] - rb[i] == targets[t][1]
    # groups: consecutive segment ranges of one capacity each, covering all
    # segments, with the group's largest S
    assert groups[0][0] == 0 and groups[-1][1] == T
    for (g0, g1, sm), nxt in zip(groups, groups[1:] + [None]):
        assert g1 > g0 and (nxt is None or nxt[0] == g1)
        seg_s = [targets[t][2] for t in order[g0:g1]]
        assert len({sample_capacity(s) for s in seg_s}) == 1 and sm == max(seg_s)
    assert len(groups) == len(set(caps))


def test_capacity_layout_rejects_oversize():
    with pytest.raises(ValueError):
        capacity_layout([(0, 2 ** 30, 32), (0, 2 ** 30, 64)])

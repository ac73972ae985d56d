"""Host-side structure of batched problems (no GPU): the disjoint union of
meshes and the per-problem coarse aggregates with their diagonal blocks."""
import numpy as np
import pytest

from nfempy_gb300 import meshes, workloads
from oracle import mesh_gen


@pytest.mark.parametrize("size", [None, 3, 5])
def test_batch_aggregates_stay_inside_problems(size):
    sides = [4, 9, 13, 6, 1]
    agg, ptr = workloads.batch_aggregates(sides, k=3, size=size, blocks=True)
    assert agg.shape == (sum(2 * n * n for n in sides),)
    assert ptr[0] == 0 and ptr[-1] == agg.max() + 1 and np.all(np.diff(ptr) >= 1)
    c0 = 0
    for b, n in enumerate(sides):
        a = agg[c0:c0 + 2 * n * n]
        # every aggregate of problem b lies in its block, and none is empty
        assert a.min() == ptr[b] and a.max() == ptr[b + 1] - 1
        assert np.all(np.bincount(a - ptr[b]) > 0)
        k = min(3, n) if size is None else max(1, min(n, int(round(n / size))))
        assert ptr[b + 1] - ptr[b] == k * k
        c0 += 2 * n * n
    assert np.array_equal(workloads.batch_aggregates(sides, k=3, size=size), agg)


def test_union_offsets_cells_and_points():
    ms = [mesh_gen.square(n) for n in (2, 3)]
    u = meshes.union(ms)
    c = [m["blocks"][-1][1] for m in ms]
    cu = u["blocks"][-1][1]
    assert cu.shape[0] == c[0].shape[0] + c[1].shape[0]
    assert np.array_equal(cu[:c[0].shape[0]], c[0])
    assert np.array_equal(cu[c[0].shape[0]:], c[1] + ms[0]["points"].shape[0])
    assert np.array_equal(u["points"][ms[0]["points"].shape[0]:], ms[1]["points"])

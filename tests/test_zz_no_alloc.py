"""pt_segment_collisions_noalloc (needs a GB300): the allocation-free entry
point, which keeps its device scratch in a static array of the library, must
return what pt_segment_collisions returns, call after call.

Tolerance: none -- counts, parameters s, normals, solid IDs and distnormal are
compared for exact equality on every slot the kernel writes (the first
min(count, max_hits) of each segment).  The file is collected last, so in a
full run it executes after every other GPU test of the process; it also
passes on its own.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene():
    from pentrack_gb300 import Scene, scenes
    sc = Scene()
    sc.add_material("m", 0.0)
    sc.add_solid(1, 0)
    sc.add_solid(2, 0, scenes.cylinder_mesh(0.2, -0.05, 0.05, 256))
    sc.add_solid(3, 0, scenes.box_mesh((-0.1, -0.1, -0.02), (0.1, 0.1, 0.02)), ignore=[(1.0, 2.0)])
    return sc


def _segments(rng, n):
    p = rng.uniform(-0.3, 0.3, (n, 3))
    d = rng.normal(size=(n, 3)) * rng.choice([1e-6, 1e-3, 0.1, 1.0], size=(n, 1))
    return np.hstack([p, p + d])


def _same(ref, got, max_hits):
    cnt = ref[0]
    assert np.array_equal(got[0], cnt)
    written = np.arange(max_hits)[None, :] < np.clip(cnt, 0, max_hits)[:, None]
    for a, b in zip(ref[1:], got[1:]):
        assert np.array_equal(a[written], b[written])
    return cnt


def test_noalloc_equals_allocating_entry_point_on_consecutive_calls(built):
    from pentrack_gb300 import Engine
    e = Engine(_scene())
    rng = np.random.default_rng(7)
    for n, max_hits in ((6000, 8), (16384, 8)):  # second call: larger, different inputs
        segs = _segments(rng, n)
        ref = e.collisions(segs, max_hits=max_hits)
        got = e.collisions_noalloc(segs, max_hits=max_hits)
        cnt = _same(ref, got, max_hits)
        assert (cnt > 0).sum() > n // 50
        assert (cnt > 1).sum() > 0


def test_noalloc_rejects_requests_beyond_its_scratch(built):
    from pentrack_gb300 import Engine
    from pentrack_gb300.engine import EngineError
    e = Engine(_scene())
    segs = np.zeros((40000, 6))
    segs[:, 3] = 1.0
    with pytest.raises(EngineError, match="static scratch"):
        e.collisions_noalloc(segs, max_hits=8)
    # the context stays usable after the rejection
    small = _segments(np.random.default_rng(8), 1000)
    _same(e.collisions(small, max_hits=4), e.collisions_noalloc(small, max_hits=4), 4)

"""Host logic of the served benchmark: the pinned output arena never hands out
overlapping live regions and frees in submission order."""
import ctypes as C
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))


class _FakeLib:
    def __init__(self):
        self.keep = []

    def mg_host_alloc(self, n):
        a = np.zeros(n, np.uint8)
        self.keep.append(a)
        return a.ctypes.data


def test_arena_ring_no_overlap():
    import bench

    lib = _FakeLib()
    arena = bench._Arena(lib, 1 << 16)
    rng = np.random.default_rng(3)
    live = []
    for step in range(5000):
        if live and (rng.random() < 0.45 or arena._fit((int(rng.integers(1, 20000)) + 63) & ~63) is None):
            arena.release()
            live.pop(0)
            continue
        size = int(rng.integers(1, 20000))
        if arena._fit((size + 63) & ~63) is None:
            continue
        v = arena.take(size)
        start = v.ctypes.data - arena.buf.ctypes.data
        end = start + len(v)
        assert 0 <= start and end <= arena.n
        for s, e in live:
            assert end <= s or start >= e, (step, start, end, s, e)
        live.append((start, end))
    while live:
        arena.release()
        live.pop(0)
    assert arena.head == 0 and not arena.live

"""Seeded synthetic inputs (libmosaic_synth.so): targets, materials, thumbnails.

Stand-ins for the reference's decoded image files: the reference reads a target
image and a directory of material images; these generators produce the same
shapes in memory from one seed (Philox4x32-10 keyed by the seed, one stream id
per input kind).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from .build import BUILD

_LIB = None


def load():
    global _LIB
    if _LIB is None:
        path = BUILD / "libmosaic_synth.so"
        if not path.exists():
            raise RuntimeError(f"{path} is not built: run mosaic_gpu.build.build()")
        lib = C.CDLL(str(path))
        u8p, i64p, ip = C.POINTER(C.c_uint8), C.POINTER(C.c_int64), C.POINTER(C.c_int)
        lib.ms_target.argtypes = [u8p, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_uint32, C.c_int]
        lib.ms_material_dims.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_uint32, ip, ip]
        lib.ms_materials.argtypes = [u8p, i64p, ip, ip, C.c_int, C.c_uint64, C.c_uint32, C.c_int]
        lib.ms_thumbnails.argtypes = [u8p, i64p, ip, ip, C.c_int, C.c_int, C.c_int, u8p, C.c_int]
        for f in (lib.ms_target, lib.ms_material_dims, lib.ms_materials, lib.ms_thumbnails):
            f.restype = None
        _LIB = lib
    return _LIB


def _threads() -> int:
    return max(1, min(32, os.cpu_count() or 1))


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def alloc_u8(nbytes: int, allocator=None) -> np.ndarray:
    """uint8 buffer, from `allocator(nbytes) -> address` (e.g. pinned memory) or numpy."""
    if allocator is None:
        return np.empty(nbytes, np.uint8)
    addr = allocator(max(nbytes, 16))
    if not addr:
        raise MemoryError("host allocation failed")
    return np.ctypeslib.as_array(C.cast(addr, C.POINTER(C.c_uint8)), shape=(max(nbytes, 16),))[:nbytes]


def target(w: int, h: int, blobs: int, seed: int, stream: int = 1, allocator=None) -> np.ndarray:
    out = alloc_u8(w * h * 3, allocator)
    load().ms_target(_p(out, C.c_uint8), w, h, blobs, seed, stream, _threads())
    return out.reshape(h, w, 3)


@dataclass
class Materials:
    """Materials packed in one buffer; material i is buf[off[i]:...] as (h[i], w[i], 3)."""
    buf: np.ndarray
    off: np.ndarray
    w: np.ndarray
    h: np.ndarray
    views: list = field(default_factory=list)

    def __len__(self):
        return len(self.w)

    def image(self, i: int) -> np.ndarray:
        o, w, h = int(self.off[i]), int(self.w[i]), int(self.h[i])
        return self.buf[o:o + w * h * 3].reshape(h, w, 3)


def materials(n: int, side: int, mode: int, seed: int, stream: int = 2, allocator=None) -> Materials:
    w = np.zeros(n, np.int32)
    h = np.zeros(n, np.int32)
    lib = load()
    lib.ms_material_dims(n, side, mode, seed, stream, _p(w, C.c_int), _p(h, C.c_int))
    sizes = (w.astype(np.int64) * h * 3 + 15) // 16 * 16
    off = np.zeros(n, np.int64)
    if n:
        off[1:] = np.cumsum(sizes)[:-1]
    buf = alloc_u8(int(sizes.sum()), allocator)
    lib.ms_materials(_p(buf, C.c_uint8), _p(off, C.c_int64), _p(w, C.c_int), _p(h, C.c_int), n, seed, stream,
                     _threads())
    return Materials(buf, off, w, h)


def thumbnails(m: Materials, tw: int, th: int, allocator=None) -> np.ndarray:
    n = len(m)
    out = alloc_u8(n * tw * th * 3, allocator)
    load().ms_thumbnails(_p(m.buf, C.c_uint8), _p(m.off, C.c_int64), _p(m.w, C.c_int), _p(m.h, C.c_int), n, tw,
                         th, _p(out, C.c_uint8), _threads())
    return out.reshape(n, th, tw, 3)

"""Whole-job helpers: workload configurations, mg_request assembly, generate and plans.

The workloads restate the mosaic configurations the path is measured on:

  small        1024x768 target, 8 blobs; 500 materials 128x128; grid 40x30;
               max usage 3; adjacency 0.25; colour 0; 500 iterations x 1 chain
  recommended  3840x2880 target, 32 blobs; 1500 materials with aspect drawn from
               {1:1, 4:3, 3:4}, long side 256; grid 80x60; max usage 3;
               adjacency 0.25; colour 0.4; 2000 iterations x 32 chains;
               48x48 output tiles
  large        7680x5760 target, 128 blobs; 5000 materials 128x128; grid 179x134;
               max usage 8; adjacency 0.25; colour 0.4; 100000 iterations x 64
               chains; 32x32 output tiles
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, replace

import numpy as np

from . import _capi as capi
from . import synth


@dataclass(frozen=True)
class JobConfig:
    name: str
    target_w: int
    target_h: int
    blobs: int
    n_materials: int
    material_side: int
    material_mode: int      # 0: all square; 1: aspect from {1:1, 4:3, 3:4}
    grid_w: int
    grid_h: int
    max_usage: int
    weight: float
    color_strength: float
    iterations: int
    chains: int
    tile_w: int = 0         # 0 -> cell size
    tile_h: int = 0
    max_materials: int = 0  # 0 -> n_materials (keep every material that passes the filter)
    aspect_tolerance: float = 0.1
    enable_optimization: bool = True
    seed: int = 20251203
    build_similarity: bool = True
    device_thumbnails: bool = False


WORKLOADS = {
    "small": JobConfig("small", 1024, 768, 8, 500, 128, 0, 40, 30, 3, 0.25, 0.0, 500, 1),
    "recommended": JobConfig("recommended", 3840, 2880, 32, 1500, 256, 1, 80, 60, 3, 0.25, 0.4, 2000, 32, 48, 48),
    "large": JobConfig("large", 7680, 5760, 128, 5000, 128, 0, 179, 134, 8, 0.25, 0.4, 100000, 64, 32, 32),
}


def scaled(cfg: JobConfig, **kw) -> JobConfig:
    return replace(cfg, **kw)


@dataclass
class Inputs:
    cfg: JobConfig
    target: np.ndarray
    mats: synth.Materials
    thumbs: np.ndarray | None

    @property
    def tile(self):
        tw = self.cfg.tile_w or self.cfg.target_w // self.cfg.grid_w
        th = self.cfg.tile_h or self.cfg.target_h // self.cfg.grid_h
        return tw, th


def make_inputs(cfg: JobConfig, allocator=None) -> Inputs:
    tgt = synth.target(cfg.target_w, cfg.target_h, cfg.blobs, cfg.seed, 1, allocator)
    mats = synth.materials(cfg.n_materials, cfg.material_side, cfg.material_mode, cfg.seed, 2, allocator)
    inp = Inputs(cfg, tgt, mats, None)
    if not cfg.device_thumbnails:
        tw, th = inp.tile
        inp.thumbs = synth.thumbnails(mats, tw, th, allocator)
    return inp


class RequestHolder:
    """An mg_request plus the ctypes arrays it points into (kept alive)."""

    def __init__(self, inp: Inputs, stream: int = 0):
        cfg = inp.cfg
        n = len(inp.mats)
        self._ptrs = (capi._u8p * max(n, 1))(
            *[C.cast(inp.mats.buf.ctypes.data + int(o), capi._u8p) for o in inp.mats.off])
        self._w = (C.c_int * max(n, 1))(*[int(v) for v in inp.mats.w])
        self._h = (C.c_int * max(n, 1))(*[int(v) for v in inp.mats.h])
        r = capi.Request()
        capi.load().mg_request_default(C.byref(r))
        r.target = capi.ptr(inp.target, C.c_uint8)
        r.target_w, r.target_h = cfg.target_w, cfg.target_h
        r.target_stride = inp.target.strides[0]
        r.n_materials = n
        r.materials = self._ptrs
        r.material_w = self._w
        r.material_h = self._h
        r.material_stride = None
        r.thumbnails = capi.ptr(inp.thumbs, C.c_uint8) if inp.thumbs is not None else None
        r.tile_w, r.tile_h = cfg.tile_w, cfg.tile_h
        r.grid_w, r.grid_h = cfg.grid_w, cfg.grid_h
        r.max_materials = cfg.max_materials or n
        r.aspect_tolerance = cfg.aspect_tolerance
        r.max_usage_per_image = cfg.max_usage
        r.adjacency_penalty_weight = cfg.weight
        r.color_adjustment_strength = cfg.color_strength
        r.enable_optimization = 1 if cfg.enable_optimization else 0
        r.optimization_iterations = cfg.iterations
        r.chains = cfg.chains
        r.seed = cfg.seed
        r.stream = stream
        r.build_similarity = 1 if cfg.build_similarity else 0
        self.req = r
        self.inp = inp

    def out_shape(self):
        tw, th = self.inp.tile
        return self.inp.cfg.grid_h * th, self.inp.cfg.grid_w * tw, 3


def new_result(holder: RequestHolder, image: np.ndarray | None = None, grid: np.ndarray | None = None):
    cfg = holder.inp.cfg
    if grid is None:
        grid = np.zeros(cfg.grid_w * cfg.grid_h, np.int32)
    if image is None:
        image = np.zeros(holder.out_shape(), np.uint8)
    res = capi.Result()
    res.grid = capi.ptr(grid, C.c_int32)
    res.image = capi.ptr(image, C.c_uint8)
    return res, grid, image


def generate(ctx: capi.Context, holder: RequestHolder, image=None, grid=None):
    res, grid, image = new_result(holder, image, grid)
    capi.check(ctx.lib.mg_generate(ctx.h, C.byref(holder.req), C.byref(res)))
    return res, grid.reshape(holder.inp.cfg.grid_h, holder.inp.cfg.grid_w), image


class Plan:
    """Device-resident job (mg_plan): inputs uploaded once, run many times."""

    def __init__(self, ctx: capi.Context, holder: RequestHolder):
        self.ctx = ctx
        self.holder = holder
        h = C.c_void_p()
        capi.check(ctx.lib.mg_plan_create(ctx.h, C.byref(holder.req), C.byref(h)))
        self.h = h

    def run(self):
        capi.check(self.ctx.lib.mg_plan_run(self.h))

    def read(self, image=None, grid=None):
        res, grid, image = new_result(self.holder, image, grid)
        capi.check(self.ctx.lib.mg_plan_read(self.h, C.byref(res)))
        return res, grid.reshape(self.holder.inp.cfg.grid_h, self.holder.inp.cfg.grid_w), image

    def stage_ms(self):
        ms = np.zeros(8, np.float32)
        n = self.ctx.lib.mg_plan_stage_ms(self.h, capi.ptr(ms, C.c_float), 8)
        if n < 0:
            capi.check(-n)
        return ms[:n]

    def launches(self) -> int:
        return int(self.ctx.lib.mg_plan_launches(self.h))

    def close(self):
        if self.h:
            self.ctx.lib.mg_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

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


# ---- resident palettes and batches -------------------------------------------------------
class Palette:
    """A resident palette (mg_palette): selection, material Lab, thumbnails, similarity."""

    def __init__(self, ctx: capi.Context, mats: synth.Materials, thumbs, tile_w: int, tile_h: int,
                 target_aspect: float, aspect_tolerance: float = 0.1, max_materials: int = 0,
                 build_similarity: bool = True):
        self.ctx = ctx
        n = len(mats)
        self._ptrs = (capi._u8p * max(n, 1))(*[C.cast(mats.buf.ctypes.data + int(o), capi._u8p) for o in mats.off])
        self._w = (C.c_int * max(n, 1))(*[int(v) for v in mats.w])
        self._h = (C.c_int * max(n, 1))(*[int(v) for v in mats.h])
        d = capi.PaletteDesc()
        ctx.lib.mg_palette_desc_default(C.byref(d))
        d.n_materials = n
        d.materials, d.material_w, d.material_h = self._ptrs, self._w, self._h
        d.material_stride = None
        d.thumbnails = capi.ptr(thumbs, C.c_uint8) if thumbs is not None else None
        d.tile_w, d.tile_h = tile_w, tile_h
        d.target_aspect, d.aspect_tolerance = target_aspect, aspect_tolerance
        d.max_materials = max_materials or n
        d.build_similarity = 1 if build_similarity else 0
        h = C.c_void_p()
        capi.check(ctx.lib.mg_palette_create(ctx.h, C.byref(d), C.byref(h)))
        self.h = h
        self.tile = (tile_w, tile_h)

    @property
    def size(self) -> int:
        return int(self.ctx.lib.mg_palette_size(self.h))

    def lab(self):
        out = np.zeros((max(self.size, 1), 3), np.float32)
        capi.check(self.ctx.lib.mg_palette_read_lab(self.h, capi.ptr(out, C.c_float)))
        return out[:self.size]

    def close(self):
        if self.h:
            self.ctx.lib.mg_palette_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mosaic_request(target: np.ndarray | int, w: int, h: int, gw: int, gh: int, *, max_usage=3, weight=0.25,
                   strength=0.4, enable_opt=True, iterations=1000, chains=1, seed=20251203, stream=0,
                   t0=100.0, decay=0.99995) -> capi.Mosaic:
    m = capi.Mosaic()
    capi.load().mg_mosaic_default(C.byref(m))
    m.target = target if isinstance(target, int) else target.ctypes.data
    m.target_w, m.target_h, m.target_stride = w, h, 3 * w
    m.grid_w, m.grid_h = gw, gh
    m.max_usage_per_image, m.adjacency_penalty_weight, m.color_adjustment_strength = max_usage, weight, strength
    m.enable_optimization = 1 if enable_opt else 0
    m.optimization_iterations, m.chains, m.seed, m.stream = iterations, chains, seed, stream
    m.initial_temperature, m.temperature_decay = t0, decay
    return m


class Batch:
    """A device-resident batch of mosaics over one palette (mg_batch)."""

    def __init__(self, ctx: capi.Context, palette: Palette, mosaics: list):
        self.ctx, self.palette = ctx, palette
        self.n = len(mosaics)
        self._arr = (capi.Mosaic * max(self.n, 1))(*mosaics)
        self._meta = [(m.grid_w, m.grid_h) for m in mosaics]
        h = C.c_void_p()
        capi.check(ctx.lib.mg_batch_create(ctx.h, palette.h, self._arr, self.n, C.byref(h)))
        self.h = h

    def run(self):
        capi.check(self.ctx.lib.mg_batch_run(self.h))

    def read(self, i: int, want_image: bool = True):
        gw, gh = self._meta[i]
        tw, th = self.palette.tile
        grid = np.zeros(gw * gh, np.int32)
        image = np.zeros((gh * th, gw * tw, 3), np.uint8) if want_image else None
        res = capi.Result()
        res.grid = capi.ptr(grid, C.c_int32)
        res.image = capi.ptr(image, C.c_uint8) if want_image else None
        capi.check(self.ctx.lib.mg_batch_read(self.h, i, C.byref(res)))
        return res, grid.reshape(gh, gw), image

    def stage_ms(self):
        ms = np.zeros(5, np.float32)
        n = self.ctx.lib.mg_batch_stage_ms(self.h, capi.ptr(ms, C.c_float), 5)
        return ms[:max(n, 0)]

    def tuning(self):
        a, b = C.c_int(), C.c_int()
        capi.check(self.ctx.lib.mg_batch_tuning(self.h, C.byref(a), C.byref(b)))
        return {"cells_per_cta": a.value, "nearest_chunk": b.value}

    def launches(self) -> int:
        return int(self.ctx.lib.mg_batch_launches(self.h))

    def close(self):
        if self.h:
            self.ctx.lib.mg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def generate_batch(ctx: capi.Context, palette: Palette, mosaics: list, outputs=None):
    """One mg_generate_batch call.  outputs: optional [(grid, image)] to write
    into (e.g. pinned buffers); fresh numpy arrays otherwise."""
    n = len(mosaics)
    arr = (capi.Mosaic * max(n, 1))(*mosaics)
    tw, th = palette.tile
    grids, images = [], []
    results = (capi.Result * max(n, 1))()
    for i, m in enumerate(mosaics):
        if outputs is not None:
            g, im = outputs[i]
        else:
            g = np.zeros(m.grid_w * m.grid_h, np.int32)
            im = np.zeros((m.grid_h * th, m.grid_w * tw, 3), np.uint8)
        results[i].grid = capi.ptr(g, C.c_int32)
        results[i].image = capi.ptr(im, C.c_uint8)
        grids.append(g.reshape(m.grid_h, m.grid_w))
        images.append(im)
    capi.check(ctx.lib.mg_generate_batch(ctx.h, palette.h, arr, n, results))
    return list(results)[:n], grids, images


# ---- the batched and served workloads ----------------------------------------------------
@dataclass
class MosaicSpec:
    w: int
    h: int
    gw: int
    gh: int
    target: np.ndarray


def uneven_grids(n: int, lo: int, hi: int, seed: int):
    """Grid widths log-uniform in [lo, hi], aspect 4:3."""
    rng = np.random.default_rng(seed)
    gw = np.exp(rng.uniform(np.log(lo), np.log(hi), n)).round().astype(int)
    gh = np.maximum(1, (gw * 3 / 4).round().astype(int))
    return gw, gh


def batched_workload(n=256, cell_px=32, n_materials=10000, seed=20251203, allocator=None, scale=1.0):
    """256 mosaics, grid widths log-uniform in 20..160 (4:3), 32 px per cell, targets from the
    blob+noise generator (8 blobs); one palette of 10 000 128x128 materials; 32x32 tiles."""
    gw, gh = uneven_grids(n, max(2, int(20 * scale)), max(3, int(160 * scale)), seed)
    specs = []
    for i in range(n):
        w, h = int(gw[i]) * cell_px, int(gh[i]) * cell_px
        specs.append(MosaicSpec(w, h, int(gw[i]), int(gh[i]), synth.target(w, h, 8, seed, 100 + i, allocator)))
    mats = synth.materials(n_materials, 128, 0, seed, 2, allocator)
    thumbs = synth.thumbnails(mats, cell_px, cell_px, allocator)
    return specs, mats, thumbs


def batched_requests(specs, iterations=5000, chains=8, max_usage=4, weight=0.25, strength=0.4, seed=20251203):
    return [mosaic_request(s.target, s.w, s.h, s.gw, s.gh, max_usage=max_usage, weight=weight, strength=strength,
                           iterations=iterations, chains=chains, seed=seed, stream=i) for i, s in enumerate(specs)]


def served_grids(n: int, seed: int, lo: int = 500, hi: int = 50000):
    """Cells per request log-uniform in [lo, hi], aspect 4:3: (grid widths, grid heights)."""
    rng = np.random.default_rng(seed)
    cells = np.exp(rng.uniform(np.log(lo), np.log(hi), n))
    gw = np.maximum(1, np.sqrt(cells * 4 / 3).round().astype(int))
    gh = np.maximum(1, (gw * 3 / 4).round().astype(int))
    return gw, gh


def served_workload(n_targets=64, cell_px=24, n_materials=20000, seed=20251203, allocator=None, scale=1.0):
    """The served stream's inputs: a pool of targets (cells log-uniform in 500..50 000 at 4:3,
    blob+noise generator with 8 blobs, 24 px per cell) and one palette of 20 000 128x128
    materials with 24x24 thumbnails.  `scale` shrinks the cell range for small runs."""
    gw, gh = served_grids(n_targets, seed, max(4, int(500 * scale)), max(12, int(50000 * scale)))
    pool = []
    for i in range(n_targets):
        w, h = int(gw[i]) * cell_px, int(gh[i]) * cell_px
        pool.append(MosaicSpec(w, h, int(gw[i]), int(gh[i]), synth.target(w, h, 8, seed, 5000 + i, allocator)))
    mats = synth.materials(n_materials, 128, 0, seed, 2, allocator)
    thumbs = synth.thumbnails(mats, cell_px, cell_px, allocator)
    return pool, mats, thumbs


def served_stream(pool, n: int, seed: int, iterations=2000, chains=4, max_usage=5, weight=0.25, strength=0.4):
    """n requests drawn from the target pool (request j: pool entry picked by a seeded draw,
    Philox stream id j): [(pool index, mg_mosaic)]."""
    rng = np.random.default_rng(seed ^ 0x5EED)
    picks = rng.integers(0, len(pool), n)
    out = []
    for j, p in enumerate(picks):
        s = pool[int(p)]
        out.append((int(p), mosaic_request(s.target, s.w, s.h, s.gw, s.gh, max_usage=max_usage, weight=weight,
                                           strength=strength, iterations=iterations, chains=chains, seed=seed,
                                           stream=j)))
    return out


def poisson_arrivals(rate: float, n: int, seed: int):
    """Arrival offsets (s) of a Poisson process of the given rate."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, n))


class Server:
    """The request loop over one resident palette (mg_server)."""

    def __init__(self, ctx: capi.Context, palette: Palette, slots: int = 3, max_batch: int = 64,
                 memory_budget_bytes: int = 120 << 30):
        self.ctx, self.palette = ctx, palette
        cfg = capi.ServerConfig()
        ctx.lib.mg_server_config_default(C.byref(cfg))
        cfg.slots, cfg.max_batch, cfg.memory_budget_bytes = slots, max_batch, memory_budget_bytes
        h = C.c_void_p()
        capi.check(ctx.lib.mg_server_create(ctx.h, palette.h, C.byref(cfg), C.byref(h)))
        self.h = h
        self._live = {}  # ticket -> (mosaic, grid, image) kept alive until completion

    def submit(self, m: capi.Mosaic, grid: np.ndarray | None = None, image: np.ndarray | None = None) -> int:
        """Queue one request; grid/image (caller-owned, e.g. pinned) receive the results."""
        m = capi.Mosaic.from_buffer_copy(m)
        t = C.c_uint64()
        capi.check(self.ctx.lib.mg_server_submit(
            self.h, C.byref(m), capi.ptr(grid, C.c_int32) if grid is not None else None,
            capi.ptr(image, C.c_uint8) if image is not None else None, C.byref(t)))
        self._live[t.value] = (m, grid, image)
        return t.value

    def _finish(self, fn, ticket: int):
        res = capi.Result()
        lat = C.c_double()
        st = fn(self.h, ticket, C.byref(res), C.byref(lat))
        if st == -1:
            return None
        self._live.pop(ticket, None)
        return st, res, lat.value

    def wait(self, ticket: int):
        """(status, Result, latency_ms) of a request, blocking until it completes."""
        return self._finish(self.ctx.lib.mg_server_wait, ticket)

    def poll(self, ticket: int):
        """(status, Result, latency_ms), or None while the request is pending."""
        return self._finish(self.ctx.lib.mg_server_poll, ticket)

    def request_bytes(self, m: capi.Mosaic) -> int:
        """Device bytes admission counts for the request against the budget."""
        return int(self.ctx.lib.mg_server_request_bytes(self.h, C.byref(m)))

    def stats(self) -> dict:
        s = capi.ServerStats()
        capi.check(self.ctx.lib.mg_server_get_stats(self.h, C.byref(s)))
        return {n: int(getattr(s, n)) for n, _ in capi.ServerStats._fields_}

    def close(self):
        if self.h:
            self.ctx.lib.mg_server_destroy(self.h)
            self.h = None
            self._live.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

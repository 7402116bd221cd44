"""ctypes binding of the C ABI in include/mosaic_gpu.h (libmosaic_gpu.so).

This is the same binding a foreign-language host writes against the ABI (the
Rust ``-sys`` crate of the integration notes declares the identical
functions); numpy arrays stand in for caller-owned host buffers.  There is no
fallback: if the CUDA library is not built, ``load()`` raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import BUILD

MG_OK, MG_ERR_ARG, MG_ERR_OOM, MG_ERR_CUDA, MG_ERR_TIMEOUT, MG_ERR_BUDGET, MG_ERR_STATE = range(7)
MG_THUMB_LANCZOS3, MG_THUMB_AREA = 0, 1
MG_SIM_FULL, MG_SIM_TRIANGULAR = 0, 1
MG_NEAREST_AUTO, MG_NEAREST_SCAN, MG_NEAREST_GRID = 0, 1, 2
MG_SCORING_CLI, MG_SCORING_GUI = 0, 1

_u8p = C.POINTER(C.c_uint8)
_f32p = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int32)
_u32p = C.POINTER(C.c_uint32)
_i64p = C.POINTER(C.c_int64)


class MosaicError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"mosaic_gpu error {code}: {msg}")
        self.code = code


class PlaceConfig(C.Structure):
    _fields_ = [("max_usage_per_image", C.c_int), ("adjacency_penalty_weight", C.c_float)]


class SaConfig(C.Structure):
    _fields_ = [("max_iterations", C.c_int64), ("initial_temperature", C.c_float),
                ("temperature_decay", C.c_float), ("chains", C.c_int), ("seed", C.c_uint64),
                ("stream", C.c_uint32), ("greedy_only", C.c_int)]


class SaResult(C.Structure):
    _fields_ = [("initial_cost", C.c_float), ("final_cost", C.c_float), ("best_cost", C.c_float),
                ("improved_count", C.c_int64), ("accepted_count", C.c_int64), ("iterations", C.c_int64),
                ("best_chain", C.c_int)]


class ColorAdjustment(C.Structure):
    _fields_ = [("brightness", C.c_float), ("contrast", C.c_float), ("hue_shift", C.c_float),
                ("saturation", C.c_float)]


class Request(C.Structure):
    _fields_ = [("target", _u8p), ("target_w", C.c_int), ("target_h", C.c_int), ("target_stride", C.c_int64),
                ("n_materials", C.c_int), ("materials", C.POINTER(_u8p)), ("material_w", C.POINTER(C.c_int)),
                ("material_h", C.POINTER(C.c_int)), ("material_stride", _i64p), ("thumbnails", _u8p),
                ("tile_w", C.c_int), ("tile_h", C.c_int), ("grid_w", C.c_int), ("grid_h", C.c_int),
                ("max_materials", C.c_int), ("aspect_tolerance", C.c_float), ("max_usage_per_image", C.c_int),
                ("adjacency_penalty_weight", C.c_float), ("color_adjustment_strength", C.c_float),
                ("enable_optimization", C.c_int), ("optimization_iterations", C.c_int64),
                ("initial_temperature", C.c_float), ("temperature_decay", C.c_float), ("chains", C.c_int),
                ("seed", C.c_uint64), ("stream", C.c_uint32), ("build_similarity", C.c_int)]


class Result(C.Structure):
    _fields_ = [("grid", _i32p), ("image", _u8p), ("out_w", C.c_int), ("out_h", C.c_int),
                ("palette_size", C.c_int), ("n_resets", C.c_int), ("best_chain", C.c_int),
                ("initial_cost", C.c_float), ("final_cost", C.c_float), ("best_cost", C.c_float),
                ("accepted_count", C.c_int64), ("improved_count", C.c_int64)]


class PaletteDesc(C.Structure):
    _fields_ = [("n_materials", C.c_int), ("materials", C.POINTER(_u8p)), ("material_w", C.POINTER(C.c_int)),
                ("material_h", C.POINTER(C.c_int)), ("material_stride", _i64p), ("thumbnails", _u8p),
                ("tile_w", C.c_int), ("tile_h", C.c_int), ("target_aspect", C.c_float),
                ("aspect_tolerance", C.c_float), ("max_materials", C.c_int), ("build_similarity", C.c_int)]


class Mosaic(C.Structure):
    _fields_ = [("target", C.c_void_p), ("target_w", C.c_int), ("target_h", C.c_int), ("target_stride", C.c_int64),
                ("grid_w", C.c_int), ("grid_h", C.c_int), ("max_usage_per_image", C.c_int),
                ("adjacency_penalty_weight", C.c_float), ("color_adjustment_strength", C.c_float),
                ("enable_optimization", C.c_int), ("optimization_iterations", C.c_int64),
                ("initial_temperature", C.c_float), ("temperature_decay", C.c_float), ("chains", C.c_int),
                ("seed", C.c_uint64), ("stream", C.c_uint32)]


class ServerConfig(C.Structure):
    _fields_ = [("slots", C.c_int), ("max_batch", C.c_int), ("memory_budget_bytes", C.c_int64)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("submitted", "completed", "rejected", "batches", "pending",
                                         "bytes_in_use", "peak_bytes_in_use")]


# (name, restype, argtypes) for every exported symbol of mosaic_gpu.h.
SIGNATURES = [
    ("mg_palette_desc_default", None, [C.POINTER(PaletteDesc)]),
    ("mg_palette_create", C.c_int, [C.c_void_p, C.POINTER(PaletteDesc), C.POINTER(C.c_void_p)]),
    ("mg_palette_size", C.c_int, [C.c_void_p]),
    ("mg_palette_device_bytes", C.c_int64, [C.c_void_p]),
    ("mg_palette_read_lab", C.c_int, [C.c_void_p, _f32p]),
    ("mg_palette_read_similarity", C.c_int, [C.c_void_p, _f32p]),
    ("mg_palette_destroy", C.c_int, [C.c_void_p]),
    ("mg_mosaic_default", None, [C.POINTER(Mosaic)]),
    ("mg_batch_create", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Mosaic), C.c_int, C.POINTER(C.c_void_p)]),
    ("mg_batch_run", C.c_int, [C.c_void_p]),
    ("mg_batch_read", C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    ("mg_batch_stage_ms", C.c_int, [C.c_void_p, _f32p, C.c_int]),
    ("mg_batch_tuning", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("mg_batch_launches", C.c_int, [C.c_void_p]),
    ("mg_batch_destroy", C.c_int, [C.c_void_p]),
    ("mg_generate_batch", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(Mosaic), C.c_int, C.c_void_p]),
    ("mg_server_config_default", None, [C.POINTER(ServerConfig)]),
    ("mg_server_create", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    ("mg_server_submit", C.c_int, [C.c_void_p, C.POINTER(Mosaic), _i32p, _u8p, C.POINTER(C.c_uint64)]),
    ("mg_server_poll", C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.POINTER(C.c_double)]),
    ("mg_server_wait", C.c_int, [C.c_void_p, C.c_uint64, C.c_void_p, C.POINTER(C.c_double)]),
    ("mg_server_get_stats", C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    ("mg_server_request_bytes", C.c_int64, [C.c_void_p, C.POINTER(Mosaic)]),
    ("mg_server_destroy", C.c_int, [C.c_void_p]),
    ("mg_version", C.c_int, []),
    ("mg_last_error", C.c_char_p, []),
    ("mg_kernel_launches", C.c_ulonglong, []),
    ("mg_ctx_create", C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    ("mg_ctx_destroy", C.c_int, [C.c_void_p]),
    ("mg_ctx_sync", C.c_int, [C.c_void_p]),
    ("mg_ctx_stream", C.c_void_p, [C.c_void_p]),
    ("mg_ctx_set_nearest_method", C.c_int, [C.c_void_p, C.c_int]),
    ("mg_ctx_set_thumbnail_filter", C.c_int, [C.c_void_p, C.c_int]),
    ("mg_resize", C.c_int, [C.c_void_p, _u8p, C.c_int, C.c_int, C.c_int64, C.c_int, C.c_int, _u8p]),
    ("mg_ctx_inject_walk_timeout", C.c_int, [C.c_void_p, C.c_int]),
    ("mg_ctx_set_scoring", C.c_int, [C.c_void_p, C.c_int]),
    ("mg_host_alloc", C.c_void_p, [C.c_size_t]),
    ("mg_host_free", None, [C.c_void_p]),
    ("mg_average_lab", C.c_int, [C.c_void_p, _u8p, C.c_int, C.c_int, C.c_int64, _f32p]),
    ("mg_is_aspect_ratio_match", C.c_int, [C.c_float, C.c_float, C.c_float]),
    ("mg_cells_lab", C.c_int, [C.c_void_p, _u8p, C.c_int, C.c_int, C.c_int64, C.c_int, C.c_int, _f32p, _u8p]),
    ("mg_cells_lab_noalloc", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int64, C.c_int, C.c_int, C.c_void_p,
                                       C.c_void_p, C.c_void_p]),
    ("mg_images_lab", C.c_int, [C.c_void_p, C.POINTER(_u8p), C.POINTER(C.c_int), C.POINTER(C.c_int), _i64p,
                                C.c_int, _f32p, _u8p]),
    ("mg_select_palette", C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, C.c_float, C.c_float,
                                    C.c_int, C.POINTER(C.c_int)]),
    ("mg_jpeg_info", C.c_int, [C.c_void_p, C.c_size_t, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("mg_jpeg_decode", C.c_int, [C.c_void_p, C.c_size_t, _u8p, C.c_int64]),
    ("mg_image_info", C.c_int, [C.c_void_p, C.c_size_t, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("mg_image_decode", C.c_int, [C.c_void_p, C.c_size_t, _u8p, C.c_int64]),
    ("mg_image_decode_batch", C.c_int, [C.POINTER(C.c_void_p), C.POINTER(C.c_size_t), C.c_int, C.POINTER(_u8p),
                                        C.POINTER(C.c_int64), C.c_int, C.POINTER(C.c_int)]),
    ("mg_png_info", C.c_int, [C.c_void_p, C.c_size_t, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("mg_png_decode", C.c_int, [C.c_void_p, C.c_size_t, _u8p, C.c_int64]),
    ("mg_png_decode_batch", C.c_int, [C.POINTER(C.c_void_p), C.POINTER(C.c_size_t), C.c_int, C.POINTER(_u8p),
                                      _i64p, C.c_int, C.POINTER(C.c_int)]),
    ("mg_png_encode_bound", C.c_size_t, [C.c_int, C.c_int]),
    ("mg_jpeg_encode_bound", C.c_size_t, [C.c_int, C.c_int]),
    ("mg_jpeg_encode", C.c_int, [_u8p, C.c_int, C.c_int, C.c_int64, C.c_int, C.c_int, _u8p, C.c_size_t,
                                 C.POINTER(C.c_size_t)]),
    ("mg_png_encode", C.c_int, [_u8p, C.c_int, C.c_int, C.c_int64, C.c_int, C.c_int, _u8p, C.c_size_t,
                                C.POINTER(C.c_size_t)]),
    ("mg_similarity_build", C.c_int, [C.c_void_p, _f32p, C.c_int, C.c_int, _f32p]),
    ("mg_lab_distance", C.c_float, [_f32p, _f32p]),
    ("mg_nearest_n", C.c_int, [C.c_void_p, _f32p, C.c_int, _f32p, C.c_int, C.c_int, _u32p, _f32p]),
    ("mg_penalty_batch", C.c_int, [C.c_void_p, _f32p, C.c_int, _i32p, C.c_int, C.c_int, C.c_float, _i32p,
                                   C.c_int, _f32p]),
    ("mg_total_cost", C.c_int, [C.c_void_p, _f32p, C.c_int, _i32p, C.c_int, C.c_int, _f32p]),
    ("mg_swap_delta_batch", C.c_int, [C.c_void_p, _f32p, C.c_int, _i32p, C.c_int, C.c_int, _i32p, C.c_int,
                                      _f32p]),
    ("mg_place_greedy", C.c_int, [C.c_void_p, _f32p, C.c_int, _f32p, C.c_int, C.c_int, C.POINTER(PlaceConfig),
                                  _i32p, C.POINTER(C.c_int)]),
    ("mg_sa_config_default", None, [C.POINTER(SaConfig)]),
    ("mg_optimize", C.c_int, [C.c_void_p, _f32p, C.c_int, _i32p, C.c_int, C.c_int, C.POINTER(SaConfig),
                              C.POINTER(SaResult), C.POINTER(SaResult), _i32p]),
    ("mg_improvement_percentage", C.c_float, [C.POINTER(SaResult)]),
    ("mg_color_adjustment_new", ColorAdjustment, [C.c_float, C.c_float, C.c_float, C.c_float]),
    ("mg_optimal_adjustment_batch", C.c_int, [C.c_void_p, _u8p, _u8p, C.c_int, C.c_float,
                                              C.POINTER(ColorAdjustment)]),
    ("mg_apply_adjustment", C.c_int, [C.c_void_p, C.POINTER(ColorAdjustment), _u8p, C.c_int, C.c_int, C.c_int64,
                                      _u8p]),
    ("mg_composite", C.c_int, [C.c_void_p, _i32p, C.c_int, C.c_int, _u8p, C.c_int, C.c_int, C.c_int, _u8p,
                               C.c_float, _u8p]),
    ("mg_request_default", None, [C.POINTER(Request)]),
    ("mg_generate", C.c_int, [C.c_void_p, C.POINTER(Request), C.POINTER(Result)]),
    ("mg_plan_create", C.c_int, [C.c_void_p, C.POINTER(Request), C.POINTER(C.c_void_p)]),
    ("mg_plan_run", C.c_int, [C.c_void_p]),
    ("mg_plan_read", C.c_int, [C.c_void_p, C.POINTER(Result)]),
    ("mg_plan_destroy", C.c_int, [C.c_void_p]),
    ("mg_plan_stage_ms", C.c_int, [C.c_void_p, _f32p, C.c_int]),
    ("mg_plan_launches", C.c_int, [C.c_void_p]),
]

_LIB = None


def library_path() -> Path:
    return BUILD / "libmosaic_gpu.so"


def load() -> C.CDLL:
    """Load libmosaic_gpu.so (built by build.build()); raise if it is missing."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not path.exists():
            raise RuntimeError(f"{path} is not built: run mosaic_gpu.build.build() (no CPU fallback exists)")
        lib = C.CDLL(str(path))
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
    return _LIB


def ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def check(status: int) -> None:
    if status != MG_OK:
        msg = load().mg_last_error()
        raise MosaicError(status, msg.decode() if msg else "")


def _lab3(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, 3))


class Context:
    """One CUDA context/stream of the library (mg_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.mg_ctx_create(device, C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.mg_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- colour statistics
    def average_lab(self, img: np.ndarray) -> np.ndarray:
        img = np.ascontiguousarray(img, dtype=np.uint8)
        out = np.zeros(3, np.float32)
        h, w = img.shape[:2]
        check(self.lib.mg_average_lab(self.h, ptr(img, C.c_uint8), w, h, img.strides[0], ptr(out, C.c_float)))
        return out

    def cells_lab(self, img: np.ndarray, gw: int, gh: int):
        img = np.ascontiguousarray(img, dtype=np.uint8)
        h, w = img.shape[:2]
        lab = np.zeros((gw * gh, 3), np.float32)
        rgb = np.zeros((gw * gh, 3), np.uint8)
        check(self.lib.mg_cells_lab(self.h, ptr(img, C.c_uint8), w, h, img.strides[0], gw, gh,
                                    ptr(lab, C.c_float), ptr(rgb, C.c_uint8)))
        return lab, rgb

    def resize(self, img: np.ndarray, dw: int, dh: int) -> np.ndarray:
        """main.rs:710-738 resize_image on the device (the context's thumbnail filter)."""
        img = np.ascontiguousarray(img, dtype=np.uint8)
        h, w = img.shape[:2]
        out = np.zeros((dh, dw, 3), np.uint8)
        check(self.lib.mg_resize(self.h, ptr(img, C.c_uint8), w, h, img.strides[0], dw, dh, ptr(out, C.c_uint8)))
        return out

    def images_lab(self, imgs: list[np.ndarray]):
        n = len(imgs)
        imgs = [np.ascontiguousarray(i, dtype=np.uint8) for i in imgs]
        ptrs = (_u8p * max(n, 1))(*[ptr(i, C.c_uint8) for i in imgs])
        ws = (C.c_int * max(n, 1))(*[i.shape[1] for i in imgs])
        hs = (C.c_int * max(n, 1))(*[i.shape[0] for i in imgs])
        lab = np.zeros((max(n, 1), 3), np.float32)
        rgb = np.zeros((max(n, 1), 3), np.uint8)
        check(self.lib.mg_images_lab(self.h, ptrs, ws, hs, None, n, ptr(lab, C.c_float), ptr(rgb, C.c_uint8)))
        return lab[:n], rgb[:n]

    # ---- similarity / nearest
    def similarity(self, lab, layout: int = MG_SIM_FULL) -> np.ndarray:
        lab = _lab3(lab)
        p = lab.shape[0]
        size = p * p if layout == MG_SIM_FULL else p * (p - 1) // 2
        out = np.zeros(max(size, 1), np.float32)
        check(self.lib.mg_similarity_build(self.h, ptr(lab, C.c_float), p, layout, ptr(out, C.c_float)))
        return out[:size].reshape(p, p) if layout == MG_SIM_FULL else out[:size]

    def set_nearest_method(self, method: int) -> None:
        """MG_NEAREST_AUTO / MG_NEAREST_SCAN / MG_NEAREST_GRID (identical results)."""
        check(self.lib.mg_ctx_set_nearest_method(self.h, method))

    def set_scoring(self, scoring: int) -> None:
        """MG_SCORING_CLI (squared distance + penalty, main.rs) or MG_SCORING_GUI
        (distance + penalty, gui/app_full.rs) for the greedy placement."""
        check(self.lib.mg_ctx_set_scoring(self.h, scoring))

    def nearest_n(self, pal, queries, k: int):
        pal, q = _lab3(pal), _lab3(queries)
        nq = q.shape[0]
        idx = np.zeros((max(nq, 1), k), np.uint32)
        dist = np.zeros((max(nq, 1), k), np.float32)
        check(self.lib.mg_nearest_n(self.h, ptr(pal, C.c_float), pal.shape[0], ptr(q, C.c_float), nq, k,
                                    ptr(idx, C.c_uint32), ptr(dist, C.c_float)))
        return idx[:nq], dist[:nq]

    # ---- adjacency
    def penalty_batch(self, pal, grid: np.ndarray, weight: float, cxy: np.ndarray) -> np.ndarray:
        pal = _lab3(pal)
        grid = np.ascontiguousarray(grid, dtype=np.int32)
        gh, gw = grid.shape
        cxy = np.ascontiguousarray(cxy, dtype=np.int32).reshape(-1, 3)
        out = np.zeros(max(len(cxy), 1), np.float32)
        check(self.lib.mg_penalty_batch(self.h, ptr(pal, C.c_float), pal.shape[0], ptr(grid, C.c_int32), gw, gh,
                                        weight, ptr(cxy, C.c_int32), len(cxy), ptr(out, C.c_float)))
        return out[:len(cxy)]

    def total_cost(self, pal, grid: np.ndarray) -> float:
        pal = _lab3(pal)
        grid = np.ascontiguousarray(grid, dtype=np.int32)
        gh, gw = grid.shape if grid.size else (0, 0)
        out = C.c_float()
        check(self.lib.mg_total_cost(self.h, ptr(pal, C.c_float), pal.shape[0], ptr(grid, C.c_int32), gw, gh,
                                     C.byref(out)))
        return out.value

    def swap_delta_batch(self, pal, grid: np.ndarray, pairs: np.ndarray) -> np.ndarray:
        pal = _lab3(pal)
        grid = np.ascontiguousarray(grid, dtype=np.int32)
        gh, gw = grid.shape
        pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 4)
        out = np.zeros(max(len(pairs), 1), np.float32)
        check(self.lib.mg_swap_delta_batch(self.h, ptr(pal, C.c_float), pal.shape[0], ptr(grid, C.c_int32), gw,
                                           gh, ptr(pairs, C.c_int32), len(pairs), ptr(out, C.c_float)))
        return out[:len(pairs)]

    # ---- placement / annealing
    def place_greedy(self, pal, cell_lab, gw: int, gh: int, max_usage: int, weight: float):
        pal, cl = _lab3(pal), _lab3(cell_lab)
        grid = np.zeros(gw * gh, np.int32)
        resets = C.c_int()
        cfg = PlaceConfig(max_usage, weight)
        check(self.lib.mg_place_greedy(self.h, ptr(pal, C.c_float), pal.shape[0], ptr(cl, C.c_float), gw, gh,
                                       C.byref(cfg), ptr(grid, C.c_int32), C.byref(resets)))
        return grid.reshape(gh, gw), resets.value

    def optimize(self, pal, grid: np.ndarray, iterations: int = 1000, t0: float = 100.0, decay: float = 0.99995,
                 chains: int = 1, seed: int = 0x5EED5EED5EED, stream: int = 0, greedy_only: bool = False):
        pal = _lab3(pal)
        g = np.ascontiguousarray(grid, dtype=np.int32).copy()
        gh, gw = g.shape if g.size else (0, 0)
        cfg = SaConfig(iterations, t0, decay, chains, seed, stream, 1 if greedy_only else 0)
        best = SaResult()
        per = (SaResult * chains)()
        cg = np.zeros((chains, max(gh * gw, 1)), np.int32)
        check(self.lib.mg_optimize(self.h, ptr(pal, C.c_float), pal.shape[0], ptr(g, C.c_int32), gw, gh,
                                   C.byref(cfg), C.byref(best), per, ptr(cg, C.c_int32)))
        return g, best, list(per), cg[:, :gh * gw].reshape(chains, gh, gw) if g.size else cg

    # ---- colour adjustment / composite
    def optimal_adjustment_batch(self, tile_rgb, target_rgb, strength: float) -> np.ndarray:
        t = np.ascontiguousarray(tile_rgb, dtype=np.uint8).reshape(-1, 3)
        g = np.ascontiguousarray(target_rgb, dtype=np.uint8).reshape(-1, 3)
        out = (ColorAdjustment * max(len(t), 1))()
        check(self.lib.mg_optimal_adjustment_batch(self.h, ptr(t, C.c_uint8), ptr(g, C.c_uint8), len(t), strength,
                                                   out))
        return np.array([[a.brightness, a.contrast, a.hue_shift, a.saturation] for a in out[:len(t)]],
                        np.float32).reshape(-1, 4)

    def apply_adjustment(self, adj, img: np.ndarray) -> np.ndarray:
        img = np.ascontiguousarray(img, dtype=np.uint8)
        h, w = img.shape[:2]
        a = ColorAdjustment(*[float(v) for v in adj])
        out = np.zeros_like(img)
        check(self.lib.mg_apply_adjustment(self.h, C.byref(a), ptr(img, C.c_uint8), w, h, img.strides[0],
                                           ptr(out, C.c_uint8)))
        return out

    def composite(self, grid: np.ndarray, thumbs: np.ndarray, cell_rgb, strength: float) -> np.ndarray:
        grid = np.ascontiguousarray(grid, dtype=np.int32)
        gh, gw = grid.shape
        thumbs = np.ascontiguousarray(thumbs, dtype=np.uint8)
        p, th, tw = thumbs.shape[:3]
        crgb = np.ascontiguousarray(cell_rgb, dtype=np.uint8).reshape(-1, 3)
        out = np.zeros((gh * th, gw * tw, 3), np.uint8)
        check(self.lib.mg_composite(self.h, ptr(grid, C.c_int32), gw, gh, ptr(thumbs, C.c_uint8), p, tw, th,
                                    ptr(crgb, C.c_uint8), strength, ptr(out, C.c_uint8)))
        return out


def improvement_percentage(r: SaResult) -> float:
    return float(load().mg_improvement_percentage(C.byref(r)))


def color_adjustment_new(b: float, c: float, h: float, s: float):
    a = load().mg_color_adjustment_new(b, c, h, s)
    return (a.brightness, a.contrast, a.hue_shift, a.saturation)


# ---- PNG files (host code: no context, no GPU) -----------------------------------------
def png_info(data: bytes) -> tuple[int, int]:
    w, h = C.c_int(), C.c_int()
    check(load().mg_png_info(data, len(data), C.byref(w), C.byref(h)))
    return w.value, h.value


def png_decode(data: bytes, out: np.ndarray | None = None) -> np.ndarray:
    """The file as an (h, w, 3) uint8 array (written into `out`, e.g. a view
    of pinned memory, when given)."""
    w, h = png_info(data)
    if out is None:
        out = np.empty((h, w, 3), np.uint8)
    if out.dtype != np.uint8 or out.ndim != 3 or out.shape != (h, w, 3) or out.strides[1:] != (3, 1):
        raise ValueError("out must be a (h, w, 3) uint8 array with contiguous rows")
    check(load().mg_png_decode(data, len(data), ptr(out, C.c_uint8), out.strides[0]))
    return out


def image_info(data: bytes) -> tuple[int, int]:
    """Width and height of a PNG or JPEG file."""
    w, h = C.c_int(), C.c_int()
    check(load().mg_image_info(data, len(data), C.byref(w), C.byref(h)))
    return w.value, h.value


def image_decode(data: bytes, out: np.ndarray | None = None) -> np.ndarray:
    """A PNG or JPEG file as an (h, w, 3) uint8 array."""
    w, h = image_info(data)
    if out is None:
        out = np.empty((h, w, 3), np.uint8)
    check(load().mg_image_decode(data, len(data), ptr(out, C.c_uint8), out.strides[0]))
    return out


def image_decode_batch(files: list[bytes], threads: int = 0) -> tuple[list[np.ndarray | None], list[int]]:
    """PNG and JPEG files on up to `threads` host threads; (images, status codes)."""
    n = len(files)
    outs, sizes = [], []
    for f in files:
        try:
            w, h = image_info(f)
        except MosaicError:
            w, h = 1, 1
        outs.append(np.zeros((h, w, 3), np.uint8))
    bufs = [C.create_string_buffer(f, len(f)) for f in files]
    data = (C.c_void_p * max(n, 1))(*[C.cast(b, C.c_void_p) for b in bufs])
    lens = (C.c_size_t * max(n, 1))(*[len(f) for f in files])
    outp = (_u8p * max(n, 1))(*[ptr(o, C.c_uint8) for o in outs])
    strides = (C.c_int64 * max(n, 1))(*[o.strides[0] for o in outs])
    status = (C.c_int * max(n, 1))()
    load().mg_image_decode_batch(data, lens, n, outp, strides, threads, status)
    st = [int(status[i]) for i in range(n)]
    return [o if s == MG_OK else None for o, s in zip(outs, st)], st


def png_decode_batch(files: list[bytes], threads: int = 0) -> tuple[list[np.ndarray | None], list[int]]:
    """Decodes every file on up to `threads` threads; (images, status codes)."""
    n = len(files)
    outs = []
    for f in files:
        try:
            w, h = png_info(f)
            outs.append(np.empty((h, w, 3), np.uint8))
        except MosaicError:
            outs.append(np.zeros((1, 1, 3), np.uint8))  # decode reports the defect
    bufs = [C.create_string_buffer(f, len(f)) for f in files]
    data = (C.c_void_p * max(n, 1))(*[C.cast(b, C.c_void_p) for b in bufs])
    sizes = (C.c_size_t * max(n, 1))(*[len(f) for f in files])
    out_p = (_u8p * max(n, 1))(*[ptr(o, C.c_uint8) for o in outs])
    strides = (C.c_int64 * max(n, 1))(*[o.strides[0] for o in outs])
    status = (C.c_int * max(n, 1))()
    load().mg_png_decode_batch(data, sizes, n, out_p, strides, threads, status)
    codes = [status[i] for i in range(n)]
    return [o if c == MG_OK else None for o, c in zip(outs, codes)], codes


def jpeg_encode(img: np.ndarray, quality: int = 75, threads: int = 0) -> bytes:
    img = np.ascontiguousarray(img, np.uint8)
    h, w = img.shape[:2]
    lib = load()
    cap = lib.mg_jpeg_encode_bound(w, h)
    out = np.empty(max(cap, 1), np.uint8)
    n = C.c_size_t()
    check(lib.mg_jpeg_encode(ptr(img, C.c_uint8), w, h, img.strides[0], quality, threads, ptr(out, C.c_uint8), cap,
                             C.byref(n)))
    return out[: n.value].tobytes()


def png_encode(img: np.ndarray, level: int = 1, threads: int = 0) -> bytes:
    img = np.ascontiguousarray(img, np.uint8)
    h, w = img.shape[:2]
    lib = load()
    cap = lib.mg_png_encode_bound(w, h)
    out = np.empty(max(cap, 1), np.uint8)
    n = C.c_size_t()
    check(lib.mg_png_encode(ptr(img, C.c_uint8), w, h, img.strides[0], level, threads, ptr(out, C.c_uint8), cap,
                            C.byref(n)))
    return out[: n.value].tobytes()

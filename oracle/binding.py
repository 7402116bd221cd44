"""ctypes binding of oracle/liboracle.so (built by oracle/Makefile).  Test infrastructure."""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "build" / "liboracle.so"

_u8p = C.POINTER(C.c_uint8)
_f32p = C.POINTER(C.c_float)
_f64p = C.POINTER(C.c_double)
_i32p = C.POINTER(C.c_int32)
_u32p = C.POINTER(C.c_uint32)
_i64p = C.POINTER(C.c_int64)
_ip = C.POINTER(C.c_int)


class OracleJob(C.Structure):
    _fields_ = [("target", _u8p), ("tw_img", C.c_int), ("th_img", C.c_int), ("tstride", C.c_long),
                ("mats", _u8p), ("mat_off", _i64p), ("mat_w", _ip), ("mat_h", _ip), ("n_mats", C.c_int),
                ("thumbs", _u8p), ("thumb_w", C.c_int), ("thumb_h", C.c_int),
                ("gw", C.c_int), ("gh", C.c_int), ("max_materials", C.c_int), ("aspect_tol", C.c_float),
                ("max_usage", C.c_int), ("weight", C.c_float), ("color_strength", C.c_float),
                ("enable_opt", C.c_int), ("iters", C.c_long), ("t0", C.c_float), ("decay", C.c_float),
                ("chains", C.c_int), ("seed", C.c_uint64), ("stream", C.c_uint32), ("threads", C.c_int),
                ("gui_scoring", C.c_int), ("ref_arith", C.c_int)]


class OracleOut(C.Structure):
    _fields_ = [("grid", _i32p), ("image", _u8p), ("pal_lab", _f32p), ("cell_lab", _f32p), ("greedy_grid", _i32p),
                ("chain_res", _f32p), ("p", C.c_int), ("n_resets", C.c_int), ("best_chain", C.c_int),
                ("initial_cost", C.c_float), ("final_cost", C.c_float), ("best_cost", C.c_float)]


_SIGS = [
    ("orc_srgb_lut", None, [_f32p]),
    ("orc_lab_pixel_f64", None, [C.c_int, C.c_int, C.c_int, _f64p]),
    ("orc_lab_mean_f64", None, [_u8p, C.c_int, C.c_int, C.c_long, _f64p]),
    ("orc_lab_mean_reffold", None, [_u8p, C.c_int, C.c_int, C.c_long, _f32p]),
    ("orc_lab_pixel_spec", None, [C.c_int, C.c_int, C.c_int, _f32p]),
    ("orc_lab_consts", None, [_f32p, _f32p, _f32p]),
    ("orc_lab_pixels_q", None, [_u8p, C.c_long, _i32p]),
    ("orc_lab_mean_spec", None, [_u8p, C.c_int, C.c_int, C.c_long, _f32p]),
    ("orc_avg_rgb", None, [_u8p, C.c_int, C.c_int, C.c_long, _u8p]),
    ("orc_resize_lanczos3", None, [_u8p, C.c_int, C.c_int, C.c_long, C.c_int, C.c_int, _u8p]),
    ("orc_cells", C.c_int, [_u8p, C.c_int, C.c_int, C.c_long, C.c_int, C.c_int, _f32p, _u8p]),
    ("orc_is_aspect_ratio_match", C.c_int, [C.c_float, C.c_float, C.c_float]),
    ("orc_select_palette", C.c_int, [_ip, _ip, C.c_int, C.c_float, C.c_float, C.c_int, _ip]),
    ("orc_lab_distance", C.c_float, [_f32p, _f32p]),
    ("orc_similarity_tri", None, [_f32p, C.c_int, _f32p]),
    ("orc_similarity_full", None, [_f32p, C.c_int, _f32p]),
    ("orc_nearest_n", None, [_f32p, C.c_int, _f32p, C.c_int, _u32p, _f32p]),
    ("orc_penalty", C.c_float, [_f32p, C.c_int, C.c_int, C.c_int, C.c_int, _i32p, C.c_int, C.c_int, C.c_float]),
    ("orc_total_cost", C.c_float, [_f32p, C.c_int, _i32p, C.c_int, C.c_int]),
    ("orc_swap_delta", C.c_float, [_f32p, C.c_int, _i32p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    ("orc_place_greedy", C.c_int, [_f32p, C.c_int, _f32p, C.c_int, C.c_int, C.c_int, C.c_float, _i32p, _ip]),
    ("orc_place_greedy_gui", C.c_int, [_f32p, C.c_int, _f32p, C.c_int, C.c_int, C.c_int, C.c_float, _i32p, _ip]),
    ("orc_philox", None, [_u32p, _u32p, _u32p]),
    ("orc_exp", C.c_float, [C.c_float]),
    ("orc_anneal", None, [_f32p, C.c_int, _i32p, C.c_int, C.c_int, C.c_long, C.c_float, C.c_float, C.c_uint64,
                          C.c_uint32, C.c_uint32, C.c_int, _f32p, _i64p]),
    ("orc_anneal_ex", None, [_f32p, C.c_int, _i32p, C.c_int, C.c_int, C.c_long, C.c_float, C.c_float, C.c_uint64,
                             C.c_uint32, C.c_uint32, C.c_int, C.c_int, _f32p, _i64p]),
    ("orc_rgb_to_hsv", None, [C.c_float, C.c_float, C.c_float, _f32p]),
    ("orc_hsv_to_rgb", None, [C.c_float, C.c_float, C.c_float, _f32p]),
    ("orc_adjustment_new", None, [C.c_float, C.c_float, C.c_float, C.c_float, _f32p]),
    ("orc_optimal_adjustment", None, [_u8p, _u8p, C.c_float, _f32p]),
    ("orc_adjust_pixel", None, [_f32p, _u8p, _u8p]),
    ("orc_adjust_pixels", None, [_f32p, _u8p, C.c_long, _u8p]),
    ("orc_composite", C.c_int, [_i32p, C.c_int, C.c_int, _u8p, C.c_int, C.c_int, _u8p, _u8p, C.c_float, _u8p]),
    ("orc_generate", C.c_int, [C.POINTER(OracleJob), C.POINTER(OracleOut)]),
]

_LIB = None


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib():
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            build_oracle()
        L = C.CDLL(str(LIB_PATH))
        for name, res, args in _SIGS:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def p(a: np.ndarray, t):
    return a.ctypes.data_as(C.POINTER(t))


# ---- numpy conveniences -------------------------------------------------------------
def lab_mean_spec(img: np.ndarray) -> np.ndarray:
    img = np.ascontiguousarray(img, np.uint8)
    out = np.zeros(3, np.float32)
    lib().orc_lab_mean_spec(p(img, C.c_uint8), img.shape[1], img.shape[0], img.strides[0], p(out, C.c_float))
    return out


def lab_mean_f64(img: np.ndarray) -> np.ndarray:
    img = np.ascontiguousarray(img, np.uint8)
    out = np.zeros(3, np.float64)
    lib().orc_lab_mean_f64(p(img, C.c_uint8), img.shape[1], img.shape[0], img.strides[0], p(out, C.c_double))
    return out


def lab_mean_reffold(img: np.ndarray) -> np.ndarray:
    img = np.ascontiguousarray(img, np.uint8)
    out = np.zeros(3, np.float32)
    lib().orc_lab_mean_reffold(p(img, C.c_uint8), img.shape[1], img.shape[0], img.strides[0], p(out, C.c_float))
    return out


def avg_rgb(img: np.ndarray) -> np.ndarray:
    img = np.ascontiguousarray(img, np.uint8)
    out = np.zeros(3, np.uint8)
    lib().orc_avg_rgb(p(img, C.c_uint8), img.shape[1], img.shape[0], img.strides[0], p(out, C.c_uint8))
    return out


def cells(img: np.ndarray, gw: int, gh: int):
    img = np.ascontiguousarray(img, np.uint8)
    lab = np.zeros((gw * gh, 3), np.float32)
    rgb = np.zeros((gw * gh, 3), np.uint8)
    rc = lib().orc_cells(p(img, C.c_uint8), img.shape[1], img.shape[0], img.strides[0], gw, gh, p(lab, C.c_float),
                         p(rgb, C.c_uint8))
    if rc != 0:
        raise ValueError("invalid grid")
    return lab, rgb


def similarity_full(lab: np.ndarray) -> np.ndarray:
    lab = np.ascontiguousarray(lab, np.float32).reshape(-1, 3)
    n = lab.shape[0]
    out = np.zeros((n, n), np.float32)
    lib().orc_similarity_full(p(lab, C.c_float), n, p(out, C.c_float))
    return out


def similarity_tri(lab: np.ndarray) -> np.ndarray:
    lab = np.ascontiguousarray(lab, np.float32).reshape(-1, 3)
    n = lab.shape[0]
    out = np.zeros(max(n * (n - 1) // 2, 1), np.float32)
    lib().orc_similarity_tri(p(lab, C.c_float), n, p(out, C.c_float))
    return out[:n * (n - 1) // 2]


def nearest_n(pal: np.ndarray, queries: np.ndarray, k: int):
    pal = np.ascontiguousarray(pal, np.float32).reshape(-1, 3)
    q = np.ascontiguousarray(queries, np.float32).reshape(-1, 3)
    kk = min(k, pal.shape[0])
    idx = np.zeros((q.shape[0], kk), np.uint32)
    dist = np.zeros((q.shape[0], kk), np.float32)
    for i in range(q.shape[0]):
        lib().orc_nearest_n(p(pal, C.c_float), pal.shape[0], p(q[i], C.c_float), kk, p(idx[i], C.c_uint32),
                            p(dist[i], C.c_float))
    return idx, dist


def place_greedy(pal, cell_lab, gw, gh, max_usage, weight, gui=False):
    """The CLI's greedy placement (main.rs:335-475), or with gui=True the GUI
    generator's scoring (gui/app_full.rs:1396-1470)."""
    pal = np.ascontiguousarray(pal, np.float32).reshape(-1, 3)
    cl = np.ascontiguousarray(cell_lab, np.float32).reshape(-1, 3)
    grid = np.zeros(gw * gh, np.int32)
    resets = C.c_int()
    fn = lib().orc_place_greedy_gui if gui else lib().orc_place_greedy
    fn(p(pal, C.c_float), pal.shape[0], p(cl, C.c_float), gw, gh, max_usage, weight, p(grid, C.c_int32),
       C.byref(resets))
    return grid.reshape(gh, gw), resets.value


def total_cost(pal, grid):
    pal = np.ascontiguousarray(pal, np.float32).reshape(-1, 3)
    g = np.ascontiguousarray(grid, np.int32)
    gh, gw = g.shape
    return lib().orc_total_cost(p(pal, C.c_float), pal.shape[0], p(g, C.c_int32), gw, gh)


def swap_delta(pal, grid, x1, y1, x2, y2):
    pal = np.ascontiguousarray(pal, np.float32).reshape(-1, 3)
    g = np.ascontiguousarray(grid, np.int32)
    gh, gw = g.shape
    return lib().orc_swap_delta(p(pal, C.c_float), pal.shape[0], p(g, C.c_int32), gw, gh, x1, y1, x2, y2)


def penalty(pal, grid, cand, x, y, weight):
    pal = np.ascontiguousarray(pal, np.float32).reshape(-1, 3)
    g = np.ascontiguousarray(grid, np.int32)
    gh, gw = g.shape
    return lib().orc_penalty(p(pal, C.c_float), pal.shape[0], cand, x, y, p(g, C.c_int32), gw, gh, weight)


def anneal(pal, grid, iters, t0=100.0, decay=0.99995, seed=0x5EED5EED5EED, stream=0, chain=0, greedy_only=False,
           libm_exp=False):
    """One annealing chain from `grid` (libm_exp: acceptance by the C library's
    expf instead of the defined exp)."""
    pal = np.ascontiguousarray(pal, np.float32).reshape(-1, 3)
    g = np.ascontiguousarray(grid, np.int32).copy()
    gh, gw = g.shape if g.size else (0, 0)
    res = np.zeros(3, np.float32)
    cnt = np.zeros(3, np.int64)
    lib().orc_anneal_ex(p(pal, C.c_float), pal.shape[0], p(g, C.c_int32), gw, gh, iters, t0, decay, seed, stream,
                        chain, 1 if greedy_only else 0, 1 if libm_exp else 0, p(res, C.c_float), p(cnt, C.c_int64))
    return g, res, cnt


def resize_lanczos3(img, dw: int, dh: int):
    """main.rs:710-738 resize_image (fast_image_resize's default Lanczos3, restated)."""
    img = np.ascontiguousarray(img, np.uint8)
    h, w = img.shape[:2]
    out = np.zeros((dh, dw, 3), np.uint8)
    lib().orc_resize_lanczos3(p(img, C.c_uint8), w, h, img.strides[0], dw, dh, p(out, C.c_uint8))
    return out


def optimal_adjustment(tile_rgb, target_rgb, strength):
    t = np.ascontiguousarray(tile_rgb, np.uint8)
    g = np.ascontiguousarray(target_rgb, np.uint8)
    out = np.zeros(4, np.float32)
    lib().orc_optimal_adjustment(p(t, C.c_uint8), p(g, C.c_uint8), strength, p(out, C.c_float))
    return out


def adjust_pixel(adj, px):
    a = np.ascontiguousarray(adj, np.float32)
    i = np.ascontiguousarray(px, np.uint8)
    o = np.zeros(3, np.uint8)
    lib().orc_adjust_pixel(p(a, C.c_float), p(i, C.c_uint8), p(o, C.c_uint8))
    return o


def adjust_pixels(adj, img):
    """adjust_pixel on every pixel of an RGB8 array (any shape ending in 3)."""
    a = np.ascontiguousarray(adj, np.float32)
    i = np.ascontiguousarray(img, np.uint8)
    o = np.zeros_like(i)
    lib().orc_adjust_pixels(p(a, C.c_float), p(i, C.c_uint8), i.size // 3, p(o, C.c_uint8))
    return o


def adjustment_new(b, c, h, s):
    out = np.zeros(4, np.float32)
    lib().orc_adjustment_new(b, c, h, s, p(out, C.c_float))
    return out


def composite(grid, thumbs, cell_rgb, thumb_rgb, strength):
    g = np.ascontiguousarray(grid, np.int32)
    gh, gw = g.shape
    t = np.ascontiguousarray(thumbs, np.uint8)
    _, th, tw = t.shape[:3]
    crgb = np.ascontiguousarray(cell_rgb, np.uint8)
    trgb = np.ascontiguousarray(thumb_rgb, np.uint8)
    out = np.zeros((gh * th, gw * tw, 3), np.uint8)
    lib().orc_composite(p(g, C.c_int32), gw, gh, p(t, C.c_uint8), tw, th, p(crgb, C.c_uint8), p(trgb, C.c_uint8),
                        strength, p(out, C.c_uint8))
    return out


def generate(inp, threads: int = 1, want_image: bool = True, stream: int = 0, gui: bool = False,
             ref_arith: bool = False):
    """Run the whole job on the CPU from mosaic_gpu.job.Inputs (Philox stream id
    `stream`; gui: the GUI generator's greedy scoring; ref_arith: Lab by the
    reference's FP32 fold and acceptance by libm expf)."""
    cfg = inp.cfg
    tw, th = inp.tile
    n = len(inp.mats)
    job = OracleJob()
    job.target = p(inp.target, C.c_uint8)
    job.tw_img, job.th_img, job.tstride = cfg.target_w, cfg.target_h, inp.target.strides[0]
    job.mats = p(inp.mats.buf, C.c_uint8)
    off = np.ascontiguousarray(inp.mats.off, np.int64)
    w = np.ascontiguousarray(inp.mats.w, np.int32)
    h = np.ascontiguousarray(inp.mats.h, np.int32)
    job.mat_off, job.mat_w, job.mat_h, job.n_mats = p(off, C.c_int64), p(w, C.c_int), p(h, C.c_int), n
    if inp.thumbs is None:
        raise ValueError("the oracle needs host thumbnails")
    job.thumbs, job.thumb_w, job.thumb_h = p(inp.thumbs, C.c_uint8), tw, th
    job.gw, job.gh = cfg.grid_w, cfg.grid_h
    job.max_materials = cfg.max_materials or n
    job.aspect_tol = cfg.aspect_tolerance
    job.max_usage, job.weight, job.color_strength = cfg.max_usage, cfg.weight, cfg.color_strength
    job.enable_opt = 1 if cfg.enable_optimization else 0
    job.iters, job.t0, job.decay = cfg.iterations, 100.0, 0.99995
    job.chains, job.seed, job.stream, job.threads = cfg.chains, cfg.seed, stream, threads
    job.gui_scoring = 1 if gui else 0
    job.ref_arith = 1 if ref_arith else 0
    N = cfg.grid_w * cfg.grid_h
    grid = np.zeros(N, np.int32)
    image = np.zeros((cfg.grid_h * th, cfg.grid_w * tw, 3), np.uint8) if want_image else None
    pal_lab = np.zeros((max(n, 1), 3), np.float32)
    cell_lab = np.zeros((N, 3), np.float32)
    greedy = np.zeros(N, np.int32)
    chain_res = np.zeros((max(cfg.chains, 1), 3), np.float32)
    out = OracleOut()
    out.grid = p(grid, C.c_int32)
    out.image = p(image, C.c_uint8) if want_image else None
    out.pal_lab, out.cell_lab, out.greedy_grid = p(pal_lab, C.c_float), p(cell_lab, C.c_float), p(greedy, C.c_int32)
    out.chain_res = p(chain_res, C.c_float)
    rc = lib().orc_generate(C.byref(job), C.byref(out))
    if rc != 0:
        raise ValueError("oracle rejected the job")
    return {
        "grid": grid.reshape(cfg.grid_h, cfg.grid_w), "image": image, "pal_lab": pal_lab[:out.p],
        "cell_lab": cell_lab, "greedy_grid": greedy.reshape(cfg.grid_h, cfg.grid_w), "chain_res": chain_res,
        "p": out.p, "n_resets": out.n_resets, "best_chain": out.best_chain, "initial_cost": out.initial_cost,
        "final_cost": out.final_cost, "best_cost": out.best_cost,
    }

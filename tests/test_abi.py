"""The C ABI library loads and exports every entry point include/mosaic_gpu.h declares (CPU only).

Only host-side helpers are called here; nothing launches a kernel.
"""
import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
HEADER = REPO / "include" / "mosaic_gpu.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert len(names) >= 30
    for must in ["mg_ctx_create", "mg_generate", "mg_plan_run", "mg_nearest_n", "mg_place_greedy", "mg_optimize",
                 "mg_composite", "mg_similarity_build", "mg_cells_lab", "mg_average_lab"]:
        assert must in names


def test_library_exports_every_declared_symbol(built):
    from mosaic_gpu import _capi

    lib = _capi.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    if shutil.which("nm"):
        out = subprocess.run(["nm", "-D", "--defined-only", str(_capi.library_path())], capture_output=True,
                             text=True).stdout
        exported = set(re.findall(r"\b(mg_[a-z0-9_]+)\b", out))
        assert set(declared_functions()) <= exported


def test_binding_covers_header(built):
    from mosaic_gpu import _capi

    bound = {name for name, _, _ in _capi.SIGNATURES}
    assert set(declared_functions()) == bound


def test_no_cuda_device_is_an_error_not_a_crash(built):
    from mosaic_gpu import _capi

    lib = _capi.load()
    h = C.c_void_p()
    rc = lib.mg_ctx_create(0, C.byref(h))
    if rc == 0:
        lib.mg_ctx_destroy(h)
        pytest.skip("a CUDA device is present")
    assert rc in (_capi.MG_ERR_CUDA, _capi.MG_ERR_ARG)
    assert lib.mg_last_error()
    assert lib.mg_ctx_create(0, None) == _capi.MG_ERR_ARG


def test_host_helpers_match_oracle(built, orc):
    from mosaic_gpu import _capi

    lib = _capi.load()
    for a, t, tol in [(16 / 9, 16 / 9, 0.1), (1.8, 16 / 9, 0.1), (4 / 3, 16 / 9, 0.1), (1.0, 1.0, -0.1)]:
        assert lib.mg_is_aspect_ratio_match(a, t, tol) == orc.lib().orc_is_aspect_ratio_match(a, t, tol)
    for args in [(2.0, -1.0, 400.0, 3.0), (-2.0, 5.0, -500.0, 10.0), (0.1, 1.0, -100.0, 1.0)]:
        assert list(_capi.color_adjustment_new(*args)) == list(orc.adjustment_new(*args))
    a = np.array([50, 0, 0], np.float32)
    b = np.array([60, 10, 10], np.float32)
    pa, pb = a.ctypes.data_as(C.POINTER(C.c_float)), b.ctypes.data_as(C.POINTER(C.c_float))
    assert lib.mg_lab_distance(pa, pb) == orc.lib().orc_lab_distance(pa, pb)
    r = _capi.SaResult(100.0, 75.0, 75.0, 10, 15, 100, 0)
    assert _capi.improvement_percentage(r) == 25.0
    r0 = _capi.SaResult(0.0, 5.0, 5.0, 0, 0, 0, 0)
    assert _capi.improvement_percentage(r0) == 0.0
    cfg = _capi.SaConfig()
    lib.mg_sa_config_default(C.byref(cfg))
    assert (cfg.max_iterations, cfg.initial_temperature, cfg.temperature_decay) == (1000, 100.0,
                                                                                   np.float32(0.99995))


def test_select_palette_matches_oracle(built, orc):
    from mosaic_gpu import _capi

    lib = _capi.load()
    rng = np.random.default_rng(11)
    for trial in range(50):
        n = int(rng.integers(0, 40))
        ws = rng.choice([100, 128, 192, 256], n).astype(np.int32)
        hs = rng.choice([100, 128, 192, 256], n).astype(np.int32)
        ta = float(rng.choice([1.0, 4 / 3, 16 / 9]))
        tol = float(rng.choice([-0.1, 0.05, 0.1, 0.5]))
        mx = int(rng.integers(0, 20))
        a = (C.c_int * max(n, 1))()
        b = (C.c_int * max(n, 1))()
        w = (C.c_int * max(n, 1))(*ws)
        h = (C.c_int * max(n, 1))(*hs)
        ca = lib.mg_select_palette(w, h, n, ta, tol, mx, a)
        cb = orc.lib().orc_select_palette(w, h, n, ta, tol, mx, b)
        assert ca == cb and list(a[:ca]) == list(b[:cb])


def test_request_defaults(built):
    from mosaic_gpu import _capi

    r = _capi.Request()
    _capi.load().mg_request_default(C.byref(r))
    # main.rs:37-79 CLI defaults
    assert (r.grid_w, r.grid_h, r.max_materials, r.max_usage_per_image) == (50, 28, 500, 3)
    assert abs(r.aspect_tolerance - 0.1) < 1e-7 and abs(r.adjacency_penalty_weight - 0.3) < 1e-7
    assert abs(r.color_adjustment_strength - 0.3) < 1e-7 and r.enable_optimization == 1
    assert r.optimization_iterations == 1000

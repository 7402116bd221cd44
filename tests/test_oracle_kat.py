"""The oracle against the reference's own known-answer unit tests (CPU only).

Each test names the reference test it ports (path:line in mosaic-art-rust).
"""
import math

import numpy as np
import pytest


def solid(w, h, rgb):
    img = np.zeros((h, w, 3), np.uint8)
    img[:] = rgb
    return img


# ---- lib.rs:133-158 calculate_average_lab known answers (tolerance 1.0) ----------------
@pytest.mark.parametrize("fn", ["lab_mean_spec", "lab_mean_f64", "lab_mean_reffold"])
def test_lab_red(orc, fn):
    lab = getattr(orc, fn)(solid(10, 10, (255, 0, 0)))
    assert abs(lab[0] - 53.24) < 1.0 and abs(lab[1] - 80.09) < 1.0 and abs(lab[2] - 67.20) < 1.0


@pytest.mark.parametrize("fn", ["lab_mean_spec", "lab_mean_f64", "lab_mean_reffold"])
def test_lab_grey(orc, fn):
    lab = getattr(orc, fn)(solid(10, 10, (128, 128, 128)))
    assert abs(lab[0] - 53.59) < 1.0 and abs(lab[1]) < 1.0 and abs(lab[2]) < 1.0


def test_lab_spec_within_1e4_of_fp64(orc):
    """The build's FP32 arithmetic (fixed-point sum) vs the FP64 oracle: ΔE <= 1e-4."""
    rng = np.random.default_rng(7)
    worst = 0.0
    for shape in [(48, 48), (25, 25), (128, 128), (192, 256), (1, 1), (3, 7)]:
        img = rng.integers(0, 256, shape + (3,), dtype=np.uint8)
        d = np.linalg.norm(orc.lab_mean_spec(img).astype(np.float64) - orc.lab_mean_f64(img))
        worst = max(worst, d)
    assert worst <= 1e-4, worst


def test_lab_pixel_exhaustive_grey_and_primaries(orc):
    """Every grey level and every pure primary level: spec vs FP64 within 1e-4."""
    import ctypes as C

    L = orc.lib()
    out = np.zeros(3, np.float32)
    ref = np.zeros(3, np.float64)
    worst = 0.0
    for v in range(256):
        for rgb in [(v, v, v), (v, 0, 0), (0, v, 0), (0, 0, v), (255 - v, v, 128)]:
            L.orc_lab_pixel_spec(*rgb, out.ctypes.data_as(C.POINTER(C.c_float)))
            L.orc_lab_pixel_f64(*rgb, ref.ctypes.data_as(C.POINTER(C.c_double)))
            worst = max(worst, float(np.linalg.norm(out - ref)))
    assert worst < 1e-4, worst


def test_kernel_lab_arithmetic_equals_the_oracle_for_every_colour(orc):
    """The reduction kernels compute each pixel's fixed-point Lab summands as
    mg_math.h's lab_pixel_q (clamps left out, the 2^20 scale folded into the
    constants, the cube root's division by 3 as a multiply-high), two pixels at
    a time in packed FP32x2 arithmetic.  For all 2^24 sRGB8 colours that equals
    the oracle's defined Lab, clamped and quantised (tests/cpp/lab_equiv.cpp)."""
    import shutil
    import subprocess
    import tempfile
    from pathlib import Path

    if not shutil.which("g++"):
        pytest.skip("no g++")
    repo = Path(__file__).resolve().parents[1]
    build = repo / "oracle" / "build"
    with tempfile.TemporaryDirectory() as d:
        exe = Path(d) / "lab_equiv"
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
               str(repo / "tests" / "cpp" / "lab_equiv.cpp"), f"-L{build}", "-loracle", f"-Wl,-rpath,{build}",
               "-o", str(exe)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "differing 0" in r.stdout, r.stdout + r.stderr


def test_composite_adjustment_equals_the_definition_for_every_colour():
    """The composite adjusts each pixel with mg_math.h's adjust_unit: the
    definition adjust_from_bc (which the oracle restates) rearranged for
    channels in [0, 1].  For twelve tile adjustments (hue shifts of both signs
    and the clamps' ends, saturation 0..2, brightness and contrast changes)
    and all 2^24 byte triples through each one's brightness/contrast table,
    the two give the same output bytes (tests/cpp/adjust_equiv.cpp)."""
    import shutil
    import subprocess
    import tempfile
    from pathlib import Path

    if not shutil.which("g++"):
        pytest.skip("no g++")
    repo = Path(__file__).resolve().parents[1]
    with tempfile.TemporaryDirectory() as d:
        exe = Path(d) / "adjust_equiv"
        r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
                            str(repo / "tests" / "cpp" / "adjust_equiv.cpp"), "-o", str(exe)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "differing 0" in r.stdout, r.stdout + r.stderr


# ---- main.rs:866-889 calculate_average_rgb -----------------------------------------------
def test_avg_rgb_red(orc):
    assert tuple(orc.avg_rgb(solid(10, 10, (255, 0, 0)))) == (255, 0, 0)


def test_avg_rgb_mixed_truncates(orc):
    img = np.array([[[255, 0, 0], [0, 255, 0]], [[0, 0, 255], [255, 255, 255]]], np.uint8)
    assert tuple(orc.avg_rgb(img)) == (127, 127, 127)


# ---- lib.rs:160-209 is_aspect_ratio_match ---------------------------------------------------------
@pytest.mark.parametrize("img,target,tol,expect", [
    (16 / 9, 16 / 9, 0.1, True), (1.8, 16 / 9, 0.1, True), (4 / 3, 16 / 9, 0.1, False),
    (16 / 9, 9 / 16, 0.1, False), (1.0, 1.0, -0.1, False), (1.0, 1.0, 1000.0, True)])
def test_aspect_ratio_match(orc, img, target, tol, expect):
    assert bool(orc.lib().orc_is_aspect_ratio_match(img, target, tol)) == expect


# ---- main.rs:166-261 load_tiles selection --------------------------------------------------------
def _select(orc, ws, hs, ta, tol, maxm):
    import ctypes as C

    n = len(ws)
    w = (C.c_int * max(n, 1))(*ws)
    h = (C.c_int * max(n, 1))(*hs)
    sel = (C.c_int * max(n, 1))()
    cnt = orc.lib().orc_select_palette(w, h, n, ta, tol, maxm, sel)
    return list(sel[:cnt])


def test_select_filter_in_order(orc):
    assert _select(orc, [256, 256, 192, 256], [192, 256, 256, 192], 4 / 3, 0.1, 10) == [0, 3]


def test_select_fallback_takes_first_2x_max(orc):
    # main.rs:215-253: no match -> first min(n, 2*max) unfiltered, then truncate to max
    assert _select(orc, [100] * 10, [100] * 10, 4 / 3, 0.1, 3) == [0, 1, 2]


def test_select_truncates(orc):
    assert _select(orc, [4] * 10, [3] * 10, 4 / 3, 0.1, 4) == [0, 1, 2, 3]


def test_select_zero_max_materials(orc):
    # main.rs:2013-2022 test_zero_max_materials
    assert _select(orc, [100, 100, 100], [100, 100, 100], 1.0, 0.1, 0) == []


# ---- similarity.rs:185-232, 320-412 ------------------------------------------------------------------
def test_similarity_self_zero_symmetric_positive(orc):
    lab = np.array([[50, 0, 0], [60, 10, 10], [40, -10, -10], [50, 0, 0]], np.float32)
    full = orc.similarity_full(lab)
    assert np.all(np.diag(full) == 0)
    assert np.array_equal(full, full.T)
    assert full[0, 1] > 0 and full[0, 3] == 0.0
    tri = orc.similarity_tri(lab)
    n = 4
    for i in range(n):
        for j in range(i + 1, n):
            assert tri[i * n - i * (i + 1) // 2 + j - i - 1] == full[i, j]


def test_lab_distance(orc):
    import ctypes as C

    a = np.array([50, 0, 0], np.float32)
    b = np.array([60, 10, 10], np.float32)
    f = orc.lib().orc_lab_distance
    pa, pb = a.ctypes.data_as(C.POINTER(C.c_float)), b.ctypes.data_as(C.POINTER(C.c_float))
    assert f(pa, pa) == 0.0
    assert abs(f(pa, pb) - math.sqrt(300)) < 1e-5


# ---- lib.rs:212-227 nearest of four Lab points -------------------------------------------------------
def test_nearest_one_red(orc):
    pal = np.array([[50, 0, 0], [53.24, 80.09, 67.20], [87.74, -86.18, 83.18], [32.30, 79.20, -107.86]], np.float32)
    idx, dist = orc.nearest_n(pal, np.array([[53, 80, 67]], np.float32), 1)
    assert idx[0, 0] == 1


def test_nearest_ties_lowest_index(orc):
    pal = np.array([[10, 0, 0], [0, 0, 0], [10, 0, 0], [0, 0, 0]], np.float32)
    idx, dist = orc.nearest_n(pal, np.array([[0, 0, 0]], np.float32), 4)
    assert list(idx[0]) == [1, 3, 0, 2]


# ---- adjacency.rs:244-290 ---------------------------------------------------------------------------------
def test_penalty_positive_with_neighbour(orc):
    lab = np.array([[50, 0, 0], [60, 10, 10], [40, -10, -10]], np.float32)
    grid = -np.ones((3, 3), np.int32)
    grid[0, 0] = 0
    grid[0, 1] = 1
    assert orc.penalty(lab, grid, 2, 1, 0, 1.0) > 0.0


def test_total_cost_identical_tiles(orc):
    lab = np.array([[50, 0, 0], [50, 0, 0]], np.float32)
    grid = -np.ones((2, 2), np.int32)
    grid[0, 0] = 0
    grid[0, 1] = 1
    assert orc.total_cost(lab, grid) > 0.5


# ---- optimizer.rs:247-662 -------------------------------------------------------------------------------------
def _grid4():
    lab = np.array([[50, 0, 0], [60, 10, 10], [40, -10, -10], [55, 5, 5]], np.float32)
    return lab, np.array([[0, 1], [2, 3]], np.int32)


def test_optimize_basic_and_greedy(orc):
    lab, grid = _grid4()
    g, res, cnt = orc.anneal(lab, grid, 10)
    assert res[1] >= 0.0
    g2, res2, cnt2 = orc.anneal(lab, grid, 10, greedy_only=True)
    assert res2[1] <= res2[0] and cnt2[0] == cnt2[1]


def test_optimize_single_tile(orc):
    lab = np.array([[50, 0, 0]], np.float32)
    g, res, cnt = orc.anneal(lab, np.array([[0]], np.int32), 100)
    assert tuple(res[:2]) == (0.0, 0.0) and cnt[0] == 0 and cnt[1] == 0


def test_optimize_sparse_grid(orc):
    lab = np.array([[50, 0, 0], [60, 10, 10]], np.float32)
    grid = -np.ones((3, 3), np.int32)
    grid[0, 0] = 0
    grid[2, 2] = 1
    g, res, cnt = orc.anneal(lab, grid, 50)
    assert res[0] == 0.0 and res[1] >= 0.0


def test_optimize_zero_iterations(orc):
    lab, grid = _grid4()
    g, res, cnt = orc.anneal(lab, grid, 0)
    assert cnt[0] == 0 and cnt[1] == 0 and res[0] == res[1]
    assert np.array_equal(g, grid)


@pytest.mark.parametrize("t0,decay", [(100.0, 0.0), (1000.0, 0.5), (0.0, 0.99995), (-5.0, 0.99995), (1e-30, 0.9)])
def test_optimize_extreme_temperatures(orc, t0, decay):
    lab, grid = _grid4()
    g, res, cnt = orc.anneal(lab, grid, 50, t0=t0, decay=decay)
    assert math.isfinite(res[1]) and res[1] >= 0.0
    assert sorted(g.ravel()) == sorted(grid.ravel())  # swaps keep the multiset


def test_optimize_preserves_multiset(orc):
    rng = np.random.default_rng(3)
    lab = rng.uniform(-50, 80, (30, 3)).astype(np.float32)
    grid = rng.integers(0, 30, (9, 11)).astype(np.int32)
    g, res, cnt = orc.anneal(lab, grid, 2000)
    assert sorted(g.ravel()) == sorted(grid.ravel())
    assert abs(orc.total_cost(lab, g) - res[1]) < 1e-3 * max(1.0, res[1])


def test_improvement_percentage():
    # optimizer.rs:279-291: (100 - 75) / 100 * 100 = 25; initial 0 -> 0
    def pct(i, f):
        return ((i - f) / i) * 100.0 if i > 0 else 0.0

    assert pct(100.0, 75.0) == 25.0 and pct(0.0, 5.0) == 0.0


# ---- color_adjustment.rs:160-499 ------------------------------------------------------------------------------------
def test_adjustment_clamps(orc):
    assert list(orc.adjustment_new(2.0, -1.0, 400.0, 3.0)) == [1.0, 0.0, 180.0, 2.0]
    assert list(orc.adjustment_new(-2.0, 5.0, -500.0, 10.0)) == [-1.0, 2.0, -180.0, 2.0]
    assert orc.adjustment_new(0.0, 1.0, -100.0, 1.0)[2] == -100.0


def test_pixel_identity(orc):
    out = orc.adjust_pixel([0.0, 1.0, 0.0, 1.0], [128, 64, 192])
    assert np.all(np.abs(out.astype(int) - [128, 64, 192]) <= 1)


def test_brightness_contrast_directions(orc):
    assert np.all(orc.adjust_pixel([0.2, 1.0, 0.0, 1.0], [100, 100, 100]) > 100)
    assert orc.adjust_pixel([0.0, 1.5, 0.0, 1.0], [50, 50, 50])[0] < 50
    assert orc.adjust_pixel([0.0, 1.5, 0.0, 1.0], [200, 200, 200])[0] > 200


def test_hue_shift_red_to_green(orc):
    out = orc.adjust_pixel([0.0, 1.0, 120.0, 1.0], [255, 0, 0])
    assert out[1] > out[0] and out[1] > out[2]


def test_saturation(orc):
    grey = orc.adjust_pixel([0.0, 1.0, 0.0, 2.0], [128, 128, 128])
    assert np.all(np.abs(grey.astype(int) - 128) <= 5)
    d = orc.adjust_pixel([0.0, 1.0, 0.0, 0.5], [255, 100, 50])
    assert int(d.max()) - int(d.min()) < 205


def test_extreme_pixels(orc):
    a = [0.5, 1.5, 60.0, 1.5]
    assert np.all(orc.adjust_pixel(a, [255, 255, 255]) >= 250)
    assert np.all(orc.adjust_pixel(a, [0, 0, 0]) > 0)


def test_optimal_adjustment_cases(orc):
    same = orc.optimal_adjustment([128, 128, 128], [128, 128, 128], 1.0)
    assert abs(same[0]) < 0.01 and abs(same[2]) < 0.01 and abs(same[3] - 1) < 0.01
    up = orc.optimal_adjustment([50, 50, 50], [200, 200, 200], 1.0)
    down = orc.optimal_adjustment([200, 200, 200], [50, 50, 50], 1.0)
    assert 0 < up[0] <= 1 and -1 <= down[0] < 0
    hue = orc.optimal_adjustment([255, 0, 0], [0, 255, 0], 1.0)
    assert 10 < abs(hue[2]) <= 180
    sat = orc.optimal_adjustment([255, 0, 0], [200, 150, 150], 1.0)
    assert 0 <= sat[3] < 1
    full = orc.optimal_adjustment([100, 100, 100], [200, 200, 200], 1.0)
    half = orc.optimal_adjustment([100, 100, 100], [200, 200, 200], 0.5)
    assert abs(half[0] - full[0] * 0.5) < 0.01
    g = orc.optimal_adjustment([128, 128, 128], [64, 64, 64], 1.0)
    assert g[0] < 0 and abs(g[2]) < 5 and abs(g[3] - 1) < 0.1
    z = orc.optimal_adjustment([255, 0, 0], [0, 255, 0], 0.0)
    assert abs(z[0]) < 0.01 and abs(z[2]) < 0.01 and abs(z[3] - 1) < 0.01
    wrap = orc.optimal_adjustment([255, 0, 0], [255, 0, 255], 1.0)
    assert abs(wrap[2]) <= 180
    low = orc.optimal_adjustment([100, 95, 105], [105, 95, 100], 1.0)
    assert abs(low[2]) < 10


# ---- the build's own definitions: Philox and exp ---------------------------------------------------------------------
def test_philox_known_answers(orc):
    import ctypes as C

    kats = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
            ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
            ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
             (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, expect in kats:
        out = (C.c_uint32 * 4)()
        orc.lib().orc_philox((C.c_uint32 * 4)(*ctr), (C.c_uint32 * 2)(*key), out)
        assert tuple(out) == expect


def test_exp_within_one_ulp(orc):
    f = orc.lib().orc_exp
    xs = np.concatenate([np.linspace(-87, 88.5, 20001), np.linspace(-1, 1, 2001)]).astype(np.float32)
    for x in xs:
        y = np.float32(f(float(x)))
        ref = math.exp(float(x))
        if ref < 1.2e-38:
            continue
        ulp = float(np.spacing(np.float32(ref)))
        assert abs(float(y) - ref) <= 1.0 * ulp, (x, y, ref)
    assert f(-100.0) == 0.0 and math.isinf(f(100.0)) and math.isnan(f(float("nan")))
    assert f(-0.0) == 1.0


# ---- main.rs:1219-1378 placement scenarios ---------------------------------------------------------------------------
def test_greedy_usage_one_forces_resets(orc):
    lab = np.array([[50, 0, 0], [52, 1, 1], [48, -1, 0]], np.float32)
    cells = np.tile(np.array([[50, 0, 0]], np.float32), (9, 1))
    grid, resets = orc.place_greedy(lab, cells, 3, 3, 1, 0.0)
    assert np.all(grid >= 0) and resets > 0
    for y in range(3):  # same-neighbour ban holds whenever a candidate passes it
        for x in range(3):
            if x > 0:
                assert grid[y, x] != grid[y, x - 1]
            if y > 0:
                assert grid[y, x] != grid[y - 1, x]


def test_greedy_empty_palette(orc):
    grid, resets = orc.place_greedy(np.zeros((0, 3), np.float32), np.zeros((4, 3), np.float32), 2, 2, 3, 0.3)
    assert np.all(grid == -1) and resets == 0


def test_greedy_single_material_falls_back_to_nearest(orc):
    grid, resets = orc.place_greedy(np.array([[50, 0, 0]], np.float32), np.zeros((4, 3), np.float32), 2, 2, 3, 0.3)
    assert np.all(grid == 0)


# ---- gui/app_full.rs:1396-1568 the GUI generator's selection ----------------------------------------------------------
def test_gui_scoring_known_answer(orc):
    """Left neighbour T0 = (50,0,0); the cell wants (52,0,0).  T1 = (51,0,0) is 1 away
    (squared 1) and 1 from T0 (penalty 1/2 per unit weight); T2 = (54,0,0) is 2 away
    (squared 4) and 4 from T0 (penalty 1/5).  At weight 5 the CLI scores 1 + 2.5 vs
    4 + 1 and keeps T1; the GUI scores sqrt: 1 + 2.5 vs 2 + 1 and takes T2."""
    lab = np.array([[50, 0, 0], [51, 0, 0], [54, 0, 0]], np.float32)
    cells = np.array([[50, 0, 0], [52, 0, 0]], np.float32)
    cli, r1 = orc.place_greedy(lab, cells, 2, 1, 10, 5.0)
    gui, r2 = orc.place_greedy(lab, cells, 2, 1, 10, 5.0, gui=True)
    assert cli.tolist() == [[0, 1]] and gui.tolist() == [[0, 2]] and r1 == r2 == 0
    f = np.float32
    assert f(1) + f(5) * f(0.5) < f(4) + f(5) * (f(1) / f(5))
    assert f(2) + f(5) * (f(1) / f(5)) < f(1) + f(5) * f(0.5)


def test_gui_equals_cli_without_penalty(orc):
    """sqrt is monotone and candidates come in ascending distance, so with weight 0
    the GUI picks the CLI's tile everywhere, fallbacks (usage resets) included."""
    rng = np.random.default_rng(5)
    resets = 0
    for p, mu in [(3, 1), (40, 2), (150, 1), (400, 3)]:
        lab = np.empty((p, 3), np.float32)
        lab[:, 0] = rng.uniform(0, 100, p)
        lab[:, 1:] = rng.uniform(-60, 60, (p, 2))
        cells = lab[rng.integers(0, p, 12 * 9)] + rng.normal(0, 2, (12 * 9, 3)).astype(np.float32)
        a, ra = orc.place_greedy(lab, cells, 12, 9, mu, 0.0)
        b, rb = orc.place_greedy(lab, cells, 12, 9, mu, 0.0, gui=True)
        assert np.array_equal(a, b) and ra == rb
        resets += ra
    assert resets > 0  # the fallback path ran


def test_gui_penalty_changes_choices(orc):
    """With a penalty the two scorings part: sqrt shrinks the colour term against it."""
    rng = np.random.default_rng(6)
    lab = np.empty((2000, 3), np.float32)
    lab[:, 0] = rng.uniform(0, 100, 2000)
    lab[:, 1:] = rng.uniform(-60, 60, (2000, 2))
    cells = lab[rng.integers(0, 2000, 400)] + rng.normal(0, 3, (400, 3)).astype(np.float32)
    a, _ = orc.place_greedy(lab, cells, 20, 20, 4, 100.0)
    b, _ = orc.place_greedy(lab, cells, 20, 20, 4, 100.0, gui=True)
    assert np.all(b >= 0) and not np.array_equal(a, b)


def test_gui_scoring_through_the_whole_job(orc):
    """orc_generate with the GUI's scoring: at weight 0 the same mosaic as the
    CLI's; at weight 2 the two part (the GPU tests compare each with the device)."""
    from mosaic_gpu import job

    for weight, same in [(0.0, True), (2.0, False)]:
        cfg = job.scaled(job.WORKLOADS["recommended"], target_w=240, target_h=180, n_materials=150, material_side=32,
                         grid_w=20, grid_h=15, tile_w=8, tile_h=8, iterations=200, chains=2, weight=weight)
        inp = job.make_inputs(cfg)
        a = orc.generate(inp, threads=4, gui=True)
        b = orc.generate(inp, threads=4)
        assert np.array_equal(a["greedy_grid"], b["greedy_grid"]) == same

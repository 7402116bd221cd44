"""Stage-by-stage parity of the CUDA path (through the C ABI) against the CPU oracle.

Bar: bit-exact for every stage (the FP32 arithmetic is defined identically on
host and device); cell Lab additionally within 1e-4 ΔE of the FP64 oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LAB_TOL_DE = 1e-4


def rand_lab(rng, n):
    lab = np.empty((n, 3), np.float32)
    lab[:, 0] = rng.uniform(0, 100, n)
    lab[:, 1:] = rng.uniform(-90, 90, (n, 2))
    return lab


# ---- (a) Lab reduce -------------------------------------------------------------------------------
@pytest.mark.parametrize("w,h,gw,gh", [(1024, 768, 40, 30), (257, 131, 7, 5), (50, 50, 50, 50), (3, 3, 1, 1),
                                       (640, 480, 13, 11), (1024, 768, 32, 24), (960, 720, 20, 15)])
def test_cells_lab_bit_exact(ctx, orc, w, h, gw, gh):
    from mosaic_gpu import synth

    img = synth.target(w, h, 4, seed=w * 7 + h, stream=5)
    lab, rgb = ctx.cells_lab(img, gw, gh)
    rlab, rrgb = orc.cells(img, gw, gh)
    assert np.array_equal(lab.view(np.uint32), rlab.view(np.uint32))
    assert np.array_equal(rgb, rrgb)
    cw, ch = w // gw, h // gh
    for c in range(0, gw * gh, max(1, gw * gh // 25)):
        y, x = divmod(c, gw)
        ref = orc.lab_mean_f64(img[y * ch:(y + 1) * ch, x * cw:(x + 1) * cw])
        assert np.linalg.norm(lab[c].astype(np.float64) - ref) <= LAB_TOL_DE


def _every_colour():
    """A 4096 x 4096 image holding each sRGB8 colour once, in an order that
    mixes all three channels inside every 16 x 16 block."""
    i = np.arange(1 << 24, dtype=np.uint32)
    j = (i * np.uint32(2654435761)) & np.uint32(0xFFFFFF)  # odd multiplier: a permutation of 0..2^24-1
    rgb = np.stack([(j >> 16) & 0xFF, (j >> 8) & 0xFF, j & 0xFF], -1).astype(np.uint8)
    return rgb.reshape(4096, 4096, 3)


@pytest.mark.parametrize("cell", [1, 4, 8, 16, 12])
def test_cells_lab_every_colour(ctx, orc, cell):
    """Every sRGB8 colour through the cell reduction: 1-pixel cells take the
    pixel-pair path (each cell one pixel, so each colour's Lab is checked on
    its own), 4-, 8- and 16-pixel cells the 12-, 24- and 48-byte vector paths,
    12-pixel cells the 12-byte path with 36-byte cell offsets.  Every cell's
    Lab equals the oracle's fixed-point mean of its pixels bit for bit."""
    import ctypes as C

    img = _every_colour()
    g = 4096 // cell
    q = np.empty((1 << 24, 3), np.int32)
    orc.lib().orc_lab_pixels_q(img.ctypes.data_as(C.POINTER(C.c_uint8)), 1 << 24,
                               q.ctypes.data_as(C.POINTER(C.c_int32)))
    sums = q.reshape(4096, 4096, 3)[:g * cell, :g * cell].astype(np.int64)
    sums = sums.reshape(g, cell, g, cell, 3).sum(axis=(1, 3)).reshape(-1, 3)
    n = np.float32(cell * cell)
    want = (sums.astype(np.float32) / n) * np.float32(2.0 ** -20)
    lab, rgb = ctx.cells_lab(img, g, g) if cell * g == 4096 else ctx.cells_lab(
        np.ascontiguousarray(img[:g * cell, :g * cell]), g, g)
    assert np.array_equal(lab.view(np.uint32), want.view(np.uint32))
    px = img[:g * cell, :g * cell].reshape(g, cell, g, cell, 3).astype(np.uint64).sum(axis=(1, 3)).reshape(-1, 3)
    assert np.array_equal(rgb, (px // np.uint64(cell * cell)).astype(np.uint8))


def test_images_lab_bit_exact(ctx, orc):
    rng = np.random.default_rng(1)
    imgs = [rng.integers(0, 256, (h, w, 3), dtype=np.uint8) for (w, h) in
            [(1, 1), (3, 7), (128, 128), (256, 192), (192, 256), (33, 1), (1, 45), (300, 200)]]
    lab, rgb = ctx.images_lab(imgs)
    for i, img in enumerate(imgs):
        assert np.array_equal(lab[i].view(np.uint32), orc.lab_mean_spec(img).view(np.uint32)), i
        assert np.array_equal(rgb[i], orc.avg_rgb(img))
        assert np.linalg.norm(lab[i].astype(np.float64) - orc.lab_mean_f64(img)) <= LAB_TOL_DE


def test_average_lab_large_and_strided(ctx, orc):
    from mosaic_gpu import synth

    img = synth.target(1600, 1200, 6, seed=99, stream=3)
    assert np.array_equal(ctx.average_lab(img).view(np.uint32), orc.lab_mean_spec(img).view(np.uint32))
    view = img[100:900, 200:1300]  # row stride 3*1600 > 3*1100
    assert np.array_equal(ctx.average_lab(np.asarray(view)).view(np.uint32),
                          orc.lab_mean_spec(np.ascontiguousarray(view)).view(np.uint32))


def test_lab_known_answers_on_gpu(ctx):
    red = np.zeros((10, 10, 3), np.uint8)
    red[:] = (255, 0, 0)
    lab = ctx.average_lab(red)
    assert abs(lab[0] - 53.24) < 1 and abs(lab[1] - 80.09) < 1 and abs(lab[2] - 67.20) < 1
    grey = np.full((10, 10, 3), 128, np.uint8)
    lab = ctx.average_lab(grey)
    assert abs(lab[0] - 53.59) < 1 and abs(lab[1]) < 1 and abs(lab[2]) < 1


# ---- (c) similarity -------------------------------------------------------------------------------------
@pytest.mark.parametrize("p", [1, 2, 5, 97, 500, 1027])
def test_similarity_bit_exact(ctx, orc, p):
    from mosaic_gpu import MG_SIM_TRIANGULAR

    lab = rand_lab(np.random.default_rng(p), p)
    full = ctx.similarity(lab)
    assert np.array_equal(full.view(np.uint32), orc.similarity_full(lab).view(np.uint32))
    if p >= 2:
        tri = ctx.similarity(lab, MG_SIM_TRIANGULAR)
        assert np.array_equal(tri.view(np.uint32), orc.similarity_tri(lab).view(np.uint32))


# ---- (b) k nearest ------------------------------------------------------------------------------------------
@pytest.mark.parametrize("p,k,nq", [(1, 1, 9), (7, 100, 13), (100, 100, 33), (101, 100, 64), (500, 100, 200),
                                    (2048, 37, 77), (4096, 100, 100), (4097, 100, 50), (9000, 100, 40),
                                    (20000, 100, 17)])
def test_nearest_bit_exact(ctx, orc, p, k, nq):
    rng = np.random.default_rng(p * 31 + k)
    pal = rand_lab(rng, p)
    if p > 10:  # duplicated palette entries exercise the lowest-index tie rule
        pal[p // 2] = pal[1]
        pal[p - 1] = pal[1]
    q = rand_lab(rng, nq)
    q[0] = pal[min(1, p - 1)]
    idx, dist = ctx.nearest_n(pal, q, k)
    ridx, rdist = orc.nearest_n(pal, q, k)
    kk = min(k, p)
    assert np.array_equal(idx[:, :kk], ridx)
    assert np.array_equal(dist[:, :kk].view(np.uint32), rdist.view(np.uint32))
    if kk < k:
        assert np.all(idx[:, kk:] == 0xFFFFFFFF) and np.all(np.isinf(dist[:, kk:]))


# ---- adjacency evaluators -------------------------------------------------------------------------------------
def test_adjacency_batches_bit_exact(ctx, orc):
    rng = np.random.default_rng(5)
    pal = rand_lab(rng, 40)
    grid = rng.integers(-1, 40, (9, 13)).astype(np.int32)
    gh, gw = grid.shape
    pairs = np.array([[rng.integers(gw), rng.integers(gh), rng.integers(gw), rng.integers(gh)] for _ in range(500)]
                     + [[3, 3, 4, 3], [3, 3, 3, 4], [0, 0, 0, 0], [12, 8, 11, 8]], np.int32)
    d = ctx.swap_delta_batch(pal, grid, pairs)
    for i, (x1, y1, x2, y2) in enumerate(pairs):
        assert np.float32(d[i]) == np.float32(orc.swap_delta(pal, grid, x1, y1, x2, y2)), i
    cxy = np.array([[rng.integers(40), rng.integers(gw), rng.integers(gh)] for _ in range(300)], np.int32)
    pen = ctx.penalty_batch(pal, grid, 0.3, cxy)
    for i, (c, x, y) in enumerate(cxy):
        assert np.float32(pen[i]) == np.float32(orc.penalty(pal, grid, c, x, y, 0.3))
    assert np.float32(ctx.total_cost(pal, grid)) == np.float32(orc.total_cost(pal, grid))


# ---- (d) greedy placement ----------------------------------------------------------------------------------------------
@pytest.mark.parametrize("p,gw,gh,max_usage,weight", [
    (600, 40, 30, 3, 0.25), (150, 20, 15, 1, 0.0), (50, 12, 9, 0, 0.3), (5, 7, 6, 2, -1.0), (1, 4, 3, 3, 0.3),
    (300, 31, 17, 8, 0.25), (120, 16, 12, 3, 5.0), (2, 9, 9, 1, 0.25)])
def test_greedy_bit_exact(ctx, orc, p, gw, gh, max_usage, weight):
    rng = np.random.default_rng(p + gw)
    pal = rand_lab(rng, p)
    # smooth-ish target: neighbouring cells have similar Lab (as real targets do)
    base = rand_lab(rng, 1)[0]
    cells = (base + np.cumsum(rng.normal(0, 3, (gw * gh, 3)), axis=0)).astype(np.float32)
    grid, resets = ctx.place_greedy(pal, cells, gw, gh, max_usage, weight)
    rgrid, rresets = orc.place_greedy(pal, cells, gw, gh, max_usage, weight)
    assert np.array_equal(grid, rgrid)
    assert resets == rresets


@pytest.mark.parametrize("p,gw,gh,max_usage,region", [
    (12000, 60, 40, 4, "smooth"), (12000, 150, 20, 4, "flat"), (12000, 90, 30, 1, "flat"), (5000, 120, 25, 3, "flat")])
def test_greedy_dense_palette_bit_exact(ctx, orc, p, gw, gh, max_usage, region):
    """Palettes too large for the walker's shared memory (Lab read from global
    memory) and regions of one colour, where a row of placements exhausts the
    nearest materials: penalty windows, deep first entries and resets."""
    rng = np.random.default_rng(p + gw + max_usage)
    pal = rand_lab(rng, p)
    base = rand_lab(rng, 1)[0]
    step = 3.0 if region == "smooth" else 0.05
    cells = (base + np.cumsum(rng.normal(0, step, (gw * gh, 3)), axis=0)).astype(np.float32)
    grid, resets = ctx.place_greedy(pal, cells, gw, gh, max_usage, 0.25)
    rgrid, rresets = orc.place_greedy(pal, cells, gw, gh, max_usage, 0.25)
    assert np.array_equal(grid, rgrid)
    assert resets == rresets
    if region == "flat":
        assert resets > 0


@pytest.mark.parametrize("p,max_usage,region", [(700, 3, "smooth"), (12000, 4, "flat")])
def test_greedy_ring_form_bit_exact(ctx, orc, p, max_usage, region):
    """A 300x150 grid (45 000 cells) is too large for the walker's shared-memory
    copy of the grid, so the placed cells are kept as a ring of tagged words and
    written to the global grid as they are placed."""
    gw, gh = 300, 150
    rng = np.random.default_rng(p + max_usage)
    pal = rand_lab(rng, p)
    base = rand_lab(rng, 1)[0]
    step = 3.0 if region == "smooth" else 0.05
    cells = (base + np.cumsum(rng.normal(0, step, (gw * gh, 3)), axis=0)).astype(np.float32)
    grid, resets = ctx.place_greedy(pal, cells, gw, gh, max_usage, 0.25)
    rgrid, rresets = orc.place_greedy(pal, cells, gw, gh, max_usage, 0.25)
    assert np.array_equal(grid, rgrid)
    assert resets == rresets


# ---- (e) annealing --------------------------------------------------------------------------------------------------------
@pytest.mark.parametrize("p,gw,gh,iters,chains,t0,decay,greedy", [
    (60, 12, 9, 3000, 4, 100.0, 0.99995, False), (30, 7, 5, 500, 3, 1.0, 0.95, False),
    (10, 4, 4, 200, 2, 100.0, 0.0, False), (10, 4, 4, 200, 2, 0.0, 0.99995, False),
    (10, 4, 4, 200, 2, -3.0, 0.99995, False), (40, 10, 8, 1000, 2, 100.0, 0.99995, True),
    (1, 1, 1, 100, 1, 100.0, 0.99995, False), (20, 6, 5, 0, 2, 100.0, 0.99995, False),
    (80, 33, 20, 20000, 5, 100.0, 0.99995, False),
    # grids of at least 12 000 cells: 32 proposals a round (four lanes each)
    (300, 150, 100, 20000, 3, 100.0, 0.99995, False), (200, 120, 100, 5000, 2, 1.0, 0.95, False),
    (150, 130, 100, 3000, 2, 100.0, 0.99995, True), (90, 150, 80, 2000, 2, 0.0, 0.99995, False)])
def test_anneal_chains_bit_exact(ctx, orc, p, gw, gh, iters, chains, t0, decay, greedy):
    rng = np.random.default_rng(p * 7 + iters)
    pal = rand_lab(rng, p)
    grid = rng.integers(0, p, (gh, gw)).astype(np.int32)
    if gw * gh > 4:
        grid[0, 1] = -1  # an empty cell
    seed = 0xABCDEF0123 + p
    g, best, per, cg = ctx.optimize(pal, grid, iterations=iters, t0=t0, decay=decay, chains=chains, seed=seed,
                                    stream=9, greedy_only=greedy)
    finals = []
    for c in range(chains):
        rg, res, cnt = orc.anneal(pal, grid, iters, t0=t0, decay=decay, seed=seed, stream=9, chain=c,
                                  greedy_only=greedy)
        assert np.array_equal(cg[c], rg), c
        assert np.float32(per[c].initial_cost) == res[0]
        assert np.float32(per[c].final_cost) == res[1]
        assert np.float32(per[c].best_cost) == res[2]
        assert per[c].accepted_count == cnt[0] and per[c].improved_count == cnt[1]
        finals.append(res[1])
    b = int(np.argmin(finals))
    assert best.best_chain == b and np.array_equal(g, cg[b])


def test_anneal_empty_grid(ctx):
    g, best, per, cg = ctx.optimize(np.zeros((1, 3), np.float32), np.zeros((0, 0), np.int32), iterations=10)
    assert best.initial_cost == 0.0 and best.final_cost == 0.0 and best.improved_count == 0


# ---- (f) colour adjustment and composite -------------------------------------------------------------------------------------
def test_optimal_adjustment_bit_exact(ctx, orc):
    rng = np.random.default_rng(9)
    t = rng.integers(0, 256, (2000, 3)).astype(np.uint8)
    g = rng.integers(0, 256, (2000, 3)).astype(np.uint8)
    t[:20] = [[v, v, v] for v in range(0, 200, 10)]
    g[20:40] = [[255, 0, 0]] * 20
    for strength in (0.0, 0.4, 1.0):
        a = ctx.optimal_adjustment_batch(t, g, strength)
        for i in range(0, 2000, 7):
            assert np.array_equal(a[i].view(np.uint32), orc.optimal_adjustment(t[i], g[i], strength).view(np.uint32))


@pytest.mark.parametrize("adj", [(0.0, 1.0, 0.0, 1.0), (0.2, 1.0, 0.0, 1.0), (0.0, 1.5, 0.0, 1.0),
                                 (0.0, 1.0, 120.0, 1.0), (0.0, 1.0, -37.5, 1.3), (-0.3, 0.7, 179.9, 0.2),
                                 (0.5, 1.5, 60.0, 1.5), (0.01, 1.0, -180.0, 2.0)])
def test_apply_adjustment_bit_exact(ctx, orc, adj):
    rng = np.random.default_rng(int(abs(adj[2]) * 10) + 1)
    img = rng.integers(0, 256, (40, 50, 3)).astype(np.uint8)
    img[0, :8] = [[0, 0, 0], [255, 255, 255], [255, 0, 0], [0, 255, 0], [0, 0, 255], [128, 128, 128],
                  [255, 255, 0], [1, 2, 3]]
    out = ctx.apply_adjustment(adj, img)
    a = np.array(adj, np.float32)
    for y in range(0, 40, 3):
        for x in range(50):
            assert np.array_equal(out[y, x], orc.adjust_pixel(a, img[y, x])), (y, x)


def test_apply_adjustment_every_colour(ctx, orc):
    """Every byte triple (a 4096 x 4096 image) through apply_to_image on the
    device -- for adjustments in adjustment_new's ranges the composite's own
    per-pixel arithmetic (the brightness/contrast table and the packed HSV
    round trip) -- against the oracle's adjust_pixel, byte for byte: hue
    shifts of both signs up to the clamp's ends and one below 2^-120,
    saturation 0..2, brightness and contrast changes, one adjustment outside
    the ranges."""
    v = np.arange(1 << 24, dtype=np.uint32)
    img = np.stack([v >> 16, (v >> 8) & 255, v & 255], axis=-1).astype(np.uint8).reshape(4096, 4096, 3)
    for adj in [(0.0, 1.0, 37.5, 1.0), (0.1, 1.0, -64.0, 0.8), (0.05, 1.3, -90.0, 1.6), (-1.0, 1.0, 5.0, 2.0),
                (0.0, 1.0, 1e-38, 1.0), (0.1, 0.9, 180.0, 2.0), (-0.1, 1.1, -180.0, 0.0), (0.0, 1.0, 0.0, 0.5),
                (0.0, 1.0, 400.0, 2.5)]:
        out = ctx.apply_adjustment(adj, img)
        ref = orc.adjust_pixels(np.array(adj, np.float32), img)
        bad = np.flatnonzero(np.any(out != ref, axis=-1).ravel())
        assert bad.size == 0, (adj, bad[:5], img.reshape(-1, 3)[bad[:5]], out.reshape(-1, 3)[bad[:5]],
                               ref.reshape(-1, 3)[bad[:5]])
        odd = np.ascontiguousarray(img[1000:1003, 77:82])  # 15 pixels: an odd count
        assert np.array_equal(ctx.apply_adjustment(adj, odd), orc.adjust_pixels(np.array(adj, np.float32), odd)), adj


@pytest.mark.parametrize("strength", [0.0, 0.4, 1.0])
@pytest.mark.parametrize("tw,th", [(12, 10), (7, 5), (48, 48)])
def test_composite_bit_exact(ctx, orc, strength, tw, th):
    rng = np.random.default_rng(21 + tw)
    p, gw, gh = 30, 9, 7
    thumbs = rng.integers(0, 256, (p, th, tw, 3)).astype(np.uint8)
    grid = rng.integers(-1, p, (gh, gw)).astype(np.int32)
    cell_rgb = rng.integers(0, 256, (gh * gw, 3)).astype(np.uint8)
    thumb_rgb = np.stack([orc.avg_rgb(t) for t in thumbs])
    out = ctx.composite(grid, thumbs, cell_rgb, strength)
    ref = orc.composite(grid, thumbs, cell_rgb, thumb_rgb, strength)
    assert np.array_equal(out, ref)

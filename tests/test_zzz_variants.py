"""The greedy scoring of the GUI generator (mg_ctx_set_scoring, gui/app_full.rs:1396-1568)
and the PNG file ends (image::open / save, main.rs:492, 548, 672) through the device
path, against the oracle and the CLI-scored paths.

The file is collected last, so that a failure here leaves every other test run.
"""
import numpy as np
import pytest

from test_gpu_batch import TILE, _palette_inputs, _requests, _single, _targets
from test_gpu_generate import _small
from test_gpu_stages import rand_lab

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("p,gw,gh,max_usage,weight,step", [
    (60, 6, 9, 2, 1.0, 3.0), (150, 20, 15, 3, 0.3, 3.0), (700, 40, 30, 2, 5.0, 0.5), (5000, 120, 25, 3, 0.25, 0.05),
    (12000, 60, 40, 4, 2.0, 0.05), (700, 300, 150, 3, 0.25, 3.0)])
def test_greedy_gui_scoring_bit_exact(ctx, orc, p, gw, gh, max_usage, weight, step):
    """The GUI generator's selection (gui/app_full.rs:1396-1470: the Lab distance,
    not its square, plus the penalty) on every form of the walk: one warp (a
    6-cell-wide grid), the scouted walk with the palette in shared and in global
    memory, and the ring form (45 000 cells).  Where the two scorings part (the
    last four cases) the device follows the GUI's."""
    from mosaic_gpu import _capi as capi

    rng = np.random.default_rng(p * 3 + gw + int(weight * 10))
    pal = rand_lab(rng, p)
    base = rand_lab(rng, 1)[0]
    cells = (base + np.cumsum(rng.normal(0, step, (gw * gh, 3)), axis=0)).astype(np.float32)
    ctx.set_scoring(capi.MG_SCORING_GUI)
    try:
        grid, resets = ctx.place_greedy(pal, cells, gw, gh, max_usage, weight)
    finally:
        ctx.set_scoring(capi.MG_SCORING_CLI)
    rgrid, rresets = orc.place_greedy(pal, cells, gw, gh, max_usage, weight, gui=True)
    assert np.array_equal(grid, rgrid)
    assert resets == rresets
    if p >= 700:
        cli, _ = orc.place_greedy(pal, cells, gw, gh, max_usage, weight)
        assert not np.array_equal(rgrid, cli)


def test_scoring_argument_checked(ctx):
    from mosaic_gpu import _capi as capi

    with pytest.raises(capi.MosaicError):
        ctx.set_scoring(5)


def test_generate_gui_scoring(ctx, orc):
    """A whole job under the GUI generator's scoring (mg_ctx_set_scoring) against
    the oracle's GUI job: grid, chains and image; the CLI scoring gives a
    different mosaic here (weight 2), and the context returns to it after."""
    from mosaic_gpu import _capi as capi
    from mosaic_gpu import job

    cfg = _small("recommended", target_w=480, target_h=360, n_materials=150, material_side=32, grid_w=20, grid_h=15,
                 tile_w=12, tile_h=12, iterations=500, chains=4, weight=2.0)
    inp = job.make_inputs(cfg)
    ctx.set_scoring(capi.MG_SCORING_GUI)
    try:
        res, grid, image = job.generate(ctx, job.RequestHolder(inp))
    finally:
        ctx.set_scoring(capi.MG_SCORING_CLI)
    ref = orc.generate(inp, threads=8, gui=True)
    assert res.palette_size == ref["p"] and res.n_resets == ref["n_resets"]
    assert np.array_equal(grid, ref["grid"])
    assert int(np.abs(image.astype(np.int16) - ref["image"].astype(np.int16)).max(initial=0)) <= 1
    assert res.best_chain == ref["best_chain"]
    assert np.float32(res.final_cost) == np.float32(ref["final_cost"])
    cli_res, cli_grid, _ = job.generate(ctx, job.RequestHolder(inp))
    assert np.array_equal(cli_grid, orc.generate(inp, threads=8, want_image=False)["grid"])
    assert not np.array_equal(cli_grid, grid)


def test_batch_gui_scoring(ctx, orc):
    """A batch set up under the GUI generator's scoring (mg_ctx_set_scoring):
    every mosaic equals mg_generate under that scoring, and the oracle's GUI
    job for the first request (whose greedy grid the GUI scoring changes in 53
    cells)."""
    from mosaic_gpu import _capi as capi
    from mosaic_gpu import job

    mats, thumbs = _palette_inputs()
    tgts = _targets()[:4]
    spec = _requests()[:4]
    ctx.set_scoring(capi.MG_SCORING_GUI)
    try:
        pal = job.Palette(ctx, mats, thumbs, TILE, TILE, target_aspect=4 / 3)
        reqs = [job.mosaic_request(t, w, h, gw, gh, stream=i, **kw)
                for i, (t, (w, h, gw, gh, kw)) in enumerate(zip(tgts, spec))]
        results, grids, images = job.generate_batch(ctx, pal, reqs)
        singles = [_single(ctx, mats, thumbs, t, w, h, gw, gh, kw, i)
                   for i, (t, (w, h, gw, gh, kw)) in enumerate(zip(tgts, spec))]
    finally:
        ctx.set_scoring(capi.MG_SCORING_CLI)
    for i, (res, grid, image) in enumerate(singles):
        assert np.array_equal(grids[i], grid) and np.array_equal(images[i], image), i
        assert results[i].n_resets == res.n_resets
    w, h, gw, gh, kw = spec[0]
    cfg = job.JobConfig("b", w, h, 0, len(mats), 24, 0, gw, gh, kw.get("max_usage", 3), kw.get("weight", 0.25),
                        kw.get("strength", 0.4), kw.get("iterations", 1000), kw.get("chains", 1), TILE, TILE,
                        enable_optimization=kw.get("enable_opt", True), seed=20251203)
    ref = orc.generate(job.Inputs(cfg, tgts[0], mats, thumbs), threads=8, gui=True)
    assert np.array_equal(grids[0], ref["grid"]) and np.array_equal(images[0], ref["image"])
    pal.close()


def test_generate_from_png_files(ctx):
    """The path's file ends (image::open of main.rs:492/548, save of main.rs:672):
    the target and every material arrive as PNG files, decoded into pinned
    memory (target) and one packed buffer (materials, on several threads), and
    the mosaic leaves as a PNG file.  Grid and image equal the same job's from
    the raw arrays, and the file decodes back to the image."""
    import ctypes as C
    import dataclasses

    from mosaic_gpu import _capi as capi
    from mosaic_gpu import job, synth

    lib = capi.load()
    cfg = _small("recommended", target_w=480, target_h=360, n_materials=150, material_side=64, grid_w=20, grid_h=15,
                 tile_w=12, tile_h=12, iterations=300, chains=4)
    inp = job.make_inputs(cfg)
    ref_res, ref_grid, ref_image = job.generate(ctx, job.RequestHolder(inp))
    # materials: files -> one packed buffer at the original offsets
    files = [capi.png_encode(inp.mats.image(i), level=i % 2) for i in range(len(inp.mats))]
    buf = np.zeros_like(inp.mats.buf)
    n = len(files)
    data = (C.c_void_p * n)(*[C.cast(C.c_char_p(f), C.c_void_p) for f in files])
    sizes = (C.c_size_t * n)(*[len(f) for f in files])
    outs = (capi._u8p * n)(*[C.cast(buf.ctypes.data + int(o), capi._u8p) for o in inp.mats.off])
    strides = (C.c_int64 * n)(*[3 * int(w) for w in inp.mats.w])
    status = (C.c_int * n)()
    capi.check(lib.mg_png_decode_batch(data, sizes, n, outs, strides, 4, status))
    mats = synth.Materials(buf, inp.mats.off, inp.mats.w, inp.mats.h)
    # target: file -> pinned memory
    h, w = inp.target.shape[:2]
    addr = lib.mg_host_alloc(h * w * 3)
    assert addr
    try:
        target = np.ctypeslib.as_array(C.cast(addr, C.POINTER(C.c_uint8)), shape=(h * w * 3,)).reshape(h, w, 3)
        capi.png_decode(capi.png_encode(inp.target), out=target)
        decoded = dataclasses.replace(inp, target=target, mats=mats)
        res, grid, image = job.generate(ctx, job.RequestHolder(decoded))
        assert np.array_equal(grid, ref_grid) and np.array_equal(image, ref_image)
        assert res.best_chain == ref_res.best_chain
        assert np.array_equal(capi.png_decode(capi.png_encode(image)), image)
    finally:
        lib.mg_host_free(addr)

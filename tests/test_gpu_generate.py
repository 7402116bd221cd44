"""Whole generate_mosaic jobs on the GPU (through the C ABI) against the CPU oracle.

Bar: grid and annealed chain bit-exact, output pixels within 1 LSB (observed:
exact), palette size and fallback count equal.  The full recommended-settings
workload (3840x2880, 1500 materials, 80x60, 32 chains x 2000 iterations) is
compared at full size.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _compare(ctx, orc, cfg, threads=8):
    from mosaic_gpu import job

    inp = job.make_inputs(cfg)
    res, grid, image = job.generate(ctx, job.RequestHolder(inp))
    ref = orc.generate(inp, threads=threads)
    assert res.palette_size == ref["p"]
    assert res.n_resets == ref["n_resets"]
    assert np.array_equal(grid, ref["grid"])
    assert int(np.abs(image.astype(np.int16) - ref["image"].astype(np.int16)).max(initial=0)) <= 1
    assert res.best_chain == ref["best_chain"]
    assert np.float32(res.final_cost) == np.float32(ref["final_cost"])
    assert np.float32(res.initial_cost) == np.float32(ref["initial_cost"])
    return inp, res, grid, image, ref


def _small(name, **kw):
    from mosaic_gpu import job

    return job.scaled(job.WORKLOADS[name], **kw)


@pytest.mark.parametrize("cfg_kw", [
    dict(name="small", target_w=320, target_h=240, n_materials=120, material_side=32, grid_w=16, grid_h=12),
    dict(name="recommended", target_w=480, target_h=360, n_materials=150, material_side=64, grid_w=20, grid_h=15,
         tile_w=12, tile_h=12, iterations=500, chains=6),
    dict(name="large", target_w=716, target_h=536, n_materials=400, material_side=32, grid_w=35, grid_h=26,
         tile_w=8, tile_h=8, iterations=3000, chains=8, blobs=16),
])
def test_generate_scaled_workloads(ctx, orc, cfg_kw):
    name = cfg_kw.pop("name")
    _compare(ctx, orc, _small(name, **cfg_kw))


def test_generate_full_large_workload(ctx, orc):
    """The large single mosaic at full size: 7680x5760 target (128 blobs), 5000
    materials of 128x128, 179x134 = 23 986 cells of 42x42 pixels, max usage 8,
    64 chains x 100 000 iterations, 32x32 output tiles (5728x4288 image).  The
    grid and the winning chain bit-exact, every chain's final cost equal to the
    CPU replay of its Philox stream, pixels within 1 LSB."""
    import os

    from mosaic_gpu import job

    cfg = job.WORKLOADS["large"]
    inp, res, grid, image, ref = _compare(ctx, orc, cfg, threads=os.cpu_count() or 8)
    assert grid.shape == (134, 179) and image.shape == (4288, 5728, 3)
    assert res.palette_size == 5000
    assert np.float32(res.best_cost) == np.float32(ref["best_cost"])
    # every chain (not only the winner): the 64 chains run again from the greedy grid
    # through mg_optimize; each chain's initial, final and best cost equal the oracle's
    g, best, per, chain_grids = ctx.optimize(ref["pal_lab"], ref["greedy_grid"], cfg.iterations, chains=cfg.chains,
                                             seed=cfg.seed, stream=0)
    # no square material passes the 4:3 filter, so every one is kept in input order (main.rs:215-253):
    # palette indices are material indices
    assert best.best_chain == ref["best_chain"] and np.array_equal(g, ref["grid"])
    got = np.array([[r.initial_cost, r.final_cost, r.best_cost] for r in per], np.float32)
    assert np.array_equal(got.view(np.uint32), ref["chain_res"][:cfg.chains].view(np.uint32))


def test_generate_edge_cases(ctx, orc):
    # every material rejected (max_materials 0) -> nothing placed, black output
    cfg = _small("small", target_w=64, target_h=48, n_materials=10, material_side=16, grid_w=8, grid_h=6,
                 max_materials=0)
    from mosaic_gpu import job

    inp = job.make_inputs(cfg)
    holder = job.RequestHolder(inp)
    holder.req.max_materials = 0
    res, grid, image = job.generate(ctx, holder)
    assert res.palette_size == 0 and np.all(grid == -1) and not image.any()
    # one material only, optimisation on, colour on
    _compare(ctx, orc, _small("recommended", target_w=96, target_h=72, n_materials=3, material_side=16,
                              material_mode=0, grid_w=8, grid_h=6, tile_w=4, tile_h=4, iterations=50, chains=2))
    # optimisation off, weight 0
    _compare(ctx, orc, _small("small", target_w=200, target_h=150, n_materials=60, material_side=16, grid_w=10,
                              grid_h=10, weight=0.0))
    _compare(ctx, orc, _small("small", target_w=200, target_h=150, n_materials=60, material_side=16, grid_w=10,
                              grid_h=10, enable_optimization=False))
    # grid that does not divide the image (remainder ignored), max usage 1
    _compare(ctx, orc, _small("recommended", target_w=203, target_h=157, n_materials=90, material_side=20,
                              grid_w=11, grid_h=9, tile_w=0, tile_h=0, max_usage=1, iterations=300, chains=3))


def test_pinned_inputs_read_in_place(ctx, orc):
    """Inputs in pinned host memory are read by the kernels over the CPU-GPU link (no staging copies)."""
    from mosaic_gpu import _capi, job

    cfg = _small("recommended", target_w=480, target_h=360, n_materials=150, material_side=64, grid_w=20, grid_h=15,
                 tile_w=12, tile_h=12, iterations=500, chains=6)
    inp = job.make_inputs(cfg, allocator=_capi.load().mg_host_alloc)
    res, grid, image = job.generate(ctx, job.RequestHolder(inp))
    ref = orc.generate(inp, threads=8)
    assert np.array_equal(grid, ref["grid"]) and np.array_equal(image, ref["image"])
    assert np.float32(res.final_cost) == np.float32(ref["final_cost"])


def test_device_thumbnails_equal_host_thumbnails(ctx, orc):
    from mosaic_gpu import job

    cfg = _small("recommended", target_w=240, target_h=180, n_materials=60, material_side=40, grid_w=10, grid_h=9,
                 tile_w=9, tile_h=7, iterations=200, chains=2)
    from mosaic_gpu import _capi

    inp = job.make_inputs(cfg)  # host thumbnails: the area rule of the synthetic generator
    res_a, grid_a, img_a = job.generate(ctx, job.RequestHolder(inp))
    inp_dev = job.Inputs(cfg, inp.target, inp.mats, None)
    assert ctx.lib.mg_ctx_set_thumbnail_filter(ctx.h, _capi.MG_THUMB_AREA) == _capi.MG_OK
    try:
        res_b, grid_b, img_b = job.generate(ctx, job.RequestHolder(inp_dev))
    finally:
        ctx.lib.mg_ctx_set_thumbnail_filter(ctx.h, _capi.MG_THUMB_LANCZOS3)
    assert np.array_equal(grid_a, grid_b) and np.array_equal(img_a, img_b)


def test_plan_rerun_is_deterministic(ctx):
    from mosaic_gpu import job

    cfg = _small("recommended", target_w=480, target_h=360, n_materials=150, material_side=64, grid_w=20, grid_h=15,
                 tile_w=12, tile_h=12, iterations=500, chains=6)
    inp = job.make_inputs(cfg)
    plan = job.Plan(ctx, job.RequestHolder(inp))
    plan.run()
    r1, g1, i1 = plan.read()
    plan.run()
    r2, g2, i2 = plan.read()
    assert np.array_equal(g1, g2) and np.array_equal(i1, i2) and r1.final_cost == r2.final_cost
    ms = plan.stage_ms()
    assert len(ms) == 8 and ms[-1] > 0
    assert plan.launches() > 0
    plan.close()


def test_full_recommended_workload(ctx, orc):
    """Full-size recommended-settings mosaic, bit-exact against the oracle."""
    from mosaic_gpu import job

    inp, res, grid, image, ref = _compare(ctx, orc, job.WORKLOADS["recommended"], threads=16)
    assert grid.shape == (60, 80) and image.shape == (2880, 3840, 3)
    assert res.palette_size > 400 and res.best_chain >= 0


@pytest.mark.parametrize("grid_h", [15, 3])
def test_generate_into_pinned_buffers(ctx, grid_h):
    """mg_generate from and into pinned host memory -- inputs read in place, the
    image downloaded band by band while the next band is composited (grids of at
    least four tile rows) -- gives the same bytes as from and into pageable memory."""
    import ctypes as C

    from mosaic_gpu import _capi as capi
    from mosaic_gpu import job

    lib = capi.load()
    cfg = _small("recommended", target_w=480, target_h=24 * grid_h, n_materials=150, material_side=64, grid_w=20,
                 grid_h=grid_h, tile_w=16, tile_h=12, iterations=300, chains=4)
    inp = job.make_inputs(cfg)
    ref_res, ref_grid, ref_image = job.generate(ctx, job.RequestHolder(inp))
    pinned = job.make_inputs(cfg, allocator=lib.mg_host_alloc)
    holder = job.RequestHolder(pinned)
    n = int(np.prod(holder.out_shape()))
    buf = np.ctypeslib.as_array(C.cast(lib.mg_host_alloc(n), C.POINTER(C.c_uint8)), shape=(n,))
    image = buf.reshape(holder.out_shape())
    for _ in range(2):  # the second call reuses the context's job buffers and staging
        image[:] = 0
        res, grid, _ = job.generate(ctx, holder, image)
        assert np.array_equal(grid, ref_grid)
        assert np.array_equal(image, ref_image)
        assert res.best_chain == ref_res.best_chain and np.float32(res.final_cost) == np.float32(ref_res.final_cost)
    lib.mg_host_free(buf.ctypes.data)

"""Batches of uneven mosaics over one resident palette, against the one-mosaic path.

Every mosaic of a batch must equal mg_generate of the same request bit for bit
(grid, image, annealing summary) -- on the autotuning run, the graph-capturing
run and graph replays -- and the one-shot mg_generate_batch must equal the
resident batch.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TILE = 8


def _palette_inputs():
    from mosaic_gpu import synth

    mats = synth.materials(160, 24, 0, seed=77, stream=2)
    thumbs = synth.thumbnails(mats, TILE, TILE)
    return mats, thumbs


def _requests():
    """(w, h, gw, gh, settings): uneven sizes, optimiser on/off, weight 0, usage 1."""
    return [
        (320, 240, 40, 30, dict(chains=4, iterations=1500)),
        (96, 72, 12, 9, dict(chains=3, iterations=800, max_usage=1)),
        (200, 150, 25, 18, dict(enable_opt=False)),
        (160, 120, 20, 15, dict(weight=0.0, chains=2)),
        (480, 360, 60, 45, dict(chains=5, iterations=3000, strength=0.0)),
        (64, 48, 8, 6, dict(chains=2, iterations=300)),
        (240, 180, 30, 22, dict(chains=6, iterations=2000, max_usage=2)),
    ]


def _targets():
    from mosaic_gpu import synth

    return [synth.target(w, h, 5, seed=1000 + i, stream=7) for i, (w, h, _, _, _) in enumerate(_requests())]


def _single(ctx, mats, thumbs, tgt, w, h, gw, gh, kw, stream):
    """The same request through mg_generate."""
    from mosaic_gpu import job

    cfg = job.JobConfig("b", w, h, 0, len(mats), 24, 0, gw, gh, kw.get("max_usage", 3), kw.get("weight", 0.25),
                        kw.get("strength", 0.4), kw.get("iterations", 1000), kw.get("chains", 1), TILE, TILE,
                        enable_optimization=kw.get("enable_opt", True), seed=20251203)
    inp = job.Inputs(cfg, tgt, mats, thumbs)
    holder = job.RequestHolder(inp, stream=stream)
    return job.generate(ctx, holder)


def test_batch_equals_single_mosaic_path(ctx):
    from mosaic_gpu import job

    mats, thumbs = _palette_inputs()
    pal = job.Palette(ctx, mats, thumbs, TILE, TILE, target_aspect=4 / 3)
    assert pal.size == len(mats)
    tgts = _targets()
    reqs = [job.mosaic_request(t, w, h, gw, gh, stream=i, **kw)
            for i, (t, (w, h, gw, gh, kw)) in enumerate(zip(tgts, _requests()))]
    batch = job.Batch(ctx, pal, reqs)
    singles = [_single(ctx, mats, thumbs, t, w, h, gw, gh, kw, i)
               for i, (t, (w, h, gw, gh, kw)) in enumerate(zip(tgts, _requests()))]
    for run in range(3):  # tuning run, graph capture, graph replay
        batch.run()
        for i, (res, grid, image) in enumerate(singles):
            r, g, im = batch.read(i)
            assert np.array_equal(g, grid), (run, i)
            assert np.array_equal(im, image), (run, i)
            assert r.best_chain == res.best_chain and np.float32(r.final_cost) == np.float32(res.final_cost)
            assert r.n_resets == res.n_resets and r.palette_size == res.palette_size
    tune = batch.tuning()
    assert tune["cells_per_cta"] in (4, 8) and tune["nearest_chunk"] in (0, 1024, 2048, 4096)
    assert len(batch.stage_ms()) == 5 and batch.launches() > 0
    # one-shot batch from host buffers
    results, grids, images = job.generate_batch(ctx, pal, reqs)
    for i, (res, grid, image) in enumerate(singles):
        assert np.array_equal(grids[i], grid) and np.array_equal(images[i], image)
    # again, twice, into pinned buffers (one of them starting one byte past a
    # 16-byte boundary), the context's batch buffers reused
    import ctypes as C

    lib = ctx.lib
    outs, blocks = [], []
    for i, r in enumerate(reqs):
        nb = 3 * r.grid_w * r.grid_h * TILE * TILE
        blk = lib.mg_host_alloc(nb + 16)
        blocks.append(blk)
        off = 1 if i == 1 else 0
        im = np.ctypeslib.as_array(C.cast(blk + off, C.POINTER(C.c_uint8)), shape=(r.grid_h * TILE, r.grid_w * TILE, 3))
        im[:] = 7
        outs.append((np.zeros(r.grid_w * r.grid_h, np.int32), im))
    for rep in range(2):
        results2, grids2, images2 = job.generate_batch(ctx, pal, reqs, outputs=outs)
        for i, (res, grid, image) in enumerate(singles):
            assert np.array_equal(grids2[i], grid) and np.array_equal(images2[i], image), (rep, i)
            assert results2[i].best_chain == results[i].best_chain and results2[i].n_resets == results[i].n_resets
    for blk in blocks:
        lib.mg_host_free(blk)
    batch.close()
    pal.close()


def test_batch_against_oracle(ctx, orc):
    from mosaic_gpu import job

    mats, thumbs = _palette_inputs()
    pal = job.Palette(ctx, mats, thumbs, TILE, TILE, target_aspect=4 / 3)
    tgts = _targets()[:3]
    reqs = [job.mosaic_request(t, w, h, gw, gh, stream=i, **kw)
            for i, (t, (w, h, gw, gh, kw)) in enumerate(zip(tgts, _requests()[:3]))]
    results, grids, images = job.generate_batch(ctx, pal, reqs)
    for i, (w, h, gw, gh, kw) in enumerate(_requests()[:3]):
        cfg = job.JobConfig("b", w, h, 0, len(mats), 24, 0, gw, gh, kw.get("max_usage", 3), kw.get("weight", 0.25),
                            kw.get("strength", 0.4), kw.get("iterations", 1000), kw.get("chains", 1), TILE, TILE,
                            enable_optimization=kw.get("enable_opt", True), seed=20251203)
        ref = orc.generate(job.Inputs(cfg, tgts[i], mats, thumbs), threads=8, stream=i)  # request i: Philox stream i
        assert np.array_equal(grids[i], ref["grid"]), i
        assert np.array_equal(images[i], ref["image"]), i
        assert results[i].best_chain == ref["best_chain"] and results[i].final_cost == ref["final_cost"], i
    pal.close()


def test_palette_lab_and_similarity_match_oracle(ctx, orc):
    import ctypes as C

    from mosaic_gpu import job

    mats, thumbs = _palette_inputs()
    pal = job.Palette(ctx, mats, thumbs, TILE, TILE, target_aspect=4 / 3)
    lab = pal.lab()
    for i in range(0, len(mats), 17):
        assert np.array_equal(lab[i].view(np.uint32), orc.lab_mean_spec(mats.image(i)).view(np.uint32))
    sim = np.zeros((pal.size, pal.size), np.float32)
    assert ctx.lib.mg_palette_read_similarity(pal.h, sim.ctypes.data_as(C.POINTER(C.c_float))) == 0
    assert np.array_equal(sim.view(np.uint32), orc.similarity_full(lab).view(np.uint32))
    pal.close()


def test_many_mosaics_take_the_batch_walk_shape(ctx):
    """A batch of 40 mosaics walks in the three-CTA cluster shape (five SMs a
    mosaic would not fit them all at once), which settles windows that are not
    clear inside its common loop; over the dense 10 000-colour palette a fifth of
    the cells have such a window.  Every mosaic must equal the same request as a
    one-mosaic batch (the five-CTA shape, which settles them on its uncommon
    path), bit for bit, with and without annealing.  The one-shot
    mg_generate_batch of these 31 529 cells runs them as four groups on
    streams of their own, and must equal the batch too."""
    from mosaic_gpu import job

    specs, mats, thumbs = job.batched_workload(n=40, seed=424242, scale=0.5)
    pal = job.Palette(ctx, mats, thumbs, 32, 32, target_aspect=4 / 3)
    for iters in (0, 600):
        reqs = job.batched_requests(specs, iterations=iters, chains=2)
        batch = job.Batch(ctx, pal, reqs)
        batch.run()
        results, grids, images = job.generate_batch(ctx, pal, reqs)
        for i, r in enumerate(reqs):
            rb, gb, imb = batch.read(i)
            assert np.array_equal(grids[i], gb) and np.array_equal(images[i], imb), (iters, i)
            assert results[i].n_resets == rb.n_resets and results[i].best_chain == rb.best_chain
            assert np.float32(results[i].final_cost) == np.float32(rb.final_cost)
            single = job.Batch(ctx, pal, [r])
            single.run()
            r1, g1, im1 = single.read(0)
            r2, g2, im2 = batch.read(i)
            assert np.array_equal(g1, g2), (iters, i)
            assert np.array_equal(im1, im2), (iters, i)
            assert r1.n_resets == r2.n_resets and np.float32(r1.final_cost) == np.float32(r2.final_cost)
            single.close()
        batch.close()
    pal.close()

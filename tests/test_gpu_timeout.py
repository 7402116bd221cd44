"""A bounded wait that runs out, on the GPU: from the kernel's error word to the
call's status to a context that still works.

Every wait inside the library's kernels gives up after a fixed number of polls
instead of hanging (the greedy walker waiting for a scout's record, scouts
waiting for a placement, TMA copies on mbarriers).  mg_ctx_inject_walk_timeout
makes the next walk's scouts withhold their records and shortens the walker's
limit, so the walker's wait runs out: nothing faults, traps or hangs -- the
kernel returns, the call reports MG_ERR_TIMEOUT with its message, the walk's
grid is left empty, and the next call on the same context matches the oracle.
(The reference has no device waits; its own failure behaviour is fallback,
main.rs:199-206.)
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cfg():
    from mosaic_gpu import job

    # rows of 20 cells and a 150-material palette: the three-CTA walk
    return job.scaled(job.WORKLOADS["recommended"], target_w=480, target_h=360, n_materials=150, material_side=64,
                      grid_w=20, grid_h=15, tile_w=12, tile_h=12, iterations=500, chains=6)


def test_generate_reports_the_timeout_and_the_context_recovers(ctx, orc):
    from mosaic_gpu import _capi, job

    inp = job.make_inputs(_cfg())
    holder = job.RequestHolder(inp)
    assert ctx.lib.mg_ctx_inject_walk_timeout(ctx.h, 1) == _capi.MG_OK
    with pytest.raises(_capi.MosaicError) as e:
        job.generate(ctx, holder)
    assert e.value.code == _capi.MG_ERR_TIMEOUT
    assert b"bounded wait" in ctx.lib.mg_last_error()
    # same context, same (reused) job buffers: the next call is exact again, twice
    ref = orc.generate(inp, threads=8)
    for _ in range(2):
        res, grid, image = job.generate(ctx, holder)
        assert np.array_equal(grid, ref["grid"]) and np.array_equal(image, ref["image"])
        assert res.best_chain == ref["best_chain"] and res.final_cost == ref["final_cost"]


def test_plan_run_reports_the_timeout_once(ctx, orc):
    from mosaic_gpu import _capi, job

    inp = job.make_inputs(_cfg())
    plan = job.Plan(ctx, job.RequestHolder(inp))
    assert ctx.lib.mg_ctx_inject_walk_timeout(ctx.h, 1) == _capi.MG_OK
    plan.run()  # asynchronous: the status comes with the results
    with pytest.raises(_capi.MosaicError) as e:
        plan.read()
    assert e.value.code == _capi.MG_ERR_TIMEOUT
    plan.run()
    res, grid, image = plan.read()
    ref = orc.generate(inp, threads=8)
    assert np.array_equal(grid, ref["grid"]) and np.array_equal(image, ref["image"])
    plan.close()


def test_place_greedy_reports_the_timeout_with_an_empty_grid(ctx, orc):
    from mosaic_gpu import _capi

    rng = np.random.default_rng(5)
    pal = np.empty((300, 3), np.float32)
    pal[:, 0] = rng.uniform(0, 100, 300)
    pal[:, 1:] = rng.uniform(-80, 80, (300, 2))
    cells = pal[rng.integers(0, 300, 24 * 18)] + rng.normal(0, 2, (24 * 18, 3)).astype(np.float32)
    assert ctx.lib.mg_ctx_inject_walk_timeout(ctx.h, 1) == _capi.MG_OK
    with pytest.raises(_capi.MosaicError) as e:
        ctx.place_greedy(pal, cells, 24, 18, 3, 0.25)
    assert e.value.code == _capi.MG_ERR_TIMEOUT
    grid, resets = ctx.place_greedy(pal, cells, 24, 18, 3, 0.25)
    want, want_resets = orc.place_greedy(pal, cells, 24, 18, 3, 0.25)
    assert np.array_equal(grid, want) and resets == want_resets


def test_injection_arguments(ctx):
    from mosaic_gpu import _capi

    assert ctx.lib.mg_ctx_inject_walk_timeout(ctx.h, -1) == _capi.MG_ERR_ARG
    assert ctx.lib.mg_ctx_inject_walk_timeout(None, 1) == _capi.MG_ERR_ARG
    assert ctx.lib.mg_ctx_inject_walk_timeout(ctx.h, 0) == _capi.MG_OK

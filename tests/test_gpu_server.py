"""The request loop (mg_server): each result is the same alone and in the mix.

Requests of uneven sizes are served one at a time (alone: one request in the
server at a time) and all at once from several submitting threads (in the mix:
folded into shared batches over several slots); grids, images and annealing
summaries must be identical, and identical to mg_generate_batch of the same
request.  A request larger than the memory budget fails with MG_ERR_BUDGET
while the others complete.
"""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TILE = 8


def _setup(ctx):
    from mosaic_gpu import job, synth

    mats = synth.materials(200, 24, 0, seed=91, stream=2)
    thumbs = synth.thumbnails(mats, TILE, TILE)
    pal = job.Palette(ctx, mats, thumbs, TILE, TILE, target_aspect=4 / 3)
    gw, gh = job.served_grids(10, seed=5, lo=20, hi=2500)
    specs = []
    for i in range(len(gw)):
        w, h = int(gw[i]) * TILE, int(gh[i]) * TILE
        specs.append(job.MosaicSpec(w, h, int(gw[i]), int(gh[i]), synth.target(w, h, 6, 300 + i, 3)))
    reqs = [job.mosaic_request(s.target, s.w, s.h, s.gw, s.gh, max_usage=5, iterations=600 + 100 * i,
                               chains=1 + i % 4, stream=i, enable_opt=(i != 3))
            for i, s in enumerate(specs)]
    return pal, specs, reqs


def _outputs(specs):
    return ([np.zeros(s.gw * s.gh, np.int32) for s in specs],
            [np.zeros((s.gh * TILE, s.gw * TILE, 3), np.uint8) for s in specs])


def test_result_same_alone_and_in_the_mix(ctx):
    from mosaic_gpu import _capi as capi
    from mosaic_gpu import job

    pal, specs, reqs = _setup(ctx)
    ref_res, ref_grids, ref_imgs = job.generate_batch(ctx, pal, reqs)

    # alone: one request in the server at a time
    srv = job.Server(ctx, pal, slots=2, max_batch=8)
    grids, imgs = _outputs(specs)
    alone = []
    for i, r in enumerate(reqs):
        t = srv.submit(r, grids[i], imgs[i])
        st, res, lat = srv.wait(t)
        assert st == capi.MG_OK and lat > 0
        alone.append(res)
    for i in range(len(reqs)):
        assert np.array_equal(grids[i], ref_grids[i].ravel()), i
        assert np.array_equal(imgs[i], ref_imgs[i]), i
        assert alone[i].best_chain == ref_res[i].best_chain
        assert np.float32(alone[i].final_cost) == np.float32(ref_res[i].final_cost)
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["batches"] == len(reqs) and st["bytes_in_use"] == 0
    srv.close()

    # in the mix: three submitting threads, reversed order, small batches over three slots
    srv = job.Server(ctx, pal, slots=3, max_batch=3)
    grids2, imgs2 = _outputs(specs)
    tickets = {}
    lock = threading.Lock()

    def submit(ids):
        for i in ids:
            t = srv.submit(reqs[i], grids2[i], imgs2[i])
            with lock:
                tickets[i] = t

    order = list(range(len(reqs)))[::-1]
    threads = [threading.Thread(target=submit, args=(order[k::3],)) for k in range(3)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    mixed = {}
    for i, t in tickets.items():
        st, res, _ = srv.wait(t)
        assert st == capi.MG_OK
        mixed[i] = res
    for i in range(len(reqs)):
        assert np.array_equal(grids2[i], grids[i]), i
        assert np.array_equal(imgs2[i], imgs[i]), i
        assert mixed[i].best_chain == alone[i].best_chain
        assert np.float32(mixed[i].final_cost) == np.float32(alone[i].final_cost)
        assert mixed[i].n_resets == alone[i].n_resets
    st = srv.stats()
    assert st["submitted"] == st["completed"] == len(reqs) and st["rejected"] == 0
    assert st["batches"] < len(reqs)  # requests were folded into shared batches
    srv.close()
    pal.close()


def test_budget_rejects_oversized_request(ctx):
    from mosaic_gpu import _capi as capi
    from mosaic_gpu import job

    pal, specs, reqs = _setup(ctx)
    big = int(np.argmax([s.gw * s.gh for s in specs]))
    small = int(np.argmin([s.gw * s.gh for s in specs]))
    probe = job.Server(ctx, pal, slots=1, max_batch=1)
    b_small, b_big = probe.request_bytes(reqs[small]), probe.request_bytes(reqs[big])
    probe.close()
    assert 0 < b_small < b_big
    # a budget the small request fits and the big one never can
    budget = b_small + (b_big - b_small) // 2
    srv = job.Server(ctx, pal, slots=2, max_batch=4, memory_budget_bytes=budget)
    grids, imgs = _outputs(specs)
    tb = srv.submit(reqs[big], grids[big], imgs[big])
    ts = srv.submit(reqs[small], grids[small], imgs[small])
    assert srv.wait(tb)[0] == capi.MG_ERR_BUDGET
    assert srv.wait(ts)[0] == capi.MG_OK
    ref_res, ref_grids, ref_imgs = job.generate_batch(ctx, pal, [reqs[small]])
    assert np.array_equal(grids[small], ref_grids[0].ravel()) and np.array_equal(imgs[small], ref_imgs[0])
    st = srv.stats()
    assert st["rejected"] == 1 and st["completed"] == 1 and st["peak_bytes_in_use"] <= budget
    srv.close()
    pal.close()


def test_poll_and_close_with_work_queued(ctx):
    from mosaic_gpu import _capi as capi
    from mosaic_gpu import job

    pal, specs, reqs = _setup(ctx)
    srv = job.Server(ctx, pal, slots=1, max_batch=2)
    grids, imgs = _outputs(specs)
    tickets = [srv.submit(r, grids[i], imgs[i]) for i, r in enumerate(reqs)]
    first = None
    deadline = time.monotonic() + 60.0
    while first is None and time.monotonic() < deadline:
        first = srv.poll(tickets[0])
        time.sleep(0.001)
    assert first is not None and first[0] == capi.MG_OK
    srv.close()  # finishes the queued requests before stopping
    ref_res, ref_grids, ref_imgs = job.generate_batch(ctx, pal, reqs)
    for i in range(len(reqs)):
        assert np.array_equal(grids[i], ref_grids[i].ravel()), i
    pal.close()

"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py from
the oracle): reduced versions of the five measured configurations.

CPU: the oracle reproduces every fixture bit for bit from regenerated inputs
(a regression pin of the oracle itself, on x86 here and Arm on the GPU machine).
GPU: the CUDA path -- mg_generate for the single mosaics, a resident palette
with one batch for the batched stream, the request loop for the served stream
-- reproduces the same grids, images and annealing summaries bit for bit.
"""
import hashlib
import json
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

NAMES = ["small", "recommended", "large", "batched", "served"]


def _load(name):
    z = np.load(GOLDEN / f"{name}.npz")
    return z, int(z["count"])


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _same_f32(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_golden(built, orc, name):
    import make_golden as mg

    z, count = _load(name)
    cases = mg.cases(name)
    assert len(cases) == count
    for j, (cfg, inp, stream) in enumerate(cases):
        assert str(z[f"{j}/target_sha"]) == _sha(inp.target), "synthetic generator changed"
        assert str(z[f"{j}/materials_sha"]) == _sha(inp.mats.buf), "synthetic generator changed"
        rec = mg.oracle_record(cfg, inp, stream, orc)
        for key in ("grid", "greedy_grid", "scalars"):
            assert np.array_equal(rec[key], z[f"{j}/{key}"]), (name, j, key)
        for key in ("cell_lab", "pal_lab", "chain_res", "costs"):
            assert _same_f32(rec[key], z[f"{j}/{key}"]), (name, j, key)
        assert str(rec["image_sha"]) == str(z[f"{j}/image_sha"]), (name, j)


def _check(z, j, grid, image, res):
    assert np.array_equal(np.asarray(grid).reshape(z[f"{j}/grid"].shape), z[f"{j}/grid"]), j
    assert _sha(image) == str(z[f"{j}/image_sha"]), j
    p, n_resets, best_chain = (int(v) for v in z[f"{j}/scalars"])
    assert res.palette_size == p and res.n_resets == n_resets and res.best_chain == best_chain, j
    costs = z[f"{j}/costs"]
    assert _same_f32([res.initial_cost, res.final_cost, res.best_cost], costs), j


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["small", "recommended", "large"])
def test_cuda_single_matches_golden(ctx, name):
    import make_golden as mg
    from mosaic_gpu import job

    z, count = _load(name)
    for j, (cfg, inp, stream) in enumerate(mg.cases(name)):
        res, grid, image = job.generate(ctx, job.RequestHolder(inp, stream=stream))
        _check(z, j, grid, image, res)


def _stream_requests(name):
    import make_golden as mg
    from mosaic_gpu import job

    cases = mg.cases(name)
    cfg0, inp0, _ = cases[0]
    reqs = [job.mosaic_request(inp.target, c.target_w, c.target_h, c.grid_w, c.grid_h, max_usage=c.max_usage,
                               weight=c.weight, strength=c.color_strength, iterations=c.iterations,
                               chains=c.chains, seed=c.seed, stream=s) for c, inp, s in cases]
    return cases, inp0, reqs


@pytest.mark.gpu
def test_cuda_batch_matches_golden(ctx):
    from mosaic_gpu import job

    z, count = _load("batched")
    cases, inp0, reqs = _stream_requests("batched")
    pal = job.Palette(ctx, inp0.mats, inp0.thumbs, 8, 8, target_aspect=4 / 3)
    batch = job.Batch(ctx, pal, reqs)
    for run in range(2):  # tuning run, then the captured graph
        batch.run()
        for j in range(count):
            res, grid, image = batch.read(j)
            _check(z, j, grid, image, res)
    batch.close()
    pal.close()


@pytest.mark.gpu
def test_cuda_server_matches_golden(ctx):
    from mosaic_gpu import _capi as capi
    from mosaic_gpu import job

    z, count = _load("served")
    cases, inp0, reqs = _stream_requests("served")
    pal = job.Palette(ctx, inp0.mats, inp0.thumbs, 8, 8, target_aspect=4 / 3)
    srv = job.Server(ctx, pal, slots=2, max_batch=3)
    outs = [(np.zeros(c.grid_w * c.grid_h, np.int32), np.zeros((c.grid_h * 8, c.grid_w * 8, 3), np.uint8))
            for c, _, _ in cases]
    tickets = [srv.submit(r, g, im) for r, (g, im) in zip(reqs, outs)]
    for j, t in enumerate(tickets):
        st, res, _ = srv.wait(t)
        assert st == capi.MG_OK
        _check(z, j, outs[j][0], outs[j][1], res)
    srv.close()
    pal.close()

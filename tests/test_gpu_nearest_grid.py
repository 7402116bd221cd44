"""The bucket-grid k-nearest search (k_nearest_grid.cu) against the oracle's
brute-force nearest_n (kiddo nearest_n of main.rs:145-151 restated): the same
indices and distance bits, forced on (MG_NEAREST_GRID) at every palette size,
on palettes built to stress the pruning -- clusters, duplicates (ties to the
lowest index), a flat axis, a single colour, queries far outside the palette's
bounding box -- and through mg_generate and resident-palette batches.
"""
import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gctx(built):
    from mosaic_gpu import _capi as capi

    c = capi.Context(0)
    yield c
    c.close()


def _uniform(rng, n):
    lab = np.empty((n, 3), np.float32)
    lab[:, 0] = rng.uniform(0, 100, n)
    lab[:, 1:] = rng.uniform(-90, 90, (n, 2))
    return lab


def _clustered(rng, n):
    centers = _uniform(rng, 6)
    lab = centers[rng.integers(0, 6, n)] + rng.normal(0, 1.5, (n, 3)).astype(np.float32)
    return lab.astype(np.float32)


def _palette(kind, rng, n):
    if kind == "uniform":
        return _uniform(rng, n)
    if kind == "clustered":
        return _clustered(rng, n)
    if kind == "duplicates":  # every colour ten times: ties everywhere
        base = _uniform(rng, max(1, n // 10))
        return np.repeat(base, 10, axis=0)[:n].copy()
    if kind == "flat_l":  # one axis without extent
        lab = _uniform(rng, n)
        lab[:, 0] = 50.0
        return lab
    if kind == "one_colour":
        return np.tile(np.array([[40.0, 10.0, -20.0]], np.float32), (n, 1))
    if kind == "integer_grid":  # entries on bucket boundaries
        v = rng.integers(-8, 9, (n, 3)).astype(np.float32) * 8.0
        v[:, 0] = np.abs(v[:, 0])
        return v
    raise ValueError(kind)


def _queries(rng, pal, nq):
    q = _uniform(rng, nq)
    q[: nq // 4] = pal[rng.integers(0, len(pal), nq // 4)]  # exact hits
    q[nq // 4: nq // 2] += rng.normal(0, 0.5, (nq // 2 - nq // 4, 3)).astype(np.float32)
    q[-3:] = np.array([[300.0, 300.0, 300.0], [-250.0, 0.0, 0.0], [50.0, -400.0, 400.0]], np.float32)
    return q


def _check(ctx, orc, pal, q, k, method):
    from mosaic_gpu import _capi as capi

    ctx.set_nearest_method(method)
    try:
        idx, dist = ctx.nearest_n(pal, q, k)
    finally:
        ctx.set_nearest_method(capi.MG_NEAREST_AUTO)
    ridx, rdist = orc.nearest_n(pal, q, k)
    kk = min(k, len(pal))
    assert np.array_equal(idx[:, :kk], ridx)
    assert np.array_equal(dist[:, :kk].view(np.uint32), rdist.view(np.uint32))
    if kk < k:
        assert np.all(idx[:, kk:] == 0xFFFFFFFF) and np.all(np.isinf(dist[:, kk:]))


@pytest.mark.parametrize("kind", ["uniform", "clustered", "duplicates", "flat_l", "one_colour", "integer_grid"])
@pytest.mark.parametrize("p,k", [(1, 1), (37, 100), (300, 100), (2500, 100), (12000, 100), (12000, 7)])
def test_grid_matches_oracle(gctx, orc, kind, p, k):
    from mosaic_gpu import _capi as capi

    rng = np.random.default_rng(zlib.crc32(f"{kind}/{p}/{k}".encode()))
    pal = _palette(kind, rng, p)
    q = _queries(rng, pal, 96)
    _check(gctx, orc, pal, q, k, capi.MG_NEAREST_GRID)


def test_grid_equals_scan_large(gctx):
    """A 60 000-colour palette: grid and scan agree bit for bit on 4000 queries."""
    from mosaic_gpu import _capi as capi

    rng = np.random.default_rng(11)
    pal = np.concatenate([_uniform(rng, 40000), _clustered(rng, 20000)])
    q = _queries(rng, pal, 4000)
    out = []
    for m in (capi.MG_NEAREST_SCAN, capi.MG_NEAREST_GRID):
        gctx.set_nearest_method(m)
        out.append(gctx.nearest_n(pal, q, 100))
    gctx.set_nearest_method(capi.MG_NEAREST_AUTO)
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1].view(np.uint32), out[1][1].view(np.uint32))


def test_method_argument_checked(gctx):
    from mosaic_gpu import _capi as capi

    with pytest.raises(capi.MosaicError):
        gctx.set_nearest_method(7)


def test_generate_and_batch_through_grid(built):
    """The golden recommended and batched fixtures, reproduced with the grid
    forced on (their palettes are below the automatic threshold)."""
    import sys
    from pathlib import Path

    from mosaic_gpu import _capi as capi
    from mosaic_gpu import job

    golden = Path(__file__).resolve().parent / "golden"
    sys.path.insert(0, str(golden))
    import make_golden as mg
    from test_golden import _check as check_fixture
    from test_golden import _load, _stream_requests

    c = capi.Context(0)
    try:
        c.set_nearest_method(capi.MG_NEAREST_GRID)
        z, _ = _load("recommended")
        for j, (cfg, inp, stream) in enumerate(mg.cases("recommended")):
            res, grid, image = job.generate(c, job.RequestHolder(inp, stream=stream))
            check_fixture(z, j, grid, image, res)
        z, count = _load("batched")
        cases, inp0, reqs = _stream_requests("batched")
        pal = job.Palette(c, inp0.mats, inp0.thumbs, 8, 8, target_aspect=4 / 3)
        batch = job.Batch(c, pal, reqs)
        batch.run()
        assert batch.tuning()["nearest_chunk"] == 0
        for j in range(count):
            res, grid, image = batch.read(j)
            check_fixture(z, j, grid, image, res)
        batch.close()
        pal.close()
    finally:
        c.close()

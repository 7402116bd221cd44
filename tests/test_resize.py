"""Lanczos3 thumbnails (main.rs:710-738 resize_image: fast_image_resize's
default Lanczos3 convolution, restated from the published resampler it
follows).

CPU: the oracle's restatement against the reference's own resize tests
(main.rs:891-921: a red image stays red, sizes as asked), against an
independent float64 numpy version of the same resampler (within 1 LSB: the
fixed-point weights round differently), constant images, and identity at the
same size.
GPU: mg_resize, and whole jobs, palettes and batches whose thumbnails are made
on the device, bit for bit against the oracle.
"""
import numpy as np
import pytest


def _lanczos3(x):
    x = np.asarray(x, np.float64)
    out = np.where(x == 0, 1.0, 0.0)
    nz = x != 0
    a = np.pi * x[nz]
    out[nz] = (np.sin(a) / a) * (np.sin(a / 3) / (a / 3))
    return np.where((x >= -3) & (x < 3), out, 0.0)


def _weights_float(n_in, n_out):
    """The resampling matrix (n_out x n_in) of one dimension, float64."""
    scale = n_in / n_out
    fs = max(scale, 1.0)
    support = 3.0 * fs
    W = np.zeros((n_out, n_in))
    for o in range(n_out):
        centre = (o + 0.5) * scale
        lo, hi = max(0, int(centre - support + 0.5)), min(n_in, int(centre + support + 0.5))
        i = np.arange(lo, hi)
        w = _lanczos3((i - centre + 0.5) / fs)
        W[o, lo:hi] = w / w.sum() if w.sum() != 0 else w
    return W


def _resize_float(img, dw, dh):
    h, w = img.shape[:2]
    x = img.astype(np.float64)
    if dw != w:
        x = np.einsum("ow,hwc->hoc", _weights_float(w, dw), x)
        x = np.clip(np.floor(x + 0.5), 0, 255)  # 8-bit intermediate
    if dh != h:
        x = np.einsum("oh,hwc->owc", _weights_float(h, dh), x)
    return np.clip(np.floor(x + 0.5), 0, 255).astype(np.uint8)


SIZES = [((100, 100), (50, 50)), ((100, 100), (200, 100)), ((256, 192), (48, 48)), ((192, 256), (48, 48)),
         ((128, 128), (32, 32)), ((128, 128), (25, 25)), ((37, 53), (11, 7)), ((5, 3), (17, 9)), ((1, 1), (4, 3)),
         ((300, 7), (300, 2)), ((64, 64), (64, 64)), ((1000, 40), (9, 40))]


def _image(rng, w, h, kind):
    if kind == "noise":
        return rng.integers(0, 256, (h, w, 3)).astype(np.uint8)
    y, x = np.mgrid[0:h, 0:w]
    return np.stack([(x * 255 // max(w - 1, 1)), (y * 255 // max(h - 1, 1)), ((x + y) * 7) % 256], -1).astype(np.uint8)


def test_reference_resize_known_answers(orc):
    """main.rs:891-921: a red 100x100 image resized to 50x50 stays red (R > 200,
    G and B < 50); 200x100 output keeps the asked size."""
    red = np.zeros((100, 100, 3), np.uint8)
    red[..., 0] = 255
    out = orc.resize_lanczos3(red, 50, 50)
    assert out.shape == (50, 50, 3) and out[25, 25, 0] > 200 and out[25, 25, 1] < 50 and out[25, 25, 2] < 50
    green = np.zeros((100, 100, 3), np.uint8)
    green[..., 1] = 255
    assert orc.resize_lanczos3(green, 200, 100).shape == (100, 200, 3)


@pytest.mark.parametrize("src,dst", SIZES)
def test_oracle_resize_against_float_restatement(orc, src, dst):
    rng = np.random.default_rng(src[0] * 31 + dst[0])
    for kind in ("noise", "ramp"):
        img = _image(rng, src[0], src[1], kind)
        got = orc.resize_lanczos3(img, *dst)
        want = _resize_float(img, *dst)
        assert np.abs(got.astype(np.int16) - want.astype(np.int16)).max() <= 1, (src, dst, kind)
        for v in (0, 1, 128, 255):  # a constant stays constant
            c = np.full((src[1], src[0], 3), v, np.uint8)
            assert np.all(orc.resize_lanczos3(c, *dst) == v)
    same = _image(rng, 23, 19, "noise")
    assert np.array_equal(orc.resize_lanczos3(same, 23, 19), same)


@pytest.mark.gpu
@pytest.mark.parametrize("src,dst", SIZES)
def test_gpu_resize_bit_exact(ctx, orc, src, dst):
    rng = np.random.default_rng(src[1] * 17 + dst[1])
    for kind in ("noise", "ramp"):
        img = _image(rng, src[0], src[1], kind)
        assert np.array_equal(ctx.resize(img, *dst), orc.resize_lanczos3(img, *dst)), (src, dst, kind)
    big = np.asarray(_image(rng, 900, 700, "noise")[100:600, 50:850])  # a view: row stride above 3 * width
    assert np.array_equal(ctx.resize(big, 31, 23), orc.resize_lanczos3(np.ascontiguousarray(big), 31, 23))


def _oracle_thumbs(orc, mats, tw, th):
    return np.stack([orc.resize_lanczos3(mats.image(i), tw, th) for i in range(len(mats))])


@pytest.mark.gpu
def test_generate_with_device_lanczos3_thumbnails(ctx, orc):
    """Thumbnails left to the library (mg_request.thumbnails NULL): the job
    equals the oracle's given the oracle's Lanczos3 thumbnails -- materials of
    three aspects (256x192, 192x256, 256x256), 48x48 and 12x12 tiles."""
    from mosaic_gpu import job

    for tile, n, side in ((48, 60, 256), (12, 90, 64)):
        cfg = job.scaled(job.WORKLOADS["recommended"], target_w=480, target_h=360, n_materials=n,
                         material_side=side, grid_w=10, grid_h=9, tile_w=tile, tile_h=tile, iterations=300, chains=3)
        inp = job.make_inputs(cfg)
        thumbs = _oracle_thumbs(orc, inp.mats, tile, tile)
        res, grid, image = job.generate(ctx, job.RequestHolder(job.Inputs(cfg, inp.target, inp.mats, None)))
        ref = orc.generate(job.Inputs(cfg, inp.target, inp.mats, thumbs), threads=8)
        assert np.array_equal(grid, ref["grid"]) and np.array_equal(image, ref["image"]), tile


@pytest.mark.gpu
def test_palette_with_device_lanczos3_thumbnails(ctx, orc):
    """A resident palette whose thumbnails are made on the device gives the same
    batch as one given the oracle's thumbnails."""
    from mosaic_gpu import job, synth

    mats = synth.materials(80, 48, 0, 99, 2)
    thumbs = _oracle_thumbs(orc, mats, 8, 8)
    reqs_t = [synth.target(160, 120, 4, 7, 100 + i) for i in range(3)]
    reqs = [job.mosaic_request(t, 160, 120, 20, 15, stream=i, iterations=200, chains=2) for i, t in enumerate(reqs_t)]
    out = []
    for th in (None, thumbs):
        pal = job.Palette(ctx, mats, th, 8, 8, target_aspect=4 / 3)
        _, grids, images = job.generate_batch(ctx, pal, reqs)
        out.append((grids, images))
        pal.close()
    for (g0, i0), (g1, i1) in zip(zip(*out[0]), zip(*out[1])):
        assert np.array_equal(g0, g1) and np.array_equal(i0, i1)

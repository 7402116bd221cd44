"""mg_cells_lab_noalloc: the cell reduction for callers that cannot allocate device memory.

A caller such as a serving process whose device memory is owned by its own pool
allocator passes device buffers it already holds; the entry point allocates
nothing and keeps its per-cell sums in a fixed array inside the library.  This
test plays that caller: the buffers come from torch's allocator, the call goes
through the C ABI, and the results must equal the allocating entry point
(mg_cells_lab) bit for bit on two calls in a row -- the second call must not
see the first call's sums, since the array is shared and kept between calls.
The file is collected after the stage, job, batch and server tests so that a failure here leaves them run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, torch, img, gw, gh):
    h, w = img.shape[:2]
    d_img = torch.from_numpy(np.ascontiguousarray(img)).cuda()
    n = gw * gh
    d_lab = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    d_rgb = torch.empty((n, 4), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.mg_cells_lab_noalloc(C.c_void_p(d_img.data_ptr()), w, h, 3 * w, gw, gh, C.c_void_p(d_lab.data_ptr()),
                                  C.c_void_p(d_rgb.data_ptr()), C.c_void_p(stream))
    torch.cuda.synchronize()
    return rc, d_lab.cpu().numpy(), d_rgb.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice(ctx):
    torch = pytest.importorskip("torch")
    from mosaic_gpu import _capi, synth

    lib = _capi.load()
    img_a = synth.target(640, 480, 5, seed=1234, stream=3)
    img_b = synth.target(640, 480, 9, seed=98765, stream=4)
    # 16x16-pixel cells are one warp each; 160x160-pixel cells (25 600 pixels)
    # are split over several warps whose sums meet in the library's array
    for gw, gh in ((40, 30), (4, 3)):
        for img in (img_a, img_b):  # two calls in a row, different inputs
            rc, lab4, rgb4 = _noalloc(lib, torch, img, gw, gh)
            assert rc == _capi.MG_OK, lib.mg_last_error()
            ref_lab, ref_rgb = ctx.cells_lab(img, gw, gh)
            assert np.array_equal(lab4[:, :3].view(np.uint32), ref_lab.view(np.uint32))
            assert np.array_equal(rgb4[:, :3], ref_rgb)


def test_noalloc_rejects_grids_beyond_its_limit(ctx):
    torch = pytest.importorskip("torch")
    from mosaic_gpu import _capi

    lib = _capi.load()
    img = np.zeros((200, 400, 3), np.uint8)
    rc, _, _ = _noalloc(lib, torch, img, 400, 100)  # 40000 cells > 32768
    assert rc == _capi.MG_ERR_ARG
    assert b"32768" in lib.mg_last_error()

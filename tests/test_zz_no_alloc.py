"""crt_render_tile_noalloc: the allocation-free render entry point.

It exists for callers that may not allocate device memory while rendering
(a host application that owns all device memory through its own pool, or a
loop that cannot afford cudaMalloc's latency and implicit synchronisation).
The caller allocates the accumulator; the library's paths in flight live in
a fixed scratch array.  These tests call it through the C ABI twice in a row
and require the same sums as crt_render_pass (bit for bit, the tolerance of
every render-equality test here), no change in free device memory across
calls, and a clear error for requests beyond the scratch capacity.

The file name sorts last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from cudart_gb300 import GB300Renderer, GB300Scene, _lib, camera_from_json, scenes

pytestmark = pytest.mark.gpu


def _tile_call(torch, g, cam, sc, acc, pixel0, count, spp0, nspp, max_depth, flags=0):
    opts = _lib.RenderOptions()
    _lib.load().crt_render_options_default(C.byref(opts))
    opts.max_depth = max_depth
    opts.flags = flags
    stream = torch.cuda.current_stream().cuda_stream
    return _lib.load().crt_render_tile_noalloc(g.handle, C.byref(cam), sc.width, sc.height,
                                               C.byref(opts), pixel0, count, spp0, nspp,
                                               acc.data_ptr(), stream)


def _reference(g, sc, spp, depth, mode="wavefront"):
    r = GB300Renderer(g, sc.width, sc.height, spp, max_depth=depth, mode=mode)
    r.render(spp)
    return r.accum()


def test_two_calls_match_render_pass(cuda):
    torch = cuda
    sc = scenes.cornell_box(width=96, height=64)
    g = GB300Scene(sc)
    cam = camera_from_json(sc.camera, sc.width, sc.height)
    npix = sc.width * sc.height
    acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    # samples 0-3, then 4-7, of the whole image: two calls in a row
    assert _tile_call(torch, g, cam, sc, acc, 0, npix, 0, 4, 5) == 0
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    assert _tile_call(torch, g, cam, sc, acc, 0, npix, 4, 4, 5) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    got = acc[:, :3].cpu().numpy()
    assert np.array_equal(got, _reference(g, sc, 8, 5, "wavefront"))
    assert np.array_equal(got, _reference(g, sc, 8, 5, "megakernel"))


def test_tiles_cover_a_larger_image(cuda):
    torch = cuda
    sc = scenes.mixed_mid(width=320, height=180, subdiv=3)
    g = GB300Scene(sc)
    cam = camera_from_json(sc.camera, sc.width, sc.height)
    npix = sc.width * sc.height
    acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
    nspp, tile = 8, _lib.NOALLOC_MAX_PATHS // 8
    for spp0 in (0, 8):
        for p0 in range(0, npix, tile):
            assert _tile_call(torch, g, cam, sc, acc, p0, min(tile, npix - p0), spp0, nspp, 8) == 0
    torch.cuda.synchronize()
    assert np.array_equal(acc[:, :3].cpu().numpy(), _reference(g, sc, 16, 8))


def test_requests_beyond_the_scratch_are_rejected(cuda):
    torch = cuda
    sc = scenes.cornell_box(width=512, height=512)
    g = GB300Scene(sc)
    cam = camera_from_json(sc.camera, sc.width, sc.height)
    acc = torch.zeros((512 * 512, 4), dtype=torch.float32, device="cuda")
    st = _tile_call(torch, g, cam, sc, acc, 0, 512 * 512, 0, 1, 5)
    assert st == 6                                   # CRT_ERR_LIMIT
    assert b"CRT_NOALLOC_MAX_PATHS" in _lib.load().crt_last_error()
    torch.cuda.synchronize()
    assert float(acc.abs().sum()) == 0.0             # nothing was launched

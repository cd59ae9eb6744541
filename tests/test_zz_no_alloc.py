"""crt_render_tile_noalloc: the allocation-free render entry point.

It exists for callers that may not allocate device memory while rendering
(a host application that owns all device memory through its own pool, or a
loop that cannot afford cudaMalloc's latency and implicit synchronisation).
The caller allocates the accumulator; the library's paths in flight live in
a fixed scratch array.  These tests call it through the C ABI twice in a row
and require the same sums as crt_render_pass (bit for bit, the tolerance of
every render-equality test here), no change in free device memory across
calls, and a clear error for requests beyond the scratch capacity.  The
launch options that change which kernels run on the scratch (node format,
lane refill, split leaf, octant queues, which this entry point ignores) are
each compared with crt_render_pass made with the same options, on a stream
other than torch's.  A traversal cut short by the scene's visit limit is
visible afterwards through crt_scene_errors, which allocates nothing either.

The file name sorts last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from cudart_gb300 import GB300Renderer, GB300Scene, _lib, camera_from_json, scenes

pytestmark = pytest.mark.gpu


def _tile_call(torch, g, cam, sc, acc, pixel0, count, spp0, nspp, max_depth, flags=0,
               node_format=-1, stream=None):
    opts = _lib.RenderOptions()
    _lib.load().crt_render_options_default(C.byref(opts))
    opts.max_depth = max_depth
    opts.flags = flags
    opts.node_format = node_format
    if stream is None:
        stream = torch.cuda.current_stream().cuda_stream
    return _lib.load().crt_render_tile_noalloc(g.handle, C.byref(cam), sc.width, sc.height,
                                               C.byref(opts), pixel0, count, spp0, nspp,
                                               acc.data_ptr(), stream)


def _reference(g, sc, spp, depth, mode="wavefront", **kw):
    r = GB300Renderer(g, sc.width, sc.height, spp, max_depth=depth, mode=mode, **kw)
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


@pytest.mark.parametrize("node_format", ["q8", "f32"])
@pytest.mark.parametrize("flags", [_lib.FLAG_LANE_REFILL, _lib.FLAG_SPLIT_LEAF, _lib.FLAG_OCTANT_QUEUES])
def test_options_match_render_pass_on_a_side_stream(cuda, node_format, flags):
    torch = cuda
    sc = scenes.mixed_mid(width=64, height=48, subdiv=2)
    g = GB300Scene(sc)
    cam = camera_from_json(sc.camera, sc.width, sc.height)
    npix = sc.width * sc.height
    fmt = _lib.NODES_F32 if node_format == "f32" else _lib.NODES_Q8
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        acc = torch.zeros((npix, 4), dtype=torch.float32, device="cuda")
        for spp0 in (0, 8):
            assert _tile_call(torch, g, cam, sc, acc, 0, npix, spp0, 8, 8, flags=flags,
                              node_format=fmt, stream=side.cuda_stream) == 0
    side.synchronize()
    ref = _reference(g, sc, 16, 8, node_format=node_format, flags=flags)
    assert np.array_equal(acc[:, :3].cpu().numpy(), ref)


def test_cut_short_traversals_are_visible_through_the_error_word(cuda):
    torch = cuda
    sc = scenes.cornell_box(width=64, height=64)
    g = GB300Scene(sc)
    cam = camera_from_json(sc.camera, sc.width, sc.height)
    acc = torch.zeros((64 * 64, 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert g.errors(stream) == 0
    g.set_visit_limit(2)                  # root + one child: most rays run out
    try:
        assert _tile_call(torch, g, cam, sc, acc, 0, 64 * 64, 0, 2, 5) == 0   # queued, not checked
        assert g.errors(stream) & _lib.SCENE_ERR_WATCHDOG
    finally:
        g.set_visit_limit(0)
        g.clear_errors()
    assert g.errors(stream) == 0
    acc.zero_()
    assert _tile_call(torch, g, cam, sc, acc, 0, 64 * 64, 0, 2, 5) == 0
    assert g.errors(stream) == 0
    assert np.array_equal(acc[:, :3].cpu().numpy(), _reference(g, sc, 2, 5))


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

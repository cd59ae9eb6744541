"""Render parity on the GPU: the megakernel and the wavefront form against
the oracle's restatement of samplePixel (renderer.cu:119-262) on the same
Philox streams, and against each other."""
import numpy as np
import pytest

import oracle
from cudart_gb300 import GB300Renderer, GB300Scene, scenes

pytestmark = pytest.mark.gpu


def _render(sc, spp, depth, mode, seed=1234, **kw):
    g = GB300Scene(sc)
    r = GB300Renderer(g, sc.width, sc.height, spp, max_depth=depth, seed=seed, mode=mode, **kw)
    r.render()
    r.synchronize()
    return r


def _oracle(sc, spp, depth, seed=1234):
    o = oracle.OracleScene(sc)
    cam = oracle.make_camera(sc.camera, sc.width, sc.height)
    return o.render(cam, seed=seed, spp=spp, max_depth=depth)


@pytest.mark.parametrize("mode", ["megakernel", "wavefront"])
def test_cornell_same_stream(cuda, mode):
    sc = scenes.cornell_box(width=96, height=96)
    r = _render(sc, 8, 5, mode, wave_paths=1 << 15)
    acc = r.accum()
    ref, _, _ = _oracle(sc, 8, 5)
    rel = float(np.sum((acc - ref) ** 2) / np.sum(ref ** 2))
    assert rel < 1e-4
    same = np.mean(np.all(acc == ref, axis=1))
    assert same > 0.5, f"only {same:.3f} of pixels bit-exact"


def test_wavefront_equals_megakernel(cuda):
    sc = scenes.mixed_mid(width=128, height=72, subdiv=3)
    a = _render(sc, 16, 8, "megakernel").accum()
    b = _render(sc, 16, 8, "wavefront", wave_paths=50000).accum()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("flags", [1, 2, 3, 4, 5, 16, 17, 18, 20, 24])
def test_scheduling_flags_do_not_change_results(cuda, flags):
    sc = scenes.cornell_box(width=96, height=64)
    a = _render(sc, 8, 5, "wavefront", wave_paths=1 << 15).accum()
    b = _render(sc, 8, 5, "wavefront", wave_paths=1 << 15, flags=flags).accum()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("mode", ["megakernel", "wavefront"])
def test_f32_nodes_render_identically(cuda, mode):
    sc = scenes.large_textured(width=96, height=54, grid=64, tex_size=64, n_spheres=12,
                               sphere_subdiv=2)
    out = []
    for fmt in ("q8", "f32"):
        g = GB300Scene(sc, node_format=fmt)
        r = GB300Renderer(g, sc.width, sc.height, 8, max_depth=8, mode=mode)
        r.render()
        out.append(r.accum())
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("shape", [dict(block_size=64), dict(block_size=256),
                                   dict(stack_depth=4), dict(stack_depth=32, block_size=256),
                                   dict(node_format="f32"), dict(wave_sets=1), dict(wave_sets=8),
                                   dict(top_nodes=0), dict(top_nodes=9), dict(top_nodes=73, node_format="f32"),
                                   dict(top_nodes=128, block_size=64, queue_chunk=128)])
def test_launch_shape_does_not_change_results(cuda, shape):
    """Block size, shared stack depth, per-render node format and the
    number of wave sets are scheduling choices: the image is unchanged."""
    sc = scenes.large_textured(width=96, height=54, grid=64, tex_size=64, n_spheres=12,
                               sphere_subdiv=2)
    g = GB300Scene(sc)
    out = []
    for kw in ({}, shape):
        r = GB300Renderer(g, sc.width, sc.height, 8, max_depth=8, mode="wavefront",
                          wave_paths=1 << 14, **kw)
        r.render()
        out.append(r.accum())
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("extra", [{}, dict(node_format="f32", flags=8), dict(wave_sets=1, wave_paths=1 << 12)])
def test_window_sort_renders_identically(cuda, extra):
    """Grouping each window's survivors by direction and its shadow requests
    by light (the default; CRT_FLAG_NO_WINDOW_SORT = 16 turns it off)
    reorders the queues only: four lights, a texture, mirrors and glass,
    many windows and partial last windows."""
    sc = scenes.large_textured(width=96, height=54, grid=64, tex_size=64, n_spheres=12,
                               sphere_subdiv=2)
    g = GB300Scene(sc)
    out = []
    for flags in (0, 16):
        kw = dict(extra)
        kw["flags"] = kw.get("flags", 0) | flags
        r = GB300Renderer(g, sc.width, sc.height, 8, max_depth=8, mode="wavefront", **kw)
        r.render()
        out.append(r.accum())
        ext, shd = r.ray_counts()
        assert ext > 0 and shd > 0
    assert np.array_equal(out[0], out[1])
    mk = GB300Renderer(g, sc.width, sc.height, 8, max_depth=8, mode="megakernel")
    mk.render()
    assert np.array_equal(out[1], mk.accum())


def test_passes_of_many_waves_render_identically(cuda):
    """A pass of up to 1024 waves runs as one graph launch; longer passes
    (here 1050 waves of 4 samples) keep per-wave launches: both schedules
    add every pixel's samples in sample order."""
    sc = scenes.cornell_box(width=128, height=128)
    g = GB300Scene(sc)
    for spp in (4096, 4200):
        wf = GB300Renderer(g, sc.width, sc.height, spp, max_depth=5, mode="wavefront", wave_paths=1 << 16)
        wf.render(spp)
        mk = GB300Renderer(g, sc.width, sc.height, spp, max_depth=5, mode="megakernel")
        mk.render(spp)
        assert np.array_equal(wf.accum(), mk.accum()), spp


def test_four_wide_bvh_renders_identically(cuda):
    sc = scenes.mixed_mid(width=128, height=72, subdiv=3)
    a = GB300Renderer(GB300Scene(sc), 128, 72, 8, max_depth=8, mode="wavefront")
    b = GB300Renderer(GB300Scene(sc, bvh_width=4), 128, 72, 8, max_depth=8, mode="wavefront")
    a.render()
    b.render()
    assert np.array_equal(a.accum(), b.accum())


def test_reference_layout_renders_identically(cuda):
    """The arrays the C++ Renderer shim passes (v1/e1/e2 per face, emission
    already scaled by 3 x light area) give the scene the standard arrays give."""
    sc = scenes.feature_mix(width=64, height=48)
    a = GB300Scene(sc)
    b = GB300Scene(sc, reference_layout=True)
    assert a.info.lights_area == b.info.lights_area
    out = []
    for g in (a, b):
        r = GB300Renderer(g, sc.width, sc.height, 8, max_depth=6, mode="wavefront")
        r.render()
        out.append(r.accum())
    assert np.array_equal(out[0], out[1])


def test_resume_from_saved_accumulator(cuda):
    """Save the sums and counters after some passes, load them into a fresh
    handle, continue: the result equals the uninterrupted render."""
    sc = scenes.cornell_box(width=64, height=48)
    g = GB300Scene(sc)
    full = GB300Renderer(g, 64, 48, 10, max_depth=5, mode="wavefront")
    full.render(10)
    part = GB300Renderer(g, 64, 48, 10, max_depth=5, mode="wavefront")
    part.render(4)
    saved, n = part.accum(), part.get_samples_rendered()
    resumed = GB300Renderer(g, 64, 48, 10, max_depth=5, mode="megakernel")
    resumed.load_accum(saved, n, 0)
    resumed.render(6)
    assert resumed.get_samples_rendered() == 10
    assert np.array_equal(resumed.accum(), full.accum())
    assert np.array_equal(resumed.copy_image_bytes(), full.copy_image_bytes())


def test_resolve_async_overlaps_next_pass(cuda):
    torch = cuda
    sc = scenes.cornell_box(width=64, height=48)
    g = GB300Scene(sc)
    r = GB300Renderer(g, 64, 48, 8, max_depth=5, mode="wavefront")
    r.render(4)
    buf = torch.empty(64 * 48 * 4, dtype=torch.uint8).pin_memory()
    r.resolve_async(buf)
    r.render(4)              # queued behind the copy
    r.synchronize()
    ref = GB300Renderer(g, 64, 48, 4, max_depth=5, mode="wavefront")
    ref.render(4)
    assert np.array_equal(buf.numpy().reshape(48, 64, 4), ref.copy_image_bytes())


def test_progressive_passes_equal_single(cuda):
    sc = scenes.cornell_box(width=64, height=64)
    g = GB300Scene(sc)
    r1 = GB300Renderer(g, 64, 64, 6, max_depth=5)
    r1.render(6)
    r2 = GB300Renderer(g, 64, 64, 6, max_depth=5)
    for _ in range(6):
        r2.render_one_sample_per_pixel()
    assert np.array_equal(r1.accum(), r2.accum())
    assert r2.get_samples_rendered() == 6


def test_resolve_matches_oracle_format(cuda):
    sc = scenes.cornell_box(width=64, height=64)
    r = _render(sc, 4, 5, "megakernel")
    img = r.copy_image_bytes().reshape(-1, 4)
    assert np.array_equal(img, oracle.resolve(r.accum(), 4))


def test_textured_mirror_glass(cuda):
    sc = scenes.large_textured(width=96, height=54, grid=64, tex_size=64, n_spheres=12,
                               sphere_subdiv=2)
    r = _render(sc, 8, 8, "megakernel")
    acc = r.accum()
    ref, _, _ = _oracle(sc, 8, 8)
    rel = float(np.sum((acc - ref) ** 2) / np.sum(ref ** 2))
    assert rel < 1e-3


@pytest.mark.parametrize("size,wave_paths", [((64, 48), 768),     # 3 whole 4-row bands per wave: 8x4 tiles
                                             ((64, 48), 1000),    # ranges cut mid-band: row order
                                             ((60, 44), 960),     # width not a multiple of 8: row order
                                             ((64, 48), 0)])      # whole images per wave: tiles
def test_pixel_order_within_waves_does_not_change_results(cuda, size, wave_paths):
    """Waves walk whole 4-row bands in 8x4 pixel tiles and other ranges in
    row order; every pixel still adds its samples in sample order."""
    sc = scenes.cornell_box(width=size[0], height=size[1])
    a = _render(sc, 6, 5, "megakernel").accum()
    b = _render(sc, 6, 5, "wavefront", wave_paths=wave_paths).accum()
    assert np.array_equal(a, b)

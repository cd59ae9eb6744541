"""The autotuner and the launch options it searches: every choice it can
make leaves the image unchanged, and the options it returns are no slower
than the ones it started from on its own clock."""
import numpy as np
import pytest

from cudart_gb300 import CrtError, GB300Renderer, GB300Scene, autotune, options_dict, scenes

pytestmark = pytest.mark.gpu


def test_autotune_returns_valid_faster_options(cuda):
    sc = scenes.mixed_mid(width=160, height=90, subdiv=3)
    g = GB300Scene(sc)
    ref = GB300Renderer(g, sc.width, sc.height, 4, max_depth=8, mode="wavefront")
    ref.render()
    res = autotune(g, sc.width, sc.height, max_depth=8, trial_spp=2, repeats=1, rounds=1)
    o = options_dict(res.options)
    assert res.candidates >= 10
    assert 0 < res.ms_per_spp <= res.start_ms_per_spp
    assert o["mode"] == 1 and o["max_depth"] == 8
    assert o["block_size"] in (64, 128, 256) and 4 <= o["stack_depth"] <= 32
    assert o["queue_chunk"] in (32, 64, 128, 256) and 1 <= o["wave_sets"] <= 8
    assert res.bvh_width in (4, 8) and g.info.bvh_width == res.bvh_width
    # the tuned render (possibly on a rebuilt BVH) gives the same image
    tuned = GB300Renderer(g, sc.width, sc.height, 4, options=res.options)
    tuned.render()
    assert np.array_equal(ref.accum(), tuned.accum())


def test_rebuilt_bvh_keeps_results_and_renders_follow(cuda):
    sc = scenes.mixed_mid(width=128, height=72, subdiv=3)
    g = GB300Scene(sc)
    r = GB300Renderer(g, 128, 72, 4, max_depth=8, mode="wavefront")
    r.render()                                  # captures its wave graphs on the 8-wide BVH
    n8 = g.info.num_nodes
    g.set_bvh_width(4)
    assert g.info.bvh_width == 4 and g.info.num_nodes > n8
    r.render()                                  # must re-capture against the new nodes
    fresh = GB300Renderer(GB300Scene(sc), 128, 72, 8, max_depth=8, mode="wavefront")
    fresh.render()
    assert np.array_equal(r.accum(), fresh.accum())
    with pytest.raises(CrtError):
        g.set_bvh_width(6)


@pytest.mark.parametrize("bad", [dict(block_size=96), dict(stack_depth=2), dict(stack_depth=40),
                                 dict(queue_chunk=48), dict(wave_sets=9), dict(top_nodes=129)])
def test_bad_launch_options_are_rejected(cuda, bad):
    sc = scenes.cornell_box(width=32, height=32)
    g = GB300Scene(sc)
    with pytest.raises(CrtError):
        GB300Renderer(g, 32, 32, 1, mode="wavefront", **bad)


@pytest.mark.parametrize("chunk", [64, 256])
def test_queue_chunk_does_not_change_results(cuda, chunk):
    sc = scenes.cornell_box(width=96, height=64)
    g = GB300Scene(sc)
    a = GB300Renderer(g, 96, 64, 8, max_depth=5, mode="wavefront", wave_paths=1 << 15)
    b = GB300Renderer(g, 96, 64, 8, max_depth=5, mode="wavefront", wave_paths=1 << 15,
                      queue_chunk=chunk)
    a.render()
    b.render()
    assert np.array_equal(a.accum(), b.accum())

"""Batched views: many cameras of one scene in one stream of waves.

Each view of a batch must equal, bit for bit, a single render of that view
(same Philox view word, same samples): the wave packing only changes which
paths share a launch, and every pixel still adds its samples in order."""
import dataclasses

import numpy as np
import pytest

from cudart_gb300 import CrtError, GB300Batch, GB300Renderer, GB300Scene, camera_from_json, scenes

pytestmark = pytest.mark.gpu


def _views(sc, n, seed=3):
    """n views of mixed small sizes and spp from the batched-views generator."""
    vs = scenes.batched_views(seed=seed, n_views=n, base=sc).views
    sizes = [(48, 32), (64, 64), (40, 24), (96, 54), (17, 9), (33, 65)]
    spps = [1, 3, 4, 2, 5]
    return [dataclasses.replace(v, width=sizes[k % len(sizes)][0], height=sizes[k % len(sizes)][1],
                                spp=spps[k % len(spps)]) for k, v in enumerate(vs)]


def _single(g, v, view_id, **kw):
    cam = camera_from_json(v.camera, v.width, v.height)
    r = GB300Renderer(g, v.width, v.height, v.spp, camera=cam, view_id=view_id, **kw)
    r.render()
    return r.accum()


@pytest.mark.parametrize("mode,wave_paths", [("wavefront", 0), ("wavefront", 4000),
                                             ("wavefront", 1000), ("megakernel", 0)])
def test_batch_views_equal_single_renders(cuda, mode, wave_paths):
    sc = scenes.mixed_mid(subdiv=2)
    g = GB300Scene(sc)
    views = _views(sc, 11)
    ids = [7 * k + 1 for k in range(len(views))]
    b = GB300Batch(g, views, view_ids=ids, max_depth=8, mode=mode, wave_paths=wave_paths)
    b.render()
    b.synchronize()
    for k, v in enumerate(views):
        ref = _single(g, v, ids[k], max_depth=8, mode="megakernel")
        assert np.array_equal(b.accum(k), ref), f"view {k}"
        info = b.view_info(k)
        assert info["samples_rendered"] == v.spp and info["view_id"] == ids[k]
    offs = [b.view_info(k)["pixel_offset"] for k in range(len(views))]
    assert offs == list(np.cumsum([0] + [v.width * v.height for v in views[:-1]]))


def test_batch_progressive_and_uniform_pass(cuda):
    sc = scenes.cornell_box()
    g = GB300Scene(sc)
    views = _views(sc, 5)
    b = GB300Batch(g, views, max_depth=5, mode="wavefront", wave_paths=3000, wave_sets=2)
    b.render()
    b.render_pass(2)         # every view two more samples
    b.render()
    for k, v in enumerate(views):
        cam = camera_from_json(v.camera, v.width, v.height)
        r = GB300Renderer(g, v.width, v.height, 2 * v.spp + 2, camera=cam, view_id=k, max_depth=5)
        r.render()
        assert np.array_equal(b.accum(k), r.accum()), f"view {k}"
        assert b.view_info(k)["samples_rendered"] == 2 * v.spp + 2
        img = b.resolve(k)
        assert img.shape == (v.height, v.width, 4) and np.array_equal(img, r.copy_image_bytes())


def test_batch_errors(cuda):
    sc = scenes.cornell_box()
    g = GB300Scene(sc)
    with pytest.raises(CrtError):
        GB300Batch(g, [])
    bad = dataclasses.replace(_views(sc, 1)[0], width=0)
    with pytest.raises(CrtError):
        GB300Batch(g, [bad])
    b = GB300Batch(g, _views(sc, 2))
    with pytest.raises(CrtError):
        b.view_info(2)

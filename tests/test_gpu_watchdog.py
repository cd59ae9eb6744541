"""Failure detection without a GPU fault: a traversal that exceeds the
scene's node-visit limit ends its ray and records CRT_ERR_WATCHDOG in the
scene's error word; the host reads the status, and after
crt_scene_clear_errors the same handles render normally again."""
import numpy as np
import pytest

from cudart_gb300 import CrtError, GB300Renderer, GB300Scene, scenes

pytestmark = pytest.mark.gpu
CRT_ERR_WATCHDOG = 5


@pytest.mark.parametrize("mode", ["megakernel", "wavefront"])
def test_visit_limit_reports_and_recovers(cuda, mode):
    sc = scenes.feature_mix(width=48, height=32)
    g = GB300Scene(sc)
    want = GB300Renderer(g, sc.width, sc.height, 4, max_depth=6, mode=mode)
    want.render()
    img0 = want.copy_image_bytes()
    r = GB300Renderer(g, sc.width, sc.height, 4, max_depth=6, mode=mode)
    r.render()                      # graphs captured under the default limit
    r.synchronize()
    g.set_visit_limit(2)            # root + one child: most rays run out
    r.reset()
    r.render()
    with pytest.raises(CrtError) as e:
        r.copy_image_bytes()
    assert e.value.status == CRT_ERR_WATCHDOG
    with pytest.raises(CrtError):   # sticky until cleared
        r.synchronize()
    g.set_visit_limit(0)
    g.clear_errors()
    r.reset()
    r.render()
    assert np.array_equal(r.copy_image_bytes(), img0)


def test_ray_queries_keep_working_after_a_watchdog(cuda):
    import torch
    sc = scenes.cornell_box(width=32, height=32)
    g = GB300Scene(sc)
    rays = torch.zeros((256, 8), dtype=torch.float32, device="cuda")
    rays[:, 2] = 3.0
    rays[:, 4:7] = torch.nn.functional.normalize(torch.randn(256, 3, device="cuda") * 0.2 +
                                                 torch.tensor([0.0, 0.0, -1.0], device="cuda"), dim=1)
    rays[:, 7] = 1e30
    idx0, t0, _ = g.trace_closest(rays)
    g.set_visit_limit(1)
    g.trace_closest(rays)
    torch.cuda.synchronize()
    g.set_visit_limit(0)
    g.clear_errors()
    idx1, t1, _ = g.trace_closest(rays)
    assert torch.equal(idx0, idx1) and torch.equal(t0, t1)


def test_visit_limit_range(cuda):
    from cudart_gb300 import load
    g = GB300Scene(scenes.cornell_box(width=16, height=16))
    L = load()
    assert L.crt_scene_set_visit_limit(g.handle, (1 << 30) + 1) == 6     # CRT_ERR_LIMIT
    assert L.crt_scene_set_visit_limit(g.handle, 1 << 30) == 0
    assert L.crt_scene_set_visit_limit(None, 5) == 1
    assert L.crt_scene_clear_errors(None) == 1


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
@pytest.mark.parametrize("builder", ["host", "gpu"])
def test_non_finite_vertices_are_an_error(cuda, bad, builder):
    import dataclasses
    sc = scenes.cornell_box(width=16, height=16)
    pos = sc.positions.copy()
    pos[7, 1, 2] = bad
    with pytest.raises(CrtError, match="non-finite vertex coordinate in face 7"):
        GB300Scene(dataclasses.replace(sc, positions=pos), builder=builder)
    g = GB300Scene(sc, builder=builder)       # the device is still usable
    assert g.info.num_triangles == sc.n_tris

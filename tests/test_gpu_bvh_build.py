"""The GPU BVH build (linear BVH + the host build's collapse and encoding):
the same invariants as the host build, and the same closest hits and
images, bit for bit (every query result is independent of the tree)."""
import numpy as np
import pytest

import oracle
from conftest import random_rays
from cudart_gb300 import GB300Renderer, GB300Scene, scenes
from test_bvh_host import check_tree

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("width", [8, 4])
def test_gpu_tree_invariants(cuda, width):
    sc = scenes.mixed_mid(subdiv=3)
    g = GB300Scene(sc, builder="gpu", bvh_width=width)
    nodes, tris = g.export_bvh()
    check_tree(np.asarray(sc.positions), nodes, tris, g.info.max_depth, width)
    assert g.info.num_nodes == len(nodes) and g.info.bvh_width == width


@pytest.mark.parametrize("fmt", ["q8", "f32"])
def test_gpu_tree_closest_hits_match_brute_force(cuda, fmt):
    sc = scenes.large_textured(grid=96, tex_size=16, n_spheres=8, sphere_subdiv=2)
    rays = random_rays(20000, 7, lo=-4.0, hi=4.0)
    g = GB300Scene(sc, builder="gpu", node_format=fmt)
    idx, t, _ = g.trace_closest(cuda.from_numpy(rays).cuda())
    oi, ot, _ = oracle.OracleScene(sc).closest_hit(rays, brute=True)
    assert np.array_equal(idx.cpu().numpy(), oi)
    assert np.array_equal(t.cpu().numpy(), ot)


@pytest.mark.parametrize("mode", ["megakernel", "wavefront"])
def test_gpu_tree_renders_identically(cuda, mode):
    sc = scenes.mixed_mid(width=128, height=72, subdiv=3)
    out = []
    for builder in ("host", "gpu"):
        r = GB300Renderer(GB300Scene(sc, builder=builder), 128, 72, 8, max_depth=8, mode=mode)
        r.render()
        out.append(r.accum())
    assert np.array_equal(out[0], out[1])


def test_gpu_tree_degenerate_inputs(cuda):
    one = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]]], np.float32)
    rng = np.random.default_rng(0)
    tiny = rng.uniform(-1, 1, (500, 1, 3)).astype(np.float32) + rng.uniform(0, 1e-3, (500, 3, 3)).astype(np.float32)
    # 100,000 identical triangles: every clustering distance ties, which the
    # pair order turns into (2k, 2k + 1) merges -- a balanced tree in
    # ~17 iterations, not one merge per iteration
    for pos in (one, np.repeat(one, 50, axis=0), np.concatenate([tiny, np.repeat(one, 7, axis=0)]),
                np.repeat(one, 100000, axis=0)):
        sc = scenes.cornell_box()
        # the Cornell box keeps its light and camera; the test geometry replaces its first faces
        n = len(pos)
        p = sc.positions.copy()
        p = np.concatenate([pos.astype(np.float32), p])
        nor = np.concatenate([np.tile([[0, 0, 1]], (n, 3, 1)).astype(np.float32), sc.normals])
        uv = np.concatenate([np.zeros((n, 3, 2), np.float32), sc.uvs])
        mid = np.concatenate([np.zeros(n, np.uint32), sc.material_ids])
        import dataclasses
        sc2 = dataclasses.replace(sc, positions=p, normals=nor, uvs=uv, material_ids=mid)
        g = GB300Scene(sc2, builder="gpu")
        nodes, tris = g.export_bvh()
        check_tree(p, nodes, tris, g.info.max_depth)
        assert g.info.max_depth <= 12

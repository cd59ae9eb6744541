"""Closest-hit parity on the GPU: face index bit-exact (ties to the lowest
index), t bit-exact, against the oracle's Moller-Trumbore restatement
(geometry.cu:38-65) over every triangle."""
import numpy as np
import pytest

import oracle
from conftest import FLT_MAX, random_rays
from cudart_gb300 import GB300Scene, scenes

pytestmark = pytest.mark.gpu


def _check(cuda, sc, rays, brute=True, node_format="q8", bvh_width=8):
    g = GB300Scene(sc, node_format=node_format, bvh_width=bvh_width)
    idx, t, uv = g.trace_closest(cuda.from_numpy(rays).cuda())
    o = oracle.OracleScene(sc)
    oi, ot, ouv = o.closest_hit(rays, brute=brute)
    gi, gt, guv = idx.cpu().numpy(), t.cpu().numpy(), uv.cpu().numpy()
    bad = np.nonzero(gi != oi)[0]
    assert len(bad) == 0, f"{len(bad)} index mismatches, first {bad[:5]}: gpu {gi[bad[:5]]} oracle {oi[bad[:5]]}"
    assert np.array_equal(gt, ot)
    hit = oi >= 0
    assert np.array_equal(guv[hit], ouv[hit])
    return oi


def test_cornell_random_rays(cuda):
    sc = scenes.cornell_box()
    oi = _check(cuda, sc, random_rays(20000, 1))
    assert (oi >= 0).mean() > 0.5


def test_cornell_ties_lowest_index(cuda):
    # the box bottoms are coplanar with the floor: rays through them tie
    sc = scenes.cornell_box()
    rng = np.random.default_rng(3)
    n = 4096
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0] = rng.uniform(-0.9, 0.9, n)
    rays[:, 2] = rng.uniform(-0.9, 0.9, n)
    rays[:, 1] = 0.5
    rays[:, 5] = -1.0
    rays[:, 3] = 1e-5
    rays[:, 7] = FLT_MAX
    oi = _check(cuda, sc, rays)
    floor = [g for g in sc.groups if g[0] == "floor"][0]
    assert np.any((oi >= floor[2]) & (oi < floor[2] + floor[3]))


@pytest.mark.parametrize("fmt", ["q8", "f32"])
def test_mixed_scene_bvh_oracle(cuda, fmt):
    sc = scenes.mixed_mid(subdiv=3)
    _check(cuda, sc, random_rays(20000, 2), node_format=fmt)


@pytest.mark.parametrize("fmt", ["q8", "f32"])
def test_four_wide_bvh(cuda, fmt):
    sc = scenes.mixed_mid(subdiv=3)
    _check(cuda, sc, random_rays(20000, 5), node_format=fmt, bvh_width=4)


@pytest.mark.parametrize("fmt", ["q8", "f32"])
def test_textured_scene(cuda, fmt):
    sc = scenes.large_textured(grid=64, tex_size=64, n_spheres=8, sphere_subdiv=2)
    _check(cuda, sc, random_rays(20000, 4, lo=-4.0, hi=4.0), node_format=fmt)


def test_f32_nodes_cornell_ties_and_windows(cuda):
    sc = scenes.cornell_box()
    rays = random_rays(6000, 8)
    rays[2000:4000, 3] = 0.3
    rays[4000:, 7] = 0.7
    _check(cuda, sc, rays, node_format="f32")


def test_axis_parallel_and_windows(cuda):
    sc = scenes.cornell_box()
    rays = random_rays(6000, 5)
    rays[:2000, 4:7] = 0.0
    rays[np.arange(2000), 4 + (np.arange(2000) % 3)] = np.where(np.arange(2000) % 2, 1.0, -1.0)
    rays[2000:4000, 3] = 0.3          # tmin window
    rays[4000:, 7] = 0.7              # tmax window
    _check(cuda, sc, rays)


def test_empty_batch_and_all_miss(cuda):
    sc = scenes.cornell_box()
    g = GB300Scene(sc)
    rays = random_rays(1000, 6)
    rays[:, :3] = 50.0                # outside, pointing away
    rays[:, 4:7] = np.abs(rays[:, 4:7])
    idx, t, _ = g.trace_closest(cuda.from_numpy(rays).cuda())
    assert (idx.cpu().numpy() == -1).all() and (t.cpu().numpy() == FLT_MAX).all()
    idx, t, _ = g.trace_closest(cuda.zeros((0, 8), dtype=cuda.float32, device="cuda"))
    assert idx.numel() == 0

"""Invariants of the host-built 8-wide quantised BVH (no GPU needed):
every face is referenced exactly once, every triangle lies inside the
decoded (exact) quantised box of its leaf slot and of every ancestor slot,
children and triangle ranges are well formed, and depth fits the traversal
stack."""
import numpy as np
import pytest

from cudart_gb300 import bvh_build_host, scenes

MAX_LEVELS = 64   # traversal stack: 16 shared-memory + 48 local entries


def _decode(node, slot):
    p = node["p"].astype(np.float64)
    scale = np.ldexp(1.0, node["e"].astype(np.int64) - 127)
    lo = p + node["qlo"][:, slot] * scale
    hi = p + node["qhi"][:, slot] * scale
    return lo, hi


def _check(positions, width=8):
    nodes, tris, depth = bvh_build_host(positions, width)
    return check_tree(positions, nodes, tris, depth, width)


def check_tree(positions, nodes, tris, depth, width=8):
    """Invariants every build must meet (also used for the GPU build)."""
    n = len(positions)
    assert depth <= MAX_LEVELS
    assert sorted(tris["face"].tolist()) == list(range(n))
    pos = positions.astype(np.float64)
    # geometry of the records equals the scene's v1, e1 = v2 - v1, e2 = v3 - v1
    f = tris["face"]
    assert np.array_equal(tris["v1"], positions[f, 0])
    assert np.array_equal(tris["e1"], positions[f, 1] - positions[f, 0])
    used = np.count_nonzero(nodes["meta"], axis=1)
    assert np.all(used >= 1) and np.all(used <= width)
    parent_boxes = {0: (np.full(3, -np.inf), np.full(3, np.inf))}
    seen_internal = 0
    for i, node in enumerate(nodes):
        plo, phi = parent_boxes[i]
        rank = 0
        for s in range(8):
            meta = int(node["meta"][s])
            internal = bool(node["imask"] & (1 << s))
            if meta == 0:
                assert not internal
                continue
            lo, hi = _decode(node, s)
            # outward rounding may push a child box past its parent's decoded
            # box by at most one quantum of this node's grid
            quantum = np.ldexp(1.0, node["e"].astype(np.int64) - 127)
            assert np.all(lo >= plo - quantum) and np.all(hi <= phi + quantum)
            if internal:
                assert meta == 0x80
                parent_boxes[int(node["child_base"]) + rank] = (lo, hi)
                rank += 1
                seen_internal += 1
            else:
                cnt, off = meta >> 5, meta & 31
                assert 1 <= cnt <= 3 and off + cnt <= 24
                for k in range(cnt):
                    face = int(tris["face"][node["tri_base"] + off + k])
                    v = pos[face]
                    assert np.all(v >= lo) and np.all(v <= hi), (i, s, face)
                    # and inside every ancestor
                    assert np.all(v >= plo) and np.all(v <= phi)
    assert seen_internal == len(nodes) - 1
    return nodes, depth


def test_cornell_bvh():
    _check(scenes.cornell_box().positions)


def test_mixed_bvh():
    nodes, depth = _check(scenes.mixed_mid(subdiv=3).positions)
    assert depth >= 3


def test_textured_bvh():
    _check(scenes.large_textured(grid=96, tex_size=16, n_spheres=6, sphere_subdiv=2).positions)


def test_degenerate_inputs():
    # one triangle, coincident triangles, a single huge triangle among tiny ones
    one = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]]], np.float32)
    _check(one)
    _check(np.repeat(one, 50, axis=0))
    rng = np.random.default_rng(0)
    tiny = rng.uniform(-1, 1, (500, 1, 3)).astype(np.float32) + rng.uniform(0, 1e-3, (500, 3, 3)).astype(np.float32)
    big = np.array([[[-1e3, -1e3, 0], [1e3, -1e3, 0], [0, 1e3, 0]]], np.float32)
    _check(np.concatenate([tiny, big]))


def test_empty_scene_is_an_error():
    from cudart_gb300 import CrtError
    with pytest.raises(CrtError):
        bvh_build_host(np.zeros((0, 3, 3), np.float32))


def test_four_wide_bvh():
    n8, d8 = _check(scenes.mixed_mid(subdiv=3).positions, width=8)
    n4, d4 = _check(scenes.mixed_mid(subdiv=3).positions, width=4)
    assert len(n4) > len(n8) and d4 >= d8


def test_bad_width_is_an_error():
    from cudart_gb300 import CrtError
    with pytest.raises(CrtError):
        bvh_build_host(scenes.cornell_box().positions, width=6)


def test_build_is_deterministic():
    # the build splits large ranges across threads; min/max bounds and
    # integer bin counts merge exactly, so repeated builds are identical
    pos = scenes.large_textured(grid=256, tex_size=16, n_spheres=8, sphere_subdiv=2).positions
    a_nodes, a_tris, _ = bvh_build_host(pos)
    b_nodes, b_tris, _ = bvh_build_host(pos)
    assert a_nodes.tobytes() == b_nodes.tobytes() and a_tris.tobytes() == b_tris.tobytes()

"""Pins the CPU oracle to the reference.

* Philox4x32-10 against the published Random123 known-answer vectors.
* Golden fixtures produced by the reference's own code (tests/golden/
  make_golden.py): scene preparation, camera, gamma table, texels, closest
  hits, per-sample radiance and long-run per-pixel statistics must come out
  of the oracle bit for bit.
"""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from golden.make_golden import load_scene

FIXTURES = ["cornell_512", "feature_mix", "mixed_sub2", "cornell_lens"]


def _fx(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def _export(fx):
    return {k[4:]: v for k, v in fx.items() if k.startswith("ref_")}


@pytest.mark.parametrize("ctr,key,expect", [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
])
def test_philox_known_answers(ctr, key, expect):
    assert list(oracle.philox(ctr, key)) == expect


@pytest.mark.parametrize("name", FIXTURES)
def test_scene_preparation_matches_reference(name):
    fx = _fx(name)
    e = _export(fx)
    sc = load_scene(fx)
    o = oracle.OracleScene(sc, lights=e["lights"])        # the reference's pick order
    t = e["tris"]
    for k, f in enumerate(["v1", "e1", "e2", "n1", "n2", "n3"]):
        assert np.array_equal(o.tris[f], t[:, 3 * k:3 * k + 3]), f
    assert np.array_equal(o.tris["uv"], t[:, 18:24])
    assert np.array_equal(o.tris["area"], t[:, 24])
    assert np.float32(o.lights_area) == np.float32(e["lights_area"])
    # the reference dedups materials; compare the rows each face ends up with
    mf, mi = e["mat_floats"], e["mat_ints"]
    om = o.mats[o.tris["material"]]
    ours = np.concatenate([om["kd"], om["ka"], om["ks"], om["ns"][:, None], om["ni"][:, None],
                           om["diffuse"][:, None]], 1)
    assert np.array_equal(ours, mf[e["mat_ids"]])
    assert np.array_equal(np.stack([om["bsdf"], om["tex"]], 1), mi[e["mat_ids"]])
    cam = oracle.make_camera(sc.camera, sc.width, sc.height)
    assert cam.tobytes() == oracle.camera_from_export(e).tobytes()
    if sc.textures:
        assert np.array_equal(o.tex_data, e["tex_data"])
        assert np.array_equal(o.tex_dims, e["tex_dims"])


@pytest.mark.parametrize("name", FIXTURES)
def test_gamma_table_matches_reference(name):
    assert np.array_equal(oracle.gamma_table(), _fx(name)["ref_gamma"])


@pytest.mark.parametrize("name", FIXTURES)
def test_closest_hit_matches_reference(name):
    fx = _fx(name)
    o = oracle.scene_from_export(_export(fx))
    rays = fx["rays"]
    ran = fx["ref_hit_idx"] != -2                       # -2: the reference's stack would overflow
    assert ran.mean() > 0.9
    bi, bt, buv = o.closest_hit(rays, brute=True)
    vi, vt, _ = o.closest_hit(rays)
    assert np.array_equal(bi, vi) and np.array_equal(bt, vt)
    ri, rt = fx["ref_hit_idx"][ran], fx["ref_hit_t"][ran]
    assert np.array_equal(bt[ran], rt)
    # equal t with a different face only at ties; the oracle takes the lowest index
    diff = bi[ran] != ri
    assert np.all(bi[ran][diff] < ri[diff])
    assert diff.mean() < 0.01
    same = ran.copy()
    same[ran] = ~diff
    hit = same & (bi >= 0)
    assert np.array_equal(buv[hit], fx["ref_hit_uv"][hit])


@pytest.mark.parametrize("name", ["cornell_512", "feature_mix", "cornell_lens"])
def test_samples_match_reference(name):
    fx = _fx(name)
    o = oracle.scene_from_export(_export(fx))
    cam = oracle.camera_from_export(_export(fx))
    W = int(cam["xpixels"][0])
    seed = int(fx["seed"])
    for (x, y, s), rgb in zip(fx["sample_xys"], fx["ref_sample_rgb"]):
        acc, _, _ = o.render(cam, seed, 1, 6, spp0=int(s), pixels=np.array([y * W + x], np.uint32))
        assert np.array_equal(acc[0], rgb), (x, y, s)


@pytest.mark.parametrize("name", ["cornell_512", "feature_mix", "cornell_lens"])
def test_long_render_statistics_match_reference(name):
    fx = _fx(name)
    o = oracle.scene_from_export(_export(fx))
    cam = oracle.camera_from_export(_export(fx))
    acc, mean, m2 = o.render(cam, int(fx["seed"]), int(fx["stats_spp"]), 6, pixels=fx["stats_pixels"])
    # Millions of paths: a handful cross a shared edge exactly (two faces at
    # equal t).  The reference breaks such ties by traversal order, the
    # oracle by lowest face index, so those few pixels may differ slightly;
    # every other pixel is bit-identical.
    same = np.all(acc == fx["ref_stats_acc"], axis=1)
    assert same.mean() >= 0.995
    assert np.array_equal(mean[same], fx["ref_stats_mean"][same])
    assert np.array_equal(m2[same], fx["ref_stats_m2"][same])
    ref = fx["ref_stats_acc"][~same]
    assert np.all(np.abs(acc[~same] - ref) <= 1e-3 * np.abs(ref).max(axis=1, keepdims=True))


def test_resolve_matches_reference_quantise_and_gamma():
    fx = _fx("feature_mix")
    spp = int(fx["stats_spp"])
    img = oracle.resolve(fx["ref_stats_acc"], spp)
    q = np.minimum(fx["ref_stats_acc"] / np.float32(spp), np.float32(1.0)) * np.float32(255.0)
    assert np.array_equal(img[:, :3], fx["ref_gamma"][q.astype(np.uint8)])
    assert (img[:, 3] == 255).all()

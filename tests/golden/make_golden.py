"""Generates the golden fixtures in tests/golden/ from the reference itself.

    python tests/golden/make_golden.py            # all fixtures
    python tests/golden/make_golden.py --one NAME # one fixture (subprocess)

Needs the CudaRT sources (the pinning harness oracle/_ref/libcrt_ref.so is
built from them by oracle/Makefile); it writes each scene as OBJ/MTL/JSON/
PNG, loads it through the reference's own Scene class, and records:

* the scene arrays given to the reference (so tests rebuild the exact scene
  on any machine), and the reference's loaded state (triangles, material
  table, light order and area, camera, texels);
* closest hits of seeded rays through the reference's intersectBVH
  (face index -2 marks rays whose traversal would overflow the reference's
  16-entry stack and were not run);
* per-sample radiance of the reference's samplePixel on Philox-keyed
  streams (rand() interposed), with the number of draws consumed;
* FP32 accumulators and FP64 per-pixel mean / M2 of long reference renders
  on a pixel subset;
* the reference's gamma table (gammaCorrectPixel for every byte value).

The reference hard-codes 6 bounces (renderer.cu:25,33), so the fixtures
above are at max depth 6.  The depth-8 fixtures of the two headline scenes
(`mixed_mid_d8`: 1280x720, 102,412 triangles; `large_textured_d8`:
1920x1080, 2,174,986 triangles) come from the reference built with its
traversal stack raised to 64 entries and c_maxBounces set to 8 (oracle/
Makefile, target ref-deep); their trees are 30 and 39 levels deep, past the
shipped 16-entry stack.  They are too large to store, so these fixtures
hold the generator's name and a fingerprint of its arrays (tests regenerate
the scene and check the fingerprint), the reference's light order, per-
sample radiance of samplePixel at depth 8, and 4096-spp statistics over a
stratified 4096-pixel subset (one pixel per cell of a 64x64 grid) plus a
64x64 crop at the image centre.

    python tests/golden/make_golden.py --one mixed_mid_d8   # ~15 min on 8 threads
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

SEED = 20240607


def _configs():
    from cudart_gb300 import scenes
    return {
        # name: (scene factory, rays, rays box, n samples, stats spp, stats pixels)
        "cornell_512": (lambda: scenes.cornell_box(), 4096, 0.95, 256, 4096, "crop+random"),
        "feature_mix": (lambda: scenes.feature_mix(), 4096, 0.95, 512, 1024, "all"),
        "mixed_sub2": (lambda: scenes.mixed_mid(width=64, height=48, subdiv=2), 4096, 0.95, 0, 0, None),
        "cornell_lens": (lambda: scenes.cornell_lens(), 1024, 0.95, 256, 2048, "crop+random"),
    }


# depth-8 fixtures: name -> (generator name, per-sample count, stats spp)
DEEP = {
    "mixed_mid_d8": ("mixed_mid", 512, 4096),
    "large_textured_d8": ("large_textured", 512, 4096),
}


def fingerprint(sc) -> np.ndarray:
    """FP64 sums that identify a generated scene up to last-bit differences
    between machines' libm: array sums and sums of squares, face and
    material counts."""
    f = []
    for a in (sc.positions, sc.normals, sc.uvs):
        a = np.asarray(a, np.float64)
        f += [a.sum(), (a * a).sum(), np.abs(a).max()]
    f += [float(np.asarray(sc.material_ids, np.int64).sum()), float(sc.n_tris), float(len(sc.materials))]
    for m in sc.materials:
        f += [float(m.bsdf), sum(m.kd), sum(m.ka), sum(m.ks), m.ni, m.diffuse, float(m.tex)]
    for img in sc.textures:
        f += [float(np.asarray(img, np.int64).sum())]
    return np.array(f, np.float64)


def stats_pixels(width: int, height: int, rng) -> np.ndarray:
    """One random pixel in each cell of a 64x64 grid over the image, plus the
    64x64 crop at the image centre (sorted, unique)."""
    px = []
    ys = np.linspace(0, height, 65).astype(int)
    xs = np.linspace(0, width, 65).astype(int)
    for j in range(64):
        for i in range(64):
            px.append(int(rng.integers(ys[j], ys[j + 1])) * width + int(rng.integers(xs[i], xs[i + 1])))
    cx, cy = width // 2 - 32, height // 2 - 32
    px += [(cy + j) * width + cx + i for j in range(64) for i in range(64)]
    return np.unique(np.array(px, np.uint32))


def make_deep(name: str) -> None:
    import time
    import oracle
    from cudart_gb300 import scenes
    gen, n_samples, stats_spp = DEEP[name]
    sc = getattr(scenes, gen)()
    out = dict(generator=np.array(gen), fingerprint=fingerprint(sc),
               size=np.array([sc.width, sc.height, sc.spp, sc.max_depth], np.int32))
    with tempfile.TemporaryDirectory() as td:
        files = scenes.write_reference_files(sc, td, name)
        R = oracle.RefHarness(files, sc.width, sc.height, deep=True)
        assert R.max_depth == sc.max_depth == 8, (R.max_depth, sc.max_depth)
        R._check_depth()
        e = R.export()
        # the reference's loaded scene must be the generator's: per face the
        # same positions and material values (its material merge, material.h:
        # 57-79, must not have changed any face's material)
        tri = e["tris"]
        p = np.asarray(sc.positions, np.float32)
        assert np.array_equal(tri[:, 0:3], p[:, 0]), "v1 differs"
        mf = e["mat_floats"][e["mat_ids"]]
        mine = np.array([list(m.kd) + list(m.ks) + [m.ni, m.diffuse] for m in sc.materials],
                        np.float32)[sc.material_ids]
        theirs = np.concatenate([mf[:, 0:3], mf[:, 6:9], mf[:, 10:12]], 1)
        assert np.array_equal(mine, theirs), "the reference merged materials of this scene"
        out["ref_lights"] = e["lights"]
        out["ref_lights_area"] = np.float32(e["lights_area"])
        out["ref_bvh_depth"] = np.int32(R.bvh_depth)
        rng = np.random.default_rng(SEED + 8)
        xs = rng.integers(0, sc.width, n_samples)
        ys = rng.integers(0, sc.height, n_samples)
        ss = rng.integers(0, 1 << 16, n_samples)
        rgb = np.zeros((n_samples, 3), np.float32)
        draws = np.zeros(n_samples, np.int32)
        for k in range(n_samples):
            rgb[k], draws[k] = R.sample_pixel(int(xs[k]), int(ys[k]), SEED, int(ss[k]))
        out.update(sample_xys=np.stack([xs, ys, ss], 1).astype(np.int32), ref_sample_rgb=rgb,
                   ref_sample_draws=draws)
        px = stats_pixels(sc.width, sc.height, rng)
        t0 = time.time()
        acc, mean, m2 = R.render(px, SEED, stats_spp)
        out.update(stats_pixels=px, stats_spp=np.int32(stats_spp), ref_stats_acc=acc,
                   ref_stats_mean=mean, ref_stats_m2=m2, ref_render_seconds=np.float64(time.time() - t0))
    out["seed"] = np.uint64(SEED)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def scene_arrays(sc) -> dict:
    m = sc.materials
    d = dict(positions=sc.positions, normals=sc.normals, uvs=sc.uvs, material_ids=sc.material_ids,
             mat_bsdf=np.array([x.bsdf for x in m], np.int32), mat_tex=np.array([x.tex for x in m], np.int32),
             mat_kd=np.array([x.kd for x in m], np.float32), mat_ka=np.array([x.ka for x in m], np.float32),
             mat_ks=np.array([x.ks for x in m], np.float32),
             mat_scalars=np.array([[x.ns, x.ni, x.diffuse] for x in m], np.float32),
             cam_fov=np.float32(sc.camera.fov_deg), cam_eye=np.array(sc.camera.eye, np.float32),
             cam_dir=np.array(sc.camera.view_dir, np.float32), cam_up=np.array(sc.camera.up, np.float32),
             cam_lens=np.array([sc.camera.focal_length, sc.camera.fstop], np.float32),
             size=np.array([sc.width, sc.height, sc.spp, sc.max_depth], np.int32),
             n_textures=np.int32(len(sc.textures)))
    for k, img in enumerate(sc.textures):
        d[f"texture{k}"] = img
    return d


def load_scene(fx) -> "object":
    """Rebuild the SceneArrays stored in a fixture."""
    from cudart_gb300 import scenes
    mats = []
    for i in range(len(fx["mat_bsdf"])):
        ns, ni, dif = fx["mat_scalars"][i]
        mats.append(scenes.Material(f"m{i}", int(fx["mat_bsdf"][i]), tuple(fx["mat_kd"][i]),
                                    tuple(fx["mat_ka"][i]), tuple(fx["mat_ks"][i]), float(ns),
                                    float(ni), float(dif), int(fx["mat_tex"][i])))
    cam = scenes.CameraSpec(float(fx["cam_fov"]), tuple(fx["cam_eye"]), tuple(fx["cam_dir"]),
                            tuple(fx["cam_up"]), float(fx["cam_lens"][0]), float(fx["cam_lens"][1]))
    w, h, spp, depth = map(int, fx["size"])
    tex = [fx[f"texture{k}"] for k in range(int(fx["n_textures"]))]
    n = len(fx["material_ids"])
    return scenes.SceneArrays(fx["positions"], fx["normals"], fx["uvs"], fx["material_ids"], mats, tex,
                              cam, w, h, spp, depth, [("all", 0, 0, n)])


def make_one(name: str) -> None:
    if name in DEEP:
        make_deep(name)
        return
    import oracle
    from cudart_gb300 import scenes
    factory, n_rays, box, n_samples, stats_spp, stats_px = _configs()[name]
    sc = factory()
    out = scene_arrays(sc)
    with tempfile.TemporaryDirectory() as td:
        files = scenes.write_reference_files(sc, td, name)
        R = oracle.RefHarness(files, sc.width, sc.height)
        e = R.export()
        for k, v in e.items():
            out["ref_" + k] = v
        out["ref_bvh_depth"] = np.int32(R.bvh_depth)
        rng = np.random.default_rng(SEED)
        rays = np.zeros((n_rays, 8), np.float32)
        rays[:, :3] = rng.uniform(-box, box, (n_rays, 3))
        d = rng.normal(size=(n_rays, 3))
        rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
        rays[:, 3] = 1e-5
        rays[:, 7] = np.finfo(np.float32).max
        idx, t, uv = R.closest_hit(rays)
        out.update(rays=rays, ref_hit_idx=idx, ref_hit_t=t, ref_hit_uv=uv)
        out["ref_gamma"] = R.gamma_table()
        if n_samples:
            xs = rng.integers(0, sc.width, n_samples)
            ys = rng.integers(0, sc.height, n_samples)
            ss = rng.integers(0, 1 << 16, n_samples)
            rgb = np.zeros((n_samples, 3), np.float32)
            draws = np.zeros(n_samples, np.int32)
            for k in range(n_samples):
                rgb[k], draws[k] = R.sample_pixel(int(xs[k]), int(ys[k]), SEED, int(ss[k]))
            out.update(sample_xys=np.stack([xs, ys, ss], 1).astype(np.int32), ref_sample_rgb=rgb,
                       ref_sample_draws=draws)
        if stats_spp:
            W, H = sc.width, sc.height
            if stats_px == "all":
                px = np.arange(W * H, dtype=np.uint32)
            else:
                cx, cy = W // 2 - 16, H // 2 - 16
                crop = np.array([(cy + j) * W + cx + i for j in range(32) for i in range(32)], np.uint32)
                extra = rng.choice(W * H, 512, replace=False).astype(np.uint32)
                px = np.unique(np.concatenate([crop, extra]))
            acc, mean, m2 = R.render(px, SEED, stats_spp)
            out.update(stats_pixels=px, stats_spp=np.int32(stats_spp), ref_stats_acc=acc,
                       ref_stats_mean=mean, ref_stats_m2=m2)
    out["seed"] = np.uint64(SEED)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def main() -> None:
    if "--one" in sys.argv:
        make_one(sys.argv[sys.argv.index("--one") + 1])
        return
    import oracle
    oracle.build()
    if not os.path.exists(oracle.REF_LIB_PATH):
        raise SystemExit("reference harness not built (needs the CudaRT sources)")
    for name in list(_configs()) + list(DEEP):
        subprocess.check_call([sys.executable, __file__, "--one", name], stdout=subprocess.DEVNULL)
        print("wrote", name)


if __name__ == "__main__":
    main()

"""Algorithmic bytes per ray: the reference's BVH layout against this
library's, on the same seeded rays of the two headline scenes.

Reference side: the oracle's restatement of the reference's binary tree
(bvh.cpp) and of intersectBVH (renderer.cu:283-330: every popped node's box
tested against the infinite line), fetching a 40-byte node per visit and a
128-byte triangle line per test (Triangle is 128-byte aligned,
geometry.h:30-51).  Library side: crt_trace_counts over the 8-wide tree,
80-byte (8-bit planes) or 208-byte (FP32 planes) nodes and 48-byte
triangle records.

Three ray families of 20,000 rays each: eye to uniform surface points;
surface points into their face's hemisphere; surface points towards a
light, clipped just short of it.  The test prints one JSON line per scene
and family (run with -s) and requires the library's layout to fetch fewer
bytes per ray than the reference's on every family.
"""
import json

import numpy as np
import pytest

import oracle
from cudart_gb300 import GB300Scene, scenes

pytestmark = pytest.mark.gpu

REF_NODE_B, REF_TRI_B = 40, 128
NODE_B = {"q8": 80, "f32": 208}
TRI_B = 48


def ray_families(sc, seed: int, n: int) -> dict:
    rng = np.random.default_rng(seed)

    def surface(k):
        f = rng.integers(0, sc.n_tris, k)
        p = sc.positions[f].astype(np.float64)
        s = np.sqrt(rng.random(k))
        r2 = rng.random(k)
        w = np.stack([1 - s, s * (1 - r2), s * r2], 1)
        nrm = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
        nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-30)
        return np.einsum("nk,nkc->nc", w, p), nrm

    def pack(o, d, tmin, tmax):
        r = np.zeros((len(d), 8), np.float32)
        r[:, :3], r[:, 4:7], r[:, 3], r[:, 7] = o, d, tmin, tmax
        return r

    fmax = np.finfo(np.float32).max
    eye = np.asarray(sc.camera.eye, np.float64)
    tgt, _ = surface(n)
    d = tgt - eye
    out = {"eye_to_surface": pack(np.broadcast_to(eye, (n, 3)), d / np.linalg.norm(d, axis=1, keepdims=True),
                                  1e-5, fmax)}
    o, nrm = surface(n)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d *= np.where(np.sum(d * nrm, 1) < 0, -1.0, 1.0)[:, None]
    out["surface_hemisphere"] = pack(o, d, 1e-4, fmax)
    o, _ = surface(n)
    lights = sc.light_indices()
    lp = sc.positions[lights[rng.integers(0, len(lights), n)]].astype(np.float64).mean(axis=1)
    d = lp - o
    dist = np.linalg.norm(d, axis=1)
    out["surface_to_light"] = pack(o, d / dist[:, None], 1e-4, dist * 0.999)
    return out


@pytest.mark.parametrize("scene", ["large_textured", "mixed_mid"])
def test_library_layout_fetches_fewer_bytes_than_the_reference(cuda, scene):
    torch = cuda
    sc = getattr(scenes, scene)()
    o = oracle.OracleScene(sc)
    gs = {fmt: GB300Scene(sc, node_format=fmt) for fmt in NODE_B}
    fams = ray_families(sc, 7, 20000)
    fams["all"] = np.concatenate(list(fams.values()))
    for name, rays in fams.items():
        rnv, rnt = o.traversal_counts(rays)
        ref_b = REF_NODE_B * rnv.mean() + REF_TRI_B * rnt.mean()
        row = {"scene": scene, "rays": name, "n": len(rays),
               "reference": {"nodes_per_ray": round(float(rnv.mean()), 2),
                             "tris_per_ray": round(float(rnt.mean()), 2),
                             "bytes_per_ray": round(float(ref_b), 1)}}
        for fmt, nb in NODE_B.items():
            nodes, tris = gs[fmt].trace_counts(torch.from_numpy(rays).cuda())
            gnv = nodes.cpu().numpy().astype(np.float64)
            gnt = tris.cpu().numpy().astype(np.float64)
            b = nb * gnv.mean() + TRI_B * gnt.mean()
            row[fmt] = {"nodes_per_ray": round(float(gnv.mean()), 2), "tris_per_ray": round(float(gnt.mean()), 2),
                        "bytes_per_ray": round(float(b), 1), "reference_over_this": round(float(ref_b / b), 2)}
            assert b < ref_b, row
        print(json.dumps(row), flush=True)

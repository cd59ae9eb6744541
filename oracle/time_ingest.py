"""Times scene-file loading on the host: the reference's loader (Scene::loadObj,
loadCamera, loadTextures, loadTriangles through oracle/_ref/libcrt_ref.so)
against the library's crt_scene_files_load + crt_camera_load_json, on the
same files.  TEST INFRASTRUCTURE: runs where the CudaRT sources are (the
reference side needs oracle/_ref); the library side alone runs anywhere.

    python oracle/time_ingest.py --scene mixed_mid [--no-ref] [--repeats 3]

Prints one JSON line.  Each reference load runs in a process of its own
(the reference keeps loader state in static variables).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)


def _ref_once(obj: str, cam: str, tex: str, w: int, h: int) -> float:
    L = C.CDLL(os.path.join(HERE, "_ref", "libcrt_ref.so"))
    L.ref_time_load.restype = C.c_double
    L.ref_time_load.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int]
    return float(L.ref_time_load(obj.encode(), cam.encode(), tex.encode(), w, h))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--scene", default="mixed_mid")
    ap.add_argument("--repeats", type=int, default=3)
    ap.add_argument("--no-ref", action="store_true")
    ap.add_argument("--ref-once", nargs=5, help=argparse.SUPPRESS)
    a = ap.parse_args()
    if a.ref_once:
        obj, cam, tex, w, h = a.ref_once
        print(_ref_once(obj, cam, tex, int(w), int(h)))
        return
    from cudart_gb300 import SceneFiles, load_camera_json, scenes
    sc = getattr(scenes, a.scene)()
    with tempfile.TemporaryDirectory() as td:
        t = time.time()
        files = scenes.write_reference_files(sc, td, a.scene)
        write_s = time.time() - t
        obj_bytes = os.path.getsize(files["obj"])
        lib_ms, parse_ms = [], []
        for _ in range(a.repeats):
            t = time.perf_counter()
            f = SceneFiles(files["obj"], files["textures"])
            load_camera_json(files["camera"], sc.width, sc.height)
            lib_ms.append((time.perf_counter() - t) * 1e3)
            parse_ms.append(float(f.info.parse_ms))
            assert f.n_tris == sc.n_tris
            f.close()
        ref_ms = None
        if not a.no_ref:
            p = subprocess.run([sys.executable, os.path.abspath(__file__), "--ref-once", files["obj"],
                                files["camera"], files["textures"], str(sc.width), str(sc.height)],
                               capture_output=True, text=True, check=True)
            ref_ms = float(p.stdout.strip().splitlines()[-1])
    out = {"scene": a.scene, "triangles": sc.n_tris, "obj_mb": round(obj_bytes / 1e6, 1),
           "library_ms": round(min(lib_ms), 1), "library_parse_ms": round(min(parse_ms), 1),
           "library_mb_per_s": round(obj_bytes / 1e3 / min(lib_ms), 1),
           "reference_ms": None if ref_ms is None else round(ref_ms, 1),
           "speedup": None if ref_ms is None else round(ref_ms / min(lib_ms), 1),
           "host_threads": os.cpu_count(), "write_s": round(write_s, 1)}
    print(json.dumps(out))


if __name__ == "__main__":
    main()

"""Generates tests/golden/ingest_cases.npz: small scene-file sets (OBJ, MTL,
camera JSON, PNG) that exercise the rules of the reference's loaders, each
with the state the reference's own Scene class made of them.

    python tests/golden/make_ingest_golden.py          # all cases
    python tests/golden/make_ingest_golden.py --one NAME DIR OUT   # one case (subprocess)

Needs the CudaRT sources (oracle/_ref/libcrt_ref.so, built by oracle/Makefile
`ref`).  The reference keeps its material map and list in static variables
(scene.cpp:24-25), so every case loads in a fresh process.  The files are
stored byte for byte in the fixture, so the tests replay exactly what the
reference read.

Every case is triangulated (the reference sizes its triangle array from the
vertex count, scene.h:27) and has at least one texture (its texture store
indexes the last texture's size, texture_store.cpp:68).
"""
from __future__ import annotations

import json
import os
import struct
import subprocess
import sys
import tempfile
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

OUT = os.path.join(HERE, "ingest_cases.npz")


# ---------------------------------------------------------------------------
# PNG writer with every filter type, palettes, 16-bit samples and Adam7
# ---------------------------------------------------------------------------
ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _filter_row(row: bytes, prev: bytes, bpp: int, ft: int) -> bytes:
    out = bytearray(len(row))
    for i in range(len(row)):
        a = row[i - bpp] if i >= bpp else 0
        b = prev[i] if prev else 0
        c = prev[i - bpp] if (prev and i >= bpp) else 0
        pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][ft]
        out[i] = (row[i] - pred) & 0xFF
    return bytes(out)


def _pack_row(samples: np.ndarray, depth: int) -> bytes:
    """samples: 1-D array of channel samples of one row."""
    if depth == 16:
        return samples.astype(">u2").tobytes()
    if depth == 8:
        return samples.astype(np.uint8).tobytes()
    per = 8 // depth
    out = bytearray((len(samples) * depth + 7) // 8)
    for i, v in enumerate(samples.tolist()):
        out[i // per] |= (int(v) & ((1 << depth) - 1)) << (8 - depth * (i % per + 1))
    return bytes(out)


def png_bytes(img: np.ndarray, color_type: int, depth: int = 8, palette=None, trns=None,
              interlace: bool = False, filters=(0, 1, 2, 3, 4), level: int = 6,
              strategy: int = zlib.Z_DEFAULT_STRATEGY) -> bytes:
    """img: [h, w, channels] samples (palette indices for colour type 3)."""
    h, w, ch = img.shape
    bpp = max(1, ch * depth // 8)
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    raw = bytearray()
    k = 0
    for x0, y0, dx, dy in passes:
        sub = img[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        prev = b""
        for y in range(sub.shape[0]):
            row = _pack_row(sub[y].reshape(-1), depth)
            ft = filters[k % len(filters)]
            k += 1
            raw += bytes([ft]) + _filter_row(row, prev, bpp, ft)
            prev = row
    z = zlib.compressobj(level, zlib.DEFLATED, 15, 9, strategy)
    data = z.compress(bytes(raw)) + z.flush()

    def chunk(tag, payload):
        return (struct.pack(">I", len(payload)) + tag + payload +
                struct.pack(">I", zlib.crc32(tag + payload) & 0xFFFFFFFF))

    out = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, color_type, 0, 0,
                                                            1 if interlace else 0))
    if palette is not None:
        out += chunk(b"PLTE", np.asarray(palette, np.uint8).tobytes())
    if trns is not None:
        out += chunk(b"tRNS", bytes(trns))
    # split the data over two IDAT chunks and add an ancillary chunk
    half = len(data) // 2
    out += chunk(b"tEXt", b"Comment\x00ingest fixture")
    out += chunk(b"IDAT", data[:half]) + chunk(b"IDAT", data[half:]) + chunk(b"IEND", b"")
    return out


def all_byte_values(h: int, w: int, ch: int, seed: int) -> np.ndarray:
    """[h, w, ch] uint8 whose every channel holds each value 0..255 (h*w >= 256)."""
    rng = np.random.default_rng(seed)
    img = np.zeros((h * w, ch), np.uint8)
    for c in range(ch):
        v = np.concatenate([np.arange(256), rng.integers(0, 256, h * w - 256)]).astype(np.uint8)
        img[:, c] = rng.permutation(v)
    return img.reshape(h, w, ch)


# ---------------------------------------------------------------------------
# cases
# ---------------------------------------------------------------------------
def _f(x: float) -> str:
    return repr(float(np.float32(x)))


def _quad_rows(p0, p1, p2, p3):
    return [p0, p1, p2, p0, p2, p3]


def case_obj_rules() -> dict:
    """Face forms, negative indices, grouping quirks and material merging."""
    rng = np.random.default_rng(11)
    L = []
    L += ["# header comment", "", "mtllib sub/rules.mtl"]
    # faces before the first group join the first mesh
    L += ["v -1 -1 -1", "v 1 -1 -1", "v 1 -1 1", "vt 0 0", "vt 1 0", "vt 1 1",
          "vn 0 1 0", "vn 0 1 0.0", "vn 0 1e0 0"]
    L += ["f 1/1/1 2/2/2 3/3/3"]
    L += ["o first", "usemtl red", "s off"]
    # P form: normals generated from the positions
    L += ["v -1 -1 1 1.0", "v -0.5 -1 1", "v -1 -0.5 1", "f -3 -2 -1"]
    # P/T form
    L += ["vt 0.25 0.75 0", "vt 0.5 0.5", "vt 0.75 0.25",
          "v -1 1 -1", "v -1 1 1", "v -1 -1 1", "f -3/-3 -2/-2 -1/-1"]
    # usemtl inside the group splits the mesh
    L += ["usemtl textured", "v 1 1 -1", "v 1 1 1", "v 1 -1 1", "vn 1 0 0",
          "f -3//-1 -2//-1 -1//-1", "f 4/4/4 5/5/4 6/6/4"]
    # a group without usemtl shifts the names of the following meshes
    L += ["g nomat", "v 0 -1 -1", "v 0.5 -1 -1", "v 0 -0.5 -1", "f -3/1/1 -2/2/2 -1/3/3"]
    L += ["g shares_kd", "usemtl blue_a", "v 0 0 -1", "v 0.5 0 -1", "v 0 0.5 -1", "f -3 -2 -1"]
    L += ["g shares_kd_too", "usemtl blue_b", "v 0 0 -0.5", "v 0.5 0 -0.5", "v 0 0.5 -0.5", "f -3 -2 -1"]
    # a line that only starts with 'g' opens a group
    L += ["group_like", "usemtl light", "v -0.25 0.99 -0.25", "v 0.25 0.99 -0.25", "v 0.25 0.99 0.25",
          "v -0.25 0.99 0.25", "vn 0 -1 0", "f -4//-1 -3//-1 -2//-1", "f -4//-1 -2//-1 -1//-1"]
    L += ["g dup_names", "usemtl twice", "v 0.2 0.2 0.2", "v 0.4 0.2 0.2", "v 0.2 0.4 0.2", "f -3 -2 -1"]
    L += ["g glass", "usemtl glass"]
    for k in range(8):   # a small fan of random triangles with their own normals
        c = rng.uniform(-0.8, 0.8, 3)
        for j in range(3):
            p = c + rng.uniform(-0.1, 0.1, 3)
            L.append("v " + " ".join(_f(x) for x in p))
        n = rng.normal(size=3)
        L.append("vn " + " ".join(_f(x) for x in n))
        L.append("f -3//-1 -2//-1 -1//-1")
    L += ["g unknown_type", "usemtl plastic", "v 0.6 0.6 0.6", "v 0.7 0.6 0.6", "v 0.6 0.7 0.6",
          "f -3 -2 -1"]
    L += ["g missing_material", "usemtl no_such_material", "v -0.6 0.6 0.6", "v -0.7 0.6 0.6",
          "v -0.6 0.7 0.6", "f -3 -2 -1"]
    obj = "\n".join(L) + "\n"
    M = []
    M += ["# materials", "newmtl red", "Kd 0.63 0.065 0.05", "Ka 0 0 0", "Ks 0 0 0", "Ns 10", "Ni 1",
          "illum 2", "d 1", "type LAMBERT"]
    M += ["newmtl textured", "Kd 0.5 0.5 0.5", "Ni 1", "type LAMBERT", "map_Kd tex_rgb.png",
          "map_Bump ignored.png"]
    M += ["newmtl only_listed", "Kd 0.3 0.3 0.3", "Ni 1", "map_Kd tex_palette.png"]
    M += ["newmtl blue_a", "Kd 0.1 0.2 0.9", "Ni 1", "type LAMBERT"]
    M += ["newmtl blue_b", "Kd 0.1 0.4 0.7", "Ni 1", "type LAMBERT", "map_Kd tex_rgba16.png"]
    M += ["newmtl light", "Kd 0 0 0", "Ka 5.6666665 4 1.3333334", "Ni 1", "type EMISSIVE"]
    M += ["newmtl twice", "Kd 0.9 0.1 0.1", "Ni 1", "type SPECULAR", "Ks 0.95 0.95 0.95"]
    M += ["newmtl twice", "Kd 0.1 0.9 0.1", "Ni 1", "type LAMBERT"]
    M += ["newmtl glass", "Kd 0 0 0", "Ks 1 1 1", "Ni 1.5", "type REFRACTIVE", "map_Kd tex_interlaced.png"]
    # Kd with one value and Ka with four are skipped; unknown type -> diffuse
    M += ["newmtl plastic", "Kd 0.2 0.6 0.2", "Kd 0.7", "Ka 1 1 1 1", "Ks 0.25 0.25 0.25", "Ns 32",
          "Ni 1.45", "type PLASTIC", "diffuse 0.75"]
    M += ["newmtl ds", "Kd 0.2 0.3 0.8", "Ks 0.9 0.9 0.9", "Ni 1", "type DIFFSPEC", "diffuse 0.6"]
    mtl = "\n".join(M) + "\n"
    pal = np.random.default_rng(5).integers(0, 256, (256, 3))
    files = {
        "rules.obj": obj.encode(),
        "sub/rules.mtl": mtl.encode(),
        "rules-camera.json": json.dumps({
            "upDirection": [0, 2, 0.0], "eye": [0.0, 0.0, 3.9], "fieldOfView": 40,
            "viewDirection": [0, 0, -1], "focalLength": 0, "fStop": 1.0}).encode(),
        "textures/tex_rgb.png": png_bytes(all_byte_values(16, 16, 3, 1), 2),
        "textures/tex_palette.png": png_bytes(np.random.default_rng(2).integers(0, 256, (16, 20, 1)), 3,
                                              palette=pal),
        "textures/tex_rgba16.png": png_bytes(np.random.default_rng(3).integers(0, 65536, (9, 13, 4)), 6,
                                             depth=16, filters=(4, 3, 2, 1, 0)),
        "textures/tex_interlaced.png": png_bytes(all_byte_values(17, 19, 4, 4), 6, interlace=True,
                                                 strategy=zlib.Z_FIXED),
    }
    return dict(files=files, obj="rules.obj", camera="rules-camera.json", textures="textures/",
                width=64, height=48)


def case_plain_groups() -> dict:
    """usemtl only (no o/g), CRLF-free, a texture in the OBJ's own folder,
    low-bit-depth palette PNG, and a thin-lens camera."""
    rng = np.random.default_rng(21)
    L = ["mtllib plain.mtl"]
    mats = ["floor", "light", "tex", "floor"]
    base = 1
    for m in mats:
        L.append(f"usemtl {m}")
        for k in range(6):
            c = rng.uniform(-1, 1, 3)
            for j in range(3):
                L.append("v " + " ".join(_f(x) for x in c + rng.uniform(-0.2, 0.2, 3)))
                L.append("vt " + " ".join(_f(x) for x in rng.uniform(0, 1, 2)))
                L.append("vn " + " ".join(_f(x) for x in rng.normal(size=3)))
            L.append(f"f {base}/{base}/{base} {base + 1}/{base + 1}/{base + 1} {base + 2}/{base + 2}/{base + 2}")
            base += 3
    M = ["newmtl floor", "Kd 0.725 0.71 0.68", "Ni 1", "type LAMBERT",
         "newmtl light", "Ka 2 3 5", "Ni 1", "type EMISSIVE",
         "newmtl tex", "Kd 1 1 1", "Ni 1", "type LAMBERT", "map_Kd p4.png"]
    pal = np.random.default_rng(6).integers(0, 256, (16, 3))
    files = {
        "plain.obj": ("\n".join(L) + "\n").encode(),
        "plain.mtl": ("\n".join(M) + "\n").encode(),
        "plain-camera.json": b'{\n  "fieldOfView" : 5.5e1, "focalLength": 35, "fStop": 2.8,\n'
                             b'  "eye": [ 1.5, -0.25, 4 ], "viewDirection": [-0.5, 0.1, -4.5],\n'
                             b'  "upDirection": [0.1, 1, 0], "note": {"a": [1, "x\\u0041"]}\n}\n',
        "tex/p4.png": png_bytes(np.random.default_rng(7).integers(0, 16, (11, 23, 1)), 3, depth=4,
                                palette=pal, level=0),
    }
    return dict(files=files, obj="plain.obj", camera="plain-camera.json", textures="tex/",
                width=40, height=30)


CASES = {"obj_rules": case_obj_rules, "plain_groups": case_plain_groups}


def write_case(case: dict, out_dir: str) -> dict:
    for rel, data in case["files"].items():
        path = os.path.join(out_dir, rel)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "wb") as f:
            f.write(data)
    return {"obj": os.path.join(out_dir, case["obj"]), "camera": os.path.join(out_dir, case["camera"]),
            "textures": os.path.join(out_dir, case["textures"])}


def run_one(name: str, out_dir: str, out_file: str) -> None:
    import oracle
    case = CASES[name]()
    paths = write_case(case, out_dir)
    R = oracle.RefHarness(paths, case["width"], case["height"])
    e = R.export()
    np.savez(out_file, **{k: np.asarray(v) for k, v in e.items()})


def main() -> None:
    if len(sys.argv) > 1 and sys.argv[1] == "--one":
        run_one(sys.argv[2], sys.argv[3], sys.argv[4])
        return
    out = {}
    for name, make in CASES.items():
        case = make()
        with tempfile.TemporaryDirectory() as td:
            res = os.path.join(td, "ref.npz")
            subprocess.run([sys.executable, os.path.abspath(__file__), "--one", name, os.path.join(td, "files"),
                            res], check=True, stdout=subprocess.DEVNULL)
            ref = dict(np.load(res))
        index = {"obj": case["obj"], "camera": case["camera"], "textures": case["textures"],
                 "width": case["width"], "height": case["height"], "files": sorted(case["files"])}
        out[f"{name}.index"] = np.frombuffer(json.dumps(index).encode(), np.uint8)
        for i, rel in enumerate(sorted(case["files"])):
            out[f"{name}.file{i}"] = np.frombuffer(case["files"][rel], np.uint8)
        for k, v in ref.items():
            out[f"{name}.ref_{k}"] = v
        print(name, "triangles", len(ref["mat_ids"]), "materials", len(ref["mat_floats"]))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


def load_cases(path: str = OUT) -> dict:
    """name -> {"index": dict, "files": {rel: bytes}, "ref": {key: array}}"""
    fx = np.load(path)
    cases = {}
    for key in fx.files:
        name, field = key.split(".", 1)
        c = cases.setdefault(name, {"files": {}, "ref": {}})
        if field == "index":
            c["index"] = json.loads(fx[key].tobytes().decode())
    for name, c in cases.items():
        for i, rel in enumerate(c["index"]["files"]):
            c["files"][rel] = fx[f"{name}.file{i}"].tobytes()
        for key in fx.files:
            if key.startswith(name + ".ref_"):
                c["ref"][key[len(name) + 5:]] = fx[key]
    return cases


if __name__ == "__main__":
    main()

"""The library's scene-file readers (OBJ/MTL, camera JSON, PNG) against what
the reference's own loaders made of the same files, plus the readers' own
rules where the reference has none (no GPU needed).

Fixtures: tests/golden/ingest_cases.npz (edge-case file sets, stored byte
for byte, with the reference's Scene state; tests/golden/
make_ingest_golden.py) and the scene fixtures of make_golden.py, whose files
the scene generators rewrite identically.
"""
import ctypes as C
import json
import os
import struct
import zlib

import numpy as np
import pytest

from golden.make_golden import _configs
from golden.make_ingest_golden import _paeth, load_cases, png_bytes, write_case
from cudart_gb300 import CrtError, SceneFiles, load_camera_json, load_png_texels, scenes, write_png

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
LUT = scenes.texel_table()


def _camera_row(cam) -> np.ndarray:
    return np.array(list(cam.eye) + list(cam.dir) + list(cam.up) + list(cam.right) +
                    [cam.fov, cam.aspect, cam.aperture, cam.focus], np.float32)


def check_against_reference(f: SceneFiles, ref: dict, camera=None) -> None:
    """Every array the reference's Scene holds after loading, compared
    exactly (the light order and the light area's summation order follow
    the reference's BVH, so those compare as a set and to a few ulps)."""
    rt = ref["tris"]
    assert f.n_tris == len(rt)
    p = f.positions
    assert np.array_equal(p[:, 0], rt[:, 0:3])
    assert np.array_equal(p[:, 1] - p[:, 0], rt[:, 3:6])
    assert np.array_equal(p[:, 2] - p[:, 0], rt[:, 6:9])
    assert np.array_equal(f.normals.reshape(-1, 9), rt[:, 9:18])
    assert np.array_equal(f.uvs.reshape(-1, 6), rt[:, 18:24])
    assert np.array_equal(f.material_ids, ref["mat_ids"])
    mf, mi = ref["mat_floats"], ref["mat_ints"]
    assert len(f.materials) == len(mf)
    kd = np.array([m.kd for m in f.materials], np.float32)
    ka = np.array([m.ka for m in f.materials], np.float32)
    ks = np.array([m.ks for m in f.materials], np.float32)
    s3 = np.array([[m.ns, m.ni, m.diffuse] for m in f.materials], np.float32)
    ints = np.array([[m.bsdf, m.tex] for m in f.materials], np.int32)
    area = np.float32(ref["lights_area"])
    assert np.array_equal(kd, mf[:, 0:3])
    assert np.array_equal((ka * np.float32(3.0)) * area, mf[:, 3:6])   # scene.cpp:163,177
    assert np.array_equal(ks, mf[:, 6:9])
    assert np.array_equal(s3, mf[:, 9:12])
    assert np.array_equal(ints, mi)
    lights = f.light_indices()
    assert sorted(lights.tolist()) == sorted(ref["lights"].tolist())
    e = (p[:, 1] - p[:, 0]).astype(np.float32), (p[:, 2] - p[:, 0]).astype(np.float32)
    c = np.cross(e[0].astype(np.float64), e[1].astype(np.float64))
    mine = np.float32(np.sum(np.sqrt((c * c).sum(1))[lights] / 2)) if len(lights) else np.float32(0)
    assert abs(float(mine) - float(area)) <= 1e-5 * max(1.0, float(area))
    n = len(f.texels)
    assert np.array_equal(f.texels, ref["tex_data"][:n])
    assert np.array_equal(f.texture_dims.reshape(-1), ref["tex_dims"])
    if camera is not None:
        assert np.array_equal(_camera_row(camera), ref["camera"])


CASES = load_cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_edge_cases_match_reference(name, tmp_path):
    case = CASES[name]
    idx = case["index"]
    paths = write_case({**idx, "files": case["files"]}, str(tmp_path))
    f = SceneFiles(paths["obj"], paths["textures"])
    cam = load_camera_json(paths["camera"], idx["width"], idx["height"])
    check_against_reference(f, case["ref"], cam)


@pytest.mark.parametrize("name", ["cornell_512", "feature_mix", "mixed_sub2"])
def test_scene_fixtures_match_reference(name, tmp_path):
    fx = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    sc = _configs()[name][0]()
    assert np.array_equal(sc.positions, fx["positions"])    # the generator is unchanged
    files = scenes.write_reference_files(sc, str(tmp_path), name)
    f = SceneFiles(files["obj"], files["textures"])
    cam = load_camera_json(files["camera"], int(fx["ref_pixels"][0]), int(fx["ref_pixels"][1]))
    ref = {k[4:]: v for k, v in fx.items() if k.startswith("ref_")}
    check_against_reference(f, ref, cam)


def test_mesh_grouping_follows_the_reference(tmp_path):
    case = CASES["obj_rules"]
    idx = case["index"]
    paths = write_case({**idx, "files": case["files"]}, str(tmp_path))
    f = SceneFiles(paths["obj"], paths["textures"])
    meshes = f.meshes()
    assert sum(c for _, _, c in meshes) == f.n_tris
    assert [m[1] for m in meshes] == sorted(m[1] for m in meshes)
    assert f.info.num_mtl_materials == 11 and f.info.num_textures == 4
    assert f.info.num_polygons == 0


def test_exact_materials(tmp_path):
    case = CASES["obj_rules"]
    idx = case["index"]
    paths = write_case({**idx, "files": case["files"]}, str(tmp_path))
    merged = SceneFiles(paths["obj"], paths["textures"])
    exact = SceneFiles(paths["obj"], paths["textures"], exact_materials=True)
    assert len(exact.materials) > len(set(merged.material_ids.tolist()))
    # same geometry; every face keeps its own MTL values
    assert np.array_equal(exact.positions, merged.positions)
    kd_exact = np.array([exact.materials[i].kd for i in exact.material_ids], np.float64)
    kd_merged = np.array([merged.materials[i].kd for i in merged.material_ids], np.float64)
    assert not np.array_equal(kd_exact, kd_merged)     # blue_b keeps its own kd
    assert {tuple(np.round(k, 6)) for k in kd_exact} >= {(0.1, 0.4, 0.7)}


# ---------------------------------------------------------------------------
# OBJ rules without a reference counterpart
# ---------------------------------------------------------------------------
def _write(tmp_path, obj: str, mtl: str = "newmtl m\nKd 0.5 0.5 0.5\nNi 1\n", name="s"):
    (tmp_path / f"{name}.obj").write_text(obj)
    (tmp_path / f"{name}.mtl").write_text(mtl)
    return str(tmp_path / f"{name}.obj")


def test_polygons_are_fanned(tmp_path):
    obj = ("mtllib s.mtl\nusemtl m\nv 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv -1 0.5 0\n"
           "vn 0 0 1\nf 1//1 2//1 3//1 4//1 5//1\nf 1 2 3\n")
    f = SceneFiles(_write(tmp_path, obj))
    assert f.n_tris == 4 and f.info.num_polygons == 1
    v = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [-1, 0.5, 0]], np.float32)
    assert np.array_equal(f.positions[:3], np.stack([v[[0, 1, 2]], v[[0, 2, 3]], v[[0, 3, 4]]]))
    assert np.array_equal(f.normals[:3], np.tile(np.float32([0, 0, 1]), (3, 3, 1)))
    # no normals: (p0 - p1) x (p2 - p1), unnormalised, on every vertex
    assert np.array_equal(f.normals[3], np.tile(np.float32([0, 0, -1]), (3, 1)))


def test_numbers_parse_like_strtof(tmp_path):
    libc = C.CDLL(None)
    libc.strtof.restype = C.c_float
    libc.strtof.argtypes = [C.c_char_p, C.c_void_p]
    rng = np.random.default_rng(0)
    toks = ["0", "-0", "+2", ".5", "5.", "1e-3", "-1.5E+2", "0x1p-2", "3.4028234e38", "1.17549435e-38",
            "0.1000000000000000055511151231257827", "2.00000011920928955078125"]
    for _ in range(600):
        digits = "".join(rng.choice(list("0123456789"), rng.integers(1, 24)))
        toks.append(f"{rng.choice(['', '-'])}{digits[:3]}.{digits[3:]}e{rng.integers(-30, 30)}")
    n = (len(toks) + 2) // 3
    toks += ["0"] * (3 * n - len(toks))
    lines = ["mtllib s.mtl", "usemtl m"]
    for i in range(n):
        lines.append("v " + " ".join(toks[3 * i:3 * i + 3]))
    for i in range(n):
        lines.append(f"f {i + 1} {i + 1} {i + 1}")
    f = SceneFiles(_write(tmp_path, "\n".join(lines) + "\n"))
    want = np.array([libc.strtof(t.encode(), None) for t in toks], np.float32).reshape(n, 3)
    assert np.array_equal(f.positions[:, 0].view(np.uint32), want.view(np.uint32))


def test_vertex_forms_and_negative_indices(tmp_path):
    obj = ("mtllib s.mtl\nusemtl m\nv 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0.25 0.5\nvt 0.5\nvn 0 0 1\n"
           "f 1/1/1 2/2/1 3//1\nf -3/-2 -2/-1/ -1\n")
    f = SceneFiles(_write(tmp_path, obj))
    assert np.array_equal(f.uvs[0], np.float32([[0.25, 0.5], [0.5, 0], [0, 0]]))
    assert np.array_equal(f.uvs[1], np.float32([[0.25, 0.5], [0.5, 0], [0, 0]]))
    assert np.array_equal(f.normals[0], np.tile(np.float32([0, 0, 1]), (3, 1)))
    # face 2 lacks normals: (p0 - p1) x (p2 - p1) = (0, 0, -1)
    assert np.array_equal(f.normals[1], np.tile(np.float32([0, 0, -1]), (3, 1)))


@pytest.mark.parametrize("obj,needle", [
    ("mtllib s.mtl\nv 0 0 0\nv 1 0 0\nf 1 2 3\n", "bad face vertex"),
    ("mtllib s.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2\n", "fewer than 3"),
    ("mtllib s.mtl\nv 0 0 0\nv 1 0 zz\nv 0 1 0\nf 1 2 3\n", "bad number"),
    ("mtllib s.mtl\nv 0 0\nf 1 1 1\n", "too few values"),
    ("mtllib s.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1/1 2/1 3/1\n", "bad face vertex"),
    ("mtllib s.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 0 1 2\n", "bad face vertex"),
    ("mtllib missing.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n", "cannot open"),
    ("mtllib s.mtl\nv 0 0 0\n", "no faces"),
])
def test_malformed_obj_is_an_error(tmp_path, obj, needle):
    with pytest.raises(CrtError, match=needle) as e:
        SceneFiles(_write(tmp_path, obj))
    assert e.value.status == 1


def test_error_names_the_line(tmp_path):
    body = "mtllib s.mtl\n" + "v 0 0 0\n" * 5000 + "v 1 x 0\n" + "f 1 2 3\n"
    with pytest.raises(CrtError, match=r"s\.obj:5002: bad number"):
        SceneFiles(_write(tmp_path, body))


def test_not_an_obj_and_missing_texture(tmp_path):
    with pytest.raises(CrtError, match="not a .obj"):
        SceneFiles(str(tmp_path / "scene.txt"))
    obj = "mtllib s.mtl\nusemtl m\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n"
    with pytest.raises(CrtError, match="cannot open"):
        SceneFiles(_write(tmp_path, obj, "newmtl m\nmap_Kd nothere.png\n"), str(tmp_path))


def test_large_file_parses_in_parallel(tmp_path):
    """Enough lines for many parse chunks; the result is the written arrays."""
    sc = scenes.mixed_mid(width=64, height=48, subdiv=4)
    files = scenes.write_reference_files(sc, str(tmp_path), "big")
    f = SceneFiles(files["obj"], files["textures"])
    assert f.n_tris == sc.n_tris and f.info.file_bytes > (8 << 20)
    assert np.array_equal(f.positions, sc.positions)
    assert np.array_equal(f.normals, sc.normals)
    assert np.array_equal(f.uvs, sc.uvs)
    names = [m.name for m in sc.materials]
    kd_file = np.array([f.materials[i].kd for i in f.material_ids], np.float32)
    kd_src = np.array([sc.materials[i].kd for i in sc.material_ids], np.float32)
    assert np.array_equal(kd_file, kd_src) and len(names) >= len(f.materials)


# ---------------------------------------------------------------------------
# camera JSON
# ---------------------------------------------------------------------------
def test_camera_matches_camera_from_json(tmp_path):
    from cudart_gb300 import camera_from_json
    spec = scenes.CameraSpec(37.5, (0.1, 1.2, 3.9), (0.0, -0.1, -1.0), (0.0, 1.0, 0.1), 50.0, 4.0)
    p = tmp_path / "c.json"
    p.write_text(json.dumps({"fieldOfView": spec.fov_deg, "focalLength": spec.focal_length,
                             "fStop": spec.fstop, "eye": list(spec.eye),
                             "viewDirection": list(spec.view_dir), "upDirection": list(spec.up)}))
    a = load_camera_json(str(p), 320, 200)
    b = camera_from_json(spec, 320, 200)
    assert _camera_row(a).tobytes() == _camera_row(b).tobytes()
    assert (a.xpixels, a.ypixels) == (320, 200)


@pytest.mark.parametrize("text,needle", [
    ('{"fieldOfView": 40}', "focalLength"),
    ('{"fieldOfView": 40, "focalLength": 0, "fStop": 1, "eye": [0, 0], "viewDirection": [0,0,-1],'
     ' "upDirection": [0,1,0]}', "eye"),
    ('{"fieldOfView": "40"}', "fieldOfView"),
    ('[1, 2, 3]', "not a JSON object"),
    ('{"fieldOfView": 40,}', "expected a string"),
    ('{"a": 1} x', "trailing"),
    ('{"a": 1e999}', "out of range"),
])
def test_bad_camera_json_is_an_error(tmp_path, text, needle):
    p = tmp_path / "c.json"
    p.write_text(text)
    with pytest.raises(CrtError, match=needle):
        load_camera_json(str(p), 64, 64)


# ---------------------------------------------------------------------------
# PNG in and out
# ---------------------------------------------------------------------------
def _expect_rgb(img: np.ndarray, ctype: int, depth: int, palette=None) -> np.ndarray:
    """8-bit rgb the decoder must produce (stb_image's rules; grey replicated)."""
    if ctype == 3:
        return np.asarray(palette, np.uint8)[img[..., 0]]
    v = img.astype(np.int64)
    if depth == 16:
        v = v >> 8
    elif depth < 8:
        v = v * (255 // ((1 << depth) - 1))
    v = v.astype(np.uint8)
    if ctype in (0, 4):
        return np.repeat(v[..., :1], 3, axis=2)
    return v[..., :3]


PNG_KINDS = [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2), (3, 4), (3, 8),
             (4, 8), (4, 16), (6, 8), (6, 16)]


@pytest.mark.parametrize("ctype,depth", PNG_KINDS)
@pytest.mark.parametrize("interlace", [False, True])
def test_png_decoder(tmp_path, ctype, depth, interlace):
    rng = np.random.default_rng(ctype * 100 + depth + 7 * interlace)
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    h, w = 13, 29
    pal = None
    if ctype == 3:
        n = 1 << depth
        pal = rng.integers(0, 256, (n, 3))
        img = rng.integers(0, n, (h, w, 1))
    else:
        img = rng.integers(0, 1 << depth, (h, w, ch))
    for level, strategy in [(0, zlib.Z_DEFAULT_STRATEGY), (9, zlib.Z_DEFAULT_STRATEGY), (6, zlib.Z_FIXED),
                            (1, zlib.Z_HUFFMAN_ONLY), (6, zlib.Z_RLE)]:
        p = tmp_path / f"t{level}{strategy}.png"
        p.write_bytes(png_bytes(img, ctype, depth, palette=pal, interlace=interlace, level=level,
                                strategy=strategy))
        got = load_png_texels(str(p))
        assert got.shape == (h, w, 3)
        assert np.array_equal(got, LUT[_expect_rgb(img, ctype, depth, pal)])


def test_png_long_matches_and_large_image(tmp_path):
    img = np.zeros((300, 517, 4), np.uint8)
    img[:, :, 0] = np.arange(517)[None, :] % 7
    img[100:200] = np.random.default_rng(1).integers(0, 256, (100, 517, 4))
    p = tmp_path / "big.png"
    p.write_bytes(png_bytes(img, 6, level=9))
    assert np.array_equal(load_png_texels(str(p)), LUT[img[..., :3]])


@pytest.mark.parametrize("mutate,needle", [
    (lambda b: b[:8] + b"\xff" + b[9:], "truncated PNG chunk"),
    (lambda b: b"GIF89a" + b[6:], "not a PNG"),
    (lambda b: b[:60], "PNG without IHDR or IDAT|truncated"),
])
def test_broken_png_is_an_error(tmp_path, mutate, needle):
    good = png_bytes(np.random.default_rng(0).integers(0, 256, (8, 8, 3)), 2)
    p = tmp_path / "bad.png"
    p.write_bytes(mutate(good))
    with pytest.raises(CrtError, match=needle):
        load_png_texels(str(p))


def test_png_bad_filter_and_short_data(tmp_path):
    w, h = 4, 2
    for raw, needle in [(b"\x05" + bytes(12) + b"\x00" + bytes(12), "filter"),
                        (b"\x00" + bytes(12), "wrong size")]:
        def chunk(tag, payload):
            return (struct.pack(">I", len(payload)) + tag + payload +
                    struct.pack(">I", zlib.crc32(tag + payload) & 0xFFFFFFFF))
        data = (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)) +
                chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))
        p = tmp_path / "x.png"
        p.write_bytes(data)
        with pytest.raises(CrtError, match=needle):
            load_png_texels(str(p))


def _decode_rgba_png(data: bytes) -> np.ndarray:
    """Independent reader for the writer's output (zlib + unfilter in Python)."""
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", None, None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        assert crc == zlib.crc32(tag + body) & 0xFFFFFFFF
        if tag == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert (depth, ctype) == (8, 6)
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    stride = 4 * w
    out = np.zeros((h, stride), np.uint8)
    for y in range(h):
        ft, row = raw[y * (stride + 1)], raw[y * (stride + 1) + 1:(y + 1) * (stride + 1)]
        prev = out[y - 1] if y else np.zeros(stride, np.uint8)
        cur = out[y]
        for i in range(stride):
            a = int(cur[i - 4]) if i >= 4 else 0
            b = int(prev[i])
            c = int(prev[i - 4]) if i >= 4 else 0
            pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][ft]
            cur[i] = (row[i] + pred) & 0xFF
    return out.reshape(h, w, 4)


def test_png_writer_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    img = np.zeros((37, 53, 4), np.uint8)
    img[..., 3] = 255
    img[:20] = rng.integers(0, 256, (20, 53, 4))
    img[20:, :, :3] = np.arange(53, dtype=np.uint8)[None, :, None] * 4
    p = tmp_path / "out.png"
    write_png(str(p), img)
    assert np.array_equal(_decode_rgba_png(p.read_bytes()), img)
    assert np.array_equal(load_png_texels(str(p)), LUT[img[..., :3]])
    assert p.stat().st_size < img.nbytes   # the smooth half compresses


def test_texel_table_pins_every_byte_value():
    """The rgb test texture of the reference fixture holds every byte value in
    every channel, so its reference texels pin the whole conversion table."""
    case = CASES["obj_rules"]
    ref = case["ref"]
    w, h = (int(x) for x in ref["tex_dims"][:2])
    tex = ref["tex_data"][:w * h]
    from golden.make_ingest_golden import all_byte_values
    img = all_byte_values(16, 16, 3, 1).reshape(-1, 3)
    assert (w, h) == (16, 16)
    assert np.array_equal(tex, LUT[img])
    assert len(np.unique(img[:, 0])) == 256


# ---------------------------------------------------------------------------
# C ABI argument checks (no GPU)
# ---------------------------------------------------------------------------
def test_c_abi_argument_errors(tmp_path):
    from cudart_gb300 import load
    L = load()
    h = C.c_void_p()
    assert L.crt_scene_files_load(None, None, 0, C.byref(h)) == 1
    assert L.crt_scene_files_load(b"x.obj", None, 0, None) == 1
    obj = _write(tmp_path, "mtllib s.mtl\nusemtl m\nv 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    assert L.crt_scene_files_load(obj.encode(), None, 0x100, C.byref(h)) == 1      # unknown flag
    assert "unknown flags" in L.crt_last_error().decode()
    assert L.crt_scene_files_load(obj.encode(), None, 0, C.byref(h)) == 0
    assert L.crt_scene_files_desc(h, None) == 1
    assert L.crt_scene_files_get_info(None, None) == 1
    assert L.crt_scene_files_mesh(h, 99, None, None, None) == 1
    assert L.crt_scene_files_destroy(h) == 0
    assert L.crt_camera_load_json(None, 1, 1, None) == 1
    dims = (C.c_uint32 * 2)()
    png = tmp_path / "t.png"
    png.write_bytes(png_bytes(np.zeros((4, 5, 3), np.uint8), 2))
    assert L.crt_texture_load_png(str(png).encode(), dims, None, 0) == 0 and tuple(dims) == (5, 4)
    buf = np.zeros(3 * 20, np.float32)
    assert L.crt_texture_load_png(str(png).encode(), dims, buf.ctypes.data, 19) == 1   # too small
    assert L.crt_texture_load_png(str(png).encode(), dims, buf.ctypes.data, 20) == 0
    img = np.zeros((2, 2, 4), np.uint8)
    assert L.crt_image_write_png(str(tmp_path / "o.png").encode(), 0, 2, img.ctypes.data) == 1
    assert L.crt_image_write_png(str(tmp_path / "o.png").encode(), 1 << 20, 1 << 12, img.ctypes.data) == 6
    assert L.crt_image_write_png(str(tmp_path / "no" / "dir" / "o.png").encode(), 2, 2, img.ctypes.data) == 1

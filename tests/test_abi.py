"""The C ABI library loads, exports every symbol include/crt_gb300.h
declares, and rejects bad scene descriptions with status codes (host-side
validation runs before any device call, so these need no GPU)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from cudart_gb300 import _lib, scenes
from cudart_gb300._lib import CrtError

HEADER = os.path.join(ROOT, "include", "crt_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"CRT_EXPORT\s+[\w\s\*]+?\b(crt_\w+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    syms = declared_symbols()
    assert len(syms) >= 20
    lib = _lib.load()
    for s in syms:
        assert hasattr(lib, s), s
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (crt_\w+)", out))
    assert exported == set(syms), exported ^ set(syms)
    assert set(_lib.SIGNATURES) == set(syms)


def test_api_version():
    assert _lib.load().crt_api_version() == 1


def _desc(sc, **over):
    pos = np.ascontiguousarray(sc.positions, np.float32)
    nor = np.ascontiguousarray(sc.normals, np.float32)
    mid = np.ascontiguousarray(sc.material_ids, np.uint32)
    mats = (_lib.Material * len(sc.materials))()
    for i, m in enumerate(sc.materials):
        mats[i].bsdf, mats[i].texture = m.bsdf, m.tex
        mats[i].kd[:] = list(m.kd)
        mats[i].ka[:] = list(m.ka)
    keep = [pos, nor, mid, mats]
    d = dict(num_triangles=sc.n_tris, positions=pos.ctypes.data, normals=nor.ctypes.data, uvs=None,
             material_ids=mid.ctypes.data, num_materials=len(sc.materials), materials=C.addressof(mats),
             num_lights=0, light_indices=None, num_textures=0, texture_dims=None, texels=None)
    d.update(over)
    return _lib.SceneDesc(**d), keep


def _create(desc):
    h = C.c_void_p()
    st = _lib.load().crt_scene_create(C.byref(desc), C.byref(h))
    return st, _lib.load().crt_last_error().decode()


def test_scene_without_lights_is_rejected():
    sc = scenes.cornell_box()
    sc.materials[3].bsdf = scenes.DIFFUSE          # the light quad stops emitting
    desc, keep = _desc(sc)
    st, msg = _create(desc)
    assert st == 1 and "emissive" in msg


def test_bad_material_index_is_rejected():
    sc = scenes.cornell_box()
    sc.material_ids = sc.material_ids.copy()
    sc.material_ids[5] = 99
    desc, keep = _desc(sc)
    st, msg = _create(desc)
    assert st == 1 and "material id" in msg


def test_bad_texture_index_is_rejected():
    sc = scenes.cornell_box()
    sc.materials[0].tex = 3
    desc, keep = _desc(sc)
    st, msg = _create(desc)
    assert st == 1 and "texture" in msg


def test_empty_scene_and_null_args_are_rejected():
    sc = scenes.cornell_box()
    desc, keep = _desc(sc, num_triangles=0)
    assert _create(desc)[0] == 1
    assert _lib.load().crt_scene_create(None, None) == 1
    assert _lib.load().crt_trace_closest(None, None, 0, None, None, None, None) == 1
    assert _lib.load().crt_scene_errors(None, None, None) == 1
    with pytest.raises(CrtError):
        _lib.check(1)


def test_gather_measurement_arguments_are_checked():
    """crt_measure_gather refuses bad shapes before it launches anything."""
    L = _lib.load()
    buf, sink = 4096, 8192          # stand-in addresses: never dereferenced on these paths
    cases = [((None, 1 << 20, 208, 256, 1, 0, sink, None), "null argument"),
             ((buf + 4, 1 << 20, 208, 256, 1, 0, sink, None), "16-byte aligned"),
             ((buf, 1 << 20, 200, 256, 1, 0, sink, None), "multiple of 16"),
             ((buf, 100, 208, 256, 1, 0, sink, None), "between 1 and"),
             ((buf, 1 << 20, 208, 100, 1, 0, sink, None), "multiple of 256"),
             ((buf, 1 << 20, 208, 256, 1, 6, sink, None), "unknown flag")]
    for args, msg in cases:
        assert L.crt_measure_gather(*args) == 1
        assert msg in L.crt_last_error().decode(), (args, L.crt_last_error())


def test_camera_from_json_matches_oracle():
    import oracle
    from cudart_gb300 import camera_from_json
    for spec, (w, h) in [(scenes.CORNELL_CAMERA, (512, 512)), (scenes.large_textured.__defaults__ and
                          scenes.CameraSpec(45.0, (0, 3.2, 7.5), (0, -3.2, -7.5)), (1920, 1080))]:
        c = camera_from_json(spec, w, h)
        o = oracle.make_camera(spec, w, h)
        assert bytes(c) == o.tobytes()


def test_renderer_shim_compiles_against_the_reference_headers():
    """The C++ Renderer subclass for the reference's tree compiles against the
    reference's own headers (where its sources are present)."""
    import shutil
    import subprocess
    shim = os.path.join(ROOT, "cudart_gb300", "shim")
    if shutil.which("nvcc") is None or shutil.which("make") is None:
        pytest.skip("nvcc/make not available")
    ref = subprocess.run(["make", "-s", "-C", shim, "print-ref"], capture_output=True, text=True).stdout.strip()
    if not os.path.isdir(os.path.join(ref, "src", "include")):
        pytest.skip("reference sources not present")
    res = subprocess.run(["make", "-C", shim, "check"], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr


def test_reference_binary_links_with_the_shim(tmp_path):
    """The reference's own main.cpp, launchers, loaders, scene, BVH and CPU
    renderer, with main.cpp's ParallelRenderer construction replaced by the
    shim (cudart_gb300/shim/Makefile, target link), link against the library
    and run.  Without a GPU the binary takes the reference's --cpu branch
    (main.cpp:157), so this checks the drop-in's build and the unchanged
    command line; the GPU branch needs the reference's sources on a GPU host."""
    import shutil
    if shutil.which("nvcc") is None or shutil.which("make") is None:
        pytest.skip("nvcc/make not available")
    shim = os.path.join(ROOT, "cudart_gb300", "shim")
    ref = subprocess.run(["make", "-s", "-C", shim, "print-ref"], capture_output=True, text=True).stdout.strip()
    if not os.path.isfile(os.path.join(ref, "src", "main.cpp")):
        pytest.skip("reference sources not present")
    res = subprocess.run(["make", "-s", "-j8", "-C", shim, "link"], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    sc = scenes.cornell_box(width=24, height=16)
    files = scenes.write_reference_files(sc, str(tmp_path / "meshes"), "box")
    os.makedirs(tmp_path / "settings")
    os.replace(files["camera"], tmp_path / "settings" / "box-camera.json")
    (tmp_path / ".env").write_text(f"MESHES_PATH={tmp_path}/meshes\nCAMERA_PATH={tmp_path}/settings\n"
                                   f"TEXTURES_PATH={files['textures'].rstrip('/')}\n")
    run_dir = tmp_path / "build"
    run_dir.mkdir()
    p = subprocess.run([os.path.join(shim, "_build", "CudaRT_gb300"), "-f", "box", "-s", "2", "-w", "24",
                        "-h", "16", "--cpu"], cwd=run_dir, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stdout[-2000:] + p.stderr[-2000:]
    assert "Rendered to box.png for 2 samples per pixel" in p.stdout
    assert (run_dir / "box.png").stat().st_size > 0


def test_header_is_valid_c_and_links():
    """include/crt_gb300.h compiles as C11 and a C host links against the
    library (running it needs a GPU: tests/test_gpu_c_host.py)."""
    import shutil
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    import tempfile
    pkg = os.path.join(ROOT, "cudart_gb300")
    with tempfile.TemporaryDirectory() as d:
        res = subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-O2", "-I", os.path.join(ROOT, "include"),
                              os.path.join(ROOT, "tests", "c", "abi_example.c"), "-L", pkg, "-lcrt_gb300",
                              "-o", os.path.join(d, "abi_example")], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr

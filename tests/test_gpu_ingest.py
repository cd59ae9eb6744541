"""Scenes read from files render exactly like the same scenes built from
arrays, through the library and through crt_render."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from cudart_gb300 import GB300Renderer, GB300Scene, SceneFiles, load_camera_json, load_png_texels, scenes

pytestmark = pytest.mark.gpu
CLI = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "cudart_gb300", "crt_render")


@pytest.mark.parametrize("mode", ["megakernel", "wavefront"])
def test_file_scene_renders_like_arrays(cuda, tmp_path, mode):
    sc = scenes.feature_mix()
    files = scenes.write_reference_files(sc, str(tmp_path), "fm")
    f = SceneFiles(files["obj"], files["textures"])
    cam = load_camera_json(files["camera"], sc.width, sc.height)
    a = GB300Renderer(GB300Scene(sc), sc.width, sc.height, 32, max_depth=6, seed=99, mode=mode)
    b = GB300Renderer(GB300Scene(f), sc.width, sc.height, 32, max_depth=6, seed=99, mode=mode, camera=cam)
    a.render()
    b.render()
    assert np.array_equal(a.accum(), b.accum())
    assert np.array_equal(a.copy_image_bytes(), b.copy_image_bytes())


def test_cli_image_matches_the_library(cuda, tmp_path):
    sc = scenes.feature_mix(width=48, height=32)
    files = scenes.write_reference_files(sc, str(tmp_path / "meshes"), "fm")
    os.makedirs(tmp_path / "settings")
    shutil.move(files["camera"], tmp_path / "settings" / "fm-camera.json")
    (tmp_path / ".env").write_text(f"MESHES_PATH={tmp_path}/meshes\nCAMERA_PATH={tmp_path}/settings\n"
                                   f"TEXTURES_PATH={files['textures']}\n")
    out = tmp_path / "img.png"
    p = subprocess.run([CLI, "-f", "fm", "-s", "8", "-w", "48", "-h", "32", "--env", str(tmp_path / ".env"),
                        "-o", str(out), "--json"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    summary = json.loads(p.stdout.strip().splitlines()[-1])
    assert summary["spp"] == 8 and summary["triangles"] == sc.n_tris
    assert "Rendered to" in p.stdout and "Average samples per pixel" in p.stdout
    got = load_png_texels(str(out))
    f = SceneFiles(str(tmp_path / "meshes" / "fm.obj"), files["textures"])
    cam = load_camera_json(str(tmp_path / "settings" / "fm-camera.json"), 48, 32)
    r = GB300Renderer(GB300Scene(f), 48, 32, 8, max_depth=6, seed=1234, mode="wavefront", camera=cam)
    r.render()
    want = r.copy_image_bytes().reshape(32, 48, 4)
    assert np.array_equal(got, scenes.texel_table()[want[..., :3]])

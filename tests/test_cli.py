"""crt_render, the command-line renderer: option handling and scene lookup
as the reference's main.cpp does them (no GPU needed for these paths)."""
import os
import subprocess

import pytest

from cudart_gb300 import scenes

CLI = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "cudart_gb300", "crt_render")


def _run(args, cwd):
    return subprocess.run([CLI] + args, cwd=cwd, capture_output=True, text=True, timeout=120)


def test_usage_without_arguments(tmp_path):
    p = _run([], tmp_path)
    assert p.returncode == 1 and "Usage: crt_render" in p.stderr and "-f" in p.stderr


@pytest.mark.parametrize("flag", ["--cpu", "--x"])
def test_cpu_and_window_flags_are_refused(tmp_path, flag):
    p = _run(["-f", "cornell", flag], tmp_path)
    assert p.returncode == 2 and flag in p.stderr


def test_env_paths_and_missing_scene(tmp_path):
    run_dir = tmp_path / "build"
    run_dir.mkdir()
    (tmp_path / ".env").write_text("# paths\nMESHES_PATH=../m\nCAMERA_PATH=../c\nTEXTURES_PATH=../t\n")
    p = _run(["-f", "nothere", "-s", "3", "-w", "32", "-h", "abc"], run_dir)
    assert "Samples: 3" in p.stdout and "Width: 32" in p.stdout and "Height: 480" in p.stdout
    assert "Invalid argument to -h!" in p.stderr
    assert "Obj path: ../m/nothere.obj" in p.stdout and "Camera path: ../c/nothere-camera.json" in p.stdout
    assert "Output: nothere.png" in p.stdout
    assert p.returncode == 1 and "cannot open ../m/nothere.obj" in p.stderr


def test_default_folders_without_env(tmp_path):
    p = _run(["-s", "1"], tmp_path)
    assert "Obj path: ../meshes/cornell.obj" in p.stdout and "Output: out.png" in p.stdout
    assert p.returncode == 1


def test_bad_camera_is_reported(tmp_path):
    sc = scenes.cornell_box(width=16, height=16)
    files = scenes.write_reference_files(sc, str(tmp_path / "meshes"), "box")
    os.makedirs(tmp_path / "settings")
    (tmp_path / "settings" / "box-camera.json").write_text('{"fieldOfView": 40}')
    (tmp_path / ".env").write_text(f"MESHES_PATH={tmp_path}/meshes\nCAMERA_PATH={tmp_path}/settings\n"
                                   f"TEXTURES_PATH={files['textures']}\n")
    p = _run(["-f", "box", "--env", str(tmp_path / ".env")], tmp_path)
    assert p.returncode == 1 and "focalLength" in p.stderr


@pytest.mark.parametrize("flag,value,message", [("--nodes", "f16", "--nodes must be f32 or q8"),
                                                ("--mode", "raster", "--mode must be wavefront or megakernel"),
                                                ("--builder", "cloud", "--builder must be host or gpu")])
def test_bad_option_values_are_refused(tmp_path, flag, value, message):
    p = _run(["-f", "box", flag, value], tmp_path)
    assert p.returncode == 1 and message in p.stderr

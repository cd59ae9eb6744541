"""The library's host code under AddressSanitizer + UndefinedBehaviorSanitizer
(no GPU): the scene-file readers on the golden edge-case files and on
seeded truncations / byte flips of them (malformed input must give an error
status, never an out-of-bounds access), and the host BVH build on random,
coincident and zero-area triangles.  Built from the product sources by g++
with -fsanitize=address,undefined -fno-sanitize-recover=all."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from golden.make_ingest_golden import load_cases, png_bytes, write_case

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = [os.path.join(ROOT, "tests", "c", "sanitize_host.cpp"),
       os.path.join(ROOT, "cudart_gb300", "csrc", "ingest.cpp"),
       os.path.join(ROOT, "cudart_gb300", "csrc", "bvh8.cpp")]
FLAGS = ["-std=c++17", "-O1", "-g", "-pthread", "-ffp-contract=off", "-fno-omit-frame-pointer",
         "-fsanitize=address,undefined", "-fno-sanitize-recover=all"]


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("san") / "sanitize_host")
    p = subprocess.run([cxx] + FLAGS + SRC + ["-o", out], capture_output=True, text=True)
    if p.returncode != 0 and "sanitize" in p.stderr and "cannot find" in p.stderr:
        pytest.skip("sanitizer runtime not installed")
    assert p.returncode == 0, p.stderr[-3000:]
    return out


def _run(driver, args, cwd=None):
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    p = subprocess.run([driver] + args, capture_output=True, text=True, timeout=600, cwd=cwd, env=env)
    assert p.returncode == 0 and "sanitize_host: ok" in p.stdout, (p.stdout[-2000:], p.stderr[-4000:])


def test_bvh_build_under_sanitizers(driver):
    _run(driver, [])


def test_readers_on_golden_files(driver, tmp_path):
    files = []
    for name, case in load_cases().items():
        d = tmp_path / name
        paths = write_case({**case["index"], "files": case["files"]}, str(d))
        files += [paths["obj"], paths["camera"]]
        files += [str(d / rel) for rel in case["files"] if rel.endswith(".png")]
    _run(driver, files)


def _mutants(data: bytes, rng, n: int):
    out = []
    for k in range(n):
        b = bytearray(data)
        kind = k % 3
        if kind == 0 and len(b) > 1:
            b = b[:rng.integers(1, len(b))]                    # truncated
        elif kind == 1:
            for _ in range(rng.integers(1, 8)):                # byte flips
                b[rng.integers(0, len(b))] ^= int(rng.integers(1, 256))
        else:
            i = rng.integers(0, len(b))                        # a run of garbage
            b[i:i + 16] = rng.integers(0, 256, 16).astype(np.uint8).tobytes()
        out.append(bytes(b))
    return out


def test_readers_on_malformed_files(driver, tmp_path):
    rng = np.random.default_rng(2024)
    case = load_cases()["obj_rules"]
    base = tmp_path / "base"
    write_case({**case["index"], "files": case["files"]}, str(base))
    files = []
    # PNGs: every colour type / depth the reader handles, interlaced or not, then mutated
    pngs = [png_bytes(rng.integers(0, 256, (9, 11, 3)), 2), png_bytes(rng.integers(0, 2, (5, 13, 1)), 0, depth=1),
            png_bytes(rng.integers(0, 16, (7, 6, 1)), 3, depth=4, palette=rng.integers(0, 256, (16, 3))),
            png_bytes(rng.integers(0, 65536, (6, 7, 4)), 6, depth=16, interlace=True),
            png_bytes(rng.integers(0, 256, (12, 12, 2)), 4, interlace=True)]
    for i, data in enumerate(pngs):
        for j, m in enumerate([data] + _mutants(data, rng, 40)):
            p = tmp_path / f"p{i}_{j}.png"
            p.write_bytes(m)
            files.append(str(p))
    # OBJ / MTL / JSON: mutated copies beside the real textures and library
    obj = case["files"]["rules.obj"]
    mtl = case["files"]["sub/rules.mtl"]
    cam = case["files"]["rules-camera.json"]
    for j, m in enumerate(_mutants(obj, rng, 30)):
        p = base / f"m{j}.obj"
        p.write_bytes(m)
        files.append(str(p))
    for j, m in enumerate(_mutants(mtl, rng, 30)):
        d = tmp_path / f"mtl{j}"
        (d / "sub").mkdir(parents=True)
        (d / "sub" / "rules.mtl").write_bytes(m)
        (d / "rules.obj").write_bytes(obj)
        files.append(str(d / "rules.obj"))
    for j, m in enumerate(_mutants(cam, rng, 30)):
        p = tmp_path / f"c{j}.json"
        p.write_bytes(m)
        files.append(str(p))
    _run(driver, files)

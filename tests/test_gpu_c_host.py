"""The C ABI from a plain C program (tests/c/abi_example.c): the header is
valid C11, the library links with gcc, and a render through it gives the
same accumulator in the plain kernel and the wavefront form."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_plain_c_host_renders(cuda, tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    pkg = os.path.join(ROOT, "cudart_gb300")
    exe = str(tmp_path / "abi_example")
    subprocess.run(["gcc", "-std=c11", "-Wall", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "abi_example.c"), "-L", pkg, "-lcrt_gb300",
                    f"-Wl,-rpath,{pkg}", "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "identical 1" in out.stdout

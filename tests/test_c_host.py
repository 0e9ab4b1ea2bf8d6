"""A plain C99 program compiled against include/tensorly_gb300.h and linked
to the built library runs on the CPU: the header is valid C, the library
links without torch, and the host-side checks answer as documented."""

import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_c_host_program(tmp_path):
    from tensorly_gb300 import _build
    so = _build.build()
    libdir = os.path.dirname(so)
    exe = tmp_path / "abi_host"
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror",
           "-I", os.path.join(REPO, "include"), os.path.join(REPO, "tests", "c_host", "abi_host.c"),
           so, "-Wl,-rpath," + libdir, "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("0 failures")
    assert "FAIL" not in out.stdout

"""The C++ mirror of the crate API (host/mosaic.hpp): the crate's own unit
tests restated in C++ (tests/cpp/host_api_test.cpp), compiled against the
built library and run host-only here and in full on a GPU."""
import os
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
PKG = REPO / "mosaic-art-rust_gb300"
BUILD = PKG / "_build"


def _compile() -> Path:
    lib = BUILD / "libmosaic_gpu.so"
    if not lib.exists():
        pytest.skip("libmosaic_gpu.so is not built")
    exe = BUILD / "host_api_test"
    src = REPO / "tests" / "cpp" / "host_api_test.cpp"
    hdr = PKG / "host" / "mosaic.hpp"
    newest = max(p.stat().st_mtime for p in (src, hdr, lib, REPO / "include" / "mosaic_gpu.h"))
    if not exe.exists() or exe.stat().st_mtime < newest:
        cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", f"-I{REPO / 'include'}", f"-I{PKG / 'host'}",
               str(src), f"-L{BUILD}", "-lmosaic_gpu", f"-Wl,-rpath,{BUILD}", "-o", str(exe)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    return exe


def test_host_mirror_host_only(built):
    exe = _compile()
    env = dict(os.environ, CUDA_VISIBLE_DEVICES=os.environ.get("CUDA_VISIBLE_DEVICES", ""))
    if os.path.exists("/dev/nvidia0"):
        pytest.skip("a GPU is present: the host-only run expects context creation to fail")
    r = subprocess.run([str(exe), "--cpu"], capture_output=True, text=True, timeout=120, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failed" in r.stdout


@pytest.mark.gpu
def test_host_mirror_on_gpu(built):
    exe = _compile()
    r = subprocess.run([str(exe), "--gpu"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failed" in r.stdout

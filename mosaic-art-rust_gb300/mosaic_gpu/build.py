"""Build the in-tree shared libraries of the mosaic GPU path.

``libmosaic_gpu.so``  -- the CUDA library behind include/mosaic_gpu.h
                         (nvcc, sm_103a only, one -gencode).
``libmosaic_synth.so`` -- the host generator of seeded synthetic inputs (g++).

Translation units compile in parallel; outputs go to ``<package>/_build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # mosaic-art-rust_gb300/
CSRC = PKG_ROOT / "csrc"
BUILD = PKG_ROOT / "_build"
REPO = PKG_ROOT.parent
INCLUDE = REPO / "include"

CUDA_SOURCES = ["k_lab.cu", "k_resize.cu", "k_scan.cu", "k_nearest_grid.cu", "k_sim.cu", "k_greedy.cu", "k_anneal.cu", "k_composite.cu", "k_batch.cu",
                "capi.cu", "capi_batch.cu", "capi_server.cu", "io_png.cpp", "io_jpeg.cpp"]  # io_png.cpp: host code, same library
GENCODE = "arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> dict[str, Path]:
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [INCLUDE / "mosaic_gpu.h"]
    flags = [
        "-gencode", GENCODE, "-lineinfo", "-O3", "-std=c++17",
        "-Xcompiler", "-fPIC,-ffp-contract=off", f"-I{INCLUDE}",
    ]
    objs = []
    jobs = []
    for src in CUDA_SOURCES:
        s = CSRC / src
        o = BUILD / (Path(src).stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, *flags, "-c", str(s), "-o", str(o)])
    synth_src = CSRC / "synth.cpp"
    synth_so = BUILD / "libmosaic_synth.so"
    if force or _stale(synth_so, [synth_src, CSRC / "mg_math.h"]):
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                     "-pthread", str(synth_src), "-o", str(synth_so)])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    lib = BUILD / "libmosaic_gpu.so"
    if force or _stale(lib, objs):
        _run([nvcc, "-shared", "-gencode", GENCODE, *[str(o) for o in objs], "-o", str(lib), "-lcudart"])
    if verbose:
        print(f"built {lib} and {synth_so}")
    return {"gpu": lib, "synth": synth_so}


if __name__ == "__main__":
    build(verbose=True)

"""Build the engine's native libraries in-tree.

libpito_recon.so  CUDA kernels (sm_103a) + the C ABI of include/pito_recon.h
libpito_synth.so  seeded synthetic syntax generators (host C++)

Compiles translation units in parallel and skips outputs newer than their
sources.  Used by __graft_entry__.build() and by the package on import when
a library is missing.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["recon_api.cu", "h264_kernels.cu", "hevc_kernels.cu", "output_order.cpp"]
SYNTH_SOURCES = ["synth_h264.cpp", "synth_hevc.cpp"]
HEADERS = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "pito_recon.h"]

RECON_LIB = PKG / "libpito_recon.so"
SYNTH_LIB = PKG / "libpito_synth.so"


def _stale(target: pathlib.Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(pathlib.Path(d).stat().st_mtime > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r


def build(verbose: bool = False) -> None:
    OUT.mkdir(exist_ok=True)
    nvcc = os.environ.get("NVCC", "nvcc")
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = CSRC / src
        o = OUT / (src + ".o")
        objs.append(o)
        if _stale(o, [s, *HEADERS]):
            jobs.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v" if verbose else "-O3", "-c", str(s), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for r in ex.map(_run, jobs):
            if verbose:
                print(r.stderr)
        if _stale(RECON_LIB, objs):
            _run([nvcc, *ARCH, "-shared", "-o", str(RECON_LIB), *map(str, objs)])
        synth_srcs = [CSRC / s for s in SYNTH_SOURCES]
        if _stale(SYNTH_LIB, [*synth_srcs, *HEADERS]):
            _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", str(SYNTH_LIB), *map(str, synth_srcs)])


if __name__ == "__main__":
    build(verbose=True)

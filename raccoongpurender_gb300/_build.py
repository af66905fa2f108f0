"""Build librgr.so: the C-ABI library with the sm_103a CUDA kernels.

nvcc compiles the .cu translation units for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); g++ compiles the host C++.
All floating-point code is compiled without contraction (``--fmad=false`` /
``-ffp-contract=off``): the kernels reproduce the reference traversal and
shading arithmetic bit for bit.  Object files go to ``_build/`` and the
library to ``raccoongpurender_gb300/_lib/librgr.so`` (both git-ignored).
Translation units compile in parallel; an unchanged tree is not rebuilt.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = ROOT / "_build" / "rgr"
LIB_DIR = PKG / "_lib"
LIB = LIB_DIR / "librgr.so"

CUDA_SOURCES = ["kernels/trace.cu", "kernels/wavefront.cu", "kernels/guide_mlp.cu", "kernels/guide_tc.cu", "kernels/guide_train_tc.cu",
                "kernels/envmap_gpu.cu", "kernels/bvh_gpu.cu",
                "host/context.cu", "host/noalloc.cu", "host/guide.cu", "host/probe.cu"]
CXX_SOURCES = ["host/scene.cpp", "host/bvh_build.cpp", "host/envmap_tables.cpp", "host/alembic.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_flags() -> list[str]:
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
        "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", str(ROOT / "include"),
        "-Xptxas", "-warn-spills",
    ]


def _cxx_flags() -> list[str]:
    # the CUDA include directory for the header-only NVTX ranges of the host sources
    cuda_include = Path(_nvcc()).resolve().parent.parent / "include"
    return ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
            "-I", str(ROOT / "include"), "-I", str(cuda_include)]


def _digest(paths: list[Path], extra: str) -> str:
    h = hashlib.sha256(extra.encode())
    for p in sorted(paths):
        h.update(str(p).encode())
        h.update(p.read_bytes())
    return h.hexdigest()


def _all_inputs() -> list[Path]:
    files = [p for p in CSRC.rglob("*") if p.suffix in (".cu", ".cuh", ".cpp", ".h")]
    files.append(ROOT / "include" / "rgr.h")
    return files


def build(verbose: bool = False, force: bool = False, defines: tuple = (), out: Path | None = None) -> Path:
    """Compile every translation unit and link librgr.so; returns its path.
    `defines` (e.g. ("RGR_TRACE_MIN_BLOCKS=6",)) and `out` build a variant of
    the library elsewhere, for launch-shape experiments."""
    lib = Path(out) if out else LIB
    bdir = BUILD if not defines else BUILD.parent / ("rgr_" + hashlib.sha1(" ".join(defines).encode()).hexdigest()[:8])
    bdir.mkdir(parents=True, exist_ok=True)
    lib.parent.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    dflags = [f"-D{d}" for d in defines]
    stamp = bdir / "stamp"
    key = _digest(_all_inputs(), " ".join(_cuda_flags() + _cxx_flags() + dflags) + os.uname().machine + str(lib))
    if not force and lib.exists() and stamp.exists() and stamp.read_text() == key:
        return lib

    jobs = []
    for src in CUDA_SOURCES:
        obj = bdir / (src.replace("/", "_") + ".o")
        jobs.append([nvcc, *_cuda_flags(), *dflags, "-c", str(CSRC / src), "-o", str(obj)])
    for src in CXX_SOURCES:
        obj = bdir / (src.replace("/", "_") + ".o")
        jobs.append(["g++", *_cxx_flags(), *dflags, "-c", str(CSRC / src), "-o", str(obj)])

    def run(cmd: list[str]) -> None:
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)

    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    objs = [str(bdir / (s.replace("/", "_") + ".o")) for s in CUDA_SOURCES + CXX_SOURCES]
    tmp = lib.with_suffix(".so.tmp")
    run([nvcc, *ARCH, "-shared", "-o", str(tmp), *objs, "-lpthread"])
    os.replace(tmp, lib)
    stamp.write_text(key)
    return lib


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))

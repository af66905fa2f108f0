"""Build the CPU oracle (test infrastructure).

* ``oracle/_build/liboracle.so`` — the C++ restatement of the reference
  kernels (rgr_oracle.cpp).  Built on every machine.
* ``oracle/_ref/libref.so`` — the reference's own OpenCL kernels
  (``kernels/*.cl``) compiled unchanged as C++ through ``oracle/ref/clshim*.h``,
  plus the step() driver ``oracle/ref/ref_step.cpp``.  Built only where the
  reference sources exist (``RGR_REFERENCE_DIR``, default ``/root/reference``);
  the GPU machines do not have them and use the committed golden fixtures.
* ``oracle/_ref/abc_tool`` — the reference's vendored Alembic library
  (``libs/abc``: Alembic, Imath, Iex, IlmThread, half) and its Houdini reader
  (``libs/houdini_alembic/houdini_alembic.cpp``) compiled from their sources,
  with ``oracle/abc/abc_tool.cpp``: writes the synthetic Alembic test scenes
  and dumps what the reference reader returns for them
  (``tests/golden/make_alembic_golden.py``).  Same condition as libref.so.

Both are compiled with ``-ffp-contract=off`` (no fused multiply-add), the
arithmetic convention shared with the CUDA kernels.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
LIB = BUILD / "liboracle.so"
REF_LIB = REF_OUT / "libref.so"
FMATH = ROOT / "raccoongpurender_gb300" / "csrc" / "rgr_fmath.h"
# -O3 without -march/-mcpu=native: the same build must give the same results on the
# x86 development machines and the Arm GPU machines
CXX = ["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off"]


def reference_dir() -> Path | None:
    d = Path(os.environ.get("RGR_REFERENCE_DIR", "/root/reference"))
    return d if (d / "kernels" / "extension_ray_cast_stackless.cl").exists() else None


def _digest(paths: list[Path]) -> str:
    h = hashlib.sha256(" ".join(CXX).encode() + os.uname().machine.encode())
    for p in sorted(paths):
        h.update(str(p).encode())
        h.update(p.read_bytes())
    return h.hexdigest()


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_oracle(force: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    srcs = [HERE / "rgr_oracle.cpp", HERE / "rgr_oracle.h", FMATH]
    stamp = BUILD / "stamp"
    key = _digest(srcs)
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == key:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    _run(CXX + ["-shared", "-pthread", str(HERE / "rgr_oracle.cpp"), "-o", str(tmp)])
    os.replace(tmp, LIB)
    stamp.write_text(key)
    return LIB


def build_ref(force: bool = False) -> Path | None:
    ref = reference_dir()
    if ref is None:
        return REF_LIB if REF_LIB.exists() else None
    REF_OUT.mkdir(parents=True, exist_ok=True)
    kern = ref / "kernels"
    tus = sorted((HERE / "ref").glob("ref_*.cpp"))
    inputs = tus + sorted((HERE / "ref").glob("*.h")) + sorted(kern.glob("*.cl")) + [
        HERE / "rgr_oracle.cpp", HERE / "rgr_oracle.h", FMATH]
    stamp = REF_OUT / "stamp"
    key = _digest(inputs)
    if not force and REF_LIB.exists() and stamp.exists() and stamp.read_text() == key:
        return REF_LIB
    flags = CXX + ["-Wno-unused-value", "-Wno-attributes", "-I", str(kern), "-I", str(HERE / "ref")]
    objs = []
    jobs = []
    for tu in tus + [HERE / "rgr_oracle.cpp"]:
        obj = REF_OUT / (tu.stem + ".o")
        objs.append(str(obj))
        jobs.append(flags + ["-c", str(tu), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    tmp = REF_LIB.with_suffix(".so.tmp")
    _run(CXX + ["-shared", "-pthread", *objs, "-o", str(tmp)])
    os.replace(tmp, REF_LIB)
    stamp.write_text(key)
    return REF_LIB


ABC_TOOL = REF_OUT / "abc_tool"


def build_abc_tool(force: bool = False) -> Path | None:
    ref = reference_dir()
    if ref is None or not (ref / "libs" / "abc" / "Alembic").exists():
        return ABC_TOOL if ABC_TOOL.exists() else None
    abc = ref / "libs" / "abc"
    hou = ref / "libs" / "houdini_alembic"
    # every Alembic / IlmBase translation unit but the Win32-only ones
    srcs = sorted(p for p in abc.rglob("*.cpp") if "Win32" not in p.name) + [hou / "houdini_alembic.cpp"]
    tool = HERE / "abc" / "abc_tool.cpp"
    stamp = REF_OUT / "abc_stamp"
    key = _digest([tool, HERE / "abc" / "windows.h"] + srcs)
    if not force and ABC_TOOL.exists() and stamp.exists() and stamp.read_text() == key:
        return ABC_TOOL
    objdir = REF_OUT / "abc_obj"
    objdir.mkdir(parents=True, exist_ok=True)
    # the pre-generated IlmBase configuration declares Windows; abc/windows.h
    # stands in for the one header that this pulls in.  houdini_alembic.hpp
    # relies on <algorithm> and <cstring> arriving through other headers.
    flags = ["g++", "-O2", "-std=c++14", "-fPIC", "-ffp-contract=off", "-w", "-include", "algorithm",
             "-include", "cstring", "-I", str(abc),
             "-I", str(abc / "Alembic"), "-I", str(hou), "-I", str(HERE / "abc")]
    objs, jobs = [], []
    for s in srcs + [tool]:
        obj = objdir / (hashlib.sha1(str(s).encode()).hexdigest()[:16] + ".o")
        objs.append(str(obj))
        jobs.append(flags + ["-c", str(s), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    tmp = ABC_TOOL.with_suffix(".tmp")
    _run(["g++", "-pthread", *objs, "-o", str(tmp)])
    os.replace(tmp, ABC_TOOL)
    stamp.write_text(key)
    return ABC_TOOL


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
    print(build_abc_tool(force="--force" in sys.argv))

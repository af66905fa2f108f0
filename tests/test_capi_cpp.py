"""A C++ program compiled against include/rgr.h and linked to librgr.so runs
the reference host's call sequence (scene, BVH, upload, render, readback,
stats, closest hit, merge_from).  On the CPU it is built and runs its
host-side part; on a GPU it runs end to end."""
import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "capi" / "integration_example.cpp"


def _build(tmp_path, rg) -> Path:
    lib = Path(rg.load_library()._name)
    exe = tmp_path / "integration_example"
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(SRC), "-o", str(exe),
           f"-L{lib.parent}", "-lrgr", f"-Wl,-rpath,{lib.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_program_builds_and_runs_host_calls(tmp_path, rg):
    exe = _build(tmp_path, rg)
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([str(exe), "--host"], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "integration host ok" in r.stdout


@pytest.mark.gpu
def test_cpp_program_end_to_end(tmp_path, rg):
    exe = _build(tmp_path, rg)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "integration ok" in r.stdout

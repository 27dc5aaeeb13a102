"""The chunk plan of the LSRK45 step on host vectors (ew_lsrk45_step_host),
checked on the host (tests/native/host_plan_check.cpp compiled with the host
C++ compiler): the chunks partition the work items and DoFs in order, each
chunk's neighbour range covers all its cells' neighbours, and the wavefront
schedule is chosen exactly when every chunk's neighbours lie in the chunk or
the two next to it (layer-by-layer numbering: yes; small or renumbered
meshes: no)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_host_step_chunk_plan(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "host_plan_check")
    src = os.path.join(HERE, "native", "host_plan_check.cpp")
    r = subprocess.run([cxx, "-std=c++17", "-O2", src, "-o", exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout[-3000:]

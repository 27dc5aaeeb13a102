"""The line kernel's shared-memory plan and bulk neighbour-copy windows,
checked on the host (tests/native/cart_layout_check.cu compiled with nvcc;
no kernel runs): alignment, sizes and containment for every dimension,
points per line, stage-input type and cells per block."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_cart_layout_and_windows(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "cart_layout_check")
    src = os.path.join(HERE, "native", "cart_layout_check.cu")
    r = subprocess.run([nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a",
                        "-diag-suppress", "128", src, "-o", exe], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout[-3000:]

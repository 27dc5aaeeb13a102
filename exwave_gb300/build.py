"""Builds libexwave_gb300.so in-tree with nvcc for sm_103a.

One object per (dimension, points-per-direction) pair from ``csrc/ew_inst.cu``
plus the C-ABI unit ``csrc/ew_api.cu``, compiled in parallel and linked into
``exwave_gb300/lib/libexwave_gb300.so``.  Objects are rebuilt only when a
source is newer.  Usage: ``python -m exwave_gb300.build``.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libexwave_gb300.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
PAIRS = [(d, n) for d in (2, 3) for n in range(2, 14)]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(ROOT, "include", "*.h"))


def _newest_source():
    return max(os.path.getmtime(p) for p in _sources())


def _compile(args):
    src, out, defs = args
    cmd = [nvcc()] + ARCH + FLAGS + defs + ["-c", src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return out


def build(jobs=None, force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    newest = _newest_source()
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tasks = []
    for d, n in PAIRS:
        out = os.path.join(OBJ, "ew_inst_d%d_n%d.o" % (d, n))
        tasks.append((os.path.join(CSRC, "ew_inst.cu"), out, ["-DEW_DIM=%d" % d, "-DEW_NP=%d" % n]))
    tasks.append((os.path.join(CSRC, "ew_api.cu"), os.path.join(OBJ, "ew_api.o"), []))
    tasks.append((os.path.join(CSRC, "ew_mesh.cpp"), os.path.join(OBJ, "ew_mesh.o"), []))
    tasks.append((os.path.join(CSRC, "ew_batch.cu"), os.path.join(OBJ, "ew_batch.o"), []))
    tasks.append((os.path.join(CSRC, "ew_diag.cu"), os.path.join(OBJ, "ew_diag.o"), []))
    todo = [t for t in tasks if force or not os.path.exists(t[1]) or os.path.getmtime(t[1]) < newest]
    jobs = jobs or min(len(todo) or 1, os.cpu_count() or 4)
    if todo:
        # the largest instantiations first
        todo.sort(key=lambda t: -sum(int(x.split("=")[1]) for x in t[2]) if t[2] else 0)
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            for out in ex.map(_compile, todo):
                if verbose:
                    print("built", os.path.basename(out), flush=True)
    objs = [t[1] for t in tasks]
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))

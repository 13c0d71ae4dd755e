"""Builds libccpgpu.so (the engine's C-ABI library) in-tree for sm_103a.

Four translation units (host C++, the analysis statistics, the CUDA engine
and the surrogate network) are compiled in parallel with nvcc and linked into tfm_gb300/libccpgpu.so. No cmake.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libccpgpu.so")
OBJ = os.path.join(HERE, "_build")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def sources():
    return [os.path.join(CSRC, f) for f in ("host.cpp", "analysis.cpp", "engine.cu", "surrogate.cu")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    for hdr in ("ccpgpu.h", "ccpgpu_surrogate.h"):
        deps.append(os.path.join(os.path.dirname(HERE), "include", hdr))
    if not force and not _stale(OUT, deps):
        return OUT
    os.makedirs(OBJ, exist_ok=True)
    nv = nvcc()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-I", os.path.join(os.path.dirname(HERE), "include")]
    jobs = []
    for src in sources():
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        cmd = [nv, ARCH, "-lineinfo", *common, "-c", src, "-o", obj]
        if src.endswith(".cu"):
            cmd[1:1] = ["-Xptxas", "-v"] if verbose else []
        jobs.append((cmd, obj))
    with ThreadPoolExecutor(len(jobs)) as ex:
        logs = list(ex.map(lambda j: _run(j[0]), jobs))
    tmp = OUT + ".tmp"
    _run([nv, ARCH, "-shared", "-o", tmp] + [o for _, o in jobs])
    os.replace(tmp, OUT)
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    return OUT


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(OUT)

"""Build recipe of the native library ``libpsi_gb300.so`` (sm_103a only).

Compiles every translation unit under ``csrc/`` in parallel -- the ``.cu``
files with ``nvcc -gencode arch=compute_103a,code=sm_103a``, the ``.cpp`` files
with the host C++ compiler -- and links them in-tree next to this file.  zlib is
linked when its header is present (``.gm.gz`` input).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpsi_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home() -> str:
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if home and os.path.isdir(home):
        return home
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _have_zlib() -> bool:
    return any(os.path.exists(os.path.join(d, "zlib.h")) for d in ("/usr/include", "/usr/local/include"))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    if r.stdout.strip():
        sys.stderr.write(r.stdout)


def build(verbose: bool = False, ptxas_verbose: bool = False) -> str:
    """Compile and link the library; returns its path."""
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OBJ, exist_ok=True)
    incs = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + os.path.join(cuda, "include")]
    defs = ["-DPSI_HAVE_ZLIB"] if _have_zlib() else []
    jobs = []
    for name in sorted(os.listdir(CSRC)):
        src = os.path.join(CSRC, name)
        obj = os.path.join(OBJ, name + ".o")
        if name.endswith(".cu"):
            cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "--expt-relaxed-constexpr", *defs, *incs, "-c", src, "-o", obj]
            if ptxas_verbose:
                cmd.insert(1, "-Xptxas=-v")
        elif name.endswith(".cpp"):
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", *defs, *incs, "-c", src, "-o", obj]
        else:
            continue
        jobs.append((cmd, obj))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(lambda j: _run(j[0]), jobs))
    link = [nvcc, ARCH, "-shared", "-cudart", "static", "-o", LIB + ".tmp", *[o for _, o in jobs], "-lpthread"]
    if defs:
        link.append("-lz")
    _run(link)
    os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_verbose="-v" in sys.argv)

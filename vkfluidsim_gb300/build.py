"""Build recipe for the in-tree shared libraries.

* ``vkfluidsim_gb300/_lib/libvfs_cuda.so`` — the product: sm_103a kernels + the C ABI of
  ``include/vfs_cuda.h`` (nvcc for ``.cu``, g++ for host ``.cpp``, linked by nvcc).
* ``oracle/_build/libvfs_oracle.so`` — the CPU oracle (test infrastructure, never linked into the
  product).

Every translation unit is compiled in parallel; nothing is rebuilt when its outputs are newer
than all sources. ``VFS_FORCE_REBUILD=1`` forces a rebuild.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "vkfluidsim_gb300"
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIB_DIR = PKG / "_lib"
OBJ_DIR = PKG / "_build"
LIB = LIB_DIR / "libvfs_cuda.so"
ORACLE_SRC = ROOT / "oracle" / "vfs_oracle.cpp"
ORACLE_LIB = ROOT / "oracle" / "_build" / "libvfs_oracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _newer(out: Path, deps) -> bool:
    if os.environ.get("VFS_FORCE_REBUILD") == "1" or not out.exists():
        return False
    t = out.stat().st_mtime
    return all(Path(d).stat().st_mtime <= t for d in deps)


def _run(cmd):
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(map(str, cmd)) + "\n" + proc.stdout)
    return proc.stdout


def build_product(verbose: bool = False) -> Path:
    cuda = cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    headers = sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(CSRC.glob("*.cpp"))
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    jobs = []
    objs = []
    for src in cu:
        obj = OBJ_DIR / (src.stem + ".o")
        objs.append(obj)
        if not _newer(obj, [src, *headers, __file__]):
            jobs.append([nvcc, "-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler",
                         "-fPIC,-ffp-contract=off",
                         "-Xptxas", "-v" if verbose else "-O3", f"-I{INCLUDE}", f"-I{CSRC}",
                         "-c", str(src), "-o", str(obj)])
    for src in cpp:
        obj = OBJ_DIR / (src.stem + ".o")
        objs.append(obj)
        if not _newer(obj, [src, *headers, __file__]):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", f"-I{INCLUDE}",
                         f"-I{CSRC}",
                         f"-I{cuda / 'include'}", "-c", str(src), "-o", str(obj)])
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            logs = list(ex.map(_run, jobs))
    if jobs or not _newer(LIB, objs):
        logs.append(_run([nvcc, "-shared", *ARCH, "-o", str(LIB), *map(str, objs)]))
    if verbose:
        for log in logs:
            if log.strip():
                print(log)
    return LIB


def build_oracle() -> Path:
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    if not _newer(ORACLE_LIB, [ORACLE_SRC, __file__]):
        _run(["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
              str(ORACLE_SRC), "-o", str(ORACLE_LIB)])
    return ORACLE_LIB


def build_all(verbose: bool = False):
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_product, verbose)
        f2 = ex.submit(build_oracle)
        return f1.result(), f2.result()


if __name__ == "__main__":
    import sys

    print(build_all(verbose="-v" in sys.argv))

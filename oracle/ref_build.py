"""Recipe that builds the reference's own WCSPH step code for the CPU, as a checker for the oracle.

TEST INFRASTRUCTURE ONLY. Usage: ``python oracle/ref_build.py <VkFluidSim source tree>``.
Everything it writes goes to ``oracle/_ref/`` (git-ignored); nothing from the reference tree is
copied into the repository.

1. The compute shaders of the step (``assets/shaders/simulation/``: wcsph_with_boundary_model,
   common, kernels/kernels_3d and spatial_hash/{update_spatial_hash, spatial_hash_3d, sort, scan,
   spatial_offsets, reorder}.slang) are read where they lie and rewritten mechanically into C++
   that compiles against ``oracle/ref_shim/slang_shim.h``. The rewrite only changes syntax that
   C++ lacks; every expression and statement of the shaders is kept:
     * ``module`` lines are dropped and each ``import`` is replaced by the imported module's text
       (once per program);
     * ``[shader(..)]``, ``[numthreads(..)]``, ``[[vk::binding(..)]]``, ``public``, ``uniform``
       and ``: SV_*`` system-value semantics are dropped; ``groupshared`` becomes
       ``static thread_local`` (one copy per host thread, which runs one workgroup at a time);
     * ``let`` becomes ``const auto`` and ``var`` becomes ``auto``;
     * namespace access written with a dot (``simulation.parameters``) becomes ``::``;
     * the ``.xyz`` swizzle becomes a call, ``.xyz()``;
     * a pointer declaration ``T* name`` becomes the bounds-checked view ``ref_ptr<T> name``;
     * a struct closed without ``;`` gets one; the identifier ``thread_local`` (a C++ keyword)
       becomes ``thread_local_``.
   Each program (one entry file with its imports) goes into its own C++ namespace of one
   translation unit, ``oracle/_ref/ref_shaders_gen.cpp``.
2. ``oracle/ref_shim/ref_harness.cpp`` (project-written) includes that unit and drives the
   shader entry points in the order of the reference's host code (WCSPHWithBoundaryModel::Step,
   SPHModel::RunSpatialHash, SpatialHash::Run, GPUCountSort::Run, GPUScan::Run,
   SpatialOffset::Run, BufferReorder), one thread at a time; it is compiled with
   ``-fsingle-precision-constant`` (Slang's unsuffixed float literals are 32-bit),
   ``-ffp-contract=off`` and OpenMP into ``oracle/_ref/libvfs_ref_shaders.so``.

3. The reference's CPU volume-map code (``src/util/``: geometry, mesh_bvh, mesh_pseudonormals,
   mesh_sdf, discretization, gaussian_quadrature, kernel, volume_map ``.cpp``) is compiled where it
   lies, unchanged, against ``oracle/ref_shim/cpu/`` (a project-written stand-in for the part of
   glm it uses, and for ``gfx/common.h`` / ``gfx/mesh.h`` without Vulkan), with the host driver
   ``oracle/ref_shim/ref_volume_map.cpp`` (MeshSDF + GenerateVolumeMap as GenericScene calls them)
   into ``oracle/_ref/libvfs_ref_volume_map.so``. This part needs the reference tree itself.

``build_generated()`` compiles an already generated ``oracle/_ref/ref_shaders_gen.cpp`` where the
reference tree is absent (the generated unit travels with the working tree).
"""
from __future__ import annotations

import re
import subprocess
import sys
from pathlib import Path

import os

HERE = Path(__file__).resolve().parent
# Where build_default() looks for the reference source tree (override: VFS_REFERENCE_TREE).
REFERENCE_TREE = Path(os.environ.get("VFS_REFERENCE_TREE", "/root/reference"))
OUT = HERE / "_ref"
SHIM = HERE / "ref_shim"
SHADERS = Path("assets/shaders/simulation")

PROGRAMS = {
    "wcsph": "wcsph_with_boundary_model.slang",
    "hash": "spatial_hash/update_spatial_hash.slang",
    "sort": "spatial_hash/sort.slang",
    "scan": "spatial_hash/scan.slang",
    "offsets": "spatial_hash/spatial_offsets.slang",
    "reorder": "spatial_hash/reorder.slang",
}


def _resolve(root: Path, importer: Path, spec: str) -> Path:
    if spec.startswith('"'):
        p = (importer.parent / (spec.strip('"') + ".slang")).resolve()
    else:
        rel = spec.replace(".", "/") + ".slang"
        p = importer.parent / rel
        if not p.exists():
            p = root / rel
    if not p.exists():
        raise FileNotFoundError(f"import {spec} from {importer}")
    return p.resolve()


def _close_structs(text: str) -> str:
    out, i = [], 0
    for m in re.finditer(r"\bstruct\s+\w+\s*\{", text):
        if m.start() < i:
            continue
        depth, j = 0, m.end() - 1
        while True:
            c = text[j]
            depth += c == "{"
            depth -= c == "}"
            j += 1
            if depth == 0:
                break
        out.append(text[i:j])
        rest = text[j:]
        if not rest.lstrip().startswith(";"):
            out.append(";")
        i = j
    out.append(text[i:])
    return "".join(out)


def translate(text: str) -> str:
    """The syntax-only rewrite of one Slang module (imports handled by the caller)."""
    t = re.sub(r"^\s*module\s+\w+\s*;\s*$", "", text, flags=re.M)
    t = re.sub(r"^\s*\[(shader|numthreads)\(.*?\)\]\s*$", "", t, flags=re.M)
    t = re.sub(r"\[\[vk::\w+\(.*?\)\]\]", "", t)
    t = re.sub(r"\bpublic\s+", "", t)
    t = re.sub(r"\buniform\s+", "", t)
    t = re.sub(r"\s*:\s*SV_\w+", "", t)
    t = re.sub(r"\bthread_local\b", "thread_local_", t)
    t = re.sub(r"\bgroupshared\b", "static thread_local", t)
    t = re.sub(r"\blet\b", "const auto", t)
    t = re.sub(r"\bvar\b", "auto", t)
    t = re.sub(r"\b(simulation|sph_model|wcsph_model)\.", r"\1::", t)
    t = re.sub(r"\.xyz\b(?!\s*\()", ".xyz()", t)
    t = re.sub(r"\b(\w+)\*\s+(\w+)", r"ref_ptr<\1> \2", t)
    return _close_structs(t)


def flatten(root: Path, entry: Path, seen=None) -> str:
    """The entry module with every imported module's text placed before it, once each."""
    seen = set() if seen is None else seen
    entry = entry.resolve()
    if entry in seen:
        return ""
    seen.add(entry)
    text = entry.read_text()
    parts = []

    def repl(m):
        parts.append(flatten(root, _resolve(root, entry, m.group(1).strip()), seen))
        return ""

    body = re.sub(r"^\s*import\s+([^;]+);\s*$", repl, text, flags=re.M)
    rel = entry.relative_to(root) if entry.is_relative_to(root) else entry
    return "".join(parts) + f"\n// ---- {SHADERS / rel}\n" + translate(body)


def generate(ref: Path) -> Path:
    root = (ref / SHADERS).resolve()
    OUT.mkdir(parents=True, exist_ok=True)
    src = ['// Generated by oracle/ref_build.py from the reference shaders; not part of the repository.',
           '#include "slang_shim.h"']
    for name, rel in PROGRAMS.items():
        src.append(f"namespace prog_{name} {{")
        src.append(flatten(root, root / rel))
        src.append(f"}}  // namespace prog_{name}")
    gen = OUT / "ref_shaders_gen.cpp"
    text = "\n".join(src) + "\n"
    if not gen.exists() or gen.read_text() != text:
        gen.write_text(text)
    return gen


def build(ref: Path) -> Path:
    generate(ref)
    return build_generated()


def build_generated() -> Path:
    gen = OUT / "ref_shaders_gen.cpp"
    if not gen.exists():
        raise FileNotFoundError(f"{gen} has not been generated")
    lib = OUT / "libvfs_ref_shaders.so"
    deps = [gen, SHIM / "ref_harness.cpp", SHIM / "slang_shim.h"]
    if lib.exists() and all(d.stat().st_mtime <= lib.stat().st_mtime for d in deps):
        return lib
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-fsingle-precision-constant",
           "-ffp-contract=off", "-U_FORTIFY_SOURCE", "-Wno-attributes", f"-I{SHIM}", f"-I{OUT}",
           str(SHIM / "ref_harness.cpp"), "-o", str(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building the reference shaders failed:\n" + " ".join(cmd) + "\n" +
                           r.stdout + r.stderr)
    return lib


VOLUME_MAP_SOURCES = ("geometry", "mesh_bvh", "mesh_pseudonormals", "mesh_sdf", "discretization",
                      "gaussian_quadrature", "kernel", "volume_map")


def build_volume_map(ref: Path) -> Path:
    """The reference's CPU volume-map code and its driver, as one shared library."""
    src = (ref / "src").resolve()
    OUT.mkdir(parents=True, exist_ok=True)
    lib = OUT / "libvfs_ref_volume_map.so"
    files = [src / "util" / f"{f}.cpp" for f in VOLUME_MAP_SOURCES] + [SHIM / "ref_volume_map.cpp"]
    deps = files + sorted((SHIM / "cpu").rglob("*.h*"))
    if lib.exists() and all(d.stat().st_mtime <= lib.stat().st_mtime for d in deps):
        return lib
    cmd = ["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-w",
           f"-I{SHIM / 'cpu'}", f"-I{src}", *map(str, files), "-o", str(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building the reference volume-map code failed:\n" + " ".join(cmd) +
                           "\n" + r.stdout + r.stderr)
    return lib


def build_default():
    """The build step's entry: regenerates and builds from the reference tree when it is present,
    else builds an already generated unit, else does nothing. Returns the library or None."""
    if (REFERENCE_TREE / SHADERS).is_dir():
        build_volume_map(REFERENCE_TREE)
        return build(REFERENCE_TREE)
    if (OUT / "ref_shaders_gen.cpp").exists():
        return build_generated()
    return None


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python oracle/ref_build.py <path of the VkFluidSim source tree>")
    print(build(Path(sys.argv[1])), build_volume_map(Path(sys.argv[1])))

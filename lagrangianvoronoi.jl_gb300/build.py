"""Builds liblvgpu.so (the C-ABI library) in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel; the mesh and physics units are
compiled with --fmad=false so that their FP64 expressions round exactly as
written (bit-identical to a sequential evaluation of the same formulas).
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblvgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]
UNITS = {
    "lv_api.cu": [],
    "lv_mesh.cu": ["--fmad=false"],
    "lv_physics.cu": ["--fmad=false"],
    "lv_solver.cu": [],
    "lv_learn.cu": [],
    "lv_fcg.cu": [],
    "lv_post.cu": ["--fmad=false"],
}


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblvgpu.so")
    return exe


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".cu", ".cuh"))] + [
        os.path.join(HERE, "..", "include", "lvgpu.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force=False, verbose=False, extra=()):
    """Compile and link liblvgpu.so unless it is newer than every source."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()
    procs = []
    objs = []
    for unit, flags in UNITS.items():
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        objs.append(obj)
        cmd = [exe, *ARCH, *COMMON, *flags, *extra, "-c", os.path.join(CSRC, unit), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((unit, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for unit, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode:
            sys.stdout.write(out.decode(errors="replace"))
        if p.returncode:
            failed.append(unit)
    if failed:
        raise RuntimeError("nvcc failed for " + ", ".join(failed))
    tmp = LIB + ".tmp"
    cmd = [exe, *ARCH, "-shared", "-o", tmp, *objs]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv,
          extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else [])
    print(LIB)

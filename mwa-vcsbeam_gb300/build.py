"""Build the GB300 library (libvcsbeam_gb300.so) in-tree with nvcc.

Each CUDA translation unit in csrc/ is compiled for sm_103a only, in
parallel, and linked into ``mwa-vcsbeam_gb300/lib/libvcsbeam_gb300.so``
(git-ignored). Plain nvcc, no cmake, no torch extension machinery: the
library exposes a C ABI (include/vcsbeam_gb300.h).
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
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libvcsbeam_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_v: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    common = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
              "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if ptxas_v:
        common += ["-Xptxas", "-v"]
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or ptxas_v or _stale(obj, [src, *headers]):
            lang = ["-x", "cu"] if src.endswith(".cu") else []
            jobs.append(common + lang + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or ptxas_v or r.returncode:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or not os.path.exists(LIB):
        link = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcuda", "-ldl"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


COMPAT_SRC = os.path.join(CSRC, "compat", "vm_compat.cu")
COMPAT_LIB = os.path.join(LIBDIR, "libvcsbeam_compat.so")


def build_compat(include_dirs, verbose: bool = False) -> str:
    """The VCSBeam-API library (lib/libvcsbeam_compat.so): csrc/compat/
    vm_compat.cu compiled against a configured VCSBeam vcsbeam.h and the
    dependency headers it includes (`include_dirs`, e.g. a VCSBeam build's
    include directories), linked to libvcsbeam_gb300.so."""
    lib = build(verbose=verbose)
    obj = os.path.join(BUILD, "vm_compat.cu.o")
    incs = []
    for d in include_dirs:
        incs += ["-I", d]
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-D__NVCC__", "-x", "cu",
           *incs, "-I", os.path.join(ROOT, "include"), "-c", COMPAT_SRC, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if verbose or r.returncode:
        sys.stderr.write(r.stdout + r.stderr)
    if r.returncode:
        raise RuntimeError("nvcc failed: " + " ".join(cmd))
    link = [nvcc(), *ARCH, "-shared", "-o", COMPAT_LIB, obj, "-L", LIBDIR, "-lvcsbeam_gb300",
            "-Xlinker", "-rpath,$ORIGIN"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return COMPAT_LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_v="-v" in sys.argv))

"""Build liblfgpu.so in-tree: every CUDA translation unit for sm_103a, compiled in
parallel with nvcc, plus the host setup code with g++/OpenMP.

    python -m lightfem_gb300.build          # or lightfem_gb300.build.build()

Output: lightfem_gb300/_lib/liblfgpu.so (git-ignored; rebuilt on every machine).
"""

from __future__ import annotations

import hashlib
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "liblfgpu.so")

CUDA_SOURCES = ["api.cu", "assemble.cu", "sparse.cu", "pcg.cu", "cg_graph.cu", "ic0.cu", "adjoint.cu", "noalloc.cu",
                "pattern.cu", "postprocess.cu", "subdomain.cu"]
HOST_SOURCES = ["host_setup.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblfgpu")


STAMP = LIB + ".stamp"


def _fingerprint() -> str:
    """Hash of every source, this script, the machine type and the compiler: a
    library built elsewhere (another architecture, other sources) never matches."""
    h = hashlib.sha256()
    files = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)) + [os.path.join(ROOT, "include", "lfgpu.h"),
                                                                        os.path.abspath(__file__)]
    for f in files:
        if os.path.isfile(f):
            h.update(os.path.basename(f).encode())
            with open(f, "rb") as fh:
                h.update(fh.read())
    h.update(platform.machine().encode())
    h.update(nvcc().encode())
    return h.hexdigest()


def _up_to_date() -> bool:
    if not (os.path.exists(LIB) and os.path.exists(STAMP)):
        return False
    with open(STAMP) as fh:
        return fh.read().strip() == _fingerprint()


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile liblfgpu.so unless a library built here from the same sources exists;
    return its path."""
    if not force and not ptxas_info and _up_to_date():
        return LIB
    os.makedirs(os.path.join(OUT_DIR, "obj"), exist_ok=True)
    nv = nvcc()
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    jobs = []
    for src in CUDA_SOURCES:
        obj = os.path.join(OUT_DIR, "obj", src + ".o")
        cmd = [nv, *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler",
               "-fPIC", *inc, "-c", os.path.join(CSRC, src), "-o", obj]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append((cmd, obj))
    cxx = os.environ.get("CXX", "g++")
    for src in HOST_SOURCES:
        obj = os.path.join(OUT_DIR, "obj", src + ".o")
        jobs.append(([cxx, "-O3", "-std=c++17", "-fPIC", "-fopenmp", *inc, "-c", os.path.join(CSRC, src),
                      "-o", obj], obj))
    procs = [(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True), cmd)
             for cmd, _ in jobs]
    failed = []
    for p, cmd in procs:
        out, _ = p.communicate()
        if verbose or ptxas_info or p.returncode != 0:
            sys.stderr.write(out)
        if p.returncode != 0:
            failed.append(" ".join(cmd))
    if failed:
        raise RuntimeError("liblfgpu build failed:\n" + "\n".join(failed))
    tmp = LIB + ".tmp"
    link = [nv, *ARCH, "-shared", "-o", tmp, *[obj for _, obj in jobs], "-Xcompiler", "-fopenmp", "-lgomp"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("liblfgpu link failed:\n" + r.stdout)
    os.replace(tmp, LIB)
    with open(STAMP, "w") as fh:
        fh.write(_fingerprint() + "\n")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))

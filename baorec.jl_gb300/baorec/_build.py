"""Compile the CUDA sources of the package into libbaorec_gb300.so (sm_103a).

Each translation unit is compiled by nvcc in parallel and linked with cuFFT;
the shared library is written next to this package's parent directory
(``baorec.jl_gb300/libbaorec_gb300.so``).  Objects go to ``_build/``.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))   # baorec.jl_gb300/
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libbaorec_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = os.path.join(home, "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def lto_sources():
    d = os.path.join(CSRC, "lto")
    return sorted(os.path.join(d, f) for f in os.listdir(d) if f.endswith(".cu")) if os.path.isdir(d) else []


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Build (incrementally) and return the path of the shared library."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    jobs = []
    objs = []
    for src in sources():
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stderr.strip() or r.stdout.strip()):
            print(r.stdout, r.stderr, flush=True)
        return r

    # cuFFT callbacks: LTO IR fatbins embedded as byte arrays (linked by cuFFT at plan creation)
    # (two IR targets: the arch-specific sm_103a and the portable sm_103; the
    # library tries them in that order)
    for src in lto_sources():
        base = os.path.basename(src)[:-3]
        blob = os.path.join(BUILD_DIR, base + "_blob.cpp")
        obj = os.path.join(BUILD_DIR, base + "_blob.o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            with open(blob, "w") as fh:
                fh.write("#include <stddef.h>\n")
                for tag, arch in (("a", "arch=compute_103a,code=lto_103a"), ("p", "arch=compute_103,code=lto_103")):
                    fat = os.path.join(BUILD_DIR, f"{base}_{tag}.fatbin")
                    run([nvcc(), "-gencode", arch, "-O3", "-std=c++17", "-dc", "-fatbin", src, "-o", fat])
                    data = open(fat, "rb").read()
                    sym = f"baorec_lto_{base}_{tag}"
                    fh.write(f'extern "C" const unsigned char {sym}[] = {{')
                    fh.write(",".join(str(b) for b in data))
                    fh.write("};\n")
                    fh.write(f'extern "C" const size_t {sym}_size = {len(data)};\n')
            jobs.append([nvcc(), *ARCH, "-O2", "-Xcompiler", "-fPIC", "-c", blob, "-o", obj])

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    if jobs or force or _stale(LIB_PATH, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB_PATH, *objs, "-lcufft", "-lnvJitLink", "-lcudart"]
        run(cmd)
    return LIB_PATH

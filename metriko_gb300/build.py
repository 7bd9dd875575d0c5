"""In-tree build of libmetriko_cuda.so for sm_103a (nvcc + g++, no cmake).

Each translation unit is compiled in parallel; the shared library lands next to this file.
Host C++ is compiled with -ffp-contract=off so that its floating-point results are the same
on x86_64 and aarch64 (no fused multiply-add contraction of the topology arithmetic), and with
OpenMP for the element-parallel host loops (each iteration writes only its own outputs).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
OUT = HERE / "libmetriko_cuda.so"
BUILD = HERE / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["mtk_ctx.cu", "mtk_field.cu", "mtk_igm.cu", "mtk_noalloc.cu", "mtk_barrier.cu", "mtk_adjoint.cu", "mtk_csr.cu",
              "mtk_topology.cu"]
CPP_SOURCES = ["mtk_pipeline.cpp"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA library cannot be built")
    return cand


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _stale(obj: Path, deps) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    inc = ["-I" + str(ROOT / "include"), "-I" + str(CSRC)]
    headers = list(CSRC.glob("*.cuh")) + list((ROOT / "include").rglob("*.h"))
    jobs = []
    for src in CU_SOURCES:
        obj = BUILD / (src + ".o")
        deps = [CSRC / src] + headers
        if force or _stale(obj, deps):
            jobs.append([nvcc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fopenmp", *inc, "-c", str(CSRC / src),
                         "-o", str(obj)])
    for src in CPP_SOURCES:
        obj = BUILD / (src + ".o")
        deps = [CSRC / src] + headers
        cuda_inc = str(Path(nvcc).resolve().parent.parent / "include")
        if force or _stale(obj, deps):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fopenmp", *inc, "-I" + cuda_inc,
                         "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr, file=sys.stderr)
    objs = [str(BUILD / (s + ".o")) for s in CU_SOURCES + CPP_SOURCES]
    if force or jobs or not OUT.exists():
        _run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fopenmp", "-o", str(OUT), *objs, "-lcudart", "-lgomp", "-lpthread"])
    return OUT


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))

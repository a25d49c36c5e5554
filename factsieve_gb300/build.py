"""In-tree build of libfactsieve.so and the factsieve CLI.

    python -m factsieve_gb300.build [--force]

nvcc compiles the CUDA sources for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), g++ the host sources with
OpenMP; the translation units compile in parallel and link into
factsieve_gb300/libfactsieve.so (CUDA runtime linked statically).  The CLI
links against that library with an $ORIGIN rpath.  Outputs are git-ignored.
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
HOST = os.path.join(HERE, "host")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfactsieve.so")
CLI = os.path.join(HERE, "bin", "factsieve")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["fs_kernels.cu", "fs_sieve2.cu", "fs_sieve4.cu", "fs_multi.cu", "fs_capi.cu", "fs_noalloc.cu",
              "fs_serve.cu", "fs_tune.cu"]
CXX_SOURCES = ["fs_host.cpp", "fs_post.cpp", "fs_putil.cpp"]
CLI_SOURCES = ["factsieve_main.cpp", "search.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def _headers(d: str) -> list[str]:
    return [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".h", ".cuh"))]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers(CSRC) + [os.path.join(INCLUDE, "factsieve.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + hdrs):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I", INCLUDE, "-c", s, "-o", o]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + hdrs):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-I", INCLUDE, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        list(ex.map(_run, jobs))
    if jobs or force or not os.path.exists(LIB):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lgomp"])
    cli_src = [os.path.join(HOST, f) for f in CLI_SOURCES]
    if all(os.path.exists(s) for s in cli_src):
        if force or jobs or not _newer(CLI, cli_src + [LIB] + _headers(HOST)):
            _run(["g++", "-O2", "-std=c++17", "-fopenmp", "-I", INCLUDE, *cli_src, "-o", CLI,
                  "-L", HERE, "-lfactsieve", "-Wl,-rpath,$ORIGIN/.."])
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)

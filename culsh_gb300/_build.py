"""Builds libculsh.so in-tree: one nvcc process per translation unit, then a link.

Only sm_103a is targeted (``-gencode arch=compute_103a,code=sm_103a``). The
library links the CUDA runtime dynamically (rpath to the toolkit), so that a
process that also loads PyTorch shares one runtime.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libculsh.so")

SOURCES = ["project.cu", "project_tc.cu", "sort.cu", "query.cu", "candidates.cu", "knn_tc.cu", "capi.cu", "serve.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libculsh")
    return cand


def _cuda_lib_dir(nvcc: str) -> str:
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        p = os.path.join(root, sub)
        if os.path.exists(os.path.join(p, "libcudart.so")):
            return p
    return os.path.join(root, "lib64")


def cflags() -> list[str]:
    return ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
            "-I", INCLUDE, "-I", CSRC] + ARCH


def build(verbose: bool = False, force: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    newest_hdr = max(os.path.getmtime(h) for h in headers)
    procs, objs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if (not force and os.path.exists(o) and os.path.getmtime(o) >= os.path.getmtime(s)
                and os.path.getmtime(o) >= newest_hdr):
            continue
        cmd = [nvcc, *cflags(), "-c", s, "-o", o]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            sys.stdout.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(src)
    if failed:
        raise RuntimeError(f"nvcc failed for {failed}")
    if procs or force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        libdir = _cuda_lib_dir(nvcc)
        cmd = [nvcc, "-shared", *ARCH, "-cudart", "shared", "-o", LIB, *objs,
               "-Xlinker", f"-rpath,{libdir}", "-L", libdir]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    build_cli(verbose)
    return LIB


CLI_SRC = os.path.join(HERE, "culsh_main.cpp")
CLI = os.path.join(HERE, "culsh_main")


def build_cli(verbose: bool = False) -> str:
    """The command-line program (culsh_main.cpp), a host C++ program over the
    drop-in header, linked against libculsh.so next to it."""
    if os.path.exists(CLI) and os.path.getmtime(CLI) >= max(
            os.path.getmtime(CLI_SRC), os.path.getmtime(LIB), os.path.getmtime(os.path.join(INCLUDE, "cuLSH.h"))):
        return CLI
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-I", INCLUDE, CLI_SRC, "-o", CLI, "-L", HERE, "-lculsh",
           "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    return CLI


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))

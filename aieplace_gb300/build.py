"""Builds libaieplace_gb300.so (sm_103a) in-tree with nvcc.

Translation units compile in parallel; the link step uses the static CUDA
runtime so the library loads on hosts without a GPU driver (the ABI symbols
can be inspected there; every compute call needs an sm_103 device).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libaieplace_gb300.so")
CLI = os.path.join(HERE, "aieplace")  # the command-line placer (csrc/cli.cpp), linked to LIB
SOURCES = ["capi.cu", "k_wirelength.cu", "k_density.cu", "k_field_simt.cu", "k_field_tc.cu", "k_surrogate.cu",
           "synth.cpp", "lefdef.cpp", "config.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-c", path, "-o", obj]
        if verbose_ptxas:
            cmd[1:1] = ["-Xptxas", "-v"]
    else:
        # no floating-point contraction: host code gives the same results on
        # x86 and Arm (the netlist generator's draws in particular)
        cmd = [nvcc(), "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-x", "c++", "-c", path,
               "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile of {src} failed:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hdrs.append(os.path.join(os.path.dirname(HERE), "include", "aieplace.h"))
    cli_src = os.path.join(CSRC, "cli.cpp")
    if not force and os.path.exists(LIB) and os.path.exists(CLI):
        newest = max(os.path.getmtime(p) for p in srcs + hdrs + [cli_src])
        if os.path.getmtime(LIB) >= newest and os.path.getmtime(CLI) >= newest:
            return LIB
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(os.path.dirname(HERE), "include"),
           cli_src, "-L", HERE, "-laieplace_gb300", "-Wl,-rpath,$ORIGIN", "-o", CLI + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build of the command-line placer failed:\n{r.stdout}\n{r.stderr}")
    os.replace(CLI + ".tmp", CLI)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    print(LIB)

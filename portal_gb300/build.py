"""Build the sm_103a shared library libportal_gb300.so in-tree.

Every translation unit is compiled by nvcc for sm_103a only, in parallel, and
linked into portal_gb300/_build/libportal_gb300.so.  No cmake, no torch
extension machinery: the library exposes a plain C ABI (include/).
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libportal_gb300.so")
SOURCES = ["ctx.cu", "rf.cu", "rf_batch.cu", "rf_static.cu", "se.cu", "image.cu", "lambda.cu", "mlp.cu",
           "warmstart.cu", "batch.cu", "adjacency.cu", "wigner.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "include", "portal_gb300.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    # host code uncontracted like the oracle (aarch64 g++ fuses a*b+c by default)
    cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd[1:1] = ["-x", "cu"]
    if verbose:
        cmd.append("-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    build_apps()
    return LIB


APPS = os.path.join(HERE, "apps")


def build_apps() -> list:
    """The drop-in executables main_portal.x and finish_portal.x (host C++
    over the C ABI), linked against the library with an $ORIGIN rpath."""
    outs = []
    io_src = os.path.join(APPS, "portal_io.cpp")
    for prog in ("main_portal", "finish_portal"):
        src = os.path.join(APPS, prog + ".cpp")
        exe = os.path.join(OUT, prog + ".x")
        deps = [src, io_src, os.path.join(APPS, "portal_io.h"), LIB]
        if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(d) for d in deps):
            # no FMA contraction: the ingestion must round exactly as the
            # reference's expressions (and the Python restatement) do on
            # every architecture
            cmd = [os.environ.get("CXX", "g++"), "-O2", "-ffp-contract=off", "-std=c++17", "-pthread",
                   "-I", os.path.join(ROOT, "include"),
                   "-I", APPS, src, io_src, "-o", exe, "-L", OUT, "-lportal_gb300", "-Wl,-rpath,$ORIGIN"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"{prog} build failed:\n{r.stderr}")
        outs.append(exe)
    return outs


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))

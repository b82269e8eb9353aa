"""Build recipe of the native library ``libfastpcc_gb300.so`` (sm_103a only).

Each ``csrc/*.cu`` translation unit is compiled by nvcc in parallel, then linked
into one shared library in this folder (in-tree, git-ignored).  The same recipe
runs on x86_64 and aarch64 hosts; nothing here depends on PyTorch.

    python -m fastpcc_gb300.native_build          # or fastpcc_gb300.build.build()
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libfastpcc_gb300.so")
OBJDIR = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-Xptxas", "-O3"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _newest_input() -> float:
    t = 0.0
    for d in (CSRC, os.path.join(HERE, "cli"), os.path.join(os.path.dirname(HERE), "include")):
        for f in os.listdir(d):
            t = max(t, os.path.getmtime(os.path.join(d, f)))
    return max(t, os.path.getmtime(__file__))


def up_to_date() -> bool:
    return (os.path.exists(OUT) and os.path.exists(CLI_OUT) and
            min(os.path.getmtime(OUT), os.path.getmtime(CLI_OUT)) >= _newest_input())


def cuda_home(cc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(cc)))


def write_jit_source() -> None:
    """The fused station kernel's source as a C++ string for run-time compilation."""
    parts = []
    for name in ("fft_core.cuh", "fused.cuh"):
        text = open(os.path.join(CSRC, name)).read()
        text = "\n".join(l for l in text.splitlines()
                         if l.strip() not in ("#pragma once", '#include "fft_core.cuh"'))
        parts.append(text)
    body = "\n".join(parts)
    assert ")FPCCJIT\"" not in body
    with open(os.path.join(OBJDIR, "jit_source.inc"), "w") as f:
        f.write('static const char* kJitSource = R"FPCCJIT(' + body + '\n)FPCCJIT";\n')


def build(force: bool = False, verbose: bool = False, extra=None) -> str:
    if not force and up_to_date():
        return OUT
    os.makedirs(OBJDIR, exist_ok=True)
    cc = nvcc()
    write_jit_source()
    home = cuda_home(cc)
    flags = NVCC_FLAGS + ARCH + ["-I" + OBJDIR, f'-DFPCC_CUDA_INCLUDE="{home}/include"'] + list(extra or [])

    def one(src):
        obj = os.path.join(OBJDIR, os.path.splitext(os.path.basename(src))[0] + ".o")
        cmd = [cc, *flags, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(one, srcs))
    tmp = OUT + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lnvrtc"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    build_cli(cc)
    return OUT


CLI_SRC = os.path.join(HERE, "cli", "fpcc_fullpair.cpp")
CLI_OUT = os.path.join(HERE, "bin", "fpcc_fullpair")


def build_cli(cc: str) -> str:
    """The command-line program (host C++), linked against the library in place."""
    os.makedirs(os.path.dirname(CLI_OUT), exist_ok=True)
    cmd = [cc, "-O2", "-std=c++17", CLI_SRC, "-o", CLI_OUT + ".tmp", "-L" + HERE, "-lfastpcc_gb300", "-lcudart",
           "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN/..", "-Xcompiler", "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the CLI failed:\n{r.stdout}\n{r.stderr}")
    os.replace(CLI_OUT + ".tmp", CLI_OUT)
    return CLI_OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra=["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else None))

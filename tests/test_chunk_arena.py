"""The server's slab sub-allocator (fastpcc_gb300/csrc/arena.h), host-only logic:
a randomised C++ check of alignment, containment, disjointness, merging of free
ranges and the return of empty chunks, compiled with the host compiler."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_chunk_arena_invariants(tmp_path, seed):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = tmp_path / "chunk_arena_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "fastpcc_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "chunk_arena_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(seed)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr

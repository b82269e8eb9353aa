"""The C-ABI library builds for sm_103a and exports every declared symbol (no GPU needed)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in ("fastpcc_gb300.h", "ccs_cuda.h"):
        path = os.path.join(ROOT, "include", h)
        if not os.path.exists(path):
            continue
        text = open(path).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:extern\s+\"C\"\s+)?[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(", text, re.M):
            name = m.group(1)
            if name not in ("defined", "if"):
                syms.add(name)
    return syms


@pytest.fixture(scope="module")
def libpath():
    from fastpcc_gb300 import native_build
    return native_build.build()


def test_library_exports_declared_symbols(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True, check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    missing = sorted(s for s in declared_symbols() if s not in exported)
    assert not missing, f"declared but not exported: {missing}"
    assert "pcc2_highlevel" in exported and "fpcc_pair_stage" in exported


def test_library_loads(libpath):
    import ctypes
    L = ctypes.CDLL(libpath)
    L.fpcc_version.restype = ctypes.c_char_p
    assert b"sm_103a" in L.fpcc_version()
    L.fpcc_choose_nz.argtypes = [ctypes.c_int] * 4
    assert L.fpcc_choose_nz(18000, -2000, 2000, 1) == 20480
    assert L.fpcc_choose_nz(18000, -2000, 2000, 0) == -1 or L.fpcc_choose_nz(18000, -2000, 2000, 0) == 32768


def test_no_cuda_calls_without_gpu(libpath):
    """Without a device, context creation fails cleanly with a message."""
    import ctypes
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    L = ctypes.CDLL(libpath)
    h = ctypes.c_void_p()
    L.fpcc_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]
    L.fpcc_last_error.restype = ctypes.c_char_p
    assert L.fpcc_create(ctypes.byref(h), 0) != 0
    assert L.fpcc_last_error()


def test_reference_cli_links_against_library(libpath):
    """The reference CLI (src/PCC_fullpair_1b.c and FFTapps.c built with -DCUDAON)
    links with libfastpcc_gb300.so in place of ccs_cuda.o and no undefined symbol
    (needs the reference sources, present only where they are mounted)."""
    from oracle import oracle as O
    if not os.path.isdir(O.reference_sources()):
        pytest.skip("reference sources not present")
    r = subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), *O.make_vars(), "-B", "cli_gb300"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    exe = os.path.join(ROOT, "oracle", "_ref", "PCC_fullpair_1b_gb300")
    out = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True, text=True, check=True).stdout
    undefined = {l.split()[-1] for l in out.splitlines()}
    assert {"pcc_highlevel", "pcc1_highlevel", "cuda_tspcc2_set_freq"} <= undefined   # resolved by the library
    ldd = subprocess.run(["ldd", exe], capture_output=True, text=True).stdout
    assert "libfastpcc_gb300.so" in ldd and "not found" not in ldd

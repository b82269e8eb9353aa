"""The allocation-free PCC2 entry point against the allocating one.

fpcc_pcc2_noalloc serves callers that cannot call cudaMalloc (a host whose pool
allocator owns all device memory, plugin frameworks that forbid device
allocation, loops that must not synchronise the device); it keeps its scratch in
a fixed device array.  This file is collected last so that a run stopping at
the first failure has already run every other test; it also passes on its own in
a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from fastpcc_gb300 import synth
from gpu_util import fp, need_gpu, relerr

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _bind(F):
    L = F.lib()
    L.fpcc_pcc2_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_void_p, C.c_int64, C.c_void_p]
    L.fpcc_pcc2_noalloc.restype = C.c_int
    L.fpcc_noalloc_scratch_bytes.restype = C.c_size_t
    L.fpcc_noalloc_last_error.restype = C.c_char_p
    return L


def test_noalloc_matches_allocating_entry_point_twice():
    need_gpu()
    import torch
    F = fp()
    L = _bind(F)
    # two calls in a row with different sizes: the second must not see the first's leftovers
    for call, (N, Tr, l1, l2, d) in enumerate([(4500, 3, -450, 450, -200), (18000, 2, -2000, 2000, 150)]):
        a, b = synth.plain_pair(N=N, n_windows=Tr, delay=d, tag=f"noalloc/{call}")
        y_ref = F.pcc2_set(a, b, l1, l2)              # the allocating entry point
        nl = abs(l2 - l1) + 1
        da = torch.from_numpy(a).cuda()
        db = torch.from_numpy(b).cuda()
        dy = torch.full((Tr, nl), float("nan"), dtype=torch.float32, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        rc = L.fpcc_pcc2_noalloc(da.data_ptr(), db.data_ptr(), N, N, Tr, l1, l2, dy.data_ptr(), nl, stream)
        torch.cuda.synchronize()
        assert rc == 0, L.fpcc_noalloc_last_error().decode()
        y = dy.cpu().numpy()
        assert np.isfinite(y).all()
        assert relerr(y, y_ref) < TOL, f"call {call}"


def test_noalloc_rejects_oversized_calls():
    need_gpu()
    import torch
    F = fp()
    L = _bind(F)
    cap = L.fpcc_noalloc_scratch_bytes()
    N = 18000
    Tr = int(cap // (N * 8)) + 1          # the analytic buffers alone exceed the array
    d = torch.zeros(1, dtype=torch.float32, device="cuda")
    rc = L.fpcc_pcc2_noalloc(d.data_ptr(), d.data_ptr(), N, N, Tr, -100, 100, d.data_ptr(), 201,
                             torch.cuda.current_stream().cuda_stream)
    assert rc == F.FpccError(-3, "").code
    assert b"scratch" in L.fpcc_noalloc_last_error()

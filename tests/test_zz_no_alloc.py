"""The allocation-free PCC2 entry point (fpcc_pcc2_noalloc).

It serves callers that cannot call cudaMalloc (a host whose pool allocator owns
all device memory, plugin frameworks that forbid device allocation, loops that
must not synchronise the device); it keeps its scratch in a fixed device array.
Checked here: two calls in a row agree with the FP64 oracle and with the
allocating entry point, device memory in use does not change across a call,
and reversed lags, strided input rows and padded output rows are honoured.
This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
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


def _call(L, torch, a, b, l1, l2, ldx=None, ldy=None):
    """a, b: (Tr, N) host arrays; rows placed at stride ldx >= N, outputs at stride ldy >= L."""
    Tr, N = a.shape
    ldx = ldx or N
    nl = abs(l2 - l1) + 1
    ldy = ldy or nl
    da = torch.zeros((Tr, ldx), dtype=torch.float32, device="cuda")
    db = torch.zeros((Tr, ldx), dtype=torch.float32, device="cuda")
    da[:, :N] = torch.from_numpy(a)
    db[:, :N] = torch.from_numpy(b)
    dy = torch.full((Tr, ldy), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.fpcc_pcc2_noalloc(da.data_ptr(), db.data_ptr(), ldx, N, Tr, l1, l2, dy.data_ptr(), ldy, stream)
    torch.cuda.synchronize()
    assert rc == 0, L.fpcc_noalloc_last_error().decode()
    assert L.fpcc_noalloc_last_error() == b""
    y = dy.cpu().numpy()
    assert np.isnan(y[:, nl:]).all()          # padding of the output rows untouched
    return y[:, :nl]


def test_noalloc_matches_oracle_and_allocating_entry_point_twice(orc):
    need_gpu()
    import torch
    F = fp()
    L = _bind(F)
    # two calls in a row with different sizes: the second must not see the first's leftovers
    for call, (N, Tr, l1, l2, d) in enumerate([(4500, 3, -450, 450, -200), (18000, 2, -2000, 2000, 150)]):
        a, b = synth.plain_pair(N=N, n_windows=Tr, delay=d, tag=f"noalloc/{call}")
        y = _call(L, torch, a, b, l1, l2)
        assert np.isfinite(y).all()
        assert relerr(y, orc.pcc2(a, b, l1, l2)) < TOL, f"call {call} vs oracle"
        assert relerr(y, F.pcc2_set(a, b, l1, l2)) < TOL, f"call {call} vs allocating path"


def test_noalloc_reversed_lags_strided_rows_padded_output(orc):
    need_gpu()
    import torch
    F = fp()
    L = _bind(F)
    a, b = synth.plain_pair(N=6000, n_windows=3, delay=45, tag="noalloc/strided")
    y = _call(L, torch, a, b, 600, -300, ldx=6144, ldy=1000)   # Lag1 > Lag2
    assert relerr(y, orc.pcc2(a, b, 600, -300)) < TOL
    assert relerr(y, F.pcc2_set(a, b, 600, -300)) < TOL


def test_noalloc_leaves_device_memory_unchanged():
    need_gpu()
    import torch
    F = fp()
    L = _bind(F)
    N, Tr, l1, l2 = 18000, 4, -2000, 2000
    a, b = synth.plain_pair(N=N, n_windows=Tr, delay=70, tag="noalloc/mem")
    da = torch.from_numpy(a).cuda()
    db = torch.from_numpy(b).cuda()
    dy = torch.empty((Tr, l2 - l1 + 1), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        rc = L.fpcc_pcc2_noalloc(da.data_ptr(), db.data_ptr(), N, N, Tr, l1, l2, dy.data_ptr(), l2 - l1 + 1,
                                 stream)
        torch.cuda.synchronize()
        assert rc == 0, L.fpcc_noalloc_last_error().decode()

    call()                                   # warm: device code loaded, kernel attributes set
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        call()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


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

"""The reference's own GPU boundary (src/ccs_cuda.h) through libfastpcc_gb300.so.

pcc_highlevel / pcc1_highlevel take analytic signals that a producer thread
publishes window by window with sem_post, as src/FFTapps.c:636-684 does;
pcc1_highlevel2 takes raw traces; cuda_tspcc2_set_freq takes the caller's
wavelet family.  Each is compared with the FP64 oracle under the normalisation
rule that reference function applies (tolerance 1e-4 relative to the peak).
"""
import ctypes as C
import threading
import time

import numpy as np
import pytest

from fastpcc_gb300 import synth
from gpu_util import fp, need_gpu, relerr

pytestmark = pytest.mark.gpu
TOL = 1e-4
SEM_T_SIZE = 32   # sizeof(sem_t) with glibc on 64-bit Linux (x86_64 and aarch64)


@pytest.fixture(scope="module")
def L():
    need_gpu()
    F = fp()
    lib = F.lib()
    fpp = C.POINTER(C.POINTER(C.c_float))
    lib.pcc_highlevel.argtypes = [fpp, C.c_void_p, C.c_void_p, C.c_int, C.c_uint, C.c_float, C.c_int, C.c_int,
                                  C.c_void_p]
    lib.pcc1_highlevel.argtypes = [fpp, C.c_void_p, C.c_void_p, C.c_int, C.c_uint, C.c_int, C.c_int, C.c_void_p]
    lib.pcc1_highlevel2.argtypes = [fpp, fpp, fpp, C.c_int, C.c_uint, C.c_int, C.c_int]
    lib.pcc1_highlevel2.restype = None
    lib.cuda_tspcc2_set_freq.argtypes = [fpp, fpp, fpp, C.c_uint, C.c_uint, C.c_uint, C.c_int, C.c_int, C.c_uint,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float]
    return lib


def rows(a, ct=C.c_float):
    r = (C.POINTER(ct) * a.shape[0])()
    for k in range(a.shape[0]):
        r[k] = a[k].ctypes.data_as(C.POINTER(ct))
    return r


def analytic_rows(orc, x):
    return np.stack([orc.analytic(r) for r in x]).astype(np.complex64)


@pytest.mark.parametrize("v", [1.0, 1.5])
def test_pcc_highlevel_with_producer_semaphores(L, orc, v):
    Tr, N, l1, l2 = 20, 3000, -300, 300
    a, b = synth.plain_pair(N=N, n_windows=Tr, delay=45, tag=f"ccs/pcc{v}")
    xa1, xa2 = analytic_rows(orc, a), analytic_rows(orc, b)
    libc = C.CDLL("libc.so.6", use_errno=True)
    sems = C.create_string_buffer(SEM_T_SIZE * Tr)
    base = C.addressof(sems)
    for t in range(Tr):
        assert libc.sem_init(C.c_void_p(base + SEM_T_SIZE * t), 0, 0) == 0
    # the producer fills the rows late and posts each window's semaphore after it
    ready1 = np.zeros_like(xa1)
    ready2 = np.zeros_like(xa2)

    def producer():
        for t in range(Tr):
            time.sleep(0.002)
            ready1[t] = xa1[t]
            ready2[t] = xa2[t]
            libc.sem_post(C.c_void_p(base + SEM_T_SIZE * t))

    y = np.zeros((Tr, l2 - l1 + 1), np.float32)
    th = threading.Thread(target=producer)
    th.start()
    r1, r2 = rows(ready1, C.c_float), rows(ready2, C.c_float)
    if v == 1.0:
        rc = L.pcc1_highlevel(rows(y), r1, r2, N, Tr, l1, l2, C.c_void_p(base))
    else:
        rc = L.pcc_highlevel(rows(y), r1, r2, N, Tr, v, l1, l2, C.c_void_p(base))
    th.join()
    assert rc == 0
    for t in range(Tr):
        libc.sem_destroy(C.c_void_p(base + SEM_T_SIZE * t))
    p1 = xa1.astype(np.complex128)
    p2 = xa2.astype(np.complex128)
    p1 = np.where(np.abs(p1) > 0, p1 / np.abs(p1), 0)
    p2 = np.where(np.abs(p2) > 0, p2 / np.abs(p2), 0)
    y64 = np.stack([orc.pccv_phase(p1[t], p2[t], v, l1, l2, norm_gpu=True) for t in range(Tr)])
    assert relerr(y, y64) < TOL


def test_pcc1_highlevel2_raw_traces(L, orc):
    Tr, N, l1, l2 = 3, 2400, -200, 200
    a, b = synth.plain_pair(N=N, n_windows=Tr, delay=-30, tag="ccs/pcc1b")
    y = np.zeros((Tr, l2 - l1 + 1), np.float32)
    L.pcc1_highlevel2(rows(y), rows(a), rows(b), N, Tr, l1, l2)
    y64 = orc.pccv(a, b, 1.0, l1, l2, rule=orc.AMP_SUMTHR, norm_gpu=True)
    assert relerr(y, y64) < TOL


def test_cuda_tspcc2_set_freq_with_callers_family(L, orc):
    N, Tr, l1, l2, pmin, pmax, V, wt = 3000, 2, -250, 250, 4.0, 60.0, 2, -3
    a, b = synth.plain_pair(N=N, n_windows=Tr, delay=37, fs=20.0, band=(0.02, 5.0), tag="ccs/wpcc")
    su = orc.wpcc_setup(N, l1, l2, pmin, pmax, V, wt)
    M = max(abs(l1), abs(l2))
    nz0 = orc.nz_rule(N, l1, l2)
    scale, Ls, center, taps = orc.wavelet_family(wt, su["J"], V, nz0, su["s0"], su["op1"])
    S = su["S"]
    wrows = []
    off = 0
    for s in range(S):
        wrows.append(np.ascontiguousarray(taps[off:off + Ls[s]]))
        off += int(Ls[s])
    wc = (C.c_void_p * S)(*[w.ctypes.data for w in wrows])
    down = np.ones(S, np.uint32)
    K0 = float(np.sum(1.0 / scale))
    Cc = 1.0 / (K0 * N)
    y = np.zeros((Tr, l2 - l1 + 1), np.float32)
    rc = L.cuda_tspcc2_set_freq(rows(y), rows(a), rows(b), N, Tr, su["Nz"], l1, l2, S, scale.ctypes.data, wc,
                                Ls.ctypes.data, center.ctypes.data, down.ctypes.data, Cc)
    assert rc == 0
    y64 = orc.wpcc(a, b, l1, l2, pmin, pmax, V=V, wtype=wt, rule=orc.AMP_THRESH)
    assert relerr(y, y64) < TOL
    down[0] = 2
    assert L.cuda_tspcc2_set_freq(rows(y), rows(a), rows(b), N, Tr, su["Nz"], l1, l2, S, scale.ctypes.data, wc,
                                  Ls.ctypes.data, center.ctypes.data, down.ctypes.data, Cc) == -2
    assert M < N

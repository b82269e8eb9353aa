"""The timed CPU baseline (oracle/cpuref.py: the reference's method layer in its
own precisions, scipy FFTs) agrees with the FP64 oracle, so the benchmark's CPU
figures time the same computation the GPU path performs."""
import numpy as np
import pytest

from fastpcc_gb300 import synth


def relerr(y, y64):
    y = np.atleast_2d(np.asarray(y, np.float64))
    y64 = np.atleast_2d(np.asarray(y64, np.float64))
    return float(np.max(np.max(np.abs(y - y64), axis=1) / np.max(np.abs(y64), axis=1)))


@pytest.fixture(scope="module")
def cr():
    from oracle import cpuref
    return cpuref


@pytest.mark.parametrize("N,l1,l2", [(3000, -300, 300), (2500, 400, -100), (4096, 10, 900)])
def test_fft_methods_match_oracle(orc, cr, N, l1, l2):
    a, b = synth.plain_pair(N=N, n_windows=3, delay=55, tag=f"cpuref/{N}")
    assert relerr(cr.pcc2_set(a, b, l1, l2), orc.pcc2(a, b, l1, l2)) < 1e-4       # single precision
    assert relerr(cr.ccgn_set(a, b, l1, l2), orc.gncc(a, b, l1, l2)) < 1e-6       # double precision
    assert relerr(cr.cc1b_set(a, b, l1, l2), orc.cc1b(a, b, l1, l2)) < 1e-5


def test_pcc1_matches_oracle(orc, cr):
    a, b = synth.plain_pair(N=2000, n_windows=2, delay=-40, tag="cpuref/pcc1")
    assert relerr(cr.pcc1_set(a, b, -200, 150), orc.pcc1(a, b, -200, 150)) < 1e-4


def test_wpcc_matches_oracle(orc, cr):
    a, b = synth.plain_pair(N=3000, n_windows=2, delay=30, fs=20.0, band=(0.02, 5.0), tag="cpuref/wpcc")
    for wt in (-1, -3):
        y64 = orc.wpcc(a, b, -300, 300, 4.0, 80.0, V=3, wtype=wt)
        assert relerr(cr.wpcc_set(a, b, -300, 300, 4.0, 80.0, V=3, wtype=wt), y64) < 1e-6


def test_reference_padding_and_cpu_model(cr):
    assert cr.nz_rule(36000, -3000, 3000) == 65536
    assert cr.nz_rule(18000, -2000, 2000) == 32768
    assert isinstance(cr.cpu_model(), str) and cr.threads() >= 1

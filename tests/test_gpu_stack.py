"""Stacks of correlation traces on the device (fpcc_stack) through the C ABI:

* ts-PWS against the same stack computed on the reference's own wavelet
  transforms (complex_1D_wavelet_dec / Re_complex_1D_wavelet_rec of src/FWTa;
  tests/golden/golden_stack.npz) for Morlet, complete Morlet and Mexican-hat
  families, odd and even trace lengths;
* linear and phase-weighted stacks against the FP64 oracle;
* several groups per call, one trace per group, rejected arguments.
Tolerance 1e-4 of the stack's peak (FP32 transforms; measured far below)."""
import os

import numpy as np
import pytest

from gpu_util import fp, need_gpu, relerr
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-4
G = os.path.join(os.path.dirname(__file__), "golden", "golden_stack.npz")


@pytest.fixture(scope="module")
def F():
    need_gpu()
    return fp()


@pytest.fixture(scope="module")
def g():
    return np.load(G)


def _case(g, i):
    L, K, wt, V, pmin, pmax, nu = g["cases"][i]
    return int(L), int(K), int(wt), int(V), float(pmin), float(pmax), float(nu)


def _stack(F, ctx, mode, c, K, **kw):
    import torch
    c = np.ascontiguousarray(c, np.float32)
    rows, L = c.shape
    ng = rows // K
    d_y = torch.from_numpy(c).cuda()
    d_o = torch.zeros((ng, L), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ctx.stack(mode, d_y.data_ptr(), L, K, L, ng, d_o.data_ptr(), L, **kw)
    ctx.sync()
    return d_o.cpu().numpy()


def test_tspws_matches_reference_transforms(F, g):
    ctx = F.Context(0)
    for i in range(len(g["cases"])):
        L, K, wt, V, pmin, pmax, nu = _case(g, i)
        y = _stack(F, ctx, F.STACK_TSPWS, g[f"c{i}"], K, nu=nu, pmin=pmin, pmax=pmax, V=V, type=wt)
        assert relerr(y, g[f"tspws{i}"][None]) < TOL, (i, relerr(y, g[f"tspws{i}"][None]))
    ctx.close()


def test_linear_and_pws_match_oracle(F, g):
    ctx = F.Context(0)
    for i in range(len(g["cases"])):
        L, K, wt, V, pmin, pmax, nu = _case(g, i)
        c = g[f"c{i}"]
        for mode in (F.STACK_LINEAR, F.STACK_PWS):
            y = _stack(F, ctx, mode, c, K, nu=nu)
            assert relerr(y, O.stack(c, mode, nu)[None]) < TOL, (i, mode)
    ctx.close()


def test_groups_in_one_call(F, g):
    ctx = F.Context(0)
    L, K, wt, V, pmin, pmax, nu = _case(g, 0)
    c = g["c0"]                                   # 24 traces -> 3 groups of 8
    for mode in (F.STACK_LINEAR, F.STACK_PWS, F.STACK_TSPWS):
        y = _stack(F, ctx, mode, c, 8, nu=nu, pmin=pmin, pmax=pmax, V=V, type=wt)
        for k in range(3):
            ref = O.stack(c[8 * k:8 * k + 8], mode, nu, pmin, pmax, V, wt)
            assert relerr(y[k], ref[None]) < TOL, (mode, k)
    ctx.close()


def test_window_major_rows(F, g):
    # an all-pairs pair stage writes row w * P + p (window-major); the stack
    # reads each pair's traces in place with ldj = P * L, ldg = L
    import torch
    ctx = F.Context(0)
    L, K, wt, V, pmin, pmax, nu = _case(g, 0)
    c = g["c0"].reshape(3, 8, L)                       # (group, trace, lag)
    wm = np.ascontiguousarray(c.transpose(1, 0, 2))    # (trace, group, lag): window-major
    d_y = torch.from_numpy(wm.reshape(24, L)).cuda()
    d_o = torch.zeros((3, L), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for mode in (F.STACK_LINEAR, F.STACK_PWS, F.STACK_TSPWS):
        ctx.stack(mode, d_y.data_ptr(), L, 8, L, 3, d_o.data_ptr(), L, nu=nu, pmin=pmin, pmax=pmax, V=V, type=wt,
                  ldg=L, ldj=3 * L)
        ctx.sync()
        y = d_o.cpu().numpy()
        for k in range(3):
            assert relerr(y[k], O.stack(c[k], mode, nu, pmin, pmax, V, wt)[None]) < TOL, (mode, k)
    ctx.close()


def test_single_trace_and_errors(F):
    ctx = F.Context(0)
    x = np.random.default_rng(5).standard_normal((1, 700)).astype(np.float32)
    # one trace: unit coherence, so PWS is the trace and ts-PWS the inverse CWT of its CWT
    assert relerr(_stack(F, ctx, F.STACK_PWS, x, 1, nu=2.0), x) < TOL
    fam = O.stack_family(700, 8.0, 150.0, 4, -3)
    ref = O.icwt(O.cwt(x[0].astype(np.float64), fam), fam, 4)
    y = _stack(F, ctx, F.STACK_TSPWS, x, 1, nu=2.0, pmin=8.0, pmax=150.0, V=4, type=-3)
    assert relerr(y, ref[None]) < TOL
    with pytest.raises(F.FpccError):
        _stack(F, ctx, F.STACK_TSPWS, x, 1, pmin=0.0, pmax=150.0, V=4, type=-1)   # pmin must be > 0
    with pytest.raises(F.FpccError):
        _stack(F, ctx, F.STACK_TSPWS, x, 1, pmin=8.0, pmax=150.0, V=4, type=5)    # unknown wavelet
    with pytest.raises(F.FpccError):
        _stack(F, ctx, 7, x, 1)                                                    # unknown mode
    ctx.close()


def test_long_traces_many_windows_and_zero_trace(F):
    # L = 12001: CWT length class 24576 is beyond the in-block menu (global
    # radix passes); K = 40 > 32 exercises the coherence's runs of 32 traces; one
    # all-zero trace contributes zero phasors; nu = 1.5 takes the general power
    rng = np.random.default_rng(11)
    L, K = 12001, 40
    t = np.arange(L) - L // 2
    pulse = np.exp(-0.5 * ((t - 800) / 30.0) ** 2) * np.cos(2 * np.pi * (t - 800) / 90.0)
    c = (0.8 * rng.standard_normal((K, L)) + (0.5 + rng.random((K, 1))) * pulse).astype(np.float32)
    c[7] = 0.0
    ctx = F.Context(0)
    for mode, kw in ((F.STACK_LINEAR, {}), (F.STACK_PWS, dict(nu=1.5)),
                     (F.STACK_TSPWS, dict(nu=1.5, pmin=20.0, pmax=80.0, V=2, type=-1))):
        y = _stack(F, ctx, mode, c, K, **kw)
        ref = O.stack(c, mode, kw.get("nu", 2.0), kw.get("pmin", 0.0), kw.get("pmax", 0.0), kw.get("V", 4),
                      kw.get("type", -1))
        assert relerr(y, ref[None]) < TOL, (mode, relerr(y, ref[None]))
    ctx.close()

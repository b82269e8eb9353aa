"""The stacking oracle (oracle64.c orc_stack) pinned against the reference's own
wavelet library: its CWT and inverse CWT against complex_1D_wavelet_dec and
Re_complex_1D_wavelet_rec (src/FWTa), and its ts-PWS against the same stack
computed on those reference transforms (tests/golden/golden_stack.npz, made by
tests/golden/make_stack_golden.py); plus known answers of the three stacks."""
import os

import numpy as np
import pytest

from oracle import oracle as O

G = os.path.join(os.path.dirname(__file__), "golden", "golden_stack.npz")


@pytest.fixture(scope="module")
def g():
    return np.load(G)


def _case(g, i):
    L, K, wt, V, pmin, pmax, nu = g["cases"][i]
    return int(L), int(K), int(wt), int(V), float(pmin), float(pmax), float(nu)


def test_cwt_and_inverse_match_reference_library(g):
    L, K, wt, V, pmin, pmax, nu = _case(g, 0)
    fam = O.stack_family(L, pmin, pmax, V, wt)
    x = g["c0"][0].astype(np.float64)
    W = O.cwt(x, fam)
    assert np.abs(W - g["cwt0"]).max() / np.abs(g["cwt0"]).max() < 1e-6
    for i in range(len(g["cases"])):
        L, K, wt, V, pmin, pmax, nu = _case(g, i)
        fam = O.stack_family(L, pmin, pmax, V, wt)
        xr = O.icwt(O.cwt(g[f"c{i}"][0].astype(np.float64), fam), fam, V)
        assert np.abs(xr - g[f"icwt{i}"]).max() / np.abs(g[f"icwt{i}"]).max() < 1e-12, i


def test_tspws_matches_stack_on_reference_transforms(g):
    for i in range(len(g["cases"])):
        L, K, wt, V, pmin, pmax, nu = _case(g, i)
        y = O.stack(g[f"c{i}"], O.STACK_TSPWS, nu, pmin, pmax, V, wt)
        assert O.relerr(y, g[f"tspws{i}"])[0] < 1e-12, i


def test_stack_known_answers():
    rng = np.random.default_rng(3)
    x = rng.standard_normal(600).astype(np.float32)
    same = np.tile(x, (5, 1))
    # linear mean of identical rows is the row; unit coherence leaves PWS equal to it
    assert np.allclose(O.stack(same, O.STACK_LINEAR), x, atol=1e-6)
    assert np.allclose(O.stack(same, O.STACK_PWS, 2.0), x, atol=1e-5)
    # ts-PWS of identical rows is the inverse CWT of the row's CWT (coherence 1)
    fam = O.stack_family(600, 8.0, 100.0, 4, -1)
    ref = O.icwt(O.cwt(x.astype(np.float64), fam), fam, 4)
    assert O.relerr(O.stack(same, O.STACK_TSPWS, 2.0, 8.0, 100.0, 4, -1), ref)[0] < 1e-10
    # nu = 0: no weighting, PWS is the linear stack
    y = rng.standard_normal((7, 600)).astype(np.float32)
    assert np.allclose(O.stack(y, O.STACK_PWS, 0.0), O.stack(y, O.STACK_LINEAR), atol=1e-12)
    # incoherent rows: the phase weights shrink the stack
    assert np.abs(O.stack(y, O.STACK_PWS, 2.0)).max() < np.abs(O.stack(y, O.STACK_LINEAR)).max()

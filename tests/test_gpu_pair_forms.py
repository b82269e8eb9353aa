"""GPU parity of the two pair kernels (fpcc_pair_form): the one-block-per-
correlation kernel and the tiled kernel (Nz/2 = R1 x 256) must both match the
FP64 oracle within 1e-4 of each correlation's peak, for PCC2 (full spectra),
GNCC and 1-bit (Hermitian half spectra), the 16-bit storage formats and the
packed descriptor launch, on lag windows that wrap around zero, lie on one
side of it, or span most of the padded length.
"""
import numpy as np
import pytest

from fastpcc_gb300 import synth
from gpu_util import fp, need_gpu, relerr

pytestmark = pytest.mark.gpu

TOL = 1e-4
NZS = (16384, 20480)   # half lengths 32 x 256 and 40 x 256


@pytest.fixture(scope="module")
def F():
    need_gpu()
    F = fp()
    yield F
    for nz in NZS:
        F.pair_form(nz, F.PAIR_TILED)


def both_forms(F, nz, fn):
    out = {}
    for form in (F.PAIR_BLOCK, F.PAIR_TILED):
        assert F.pair_form(nz, form) == form
        out[form] = fn()
    F.pair_form(nz, F.PAIR_TILED)
    return out[F.PAIR_BLOCK], out[F.PAIR_TILED]


@pytest.mark.parametrize("nz", NZS)
@pytest.mark.parametrize("N,l1,l2", [(4500, -450, 450), (6000, -2999, 800), (7000, 30, 3100),
                                     (8000, -7000, -6000), (4096, -4095, 4095)])
def test_pcc2_both_forms(F, orc, nz, N, l1, l2):
    a, b = synth.plain_pair(N=N, n_windows=2, delay=min(300, N // 20), tag=f"gpu/forms/{N}")
    if N + max(abs(l1), abs(l2)) > nz:
        pytest.skip("lags beyond the padded length")
    y64 = orc.pcc2(a, b, l1, l2)
    yb, yt = both_forms(F, nz, lambda: F.pcc2_set(a, b, l1, l2, nz_mode=nz))
    assert relerr(yb, y64) < TOL
    assert relerr(yt, y64) < TOL


@pytest.mark.parametrize("nz", NZS)
def test_row_pass_pruning_edges(F, orc, nz):
    """The tiled kernel's last row pass forms only the row outputs q in
    [-32, 32) when every stored lag lies in [-64 R1, 64 R1) (R1 = Nz / 512):
    lag windows exactly at that edge (even and odd first lag) and one lag past
    it on either side (full pass)."""
    e = nz // 8
    a, b = synth.plain_pair(N=4000, n_windows=2, delay=120, tag="gpu/forms/edges")
    for l1, l2 in ((-e, e - 1), (-e + 1, e - 2), (-e - 1, e - 1), (-e, e), (e - 700, e - 1), (-e, -e + 500)):
        y64 = orc.pcc2(a, b, l1, l2)
        yb, yt = both_forms(F, nz, lambda: F.pcc2_set(a, b, l1, l2, nz_mode=nz))
        assert relerr(yb, y64) < TOL, (l1, l2)
        assert relerr(yt, y64) < TOL, (l1, l2)


@pytest.mark.parametrize("nz", NZS)
def test_gncc_and_1bit_both_forms(F, orc, nz):
    a, b = synth.plain_pair(N=7000, n_windows=2, delay=-180, tag="gpu/forms/herm")
    for f, o in ((F.ccgn_set, orc.gncc), (F.cc1b_set, orc.cc1b)):
        y64 = o(a, b, -1500, 1200)
        yb, yt = both_forms(F, nz, lambda: f(a, b, -1500, 1200, nz_mode=nz))
        assert relerr(yb, y64) < TOL, f.__name__
        assert relerr(yt, y64) < TOL, f.__name__


@pytest.mark.parametrize("nz", NZS)
def test_int16_storage_both_forms(F, orc, nz):
    a, b = synth.plain_pair(N=6000, n_windows=2, delay=90, tag="gpu/forms/i16")
    y64 = orc.pcc2(a, b, -900, 900)
    yb, yt = both_forms(F, nz, lambda: F.pcc2_set(a, b, -900, 900, nz_mode=nz, fmt=F.I16))
    assert relerr(yb, y64) < TOL
    assert relerr(yt, y64) < TOL


def test_all_pairs_window_many_blocks(F, orc):
    """All-pairs size (N = 18000, lags +-2000, Nz = 20480) with more correlations
    than resident blocks, so each tiled block loops over several correlations;
    both forms agree with each other and with the oracle on a sample."""
    import torch
    n_sta, n_win, N, lag = 40, 2, 18000, 2000
    x, _ = synth.all_pairs(n_stations=n_sta, n_windows=n_win, N=N, tag="gpu/forms/allpairs")
    x = np.ascontiguousarray(x.reshape(n_sta * n_win, N))
    iu, ju = np.triu_indices(n_sta, k=1)
    w = np.repeat(np.arange(n_win), iu.size)
    pairs = np.ascontiguousarray(np.stack([np.tile(iu, n_win) * n_win + w, np.tile(ju, n_win) * n_win + w],
                                          axis=1).astype(np.int32))
    P, L = pairs.shape[0], 2 * lag + 1
    Nz = F.choose_nz(N, -lag, lag, F.NZ_FAST)
    assert Nz == 20480
    ctx = F.Context(0)
    d_x = torch.from_numpy(x).cuda()
    d_p = torch.from_numpy(pairs).cuda()
    d_s = torch.empty((x.shape[0], 2 * Nz), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ctx.station_stage(F.PCC2, d_x.data_ptr(), N, x.shape[0], N, Nz, F.F32, F.AMP_F_REG, d_s.data_ptr(), Nz)

    def run():
        d_y = torch.full((P, L), float("nan"), dtype=torch.float32, device="cuda")
        ctx.pair_stage(F.PCC2, d_s.data_ptr(), Nz, F.F32, d_p.data_ptr(), P, N, Nz, -lag, lag,
                       d_y=d_y.data_ptr(), ldy=L)
        ctx.sync()
        return d_y.cpu().numpy()

    yb, yt = both_forms(F, Nz, run)
    ctx.close()
    assert np.isfinite(yt).all()
    assert np.max(np.abs(yt - yb)) <= 2e-5 * np.max(np.abs(yb))
    sel = np.random.default_rng(3).choice(P, 5, replace=False)
    assert relerr(yt[sel], orc.pcc2(x[pairs[sel, 0]], x[pairs[sel, 1]], -lag, lag)) < TOL


def test_packed_descriptors_both_forms(F, orc):
    """Packed launch (fpcc_pair_stage_packed) at Nz = 20480: windows of
    different lengths and lag windows in one launch, more descriptors than
    resident blocks."""
    import ctypes as C
    import torch
    nz = 20480
    cases = [(9000, -1000, 1000), (6000, 20, 2500), (8500, -3000, -100), (4000, -50, 3999)]
    reps = 200
    ctx = F.Context(0)
    rows, y64, keep = [], [], []
    for k, (n, l1, l2) in enumerate(cases):
        a, b = synth.plain_pair(N=n, n_windows=1, delay=77, tag=f"gpu/forms/packed/{k}")
        y64.append(orc.pcc2(a, b, l1, l2))
        d_x = torch.from_numpy(np.concatenate([a, b])).cuda()
        d_s = torch.empty((2, 2 * nz), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        ctx.station_stage(F.PCC2, d_x.data_ptr(), n, 2, n, nz, F.F32, F.AMP_F_REG, d_s.data_ptr(), nz)
        keep += [d_x, d_s]
        rows.append(d_s)
    ctx.sync()
    Lmax = max(abs(l2 - l1) + 1 for _, l1, l2 in cases)
    d_y = torch.zeros((reps * len(cases), Lmax), dtype=torch.float32, device="cuda")
    desc = (F.PairDesc * (reps * len(cases)))()
    for r in range(reps):
        for k, (n, l1, l2) in enumerate(cases):
            i = r * len(cases) + k
            desc[i] = F.PairDesc(rows[k].data_ptr(), rows[k].data_ptr() + 2 * nz * 4, None, None,
                                 d_y.data_ptr() + i * Lmax * 4, n, min(l1, l2), abs(l2 - l1) + 1, 0.0)
    raw = torch.frombuffer(bytearray(C.string_at(C.addressof(desc), C.sizeof(desc))), dtype=torch.uint8).cuda()

    def run():
        d_y.zero_()
        ctx.pair_stage_packed(F.PCC2, F.F32, nz, raw.data_ptr(), reps * len(cases), Lmax)
        ctx.sync()
        return d_y.cpu().numpy()

    yb, yt = both_forms(F, nz, run)
    ctx.close()
    for k, (n, l1, l2) in enumerate(cases):
        L = abs(l2 - l1) + 1
        for y in (yb, yt):
            got = y[k::len(cases), :L]
            assert np.array_equal(got, np.repeat(got[:1], reps, axis=0))
            assert relerr(got[:1], y64[k]) < TOL


def test_form_query_and_unsupported(F):
    assert F.pair_form(20480) == F.PAIR_TILED
    assert F.pair_form(4096) == F.PAIR_BLOCK
    with pytest.raises(F.FpccError):
        F.pair_form(4096, F.PAIR_TILED)

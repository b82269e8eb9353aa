"""GPU parity: every method through the C ABI against the FP64 oracle.

Error metric: max over lags of |y - y64| divided by max |y64| of the same
correlation (relative to its own peak).  Tolerance 1e-4 for every FP32 path and
for block-scaled int16 storage (the 4-byte storage format the library offers
for the 1e-4 target); the 1-bit popcount numerators must be bit-exact.  FP16
storage is not within 1e-4 (see test_pcc2_fp16_storage) and is not offered for it.
"""
import numpy as np
import pytest

from fastpcc_gb300 import synth
from gpu_util import fp, need_gpu, relerr

pytestmark = pytest.mark.gpu

TOL = 1e-4
CASES = [
    # N, Tr, Lag1, Lag2, delay
    (1000, 3, -100, 100, 37),
    (1200, 2, -400, -20, -150),
    (2048, 2, 10, 300, 120),
    (3000, 2, 250, -250, 60),
    (4500, 2, -450, 450, -200),
]


@pytest.fixture(scope="module")
def F():
    need_gpu()
    return fp()


def _data(N, Tr, d, tag):
    return synth.plain_pair(N=N, n_windows=Tr, delay=d, tag=f"gpu/{tag}/{N}")


@pytest.mark.parametrize("N,Tr,l1,l2,d", CASES)
def test_pcc2(F, orc, N, Tr, l1, l2, d):
    a, b = _data(N, Tr, d, "pcc2")
    y64 = orc.pcc2(a, b, l1, l2)
    assert relerr(F.pcc2_set(a, b, l1, l2), y64) < TOL
    assert relerr(F.pcc2_set(a, b, l1, l2, plain=True), y64) < TOL
    assert relerr(F.pcc2_highlevel(a, b, l1, l2), y64) < TOL


@pytest.mark.parametrize("N,Tr,l1,l2,d", CASES)
def test_gncc(F, orc, N, Tr, l1, l2, d):
    a, b = _data(N, Tr, d, "gncc")
    assert relerr(F.ccgn_set(a, b, l1, l2), orc.gncc(a, b, l1, l2)) < TOL


def test_gncc_normalisation_tables(F, orc):
    # energy rows with room for the normalisation tables (ldE = 2 (N + 1)) give
    # the pair stage the same results, bit for bit, as rows of FP64 prefix sums
    # only (ldE = N + 1), over every lag of the window: rows of ordinary scale,
    # a row ending in zeros (empty overlaps: the FP64 branch), rows scaled by
    # 1e-17 and 1e15 (energies outside the tables' range: the FP64 branch)
    import torch
    N, lag = 1000, 999
    a, b = _data(N, 3, 41, "gncc-tables")
    x = np.concatenate([a, b]).astype(np.float32)
    x[1, 800:] = 0.0
    x[2] *= np.float32(1e-17)
    x[3] *= np.float32(1e15)
    rows = x.shape[0]
    iu, ju = np.triu_indices(rows)
    pairs = np.ascontiguousarray(np.stack([iu, ju], axis=1).astype(np.int32))
    P, L = pairs.shape[0], 2 * lag + 1
    Nz = F.choose_nz(N, -lag, lag, F.NZ_FAST)
    H = Nz // 2 + 1
    ctx = F.Context(0)
    d_x = torch.from_numpy(x).cuda()
    d_p = torch.from_numpy(pairs).cuda()
    d_s = torch.empty((rows, 2 * H), dtype=torch.float32, device="cuda")
    ctx.station_stage(F.GNCC, d_x.data_ptr(), N, rows, N, Nz, F.F32, 0, d_s.data_ptr(), H)
    ys, Es = [], []
    for ldE in (N + 1, 2 * (N + 1)):
        E = torch.empty((rows, ldE), dtype=torch.float64, device="cuda")
        d_y = torch.empty((P, L), dtype=torch.float32, device="cuda")
        ctx.energy_stage(d_x.data_ptr(), N, rows, N, E.data_ptr(), ldE)
        ctx.pair_stage(F.GNCC, d_s.data_ptr(), H, F.F32, d_p.data_ptr(), P, N, Nz, -lag, lag,
                       d_E=E.data_ptr(), ldE=ldE, d_y=d_y.data_ptr(), ldy=L)
        ctx.sync()
        ys.append(d_y.cpu().numpy())
        Es.append(E.cpu().numpy())
    ctx.close()
    assert np.array_equal(ys[0], ys[1], equal_nan=True)
    # the sums are the same; E[0] carries the sign flag of the tables
    assert np.array_equal(Es[0][:, 1:], Es[1][:, 1:N + 1])
    assert np.all(Es[0][:, 0] == 0) and not np.any(np.signbit(Es[0][:, 0]))
    assert np.all(np.signbit(Es[1][:, 0]))
    # against the oracle on the lags whose overlaps are not empty
    m = 700
    sel = slice(lag - m, lag + m + 1)
    y64 = orc.gncc(x[pairs[:, 0]], x[pairs[:, 1]], -m, m)
    assert relerr(ys[1][:, sel], y64) < TOL


@pytest.mark.parametrize("N,Tr,l1,l2,d", CASES)
def test_cc1b_fft(F, orc, N, Tr, l1, l2, d):
    a, b = _data(N, Tr, d, "cc1b")
    assert relerr(F.cc1b_set(a, b, l1, l2), orc.cc1b(a, b, l1, l2)) < TOL


@pytest.mark.parametrize("N,Tr,l1,l2,d", CASES)
def test_cc1b_popcount_bit_exact(F, orc, N, Tr, l1, l2, d):
    a, b = _data(N, Tr, d, "cc1b")
    a[:, ::97] = 0.0   # exact zeros exercise the asymmetric sign rule
    b[:, ::89] = 0.0
    num = F.cc1b_numerators(a, b, l1, l2)
    ref = orc.cc1b_num(a, b, l1, l2)
    assert np.array_equal(num, ref)
    y = F.cc1b_set(a, b, l1, l2, popcount=True)
    assert np.max(np.abs(y - orc.cc1b(a, b, l1, l2))) < 1e-6


@pytest.mark.parametrize("N,l1,l2", [
    (70001, -1500, 1500),   # 2188 words: the exact kernel's shared-memory tiles (1024 words) and their seams
    (40, -39, 39),          # every lag the window allows, windows shorter than two words
    (33, -1, 31),           # one partial word at each end of every overlap
])
def test_cc1b_popcount_long_and_edge_windows(F, orc, N, l1, l2):
    a, b = _data(N, 2, 7, "cc1b-edge")
    a[:, ::53] = 0.0
    num = F.cc1b_numerators(a, b, l1, l2)
    assert np.array_equal(num, orc.cc1b_num(a, b, l1, l2))


@pytest.mark.parametrize("N,Tr,l1,l2,d", [c for c in CASES if c[2] <= c[3]])
def test_pcc1(F, orc, N, Tr, l1, l2, d):
    a, b = _data(N, Tr, d, "pcc1")
    assert relerr(F.pcc1_set(a, b, l1, l2), orc.pcc1(a, b, l1, l2)) < TOL


@pytest.mark.parametrize("N,l1,l2,gaps", [(3000, -300, 300, False), (4500, -450, 200, True),
                                         (70001, -600, 600, False), (1200, -1199, 1199, True)])
def test_pcc1_pure_phase_rule(F, orc, N, l1, l2, gaps):
    """PCC1 of pure-phase signals (x/|x|, the reference GPU rule): tiles whose
    samples are all unit-modulus or zero take the one-root form of each term,
    the others (zero-padded edges included) the two-root form; both against
    the FP64 oracle with the same rule, with gaps, several tiles and lag
    windows covering the whole window."""
    import torch
    a, b = _data(N, 2, N // 40, "pcc1-pure")
    if gaps:
        a = np.stack([synth.gaps(a[k], seed_tag=f"pa{k}") for k in range(2)])
        b = np.stack([synth.gaps(b[k], seed_tag=f"pb{k}") for k in range(2)])
    y64 = orc.pcc1(a, b, l1, l2, rule=orc.AMP_PURE)
    ctx = F.Context(0)
    x = torch.from_numpy(np.ascontiguousarray(np.concatenate([a, b]))).cuda()
    ph = torch.empty((4, 2 * N), dtype=torch.float32, device="cuda")
    pairs = torch.tensor([[0, 2], [1, 3]], dtype=torch.int32, device="cuda")
    L = l2 - l1 + 1
    y = torch.empty((2, L), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ctx.station_stage(F.PCC1, x.data_ptr(), N, 4, N, 0, F.F32, F.AMP_PURE, ph.data_ptr(), N)
    ctx.pair_stage(F.PCC1, ph.data_ptr(), N, F.F32, pairs.data_ptr(), 2, N, 0, l1, l2, d_y=y.data_ptr(), ldy=L)
    ctx.sync()
    ctx.close()
    assert relerr(y.cpu().numpy(), y64) < TOL


def test_pccv_gpu_normalisation(F, orc):
    a, b = _data(2000, 2, 40, "pccv")
    y64 = orc.pccv(a, b, 1.5, -150, 150, norm_gpu=True)
    assert relerr(F.pcc_set(a, b, 1.5, -150, 150), y64) < TOL


def test_pcc2_fp16_storage(F, orc):
    """FP16 phase spectra: each stored value carries a relative rounding error up
    to 2^-11, about 1e-4 of the peak after the inverse transform (1.0-1.3e-4
    measured on the all-pairs windows), so FP16 does not meet the 1e-4 target and
    int16 is the 4-byte format for it.  This guards the FP16 path against
    regressions at its own measured level, 3e-4."""
    a, b = _data(4500, 3, -200, "f16")
    y64 = orc.pcc2(a, b, -450, 450)
    err = relerr(F.pcc2_set(a, b, -450, 450, fmt=F.F16), y64)
    assert err < 3e-4
    assert relerr(F.pcc2_set(a, b, -450, 450, fmt=F.I16), y64) < TOL


@pytest.mark.parametrize("N,l1,l2,nz", [(1000, -100, 100, 1), (4500, -450, 450, 1), (18000, -2000, 2000, 1),
                                         (36000, -3000, 3000, 1 << 17)])
def test_int16_storage_within_1e4(F, orc, N, l1, l2, nz):
    """Block-scaled int16 phase spectra (PCC2) and fixed-scale int16 phase
    signals (PCC1): 4 bytes per complex value, within 1e-4 of the FP64 oracle
    (in-block, run-time specialised and four-step station paths)."""
    a, b = _data(N, 2, -N // 30, "i16")
    y64 = orc.pcc2(a, b, l1, l2)
    assert relerr(F.pcc2_set(a, b, l1, l2, fmt=F.I16, nz_mode=nz), y64) < TOL
    assert relerr(F.pcc2_set(a, b, l1, l2, fmt=F.I16, nz_mode=nz, plain=True), y64) < TOL
    if N <= 4500:
        assert relerr(F.pcc1_set(a, b, l1, l2, fmt=F.I16), orc.pcc1(a, b, l1, l2)) < TOL


def test_pcc2_reference_padding_rule(F, orc):
    a, b = _data(3000, 2, 60, "nzref")
    y64 = orc.pcc2(a, b, -500, 500)
    assert relerr(F.pcc2_set(a, b, -500, 500, nz_mode=F.NZ_REFERENCE), y64) < TOL


def test_all_pairs_size_window(F, orc):
    """One window of the all-pairs workload size (N = 18000, lags +-2000)."""
    x, _ = synth.all_pairs(n_stations=3, n_windows=1, N=18000, tag="gpu/allpairs-size")
    a = x[[0, 0, 1], 0]
    b = x[[1, 2, 2], 0]
    for name, f, o in (("pcc2", F.pcc2_set, orc.pcc2), ("cc1b", F.cc1b_set, orc.cc1b)):
        assert relerr(f(a, b, -2000, 2000), o(a, b, -2000, 2000)) < TOL, name


def test_identity_and_shift(F):
    a, b = synth.plain_pair(N=3000, n_windows=1, delay=37, snr=3.0, tag="gpu/shift")
    y = F.pcc2_set(a, a, -50, 50)
    assert abs(y[0, 50] - 1.0) < 1e-4
    for f in (F.pcc2_set, F.ccgn_set, F.cc1b_set, F.pcc1_set):
        y = f(a, b, -200, 200)
        assert int(np.argmax(y[0])) - 200 == 37, f.__name__


def test_bad_lags_raise(F):
    a, b = _data(1000, 1, 0, "bad")
    with pytest.raises(F.FpccError):
        F.pcc2_set(a, b, -1000, 10)


# ---- lengths above the in-block menu (four-step transforms) --------------------
@pytest.mark.parametrize("nz", [0, 131072])
def test_plain_pair_config_sizes(F, orc, nz):
    """36,000-sample windows, lags +-3000: default padding and 2^17 (four-step)."""
    a, b = synth.plain_pair(N=36000, n_windows=2, delay=150, tag="gpu/plain36k")
    mode = nz if nz else F.NZ_FAST
    y64 = orc.pcc2(a, b, -3000, 3000)
    assert relerr(F.pcc2_set(a, b, -3000, 3000, nz_mode=mode), y64) < TOL
    assert relerr(F.ccgn_set(a, b, -3000, 3000, nz_mode=mode), orc.gncc(a, b, -3000, 3000)) < TOL
    assert relerr(F.cc1b_set(a, b, -3000, 3000, nz_mode=mode), orc.cc1b(a, b, -3000, 3000)) < TOL


def test_long_window_pcc2(F, orc):
    a, b = synth.plain_pair(N=65536, n_windows=1, delay=-300, fs=20.0, band=(0.02, 5.0), tag="gpu/long")
    assert relerr(F.pcc2_set(a, b, -4000, 4000), orc.pcc2(a, b, -4000, 4000)) < TOL


def test_explicit_padding_lengths(F, orc):
    a, b = _data(4500, 2, 80, "explicit-nz")
    y64 = orc.pcc2(a, b, -450, 450)
    for nz in (6144, 8192, 16384, 32768):   # in-block and four-step pair transforms
        assert relerr(F.pcc2_set(a, b, -450, 450, nz_mode=nz), y64) < TOL, nz


# ---- wavelet PCC -----------------------------------------------------------------
def test_wpcc_golden(F, orc):
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_wpcc_n3000.npz"))
    x1, x2 = g["x1"], g["x2"]
    l1, l2, pmin, pmax, V = int(g["Lag1"]), int(g["Lag2"]), float(g["pmin"]), float(g["pmax"]), int(g["V"])
    for key, wt in (("wpcc_mexhat", -3), ("wpcc_morlet", -1)):
        y64 = orc.wpcc(x1, x2, l1, l2, pmin, pmax, V=V, wtype=wt)
        assert relerr(g[key], y64) < 1e-6, key          # oracle pinned to the reference
        y = F.wpcc_set(x1, x2, l1, l2, pmin, pmax, V=V, type=wt)
        assert relerr(y, y64) < TOL, key
        y_ref_len = F.wpcc_set(x1, x2, l1, l2, pmin, pmax, V=V, type=wt, nz_mode=F.NZ_REFERENCE)
        assert relerr(y_ref_len, y64) < TOL, key


def test_wpcc_gpu_rule(F, orc):
    a, b = synth.plain_pair(N=4000, n_windows=2, delay=-60, fs=20.0, band=(0.02, 5.0), tag="gpu/wpcc-thr")
    y64 = orc.wpcc(a, b, -300, 300, 4.0, 80.0, V=3, wtype=-1, rule=orc.AMP_THRESH)
    assert relerr(F.wpcc_set(a, b, -300, 300, 4.0, 80.0, V=3, type=-1, rule=F.AMP_THRESH), y64) < TOL


def test_wpcc_wavelet_config_size(F, orc, monkeypatch):
    """65,536 samples at 20 Hz, Morlet, 40 scales (V=5, 4 to 1000 samples), lags +-4000,
    at the fast padded length (81920: rows on clusters of four blocks) and the
    reference's (2^17: clusters of eight), and both again as four-step passes."""
    x1, x2, _ = synth.wavelet_pairs(n_pairs=1, n_windows=1, tag="gpu/wpcc-c3")
    a, b = x1[0], x2[0]
    y64 = orc.wpcc(a, b, -4000, 4000, 4.0, 1000.0, V=5, wtype=-1)
    for cluster in ("1", "0"):
        monkeypatch.setenv("FPCC_WPCC_CLUSTER", cluster)
        for nz_mode in (F.NZ_FAST, F.NZ_REFERENCE):
            y = F.wpcc_set(a, b, -4000, 4000, 4.0, 1000.0, V=5, type=-1, nz_mode=nz_mode)
            assert relerr(y, y64) < TOL, (cluster, nz_mode)


# ---- window lengths with prime factors above 5 (Bluestein analytic signal) -----
@pytest.mark.parametrize("N,l1,l2", [(997, -100, 100), (1007, -50, 300), (4099, -400, 400), (37123, -3000, 2500)])
def test_non_smooth_window_lengths(F, orc, N, l1, l2):
    a, b = synth.plain_pair(N=N, n_windows=2, delay=min(150, N // 20), tag=f"gpu/blue/{N}")
    assert relerr(F.pcc2_set(a, b, l1, l2), orc.pcc2(a, b, l1, l2)) < TOL
    lo, hi = min(l1, l2), max(l1, l2)
    assert relerr(F.pcc1_set(a, b, lo, hi), orc.pcc1(a, b, lo, hi)) < TOL
    assert relerr(F.ccgn_set(a, b, l1, l2), orc.gncc(a, b, l1, l2)) < TOL


def test_wpcc_error_per_octave_band(F, orc):
    """Wavelet config shape (20 Hz, 0.02-5 Hz, Morlet, V=5): error of each octave's
    partial sum against the oracle's, relative to that band's own peak."""
    import torch
    x1, x2, _ = synth.wavelet_pairs(n_pairs=1, n_windows=1, N=16384, tag="gpu/wpcc-bands")
    a, b = x1[0], x2[0]
    l1, l2, pmin, pmax, V = -1000, 1000, 4.0, 256.0, 5
    ctx = F.Context(0)
    plan = F.WpccPlan(ctx, a.shape[1], l1, l2, pmin, pmax, V=V, type=-1)
    xs = torch.from_numpy(np.concatenate([a, b])).cuda()
    P = torch.empty((2, plan.S, plan.Nz, 2), dtype=torch.float32, device="cuda")
    plan.station_stage(xs.data_ptr(), a.shape[1], 2, P.data_ptr())
    pairs = torch.tensor([[0, 1]], dtype=torch.int32, device="cuda")
    y = torch.empty((1, plan.L), dtype=torch.float32, device="cuda")
    errs = []
    for lo in range(0, plan.S, V):
        plan.set_band(lo, lo + V)
        plan.pair_stage(P.data_ptr(), pairs.data_ptr(), 1, y.data_ptr(), plan.L)
        ctx.sync()
        y64 = orc.wpcc_band(a, b, l1, l2, pmin, pmax, lo, lo + V, V=V, wtype=-1)
        errs.append(relerr(y.cpu().numpy(), y64))
    plan.close()
    ctx.close()
    assert max(errs) < TOL, errs


@pytest.mark.parametrize("N,M", [(2500, 200), (4099, 300), (18000, 1500), (40000, 2000)])
def test_phase_methods_on_gapped_windows(F, orc, N, M):
    # 5 % of the samples zeroed in gaps of 50-2000 samples: the analytic signals
    # of such windows are computed in FP64 (FP32 transforms lose their phase
    # inside the gaps and drift by a few 1e-4)
    a, b = synth.plain_pair(N=N, n_windows=2, delay=-M // 3, tag=f"gpu/gaps/{N}")
    a = np.stack([synth.gaps(a[k], seed_tag=f"a{k}") for k in range(2)])
    b = np.stack([synth.gaps(b[k], seed_tag=f"b{k}") for k in range(2)])
    y64 = orc.pcc2(a, b, -M, M)
    assert relerr(F.pcc2_set(a, b, -M, M), y64) < TOL
    assert relerr(F.pcc2_set(a, b, -M, M, plain=True), y64) < TOL
    if N <= 18000:
        assert relerr(F.pcc1_set(a, b, -M // 4, M // 4), orc.pcc1(a, b, -M // 4, M // 4)) < TOL


def test_example_records_against_reference_cli(F, orc):
    """Three days of the reference's GEOSCOPE example records (N = 21600, lags
    +-3000): every method against the reference CLI's own outputs and the oracle."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_cli_geoscope.npz"))
    x1, x2, l1, l2 = g["x1"], g["x2"], int(g["Lag1"]), int(g["Lag2"])
    got = {"pcc2": F.pcc2_set(x1, x2, l1, l2), "pcc1": F.pcc1_set(x1, x2, l1, l2),
           "ccgn": F.ccgn_set(x1, x2, l1, l2), "cc1b": F.cc1b_set(x1, x2, l1, l2),
           "wpcc2": F.wpcc_set(x1, x2, l1, l2, float(g["pmin"]), float(g["pmax"]), V=2, type=-3)}
    ref64 = {"pcc2": orc.pcc2(x1, x2, l1, l2), "pcc1": orc.pcc1(x1, x2, l1, l2), "ccgn": orc.gncc(x1, x2, l1, l2),
             "cc1b": orc.cc1b(x1, x2, l1, l2),
             "wpcc2": orc.wpcc(x1, x2, l1, l2, float(g["pmin"]), float(g["pmax"]), V=2, wtype=-3)}
    for k, y in got.items():
        assert relerr(y, ref64[k]) < TOL, k
        assert relerr(y, g[k]) < TOL, k
    assert np.array_equal(F.cc1b_numerators(x1, x2, l1, l2), orc.cc1b_num(x1, x2, l1, l2))


def test_allpairs_host_first_use_pipeline(F, orc):
    # pinned host buffers: the rows go up in the order the pair list first uses
    # them (one strided copy per window here), the station stage runs on chunks
    # of them as they arrive, with each chunk's FP64 rows chosen from gap counts
    # read back on the upload stream, and pieces of pairs start as soon as their
    # rows are ready.  Every method's results equal the pageable-buffer path's bit
    # for bit (same station and pair kernels, same FP64 rows), on windows with
    # gaps as well, and agree with the oracle; a shuffled pair list (no row
    # structure) falls back to the chunked path with the same results
    import torch
    n_sta, n_win, N, lag = 32, 25, 2000, 100
    x, _ = synth.all_pairs(n_stations=n_sta, n_windows=n_win, N=N, max_delay=60, tag="gpu/allpairs-first-use")
    x = np.ascontiguousarray(x.reshape(n_sta * n_win, N))
    x[3 * n_win + 2, 500:900] = 0.0       # gaps: FP64 analytic signals for these rows
    x[17 * n_win + 11, 0:40] = 0.0
    iu, ju = np.triu_indices(n_sta, k=1)
    w = np.repeat(np.arange(n_win), iu.size)
    pairs = np.ascontiguousarray(np.stack([np.tile(iu, n_win) * n_win + w, np.tile(ju, n_win) * n_win + w],
                                          axis=1).astype(np.int32))
    P, L = pairs.shape[0], 2 * lag + 1
    xp = torch.from_numpy(x).pin_memory()
    yp = torch.zeros((P, L), dtype=torch.float32).pin_memory()
    sel = np.concatenate([np.flatnonzero((pairs[:, 0] == 3 * n_win + 2) | (pairs[:, 1] == 3 * n_win + 2))[:3],
                          np.random.default_rng(8).choice(P, 3, replace=False)])
    ctx = F.Context(0)
    refs = {F.PCC2: orc.pcc2, F.GNCC: orc.gncc, F.PCC1: orc.pcc1}
    for method, ref in refs.items():
        y = np.zeros((P, L), np.float32)
        ctx.allpairs_host(method, x, pairs, -lag, lag, y)          # pageable: chunked path
        yp.zero_()
        ctx.allpairs_host(method, xp.numpy(), pairs, -lag, lag, yp.numpy())   # pinned: first-use order
        assert np.array_equal(yp.numpy(), y), method
        assert relerr(y[sel], ref(x[pairs[sel, 0]], x[pairs[sel, 1]], -lag, lag)) < TOL, method
    perm = np.random.default_rng(12).permutation(P)
    yp.zero_()
    ctx.allpairs_host(F.PCC2, xp.numpy(), np.ascontiguousarray(pairs[perm]), -lag, lag, yp.numpy())
    y = np.zeros((P, L), np.float32)
    ctx.allpairs_host(F.PCC2, x, pairs, -lag, lag, y)
    assert np.array_equal(yp.numpy(), y[perm])
    # a row index outside the station rows is refused before any result is
    # written, early or late in the pair list; the context stays usable
    for at in ((7, 0), (P - 5, 1)):
        bad = pairs.copy()
        bad[at] = -1 if at[1] == 0 else n_sta * n_win
        yp.fill_(7.0)
        with pytest.raises(F.FpccError):
            ctx.allpairs_host(F.PCC2, xp.numpy(), bad, -lag, lag, yp.numpy())
        assert (yp.numpy() == 7.0).all()
    yp.zero_()
    ctx.allpairs_host(F.PCC2, xp.numpy(), pairs, -lag, lag, yp.numpy())
    assert np.array_equal(yp.numpy(), y)
    ctx.close()


def test_allpairs_host_chunked_transfers(F, orc):
    # all station pairs of every window with host buffers (fpcc_allpairs_host):
    # 32 stations x 25 windows -> 12,400 correlations, so the windows go up in
    # four row chunks and the results come down in two chunks on the second
    # stream; PCC2 equals the device-resident stages bit for bit, and PCC2, GNCC
    # and 1-bit (two sign rules) agree with the oracle
    import torch
    n_sta, n_win, N, lag = 32, 25, 2000, 100
    x, _ = synth.all_pairs(n_stations=n_sta, n_windows=n_win, N=N, max_delay=60, tag="gpu/allpairs-host")
    x = np.ascontiguousarray(x.reshape(n_sta * n_win, N))
    iu, ju = np.triu_indices(n_sta, k=1)
    w = np.repeat(np.arange(n_win), iu.size)
    pairs = np.ascontiguousarray(np.stack([np.tile(iu, n_win) * n_win + w, np.tile(ju, n_win) * n_win + w],
                                          axis=1).astype(np.int32))
    P, L = pairs.shape[0], 2 * lag + 1
    sel = np.random.default_rng(7).choice(P, 6, replace=False)
    ctx = F.Context(0)
    y = np.zeros((P, L), np.float32)
    ctx.allpairs_host(F.PCC2, x, pairs, -lag, lag, y)
    # device-resident stages, the same kernels
    Nz = F.choose_nz(N, -lag, lag, F.NZ_FAST)
    d_x = torch.from_numpy(x).cuda()
    d_p = torch.from_numpy(pairs).cuda()
    d_s = torch.empty((x.shape[0], 2 * Nz), dtype=torch.float32, device="cuda")
    d_y = torch.empty((P, L), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ctx.station_stage(F.PCC2, d_x.data_ptr(), N, x.shape[0], N, Nz, F.F32, F.AMP_F_REG, d_s.data_ptr(), Nz)
    ctx.pair_stage(F.PCC2, d_s.data_ptr(), Nz, F.F32, d_p.data_ptr(), P, N, Nz, -lag, lag, d_y=d_y.data_ptr(), ldy=L)
    ctx.sync()
    assert np.array_equal(y, d_y.cpu().numpy())
    assert relerr(y[sel], orc.pcc2(x[pairs[sel, 0]], x[pairs[sel, 1]], -lag, lag)) < TOL
    for method, ref in ((F.GNCC, orc.gncc), (F.CC1B, orc.cc1b)):
        y[:] = 0
        ctx.allpairs_host(method, x, pairs, -lag, lag, y)
        assert relerr(y[sel], ref(x[pairs[sel, 0]], x[pairs[sel, 1]], -lag, lag)) < TOL, method
    # a shuffled pair list gives the same rows in its own order (the chunked
    # downloads follow the caller's pair order)
    perm = np.random.default_rng(11).permutation(P)
    ys = np.zeros((P, L), np.float32)
    ctx.allpairs_host(F.PCC2, x, np.ascontiguousarray(pairs[perm]), -lag, lag, ys)
    assert np.array_equal(ys, d_y.cpu().numpy()[perm])
    # a row index outside the station rows is refused before any work
    bad = pairs.copy()
    bad[5, 1] = x.shape[0]
    with pytest.raises(F.FpccError):
        ctx.allpairs_host(F.PCC2, x, bad, -lag, lag, ys)
    ctx.close()

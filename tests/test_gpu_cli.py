"""The command-line program and its preprocessing against the reference CLI's
own outputs on its GEOSCOPE example records (three days of CAN and ECH, 24 h at
4 s, N = 21600, lags +-3000), from tests/golden/golden_cli_geoscope.npz:

* fpcc_clip_rows against the CLI's clipping() (bit-exact) on the records and on
  synthetic windows with gaps, odd and even lengths;
* fpcc_whiten_rows against the CLI's AveWhite();
* bin/fpcc_fullpair end to end — SAC inputs written from the recorded headers,
  SAC and binary outputs — against PCC_fullpair_1b's files for PCC2, PCC1, GNCC,
  1-bit, WPCC, and PCC2/GNCC after clipping and whitening.
"""
import os
import struct
import subprocess

import numpy as np
import pytest

from gpu_util import fp, need_gpu, relerr

pytestmark = pytest.mark.gpu
TOL = 1e-4
G = os.path.join(os.path.dirname(__file__), "golden", "golden_cli_geoscope.npz")


@pytest.fixture(scope="module")
def F():
    need_gpu()
    return fp()


@pytest.fixture(scope="module")
def g():
    return np.load(G)


def _device_rows(a):
    import torch
    d = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()
    torch.cuda.synchronize()   # the library works on its own stream
    return d


def _ok(F, rc):
    assert rc == 0, F.lib().fpcc_prep_last_error().decode()


def test_clip_rows_bit_exact(F, g):
    import torch
    ctx = F.Context(0)
    syn = g["clip_in_syn"]
    for name, xin in (("x1", g["x1"]), ("syn_odd", syn), ("syn_even", syn[:, :5000])):
        d = _device_rows(xin)
        _ok(F, F.lib().fpcc_clip_rows(ctx.handle, d.data_ptr(), d.shape[1], d.shape[0], d.shape[1]))
        ctx.sync()
        torch.cuda.synchronize()
        assert np.array_equal(d.cpu().numpy(), g[f"clip_out_{name}"]), name
    ctx.close()


def test_whiten_rows_matches_reference(F, g):
    import torch
    ctx = F.Context(0)
    d = _device_rows(g["x1"])
    f1, f2 = (float(v) for v in g["awhite"])
    _ok(F, F.lib().fpcc_whiten_rows(ctx.handle, d.data_ptr(), d.shape[1], d.shape[0], d.shape[1], f1, f2,
                                    float(g["dt"])))
    ctx.sync()
    torch.cuda.synchronize()
    assert relerr(d.cpu().numpy(), g["white_out_x1"]) < 1e-5
    ctx.close()


def _write_inputs(tmp, g):
    lists = []
    for st, key in (("CAN", "hdr1"), ("ECH", "hdr2")):
        names = []
        for k in range(g[key].shape[0]):
            p = os.path.join(tmp, f"{st}_{k}.SAC")
            with open(p, "wb") as f:
                f.write(g[key][k].tobytes())
                f.write(np.ascontiguousarray(g["x1" if st == "CAN" else "x2"][k], "<f4").tobytes())
            names.append(p)
        lp = os.path.join(tmp, f"{st}.txt")
        with open(lp, "w") as f:
            f.write("\n".join(names) + "\n")
        lists.append(lp)
    return lists


def _read_sac(p):
    raw = open(p, "rb").read()
    n = struct.unpack("<i", raw[280 + 36:280 + 40])[0]
    return np.frombuffer(raw[632:632 + 4 * n], "<f4"), raw[:632]


def _run(F, args, cwd):
    exe = os.path.join(os.path.dirname(F.LIB_PATH), "bin", "fpcc_fullpair")
    r = subprocess.run([exe, *args], cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def _outputs(cwd, tag):
    # per-window files: the window's start date follows the method tag (stack files end in _lin/_pws/_tspws)
    fs = sorted(f for f in os.listdir(cwd)
                if f.endswith(".sac") and f"_{tag}_" in f and f.split(f"_{tag}_")[1][:1].isdigit())
    return fs, np.stack([_read_sac(os.path.join(cwd, f))[0] for f in fs])


def test_cli_matches_reference_cli(F, g, tmp_path):
    l1, l2 = _write_inputs(str(tmp_path), g)
    runs = {"plain": ["pcc", "ccgn", "cc1b"], "pcc1": ["pcc", "v=1"], "wpcc": ["wpcc", "pmin=25", "pmax=330"],
            "prep": ["pcc", "ccgn", "clip", f"awhite={g['awhite'][0]},{g['awhite'][1]}"]}
    for name, extra in runs.items():
        d = tmp_path / name
        d.mkdir()
        out = _run(F, [l1, l2, "tl1=-12000", "tl2=12000", *extra], str(d))
        assert "L = 6001 smpl" in out and "Tr = 3" in out, out
    for run, tag, key in (("plain", "pcc2", "pcc2"), ("plain", "ccgn", "ccgn"), ("plain", "cc1b", "cc1b"),
                          ("pcc1", "pcc1", "pcc1"), ("wpcc", "wpcc2", "wpcc2"), ("prep", "pcc2", "pcc2_prep"),
                          ("prep", "ccgn", "ccgn_prep")):
        names, y = _outputs(str(tmp_path / run), tag)
        assert len(names) == 3 and names[0] == f"G.CAN.00.LHZ.G.ECH.00.LHZ_{tag}_2017.002.00.00.00.sac", names
        assert relerr(y, g[key]) < TOL, (run, tag)
    # header fields of the output SAC files (delta, b, npts, kinst, station fields, zero-lag time)
    _, h = _read_sac(str(tmp_path / "plain" / "G.CAN.00.LHZ.G.ECH.00.LHZ_pcc2_2017.002.00.00.00.sac"))
    ref = g["out_header"].tobytes()
    f_ours, f_ref = np.frombuffer(h[:280], "<f4"), np.frombuffer(ref[:280], "<f4")
    for k in (0, 5, 7, 31, 32, 35, 36):          # delta, b, o, stla, stlo, evla, evlo
        assert f_ours[k] == f_ref[k], k
    i_ours, i_ref = np.frombuffer(h[280:440], "<i4"), np.frombuffer(ref[280:440], "<i4")
    for k in (0, 1, 2, 3, 4, 5, 9, 17):          # nz date fields, npts, iztype
        assert i_ours[k] == i_ref[k], k
    assert h[440:632] == ref[440:632]            # all character fields


def test_cli_binary_output(F, g, tmp_path):
    l1, l2 = _write_inputs(str(tmp_path), g)
    d = tmp_path / "bin"
    d.mkdir()
    _run(F, [l1, l2, "tl1=-12000", "tl2=12000", "pcc", "obin"], str(d))
    name = str(g["obin_name"])
    ours = open(d / name, "rb").read()
    ref = g["obin_bytes"].tobytes()
    assert len(ours) == len(ref)
    nseq, L = 3, 6001
    head = 116 + nseq * 8 + nseq * 4
    assert ours[:head] == ref[:head]             # header, start times, zero-lag offsets
    y, yr = np.frombuffer(ours[head:], "<f4").reshape(nseq, L), np.frombuffer(ref[head:], "<f4").reshape(nseq, L)
    assert relerr(y, yr) < TOL


def test_cli_stacks_over_windows(F, g, tmp_path):
    # stack=lin,pws,tspws: each channel pair's windows stacked on the device, one
    # SAC file per kind; checked against the oracle's stacks of the program's own
    # per-window outputs and of the reference CLI's (ts-PWS family: the WPCC
    # options, pmin/pmax in seconds, Mexican hat, 2 voices by default)
    from oracle import oracle as O
    l1, l2 = _write_inputs(str(tmp_path), g)
    d = tmp_path / "stack"
    d.mkdir()
    _run(F, [l1, l2, "tl1=-12000", "tl2=12000", "pcc", "stack=lin,pws,tspws", "nu=2", "pmin=25", "pmax=330"], str(d))
    _, per_window = _outputs(str(d), "pcc2")
    dt = float(g["dt"])
    for mode, kind in ((O.STACK_LINEAR, "lin"), (O.STACK_PWS, "pws"), (O.STACK_TSPWS, "tspws")):
        y, _ = _read_sac(str(d / f"G.CAN.00.LHZ.G.ECH.00.LHZ_pcc2_{kind}.sac"))
        ours = O.stack(per_window, mode, 2.0, 25.0 / dt, 330.0 / dt, 2, -3)
        assert relerr(y[None], ours[None]) < TOL, kind
        ref = O.stack(g["pcc2"], mode, 2.0, 25.0 / dt, 330.0 / dt, 2, -3)
        assert relerr(y[None], ref[None]) < 3 * TOL, kind

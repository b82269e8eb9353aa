"""Golden fixture from the reference's own CLI on its bundled example records.

Run in a container that holds the reference: it builds the reference CLI
(src/PCC_fullpair_1b.c with its reader, FFTapps.c and the wavelet files,
unmodified) against the oracle's FFTW-API and SAC-I/O shims (``make -C oracle
cli``), correlates a few days of the GEOSCOPE example records
(examples/G/CAN and examples/G/ECH, 24 h at 4 s: N = 21600) with PCC2, PCC1,
GNCC, 1-bit GNCC and WPCC at lags +-12000 s (+-3000 samples), once more with
clipping and whitening, and once with the binary output, and stores the input
windows and SAC headers with the CLI's outputs, plus the CLI's own clipping and
whitening functions applied to these and to synthetic windows, as
``golden_cli_geoscope.npz``.

    python tests/golden/make_cli_golden.py
"""
import glob
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as _O   # noqa: E402

EXAMPLES = os.path.join(os.path.dirname(os.path.normpath(_O.reference_sources())), "examples", "G")
DAYS = 3
WPCC = dict(pmin=25.0, pmax=330.0)   # seconds, as in the reference's example script
AWHITE = (0.005, 0.03)                # Hz, whitening band for the preprocessing run


def read_sac(path):
    """(samples, header floats, header ints) of a little-endian SAC v6 file."""
    with open(path, "rb") as f:
        raw = f.read()
    hf = np.frombuffer(raw[:280], "<f4")
    hi = np.frombuffer(raw[280:420], "<i4")
    npts = int(hi[9])
    return np.frombuffer(raw[632:632 + 4 * npts], "<f4").copy(), hf, hi


def main():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), *_O.make_vars(), "cli"], check=True)
    cli = os.path.join(ROOT, "oracle", "_ref", "PCC_fullpair_1b")
    can = sorted(glob.glob(f"{EXAMPLES}/CAN/*.LHZ.*.SACvelbp"))
    ech = sorted(glob.glob(f"{EXAMPLES}/ECH/*.LHZ.*.SACvelbp"))
    day = lambda p: os.path.basename(p)[:17]   # yyyy.ddd.hh.mm.ss
    common = sorted(set(map(day, can)) & set(map(day, ech)))[:DAYS]
    can = [p for p in can if day(p) in common]
    ech = [p for p in ech if day(p) in common]
    rec = {"days": np.array(common)}
    with tempfile.TemporaryDirectory() as tmp:
        for name, lst in (("can.txt", can), ("ech.txt", ech)):
            with open(os.path.join(tmp, name), "w") as f:
                f.write("\n".join(lst) + "\n")
        runs = [["pcc", "ccgn", "cc1b"], ["pcc", "v=1"],
                ["wpcc", f"pmin={WPCC['pmin']}", f"pmax={WPCC['pmax']}"]]
        for extra in runs:
            subprocess.run([cli, "can.txt", "ech.txt", "tl1=-12000", "tl2=12000"] + extra, cwd=tmp, check=True,
                           stdout=subprocess.DEVNULL)
        outs = sorted(glob.glob(os.path.join(tmp, "*.sac")))
        for tag in ("pcc2", "pcc1", "ccgn", "cc1b", "wpcc2"):
            files = [p for p in outs if f"_{tag}_" in os.path.basename(p)]
            assert len(files) == DAYS, (tag, files)
            rec[tag] = np.stack([read_sac(p)[0] for p in sorted(files)])
        # preprocessing (clipping + whitening) and the binary output, in fresh folders
        for sub, extra in (("prep", ["pcc", "ccgn", "clip", f"awhite={AWHITE[0]},{AWHITE[1]}"]),
                           ("bin", ["pcc", "obin"])):
            d = os.path.join(tmp, sub)
            os.makedirs(d)
            subprocess.run([cli, "../can.txt", "../ech.txt", "tl1=-12000", "tl2=12000"] + extra, cwd=d, check=True,
                           stdout=subprocess.DEVNULL)
            if sub == "prep":
                outs = sorted(glob.glob(os.path.join(d, "*.sac")))
                for tag in ("pcc2", "ccgn"):
                    rec[tag + "_prep"] = np.stack([read_sac(p)[0] for p in outs if f"_{tag}_" in p])
            else:
                (binf,) = glob.glob(os.path.join(d, "*.bin"))
                rec["obin_name"] = os.path.basename(binf)
                rec["obin_bytes"] = np.frombuffer(open(binf, "rb").read(), np.uint8)
        # output SAC headers of the first pair (field checks)
        rec["out_header"] = np.frombuffer(open(sorted(glob.glob(os.path.join(tmp, "*_pcc2_*.sac")))[0], "rb")
                                          .read()[:632], np.uint8)
    # the raw input SAC headers, so that tests can write the same files
    rec["hdr1"] = np.stack([np.frombuffer(open(p, "rb").read()[:632], np.uint8) for p in can])
    rec["hdr2"] = np.stack([np.frombuffer(open(p, "rb").read()[:632], np.uint8) for p in ech])
    rec["awhite"] = np.array(AWHITE)
    rec["x1"] = np.stack([read_sac(p)[0] for p in can])
    rec["x2"] = np.stack([read_sac(p)[0] for p in ech])
    _, hf, _ = read_sac(can[0])
    rec["dt"] = float(hf[0])
    rec["Lag1"], rec["Lag2"] = -3000, 3000
    rec["pmin"], rec["pmax"] = WPCC["pmin"] / rec["dt"], WPCC["pmax"] / rec["dt"]
    # the CLI's own clipping and whitening functions on these windows and on
    # synthetic windows with gaps (odd and even lengths)
    import ctypes as C
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_cli.so"))
    fpp = C.POINTER(C.POINTER(C.c_float))

    def rows(a):
        r = (C.POINTER(C.c_float) * a.shape[0])()
        for k in range(a.shape[0]):
            r[k] = a[k].ctypes.data_as(C.POINTER(C.c_float))
        return r
    sys.path.insert(0, ROOT)
    from fastpcc_gb300 import synth
    rng = np.random.default_rng(12)
    syn = np.stack([synth.gaps((rng.standard_normal(5001) * (1 + 9 * (rng.random(5001) < 0.01))).astype(np.float32),
                               seed_tag=f"clip/{k}") for k in range(2)])
    rec["clip_in_syn"] = syn   # odd length; the even case uses its first 5000 samples
    for name, xin in (("x1", rec["x1"]), ("syn_odd", syn), ("syn_even", np.ascontiguousarray(syn[:, :5000]))):
        xc = np.ascontiguousarray(xin.copy())
        for k in range(xc.shape[0]):
            lib.clipping(xc[k].ctypes.data_as(C.POINTER(C.c_float)), C.c_uint(xc.shape[1]))
        rec[f"clip_out_{name}"] = xc
    xw = np.ascontiguousarray(rec["x1"].copy())
    freq = (C.c_double * 2)(*AWHITE)
    lib.AveWhite.argtypes = [fpp, C.c_uint, C.c_uint, C.POINTER(C.c_double), C.c_double]
    lib.AveWhite(rows(xw), xw.shape[1], xw.shape[0], freq, float(rec["dt"]))   # its status is not set on success
    rec["white_out_x1"] = xw
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_cli_geoscope.npz")
    np.savez_compressed(out, **rec)
    print("wrote", out, {k: getattr(v, "shape", v) for k, v in rec.items()})


if __name__ == "__main__":
    main()

"""Golden fixture from the reference's own CLI on its bundled example records.

Run in a container that holds the reference: it builds the reference CLI
(src/PCC_fullpair_1b.c with its reader, FFTapps.c and the wavelet files,
unmodified) against the oracle's FFTW-API and SAC-I/O shims (``make -C oracle
cli``), correlates a few days of the GEOSCOPE example records
(examples/G/CAN and examples/G/ECH, 24 h at 4 s: N = 21600) with PCC2, PCC1,
GNCC, 1-bit GNCC and WPCC at lags +-12000 s (+-3000 samples), and stores the
input windows (read from the SAC files) with the CLI's SAC outputs as
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
EXAMPLES = "/root/reference/examples/G"
DAYS = 3
WPCC = dict(pmin=25.0, pmax=330.0)   # seconds, as in the reference's example script


def read_sac(path):
    """(samples, header floats, header ints) of a little-endian SAC v6 file."""
    with open(path, "rb") as f:
        raw = f.read()
    hf = np.frombuffer(raw[:280], "<f4")
    hi = np.frombuffer(raw[280:420], "<i4")
    npts = int(hi[9])
    return np.frombuffer(raw[632:632 + 4 * npts], "<f4").copy(), hf, hi


def main():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "cli"], check=True)
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
    rec["x1"] = np.stack([read_sac(p)[0] for p in can])
    rec["x2"] = np.stack([read_sac(p)[0] for p in ech])
    _, hf, _ = read_sac(can[0])
    rec["dt"] = float(hf[0])
    rec["Lag1"], rec["Lag2"] = -3000, 3000
    rec["pmin"], rec["pmax"] = WPCC["pmin"] / rec["dt"], WPCC["pmax"] / rec["dt"]
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_cli_geoscope.npz")
    np.savez_compressed(out, **rec)
    print("wrote", out, {k: getattr(v, "shape", v) for k, v in rec.items()})


if __name__ == "__main__":
    main()

"""Generate the golden fixtures in this folder from the reference's own CPU path.

Run in a container that holds the reference sources: it compiles src/FFTapps.c
and the src/FWTa wavelet files unmodified against the oracle's FFTW-API shim
(``make -C oracle ref``), runs each method on small seeded synthetic windows and
stores inputs and outputs as ``golden_<case>.npz``.  The fixtures pin the FP64
oracle (tests/test_oracle.py) on machines where the reference is absent.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from fastpcc_gb300 import synth  # noqa: E402

CASES = [
    # name, N, Tr, Lag1, Lag2, delay
    ("n1000_sym", 1000, 2, -100, 100, 37),
    ("n997_prime", 997, 2, -50, 80, -21),
    ("n2048_pos", 2048, 2, 10, 300, 120),
    ("n1200_neg", 1200, 2, -400, -20, -150),
    ("n3000_swapped", 3000, 1, 250, -250, 60),
]


def main():
    O.build(ref=True)
    out = os.path.dirname(os.path.abspath(__file__))
    for name, N, Tr, l1, l2, d in CASES:
        a, b = synth.plain_pair(N=N, n_windows=Tr, delay=d, tag=f"golden/{name}")
        rec = dict(x1=a, x2=b, N=N, Lag1=l1, Lag2=l2)
        rec["pcc2"] = O.ref_call("pcc2", a, b, l1, l2)
        rec["cc1b"] = O.ref_call("cc1b", a, b, l1, l2)
        if max(l1, l2) >= 0:   # src/FFTapps.c:925 + :351 overflow yd when Lag2 < 0
            rec["ccgn"] = O.ref_call("ccgn", a, b, l1, l2)
        lo, hi = min(l1, l2), max(l1, l2)
        rec["pcc1"] = O.ref_call("pcc1", a, b, lo, hi)
        rec["pcc_v1.5"] = O.ref_call("pcc", a, b, lo, hi, v=1.5)
        np.savez_compressed(os.path.join(out, f"golden_{name}.npz"), **rec)
    # wavelet PCC, both complex wavelet types of the reference CLI
    N = 3000
    a, b = synth.plain_pair(N=N, n_windows=2, delay=37, fs=20.0, band=(0.02, 5.0), tag="golden/wpcc")
    rec = dict(x1=a, x2=b, N=N, Lag1=-200, Lag2=200, pmin=4.0, pmax=60.0, V=2)
    rec["wpcc_mexhat"] = O.ref_call("wpcc", a, b, -200, 200, pmin=4.0, pmax=60.0, V=2, wtype=-3)
    rec["wpcc_morlet"] = O.ref_call("wpcc", a, b, -200, 200, pmin=4.0, pmax=60.0, V=2, wtype=-1)
    np.savez_compressed(os.path.join(out, "golden_wpcc_n3000.npz"), **rec)
    print("fixtures written to", out)


if __name__ == "__main__":
    main()

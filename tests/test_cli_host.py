"""Host side of bin/fpcc_fullpair (no GPU needed): argv grammar, SAC reading,
removal of all-zero traces, pairing by start time, lags and the interstation
distance, checked through the summary line the program prints before it
creates its GPU context — the same line the reference CLI prints
(src/PCC_fullpair_1b.c:432-433) for the same records."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
G = os.path.join(ROOT, "tests", "golden", "golden_cli_geoscope.npz")
# printed by the reference CLI for the three example days at lags +-12000 s
REF_LINE = ("Lag1 = -3000 smpl (-12000 s), Lag2 = 3000 smpl (12000 s), L = 6001 smpl (24000 s), "
            "N = 21600 smpl, Tr = {tr}, gcarc = 149.155696 deg")


@pytest.fixture(scope="module")
def exe():
    from fastpcc_gb300 import native_build
    native_build.build()
    return native_build.CLI_OUT


def _inputs(tmp, zero=(), drop1=()):
    g = np.load(G)
    lists = []
    for st, key, xk in (("CAN", "hdr1", "x1"), ("ECH", "hdr2", "x2")):
        names = []
        for k in range(3):
            if st == "CAN" and k in drop1:
                continue
            p = os.path.join(tmp, f"{st}_{k}.SAC")
            x = np.zeros(21600, "<f4") if (st, k) in zero else np.ascontiguousarray(g[xk][k], "<f4")
            with open(p, "wb") as f:
                f.write(g[key][k].tobytes() + x.tobytes())
            names.append(p)
        lp = os.path.join(tmp, f"{st}.txt")
        with open(lp, "w") as f:
            f.write("\n".join(reversed(names)) + "\n")    # out of time order: the program sorts
        lists.append(lp)
    return lists


def _summary(exe, args):
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=120)
    lines = [l for l in r.stdout.splitlines() if l.startswith("Lag1 =")]
    return lines[0] if lines else r.stdout


def test_summary_line_matches_reference(exe, tmp_path):
    l1, l2 = _inputs(str(tmp_path))
    assert _summary(exe, [l1, l2, "pcc", "tl1=-12000", "tl2=12000"]) == REF_LINE.format(tr=3)
    # sample lags override time lags; swapped lags are ordered
    assert _summary(exe, [l1, l2, "pcc", "nl1=3000", "nl2=-3000"]) == REF_LINE.format(tr=3)


def test_pairing_drops_unmatched_and_zero_traces(exe, tmp_path):
    l1, l2 = _inputs(str(tmp_path), zero={("ECH", 1)}, drop1={2})
    # day 3 exists only at ECH, day 2 is all zeros at ECH: one pair is left
    assert _summary(exe, [l1, l2, "pcc", "tl1=-12000", "tl2=12000"]) == REF_LINE.format(tr=1)

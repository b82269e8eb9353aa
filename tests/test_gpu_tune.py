"""The autotuner: a measured table of padded lengths and pair-kernel forms on
this GPU, lengths chosen from it, the chosen kernel form in use, results
unchanged (any length >= N + max|lag| gives the same lags)."""
import json
import os

import numpy as np
import pytest

from fastpcc_gb300 import synth
from gpu_util import fp, need_gpu, relerr

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def F():
    need_gpu()
    return fp()


def test_autotune_table_drives_tuned_lengths(F, orc, tmp_path):
    path = str(tmp_path / "tune.json")
    ctx = F.Context(0)
    table = ctx.autotune(min_nz=512, max_nz=1 << 17, reuse=8.0, path=path)
    ctx.close()
    assert len(table) > 20 and os.path.exists(path)
    assert all(v[0] > 0 and v[1] > 0 for v in table.values())
    # lengths that two pair kernels run carry the faster form, and that form is in use
    for nz in (16384, 20480):
        assert table[nz][2] in (F.PAIR_BLOCK, F.PAIR_TILED)
        assert F.pair_form(nz) == table[nz][2]
    assert table[4096][2] == 0
    for N, M in [(1000, 100), (3001, 250), (18000, 2000), (36000, 3000)]:
        nz = F.choose_nz(N, -M, M, F.NZ_TUNED)
        assert nz >= N + M and nz in table
        cost = lambda z: table[z][0] + table[z][1] / 8.0
        assert all(cost(nz) <= cost(z) for z in table if N + M <= z <= 2 * (N + M) + 64)
    a, b = synth.plain_pair(N=3001, n_windows=2, delay=40, tag="gpu/tune")
    y64 = orc.pcc2(a, b, -250, 250)
    assert relerr(F.pcc2_set(a, b, -250, 250, nz_mode=F.NZ_TUNED), y64) < 1e-4
    assert relerr(F.ccgn_set(a, b, -250, 250, nz_mode=F.NZ_TUNED), orc.gncc(a, b, -250, 250)) < 1e-4
    assert F.load_tuning(path) == table
    # a loaded table sets the forms it names
    d = json.load(open(path))
    other = F.PAIR_BLOCK if table[20480][2] == F.PAIR_TILED else F.PAIR_TILED
    d["lengths"]["20480"][2] = other
    with open(path, "w") as f:
        f.write('{"reuse": %g, "lengths": {\n' % d["reuse"])
        f.write(",\n".join('  "%s": [%g, %g, %d]' % (k, *v) for k, v in d["lengths"].items()))
        f.write("\n}}\n")
    F.load_tuning(path)
    assert F.pair_form(20480) == other
    F.pair_form(20480, table[20480][2])

"""The padded-length autotuner: a measured table on this GPU, lengths chosen
from it, results unchanged (any length >= N + max|lag| gives the same lags)."""
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
    assert all(p > 0 and s > 0 for p, s in table.values())
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

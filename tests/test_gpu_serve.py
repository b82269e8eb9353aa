"""The continuous-batching server: mixed methods and lengths against the oracle,
each result identical alone and in the mix, eviction under a small HBM budget,
and concurrent submitters."""
import threading

import numpy as np
import pytest

from fastpcc_gb300 import synth
from gpu_util import fp, need_gpu, relerr

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture(scope="module")
def F():
    need_gpu()
    return fp()


def _stations(n_sta, n_win, N, tag):
    x, _ = synth.all_pairs(n_stations=n_sta, n_windows=n_win, N=N, max_delay=min(750, N // 10), tag=tag)
    return x


def _mix():
    """(method, sta1, sta2, window, Lag1, Lag2, v, N-class) requests over two window lengths."""
    rng = np.random.default_rng(0)
    reqs = []
    methods = [0, 1, 2, 3, 4, 5]
    for k in range(60):
        m = methods[k % len(methods)]
        big = (k % 3 == 0)
        n_sta = 4 if big else 6
        s1, s2 = rng.choice(n_sta, 2, replace=False)
        w = int(rng.integers(0, 2))
        M = int(rng.integers(20, 300))
        l1, l2 = -M, int(rng.integers(0, M + 1))
        v = 1.5 if m == 5 else 0.0
        reqs.append((m, int(s1) + (100 if big else 0), int(s2) + (100 if big else 0), w, l1, l2, v))
    return reqs


def _register(srv, xa, xb):
    for s in range(xa.shape[0]):
        for w in range(xa.shape[1]):
            srv.put(s, w, xa[s, w])
    for s in range(xb.shape[0]):
        for w in range(xb.shape[1]):
            srv.put(100 + s, w, xb[s, w])


def _oracle(orc, m, a, b, l1, l2, v):
    a, b = a[None], b[None]
    if m == 0:
        return orc.pcc2(a, b, l1, l2)[0]
    if m == 1:
        return orc.gncc(a, b, l1, l2)[0]
    if m in (2, 3):
        return orc.cc1b(a, b, l1, l2)[0]
    if m == 4:
        return orc.pcc1(a, b, l1, l2)[0]
    return orc.pccv(a, b, v, l1, l2, norm_gpu=True)[0]


def _run(F, srv, reqs):
    outs = []
    for (m, s1, s2, w, l1, l2, v) in reqs:
        L = abs(l2 - l1) + 1
        out = np.zeros(L, np.int64 if m == F.CC1B_POPCOUNT else np.float32)
        outs.append(out)
        srv.submit(m, s1, s2, w, l1, l2, out, v=v)
    srv.drain()
    return outs


def test_server_mixed_methods_against_oracle_and_alone(F, orc):
    xa = _stations(6, 2, 3000, "serve/a")
    xb = _stations(4, 2, 4800, "serve/b")
    xa[:, :, 500:700] = 0.0   # gaps exercise the zero-sample rules
    reqs = _mix()
    srv = F.Server(hbm_budget=2 << 30, max_batch=64)
    _register(srv, xa, xb)
    outs = _run(F, srv, reqs)
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["p99_ms"] >= st["p50_ms"] > 0
    srv.close()
    for (m, s1, s2, w, l1, l2, v), out in zip(reqs, outs):
        X = xb if s1 >= 100 else xa
        a, b = X[s1 % 100, w], X[s2 % 100, w]
        if m == F.CC1B_POPCOUNT:
            assert np.array_equal(out, orc.cc1b_num(a[None], b[None], l1, l2)[0])
        else:
            assert relerr(out, _oracle(orc, m, a, b, l1, l2, v)) < TOL, (m, l1, l2)
    # every result is the same when computed alone on a fresh server
    for i in range(0, len(reqs), 7):
        alone = F.Server(hbm_budget=1 << 30)
        _register(alone, xa, xb)
        (o,) = _run(F, alone, [reqs[i]])
        alone.close()
        assert np.array_equal(o, outs[i]), reqs[i]


def test_server_eviction_under_small_budget(F, orc):
    x = _stations(8, 1, 3000, "serve/evict")
    srv = F.Server(hbm_budget=200 << 10, max_batch=1)    # room for a few station products only
    for s in range(8):
        srv.put(s, 0, x[s, 0])
    reqs = [(0, i, j, 0, -200, 200, 0.0) for i in range(8) for j in range(8) if i < j]
    outs = _run(F, srv, reqs)
    assert srv.stats()["station_rows"] > 8        # products were evicted and rebuilt
    srv.close()
    for (m, s1, s2, w, l1, l2, v), out in zip(reqs, outs):
        assert relerr(out, orc.pcc2(x[s1, 0][None], x[s2, 0][None], l1, l2)[0]) < TOL


def test_server_concurrent_submitters(F, orc):
    x = _stations(5, 2, 2400, "serve/conc")
    srv = F.Server(hbm_budget=1 << 30, max_batch=16)
    for s in range(5):
        for w in range(2):
            srv.put(s, w, x[s, w])
    jobs = [(0, i, j, w, -150, 150, 0.0) for w in range(2) for i in range(5) for j in range(5) if i != j]
    outs = [np.zeros(301, np.float32) for _ in jobs]

    def worker(k):
        for idx in range(k, len(jobs), 3):
            m, s1, s2, w, l1, l2, v = jobs[idx]
            srv.submit(m, s1, s2, w, l1, l2, outs[idx])

    ths = [threading.Thread(target=worker, args=(k,)) for k in range(3)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    srv.drain()
    srv.close()
    for (m, s1, s2, w, l1, l2, v), out in zip(jobs, outs):
        assert relerr(out, orc.pcc2(x[s1, w][None], x[s2, w][None], l1, l2)[0]) < TOL

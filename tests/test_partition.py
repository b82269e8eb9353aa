"""Sharding of the correlation work across ranks (CPU, gloo, world size 2).

The union of the shards must equal the whole job exactly once, and results
computed rank by rank (with the FP64 oracle standing in for each rank's GPU)
and gathered to rank 0 must equal the single-rank result.
"""
import os
import socket

import numpy as np
import pytest

from fastpcc_gb300 import partition


@pytest.mark.parametrize("n_sta,n_win,world", [(6, 4, 2), (7, 5, 3), (9, 1, 4), (5, 2, 8), (16, 1, 2)])
def test_shards_cover_the_job_once(n_sta, n_win, world):
    shards = partition.shard_all_pairs(n_sta, n_win, world)
    allrows = np.concatenate([s.pairs for s in shards if s.n])
    assert allrows.shape[0] == n_sta * (n_sta - 1) // 2 * n_win
    assert len(set(map(tuple, allrows.tolist()))) == allrows.shape[0]
    assert np.all(allrows[:, 0] < allrows[:, 1])


def test_window_split_duplicates_no_station_product():
    shards = partition.shard_all_pairs(8, 6, 3)
    needs = [partition.stations_needed(s) for s in shards]
    for a in range(3):
        for b in range(a + 1, 3):
            assert not (needs[a] & needs[b])
    loads = [s.n for s in shards]
    assert max(loads) - min(loads) <= 28


@pytest.mark.parametrize("n_sta,n_win,world", [(6, 4, 2), (7, 5, 3), (9, 1, 4), (64, 8, 1)])
def test_shard_rows_window_major(n_sta, n_win, world):
    # each rank's station-major rows address exactly its shard's (i, j, w) triples,
    # window-major; one rank over the whole job gives the plain all-pairs order
    for sh in partition.shard_all_pairs(n_sta, n_win, world):
        rows = partition.shard_rows(sh, n_sta)
        W = len(sh.windows)
        assert rows.shape == (sh.n, 2)
        k = rows[:, 0] % W
        assert np.array_equal(k, rows[:, 1] % W)
        got = set(zip((rows[:, 0] // W).tolist(), (rows[:, 1] // W).tolist(),
                      np.asarray(sh.windows)[k].tolist()))
        assert got == set(map(tuple, sh.pairs.tolist()))
        assert np.all(np.diff(k) >= 0)
    if world == 1:
        iu, ju = np.triu_indices(n_sta, k=1)
        w = np.repeat(np.arange(n_win), iu.size)
        ref = np.stack([np.tile(iu, n_win) * n_win + w, np.tile(ju, n_win) * n_win + w], axis=1)
        assert np.array_equal(partition.shard_rows(partition.shard_all_pairs(n_sta, n_win, 1)[0], n_sta), ref)


def test_route_is_stable_and_symmetric():
    for a in range(20):
        for b in range(20):
            assert partition.route(a, b, 4) == partition.route(b, a, 4)
            assert 0 <= partition.route(a, b, 4) < 4
    counts = np.bincount([partition.route(a, b, 4) for a in range(40) for b in range(a + 1, 40)], minlength=4)
    assert counts.min() > 0.5 * counts.mean()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, n_sta, n_win, N, lag, q):
    import torch
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from fastpcc_gb300 import synth
    from oracle import oracle as O
    x, _ = synth.all_pairs(n_stations=n_sta, n_windows=n_win, N=N, max_delay=100, tag="partition")
    sh = partition.shard_all_pairs(n_sta, n_win, world)[rank]
    p = sh.pairs
    y = O.pcc2(x[p[:, 0], p[:, 2]], x[p[:, 1], p[:, 2]], -lag, lag) if sh.n else np.zeros((0, 2 * lag + 1))
    # gather rows and their keys to rank 0 (host-side result gathering, no data-path collective)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([sh.n], dtype=torch.int64))
    mx = int(max(s.item() for s in sizes))
    buf = torch.zeros((mx, 3 + y.shape[1]), dtype=torch.float64)
    if sh.n:
        buf[: sh.n, :3] = torch.from_numpy(p.astype(np.float64))
        buf[: sh.n, 3:] = torch.from_numpy(y)
    out = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(out, buf)
    if rank == 0:
        rows = np.concatenate([o[: int(s.item())].numpy() for o, s in zip(out, sizes)])
        q.put(rows)
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks_equal_single_rank():
    import torch.multiprocessing as mp

    n_sta, n_win, N, lag, world = 5, 3, 1200, 100, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, n_sta, n_win, N, lag, q)) for r in range(world)]
    for p in procs:
        p.start()
    rows = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    from fastpcc_gb300 import synth
    from oracle import oracle as O
    x, _ = synth.all_pairs(n_stations=n_sta, n_windows=n_win, N=N, max_delay=100, tag="partition")
    keys = rows[:, :3].astype(int)
    order = np.lexsort((keys[:, 2], keys[:, 1], keys[:, 0]))
    keys, ys = keys[order], rows[order, 3:]
    full = partition.shard_all_pairs(n_sta, n_win, 1)[0].pairs
    full = full[np.lexsort((full[:, 2], full[:, 1], full[:, 0]))]
    assert np.array_equal(keys, full)
    y1 = O.pcc2(x[full[:, 0], full[:, 2]], x[full[:, 1], full[:, 2]], -lag, lag)
    assert np.array_equal(ys, y1)

"""Work partitioning across GPUs (one process per GPU).

Every (station pair, window) correlation is independent and every station
product belongs to one (station, window), so the correlations shard with no
data-path collective:

* ``shard_all_pairs`` splits an all-pairs job.  Windows are dealt to ranks
  first — a rank then computes the products of its windows only and no product
  is computed twice.  With fewer windows than ranks, the upper triangle of the
  station x station matrix is cut into square blocks that are dealt out so that
  each rank recomputes only the products of its blocks' rows and columns.
* ``route`` sends a served request to a replica by a stable hash of its
  station pair, so one pair's windows always meet the same spectrum cache.

Results are gathered on the host per pair (each rank returns its own rows).
"""
from __future__ import annotations

import hashlib
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Shard:
    rank: int
    windows: list = field(default_factory=list)        # window ids this rank correlates
    pairs: np.ndarray = None                            # (P, 3) int32: station 1, station 2, window

    @property
    def n(self) -> int:
        return 0 if self.pairs is None else int(self.pairs.shape[0])


def _upper_pairs(n_sta):
    i, j = np.triu_indices(n_sta, k=1)
    return np.stack([i, j], axis=1)


def shard_all_pairs(n_sta: int, n_win: int, world: int, block: int = 0) -> list:
    """Shards of the job {(i, j, w): i < j < n_sta, w < n_win} for `world` ranks."""
    if world < 1:
        raise ValueError("world must be >= 1")
    shards = [Shard(rank=r) for r in range(world)]
    up = _upper_pairs(n_sta)
    if n_win >= world:
        # deal windows round-robin by descending share so counts differ by at most one
        for w in range(n_win):
            shards[w % world].windows.append(w)
        for sh in shards:
            ws = np.asarray(sh.windows, dtype=np.int64)
            if ws.size:
                p = np.repeat(up, ws.size, axis=0)
                wcol = np.tile(ws, up.shape[0])
                sh.pairs = np.ascontiguousarray(np.column_stack([p, wcol]).astype(np.int32))
            else:
                sh.pairs = np.zeros((0, 3), np.int32)
        return shards
    # fewer windows than ranks: block the upper triangle
    b = block or max(1, int(np.ceil(n_sta / np.ceil(np.sqrt(2 * world)))))
    nb = (n_sta + b - 1) // b
    blocks = [(bi, bj) for bi in range(nb) for bj in range(bi, nb)]
    # greedy: heaviest block to the least-loaded rank
    def weight(blk):
        bi, bj = blk
        ri = np.arange(bi * b, min(n_sta, (bi + 1) * b))
        rj = np.arange(bj * b, min(n_sta, (bj + 1) * b))
        return int(np.sum(ri[:, None] < rj[None, :]))
    blocks.sort(key=weight, reverse=True)
    load = [0] * world
    owned = [[] for _ in range(world)]
    for blk in blocks:
        r = int(np.argmin(load))
        owned[r].append(blk)
        load[r] += weight(blk) * n_win
    for r, sh in enumerate(shards):
        sh.windows = list(range(n_win))
        rows = []
        for (bi, bj) in owned[r]:
            for i in range(bi * b, min(n_sta, (bi + 1) * b)):
                for j in range(bj * b, min(n_sta, (bj + 1) * b)):
                    if i < j:
                        for w in range(n_win):
                            rows.append((i, j, w))
        sh.pairs = np.asarray(rows, np.int32).reshape(-1, 3)
    return shards


def shard_rows(shard: Shard, n_sta: int) -> np.ndarray:
    """The shard's pair list as (row of station 1, row of station 2), int32,
    for a rank that holds its windows station-major: row = station * W + k,
    where k is the window's position in ``shard.windows`` and W their number.
    Ordered window-major (then station 1, station 2), the order in which one
    window's station products are read by consecutive pairs."""
    W = len(shard.windows)
    if shard.n == 0 or W == 0:
        return np.zeros((0, 2), np.int32)
    local = np.full(max(shard.windows) + 1, -1, np.int64)
    local[np.asarray(shard.windows, np.int64)] = np.arange(W)
    p = shard.pairs.astype(np.int64)
    k = local[p[:, 2]]
    if np.any(k < 0) or np.any(p[:, :2] >= n_sta):
        raise ValueError("shard pairs outside its windows or stations")
    order = np.lexsort((p[:, 1], p[:, 0], k))
    rows = np.stack([p[order, 0] * W + k[order], p[order, 1] * W + k[order]], axis=1)
    return np.ascontiguousarray(rows.astype(np.int32))


def stations_needed(shard: Shard) -> set:
    """(station, window) products a shard computes."""
    if shard.n == 0:
        return set()
    p = shard.pairs
    return set(map(tuple, np.concatenate([p[:, [0, 2]], p[:, [1, 2]]]).tolist()))


def route(sta1: int, sta2: int, world: int) -> int:
    """Replica for a served request: stable in the (unordered) station pair."""
    a, b = (sta1, sta2) if sta1 <= sta2 else (sta2, sta1)
    h = hashlib.blake2b(f"{a}:{b}".encode(), digest_size=8).digest()
    return int.from_bytes(h, "little") % world

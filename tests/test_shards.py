"""Multi-GPU host logic on the CPU: row sharding of a domain across ranks and the
max-over-ranks timing reduction, with two `gloo` ranks.  Each rank steps its block
of columns (the oracle stands in for the device step; columns are independent, so
the union of the blocks must equal one whole-domain step bit for bit)."""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]

from tempo_gb300.shards import shard_bounds, shard_rows  # noqa: E402


@pytest.mark.parametrize("n,world", [(1, 1), (8, 2), (7, 2), (3, 4), (0, 3), (1024, 8), (5, 5)])
def test_shard_rows_partition(n, world):
    rows = []
    sizes = []
    for r in range(world):
        a, b = shard_rows(1, n, r, world)
        assert b >= a - 1
        rows.extend(range(a, b + 1))
        sizes.append(b - a + 1)
    assert rows == list(range(1, n + 1))
    assert max(sizes) - min(sizes) <= 1


def test_shard_bounds_only_narrows_tile_rows():
    b = list(range(1, 19))
    b[14], b[15] = 3, 10
    s = shard_bounds(b, 1, 2)
    assert s[:14] == b[:14] and s[16:] == b[16:]
    assert (s[14], s[15]) == (7, 10)
    with pytest.raises(ValueError):
        shard_rows(1, 4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    sys.path.insert(0, str(REPO))
    sys.path.insert(0, str(REPO / "tests"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist
    import oracle
    from parity_util import make_diags
    from tempo_gb300 import workloads as W
    from tempo_gb300.shards import max_over_ranks, shard_bounds, sum_over_ranks

    dist.init_process_group("gloo", rank=rank, world_size=world)
    oracle.build()
    oracle.init(False, REPO / "tables" / "ccn_activate.bin")
    oracle.build_big_tables(nthreads=2)
    wl = W.stretched_grid(seed=3, ni=12, nj=7, steps=1)
    f = {k: v.copy() for k, v in wl.fields.items()}
    nj, nk, ni = f["p"].shape
    full = [1, ni, 1, nj, 1, nk] * 3
    b = shard_bounds(full, rank, world)
    d = make_diags(f["p"].shape)
    rc = oracle.run(oracle.default_cfgs(hailaware_flag=0), wl.dt, 1, f, d, bounds=b, nthreads=1)
    assert rc == 0
    # gather every rank's block of t/qs/qr on rank 0 (a test-side exchange;
    # the step itself needs none)
    j0, j1 = b[14] - 1, b[15]
    mine = np.concatenate([f["t"][j0:j1].ravel(), f["qs"][j0:j1].ravel(),
                           f["qr"][j0:j1].ravel()])
    parts = [None] * world
    dist.all_gather_object(parts, (j0, j1, mine))
    tmax = max_over_ranks(float(rank + 1))
    tsum = sum_over_ranks(float(rank + 1))
    if rank == 0:
        np.save(Path(outdir) / "gathered.npy", np.array(parts, dtype=object), allow_pickle=True)
        np.save(Path(outdir) / "reduced.npy", np.array([tmax, tsum]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_match_whole_domain(tmp_path, oracle_mod):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from parity_util import make_diags
    from tempo_gb300 import workloads as W

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    tmax, tsum = np.load(tmp_path / "reduced.npy")
    assert tmax == 2.0 and tsum == 3.0

    o = oracle_mod
    o.init(False, REPO / "tables" / "ccn_activate.bin")
    o.build_big_tables(nthreads=2)
    wl = W.stretched_grid(seed=3, ni=12, nj=7, steps=1)
    f = {k: v.copy() for k, v in wl.fields.items()}
    d = make_diags(f["p"].shape)
    assert o.run(o.default_cfgs(hailaware_flag=0), wl.dt, 1, f, d, nthreads=1) == 0
    parts = np.load(tmp_path / "gathered.npy", allow_pickle=True)
    covered = 0
    for j0, j1, mine in parts:
        want = np.concatenate([f["t"][j0:j1].ravel(), f["qs"][j0:j1].ravel(),
                               f["qr"][j0:j1].ravel()])
        assert np.array_equal(mine, want)
        covered += j1 - j0
    assert covered == f["p"].shape[0] == 7
    assert all(j1 > j0 for j0, j1, _ in parts)

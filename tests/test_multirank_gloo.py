"""Blocks sharded over two ranks (gloo, CPU): each rank computes the density
of its own blocks with the data bounds of the whole decomposition; the sum of
the ranks' grids equals the single-process grid bit for bit, because every
grid point belongs to exactly one block's box.  Timing uses the max over
ranks, as bench.py does."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import ROOT, load_blocks


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, alg, out):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch
    from oracle.oracle import Restated
    from tess2_gb300 import host
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    d, blocks = load_blocks("blocks8_mix8192_seed3")
    gni = [int(x) for x in d["glo_num_idx"]]
    mn, mx = host.data_bounds_of(blocks)
    mine = host.shard_blocks(blocks, rank, world)
    O = Restated()
    if alg == "dtfe":
        grid = O.dtfe(mine, gni, want_owner=False, want_rho=False, data6=np.concatenate([mn, mx]))["grid"]
    else:
        grid = O.dense(1, mine, gni, data6=np.concatenate([mn, mx]))["grid"]
    t = torch.from_numpy(grid.astype(np.float64).ravel().copy())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    ms = torch.tensor([float(rank + 1)])
    dist.all_reduce(ms, op=dist.ReduceOp.MAX)
    if rank == 0:
        np.save(out, t.numpy())
        np.save(out + ".ms.npy", ms.numpy())
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("alg", ["dtfe", "cic"])
def test_two_ranks_partition_blocks(tmp_path, oracle, alg):
    out = str(tmp_path / "sum.npy")
    mp.start_processes(_rank_main, args=(2, _free_port(), alg, out), nprocs=2, join=True, start_method="spawn")
    summed = np.load(out)
    d, blocks = load_blocks("blocks8_mix8192_seed3")
    gni = [int(x) for x in d["glo_num_idx"]]
    ref = oracle.dtfe(blocks, gni, want_owner=False, want_rho=False)["grid"] if alg == "dtfe" \
        else oracle.dense(1, blocks, gni)["grid"]
    if alg == "dtfe":
        # one owner per grid point: the sum over ranks is the single-process grid exactly
        assert np.array_equal(summed.astype(np.float32), ref.ravel())
    else:
        # CIC deposits that cross blocks are dropped by each rank's single-rank
        # exchange; the owned-box deposits add up
        assert summed.sum() <= ref.astype(np.float64).sum() + 1e-3
    assert float(np.load(out + ".ms.npy")[0]) == 2.0


def test_shard_blocks_round_robin():
    from tess2_gb300 import host
    blocks = list(range(8))
    assert host.shard_blocks(blocks, 0, 3) == [0, 3, 6]
    assert host.shard_blocks(blocks, 2, 3) == [2, 5]
    assert sorted(sum((host.shard_blocks(blocks, r, 3) for r in range(3)), [])) == blocks
    with pytest.raises(ValueError):
        host.shard_blocks(blocks, 3, 3)

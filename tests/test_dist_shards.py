"""The multi-GPU path on CPU: two gloo ranks, each solving its own column shard with
the oracle, and the bench's aggregation.  Checks that the shards are disjoint, that a
shard's results do not depend on the world size, and that the whole-job throughput is
the units of all ranks over the slowest rank's time (bench.aggregate_throughput)."""
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NC, CFG = 48, 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _shard_checksum(rank):
    """Rank `rank`'s shard, one step through the oracle: checksums of its outputs."""
    sys.path.insert(0, ROOT)
    import bench
    from clmgb import abi, synth
    from oracle import oracle as orc
    wl = synth.make_workload(CFG, nc=NC, seed=bench.shard_seed(CFG, rank), nsteps=1)
    st = wl.state
    G, I = wl.forcing_block([0])
    orc.run_steps(st, wl.dtime, G, I, abi.SwmConfig.clm5_default(), nthreads=1)
    return np.array([st["h2osoi_liq"].sum(), st["t_soisno"].sum(), st["qcharge"].sum()], dtype=np.float64)


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sums = torch.from_numpy(_shard_checksum(rank))
        gathered = [torch.zeros_like(sums) for _ in range(world)]
        dist.all_gather(gathered, sums)
        # rank r "took" 10 + 5r ms for 1000 units
        value, ms = bench.aggregate_throughput(10.0 + 5.0 * rank, 1000, world, device="cpu")
        if rank == 0:
            torch.save({"sums": torch.stack(gathered), "value": value, "ms": ms}, out)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_solve_disjoint_shards(tmp_path):
    mp = torch.multiprocessing.get_context("spawn")
    out = str(tmp_path / "r0.pt")
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
        assert p.exitcode == 0
    res = torch.load(out)
    sums = res["sums"].numpy()
    assert not np.array_equal(sums[0], sums[1])                     # disjoint shards
    for r in range(2):                                              # independent of the world size
        assert np.array_equal(sums[r], _shard_checksum(r))
    assert res["ms"] == 15.0                                        # the slowest rank's time
    assert res["value"] == pytest.approx(2 * 1000 / 0.015)

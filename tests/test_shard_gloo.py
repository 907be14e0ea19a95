"""The N > 1 path on CPU: two gloo ranks each solve their contiguous shard of
the calcite column with the oracle and reduce the statistics; the union must
equal the single-process solve and the reduced statistics its totals."""
import os

import numpy as np
import torch.multiprocessing as mp

from pflotran_gb300.shard import shard_bounds


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist
    from oracle import oracle
    from pflotran_gb300 import workloads
    from pflotran_gb300.shard import reduce_stats, shard_bounds
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    net, opt, cells, dt = workloads.calcite_cells(257, seed=3)
    lo, hi = shard_bounds(cells.ncells, rank, world)
    sub = cells.subset(np.arange(lo, hi), net)
    oracle.react(net.as_struct(), opt, dt, sub, 0, 1)
    stats = reduce_stats(hi - lo, int(sub.iterations.sum()), int(sub.iterations.max()), int((sub.status != 0).sum()))
    q.put((rank, lo, hi, sub.pri_molal.copy(), stats))
    dist.barrier()
    dist.destroy_process_group()


def test_shard_bounds_cover_exactly():
    for n in (0, 1, 7, 100, 257):
        for w in (1, 2, 3, 8):
            ranges = [shard_bounds(n, r, w) for r in range(w)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(ranges[i][1] == ranges[i + 1][0] for i in range(w - 1))
            assert max(h - l for l, h in ranges) - min(h - l for l, h in ranges) <= 1


def test_two_gloo_ranks_match_single_process(oracle):
    from pflotran_gb300 import workloads
    net, opt, cells, dt = workloads.calcite_cells(257, seed=3)
    full = cells.copy()
    oracle.react(net.as_struct(), opt, dt, full, 0, 1)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    m = full.pri_molal.reshape(net.N, -1)
    for rank, lo, hi, pm, stats in res:
        assert np.array_equal(pm.reshape(net.N, -1), m[:, lo:hi])
        assert stats == (257, int(full.iterations.sum()), int(full.iterations.max()), int((full.status != 0).sum()))

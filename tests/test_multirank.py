"""Multi-process paths on CPU: two ranks over gloo at 127.0.0.1.

`bench.py --gpus N` runs one replica per GPU; the ranks meet at a barrier and
every rank takes the longest time over ranks (bench.max_over_ranks) before
rank 0 reports.  A pass split across ranks would give each rank a disjoint
packet range and sum jmean once: with packet-id keyed Philox streams that sum
equals the single-range pass (the oracle's transport stands in for each
rank's device).  No GPU is used.
"""
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case():
    mats = [(0.0, 0.0, 0.0, 1.0), (0.5, 30.0, 0.9, 1.4)]
    grid = np.ones((12, 12, 12), dtype=np.uint8, order="F")
    grid[:, :, 8:] = 0  # an air layer
    return mats, grid


def _worker(rank, world, port, kind, out_dir):
    for p in (ROOT, os.path.join(ROOT, "oracle")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        if kind == "max":
            import bench

            got = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
            np.save(os.path.join(out_dir, f"max{rank}.npy"), np.array([got]))
        else:
            import oracle

            oracle.load()
            mats, grid = _case()
            d = oracle.mc_desc(12, 12, 12, 0.3, 0.3, 0.3, materials=mats, source_radius=0.05)
            n = 4000
            p0, p1 = n * rank // world, n * (rank + 1) // world
            j, tal = oracle.mc_transport(d, grid, p1 - p0, seed=8, p0=p0, nthreads=1)
            t = torch.from_numpy(np.ascontiguousarray(j.ravel(order="F")))
            dist.all_reduce(t)  # the one data-path collective: jmean sum
            np.save(os.path.join(out_dir, f"j{rank}.npy"), t.numpy())
    finally:
        dist.destroy_process_group()


def _spawn(kind, tmp_path, world=2):
    mp.spawn(_worker, args=(world, _free_port(), kind, str(tmp_path)), nprocs=world, join=True)


def test_bench_max_over_ranks_gloo(tmp_path):
    _spawn("max", tmp_path)
    for r in range(2):
        assert float(np.load(tmp_path / f"max{r}.npy")[0]) == 15.0


def test_sharded_pass_sums_to_single_pass_gloo(tmp_path, orc):
    _spawn("shard", tmp_path)
    mats, grid = _case()
    d = orc.mc_desc(12, 12, 12, 0.3, 0.3, 0.3, materials=mats, source_radius=0.05)
    j_all, _ = orc.mc_transport(d, grid, 4000, seed=8, nthreads=1)
    want = j_all.ravel(order="F")
    assert want.sum() > 0
    for r in range(2):
        got = np.load(tmp_path / f"j{r}.npy")
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-15 * want.max())

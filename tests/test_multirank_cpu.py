"""Multi-rank host logic on the CPU (gloo, world size 2): every rank generates its own slice of the
ensemble from the counter-based seed, the slices tile the single-process workload exactly, and
the timing reduction is a max over ranks (what bench.py does under torchrun)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from degpu import workloads as W  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    first, count = W.rank_slice(n, rank)
    e = W.config1(n=count, first=first)
    np.save(os.path.join(out_dir, f"rank{rank}.npy"), np.concatenate([e.tf, e.rtol, e.y0.ravel()]))
    t = torch.tensor([float(rank + 1) * 1.5])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    np.save(os.path.join(out_dir, f"max{rank}.npy"), t.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_partition_and_max_reduction(tmp_path):
    n, world = 300, 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_worker, args=(r, world, port, n, str(tmp_path))) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    whole = W.config1(n=world * n)
    for r in range(world):
        sl = W.config1(n=n, first=r * n)
        got = np.load(tmp_path / f"rank{r}.npy")
        exp = np.concatenate([whole.tf[r * n:(r + 1) * n], whole.rtol[r * n:(r + 1) * n],
                              whole.y0[:, r * n:(r + 1) * n].ravel()])
        assert np.array_equal(got, exp)
        assert np.array_equal(sl.family, whole.family[r * n:(r + 1) * n])
        assert float(np.load(tmp_path / f"max{r}.npy")[0]) == 3.0

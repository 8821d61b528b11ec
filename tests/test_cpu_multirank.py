"""Multi-GPU is replicas only: each rank integrates its own cells, no collective
on the data path, the step time is the max over ranks. The rank logic of
bench.py runs here on CPU with two gloo ranks (each rank's cells integrated by
the oracle, the CPU stand-in for its GPU)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, cells, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    import simstack_gb300 as sg
    from oracle import oracle as O

    grp = bench.Group(world)
    w, r, _ = bench.dist_env()
    z = sg.air_cells(cells, seed=1, first_cell=r * cells)    # this rank's partition
    O.Mechanism.air().advance("rodas3", O.control(), z.as_dict(), z.padded, 0, cells, 0.2, 0, 1)
    t = grp.max(float(r + 1))                               # max over ranks
    grp.barrier()
    out[r] = (z["y"][:, :cells].copy(), t)
    grp.close()


def test_two_rank_replicas():
    cells, world = 16, 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(world, port, cells, out), nprocs=world, join=True)
    from oracle import oracle as O
    import simstack_gb300 as sg

    whole = sg.air_cells(cells * world, seed=1)
    O.Mechanism.air().advance("rodas3", O.control(), whole.as_dict(), whole.padded, 0, cells * world, 0.2, 0, 1)
    got = np.concatenate([out[0][0], out[1][0]], axis=1)
    assert got.tobytes() == whole["y"][:, :cells * world].tobytes()   # partitions compose to the whole
    assert out[0][1] == out[1][1] == 2.0

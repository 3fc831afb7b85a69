"""Shot-parallel path on CPU: two gloo ranks shard a list of window shots,
run their shots with the oracle and gather the seismograms on rank 0; the
gathered traces equal a serial run of every shot (no GPU needed)."""

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from cgfd3d_gb300 import shots as S


def test_shard_is_a_partition():
    for n in (1, 5, 64, 67):
        for w in (1, 2, 3, 8):
            got = [S.shard(n, r, w) for r in range(w)]
            flat = [i for g in got for i in g]
            assert flat == list(range(n))
            assert max(map(len, got)) - min(map(len, got)) <= 1


def _problems():
    from cgfd3d_gb300 import models
    base = models._topo_base(60, 56, 40, 3)
    return models.window_shots(3, base=(60, 56, 40), wmin=(40, 36, 30),
                               wmax=(48, 44, 34), steps=4, base_model=base,
                               seed=5, nrecv=4, npml=4)


def _worker(rank, world, port, out_path):
    import torch.distributed as dist
    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    probs = _problems()
    mine = S.shard(len(probs), rank, world)
    local = {}
    for k in mine:
        oracle.allstep(probs[k], oracle.TIMG_ZERO, 1)
        local[k] = S.traces(probs[k])
    got = S.gather_to_root(local, rank, world)
    if rank == 0:
        merged = {}
        for d in got:
            merged.update(d)
        np.savez(out_path, **{str(k): v for k, v in merged.items()})
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_gather_equals_serial(tmp_path):
    import oracle
    import torch.multiprocessing as mp
    out = str(tmp_path / "traces.npz")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2,
                       start_method="spawn")
    got = np.load(out)
    probs = _problems()
    assert sorted(int(k) for k in got.files) == list(range(len(probs)))
    for k, p in enumerate(probs):
        oracle.allstep(p, oracle.TIMG_ZERO, 1)
        np.testing.assert_array_equal(got[str(k)], S.traces(p))

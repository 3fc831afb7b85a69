"""Data-parallel surrogate training on CPU: two gloo ranks each take half of
a batch, compute the float64 gradient of their half with the restatement
(oracle/surrogate_ref.py) and average it with surrogate.allreduce_mean, the
all-reduce Surrogate.sync_gradients issues; the result is the gradient and
loss of the whole batch in one process (no GPU needed)."""

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _batch():
    import surrogate_ref as sr
    rng = np.random.default_rng(4)
    nrec, B, nt = 1, 4, 1000
    enc, dec = sr.layers(nrec)
    params = np.concatenate([np.concatenate([rng.standard_normal(o * i) * np.sqrt(2.0 / i),
                                             0.01 * rng.standard_normal(o)])
                             for o, i in enc + dec])
    pos = rng.uniform(-1, 1, (B, 3))
    M = rng.standard_normal((B, 6))
    U = rng.standard_normal((B, nt, 3 * nrec))
    return params, pos, M, U, nrec


def _worker(rank, world, port, out_path):
    import torch.distributed as dist
    import surrogate_ref as sr
    from cgfd3d_gb300 import shots, surrogate
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    params, pos, M, U, nrec = _batch()
    mine = shots.shard(len(pos), rank, world)
    loss, g = sr.loss_and_grad(params, pos[mine], M[mine], U[mine], nrec, 1.0)
    tg = torch.from_numpy(g.copy())
    tl = torch.tensor([loss], dtype=torch.float64)
    surrogate.allreduce_mean(tg)
    surrogate.allreduce_mean(tl)
    if rank == 0:
        np.savez(out_path, g=tg.numpy(), loss=tl.numpy())
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_give_the_whole_batch_gradient(tmp_path):
    import surrogate_ref as sr
    import torch.multiprocessing as mp
    out = str(tmp_path / "dp.npz")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True,
                       start_method="spawn")
    got = np.load(out)
    params, pos, M, U, nrec = _batch()
    loss, g = sr.loss_and_grad(params, pos, M, U, nrec, 1.0)
    assert abs(float(got["loss"][0]) - loss) <= 1e-12 * abs(loss)
    np.testing.assert_allclose(got["g"], g, rtol=1e-10, atol=1e-12 * np.abs(g).max())


def test_one_process_is_a_no_op():
    from cgfd3d_gb300 import surrogate
    t = torch.arange(5, dtype=torch.float64)
    assert torch.equal(surrogate.allreduce_mean(t.clone()), t)

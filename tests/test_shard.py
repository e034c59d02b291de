"""Sharding independent junctions over ranks (cmtj_gb300.shard), on CPU:
the partition's properties, and a world_size-2 gloo run in which each rank
integrates only its own rows (with the oracle, the CPU stand-in for one
rank's GPU) and rank 0 gathers them.  The gathered result must equal the
unsharded run bit for bit: sharding adds no exchange on the data path."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

import cmtj_gb300 as cm
from cmtj_gb300 import shard, sweeps

DT = 1e-13


def test_partition_covers_every_row_once_and_balances():
    rng = np.random.default_rng(0)
    cost = rng.integers(1, 1000, size=101).astype(float)
    for world in (1, 2, 3, 8):
        parts = shard.partition(cost, world)
        assert len(parts) == world
        assert np.array_equal(np.sort(np.concatenate(parts)), np.arange(101))
        loads = [cost[p].sum() for p in parts]
        # LPT: the heaviest rank exceeds the lightest by at most one row
        assert max(loads) - min(loads) <= cost.max()
        assert all(np.all(np.diff(p) > 0) for p in parts)
    a, b = shard.partition(cost, 3), shard.partition(cost, 3)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))


def test_partition_edges():
    parts = shard.partition([5.0, 3.0], 4)
    assert [p.tolist() for p in parts] == [[0], [1], [], []]
    assert [p.tolist() for p in shard.partition([], 2)] == [[], []]
    with pytest.raises(ValueError):
        shard.partition([1.0], 0)
    with pytest.raises(ValueError):
        shard.partition([1.0, -2.0], 2)
    spec, n_steps = _spec()
    with pytest.raises(ValueError):
        shard.rows_of(spec, n_steps, 2, 2)


def test_uneven_rows_balance_by_layer_steps():
    spec, n_steps = _spec()
    cost = shard.row_cost(spec, n_steps)
    assert np.array_equal(cost, n_steps * spec.n_layers)
    parts = shard.partition(cost, 2)
    loads = [cost[p].sum() for p in parts]
    assert max(loads) - min(loads) <= cost.max()


def _spec():
    # uneven 1-4 layer spin-diode junctions, 200-600 steps each
    return sweeps.vsd_config(n_f=2, n_h=5, seed=11, dt=DT, t_min=2e-11, t_max=6e-11, amp=5e3)


def _oracle_runner(sub, n_steps):
    """One rank's work: every row of `sub` for its own n_steps on the oracle;
    returns the final m [rows, 4, 3] and the step count."""
    import oracle_harness
    from cases import junctions_from_spec
    m = np.zeros((sub.n, 4, 3))
    for q in range(sub.n):
        f = float(sub.vsd_freq[q])
        j = junctions_from_spec(sub, [q], lambda k: cm.AxialDriver(cm.NullDriver(), cm.sineDriver(0, 5e3, f, 0),
                                                                    cm.NullDriver()))[0]
        oracle_harness.run_oracle([j], int(n_steps[q]) * DT, DT, DT)
        for l, ly in enumerate(j.layers):
            m[q, l] = [ly.mag.x, ly.mag.y, ly.mag.z]
    return {"m": m, "steps": np.asarray(n_steps, dtype=np.int64)}


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        spec, n_steps = _spec()
        res = shard.run_sharded(spec, n_steps, _oracle_runner, rank, world)
        if rank == 0:
            np.savez(out, **res)
        else:
            assert res is None
        dist.barrier()
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_sweep_gloo_world2_equals_unsharded(tmp_path):
    out = str(tmp_path / "sharded.npz")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    got = np.load(out)
    spec, n_steps = _spec()
    want = _oracle_runner(spec, n_steps)
    assert np.array_equal(got["steps"], n_steps)
    assert np.array_equal(got["m"], want["m"])


def _gpu_runner(sub, n_steps):
    """One rank's work on its GPU: the FP32 batched form over its rows, with
    the on-device <I R> reduction; final m, reductions and step counts."""
    from cmtj_gb300 import batch
    run = batch.BatchRun(batch.lower(sub, DT, n_steps), DT, cm.SolverMode.RK4, batch.LOG_NONE, 0, red_every=1)
    run.launch()
    st = run.state()
    return {"m": st["m"].copy(), "v": st["v_sum"].copy(), "status": st["status"].copy(),
            "steps": st["step"].astype(np.int64)}


def _gpu_worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.cuda.set_device(0)  # one GPU here: the ranks share it, and nothing on it waits on another rank
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        spec, n_steps = sweeps.vsd_config(n_f=8, n_h=64, seed=11, dt=DT, t_min=2e-10, t_max=6e-10)
        res = shard.run_sharded(spec, n_steps, _gpu_runner, rank, world)
        if rank == 0:
            np.savez(out, **res)
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.gpu
def test_sharded_gpu_sweep_equals_unsharded(gpu_lib, tmp_path):
    """The sharded path with the GPU solver: two gloo ranks, each running its
    own rows of an uneven spin-diode sweep on the GPU (FP32 batched form),
    gathered on rank 0, equal the unsharded GPU run bit for bit."""
    out = str(tmp_path / "sharded_gpu.npz")
    mp.spawn(_gpu_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    got = np.load(out)
    spec, n_steps = sweeps.vsd_config(n_f=8, n_h=64, seed=11, dt=DT, t_min=2e-10, t_max=6e-10)
    want = _gpu_runner(spec, n_steps)
    assert np.all(got["status"] == 0) and np.array_equal(got["steps"], n_steps)
    for k in ("m", "v"):
        assert got[k].tobytes() == want[k].tobytes(), k

"""Sharding a batch of independent junctions over ranks, one GPU per rank.

The reference parallelises sweeps as independent solves in a process pool
(cmtj/utils/parallel.py:13-51); nothing couples two junctions outside a
Stack (core/stack.hpp).  So a sweep splits by junction with no exchange
step on the data path: each rank lowers and runs only its own rows, and the
per-row results are gathered to one rank on the host after the runs end.

* partition()   -- rows per rank, balanced by cost (layer-steps), with the
                   longest-processing-time-first rule: deterministic, every
                   row exactly once, max load within one row of optimal.
* run_sharded() -- this rank's rows through a runner, then the gather.

The collective here is one host-side gather_object after the work (gloo on
CPU, NCCL on GPUs); nothing waits on another rank while junctions run.
"""
import numpy as np


def row_cost(spec, n_steps):
    """Layer-steps of each row: n_steps[k] (or a scalar) x n_layers[k]."""
    steps = np.broadcast_to(np.asarray(n_steps, dtype=np.float64), (spec.n,))
    return steps * spec.n_layers.astype(np.float64)


def partition(cost, world):
    """Split rows 0..n-1 over `world` ranks: rows in decreasing cost (ties by
    index) each go to the least-loaded rank (ties to the lowest rank).
    Returns a list of `world` sorted index arrays."""
    cost = np.asarray(cost, dtype=np.float64)
    if world < 1:
        raise ValueError("world must be >= 1, got %d" % world)
    if np.any(cost < 0) or not np.all(np.isfinite(cost)):
        raise ValueError("row costs must be finite and >= 0")
    order = np.lexsort((np.arange(len(cost)), -cost))
    load = np.zeros(world)
    owner = np.empty(len(cost), dtype=np.int64)
    for k in order:
        r = int(np.argmin(load))
        owner[k] = r
        load[r] += cost[k]
    return [np.flatnonzero(owner == r) for r in range(world)]


def rows_of(spec, n_steps, rank, world):
    """This rank's rows of `spec` (see partition)."""
    if not 0 <= rank < world:
        raise ValueError("rank %d outside [0, %d)" % (rank, world))
    return partition(row_cost(spec, n_steps), world)[rank]


def gather_rows(rows, values, n, dst=0, group=None):
    """Collect per-row results from every rank onto rank `dst`.  `values` is a
    dict name -> array whose first axis follows `rows`.  Returns on dst a
    dict name -> array [n, ...] in global row order, else None."""
    import torch.distributed as dist
    payload = (np.asarray(rows), {k: np.asarray(v) for k, v in values.items()})
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    bucket = [None] * world if rank == dst else None
    dist.gather_object(payload, bucket, dst=dst, group=group)
    if rank != dst:
        return None
    out = {}
    seen = np.zeros(n, dtype=bool)
    for r_rows, r_vals in bucket:
        if np.any(seen[r_rows]):
            raise RuntimeError("a row was returned by two ranks")
        seen[r_rows] = True
        for k, v in r_vals.items():
            if k not in out:
                out[k] = np.zeros((n,) + v.shape[1:], dtype=v.dtype)
            out[k][r_rows] = v
    if not np.all(seen):
        raise RuntimeError("rows %s were returned by no rank" % np.flatnonzero(~seen)[:8].tolist())
    return out


def run_sharded(spec, n_steps, runner, rank, world, dst=0, group=None):
    """Run this rank's rows: runner(sub_spec, sub_n_steps) -> dict of per-row
    arrays (for instance final m and spectra from a BatchRun on this rank's
    GPU).  Returns the gathered dict on rank dst, None elsewhere."""
    rows = rows_of(spec, n_steps, rank, world)
    steps = np.asarray(n_steps)
    sub_steps = steps[rows] if steps.ndim else steps
    values = runner(spec.take(rows), sub_steps) if len(rows) else {}
    return gather_rows(rows, values, spec.n, dst=dst, group=group)

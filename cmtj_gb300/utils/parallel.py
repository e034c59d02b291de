"""`cmtj.utils.parallel.distribute` (cmtj/utils/parallel.py:13-51).

The reference maps a simulation function over the product of parameter
spaces with a process pool, yielding (index, output) as results arrive.
Here the calls run on a thread pool in this process: each call's GPU work
is a kernel launch that releases the GIL while it runs, so calls overlap on
the device, and no CUDA context is forked.  For sweeps of many junctions
the batched forms are far faster: a list of junctions to one launch
(cmtj_gb300.engine.run_junctions, the procedures with a list), or
cmtj_gb300.batch / sweeps for FP32.
"""
import concurrent.futures
import os
from itertools import product

import numpy as np

__all__ = ["distribute"]


def distribute(simulation_fn, spaces, n_cores=None, shuffle=False):
    """Yield (index, simulation_fn(*values)) for every combination of
    `spaces`, in completion order; index[i] is the position of values[i] in
    spaces[i].  shuffle submits the combinations in random order (numpy's
    global generator, as the reference)."""
    spaces = [np.asarray(space) for space in spaces]
    iterables = list(product(*spaces))
    indexes = [[int(np.argwhere(space == v[i]).ravel()[0]) for i, space in enumerate(spaces)] for v in iterables]
    order = np.arange(len(iterables))
    if shuffle:
        np.random.shuffle(order)
    workers = n_cores if n_cores else min(32, os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(max_workers=workers) as ex:
        futures = {ex.submit(simulation_fn, *iterables[k]): k for k in order}
        for fut in concurrent.futures.as_completed(futures):
            yield indexes[futures[fut]], fut.result()

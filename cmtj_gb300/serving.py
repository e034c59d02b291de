"""Continuous-batching request loop over the FP32 batched form.

Requests (sweeps or fits: 64-16,384 independent solves each) arrive over
time.  The engine keeps a pool of device-resident junction slots sized by
an HBM budget; a request is admitted when a contiguous range of free slots
holds it, its records are copied into those slots once, and from then on
its state stays on the device.  The GPU advances every admitted junction in
ticks of `chunk_steps` iterations (one persistent launch per kernel variant
present), so requests that arrive while others run join at the next tick
and overlap with them on the device.  A request completes when all its
junctions have run their steps; only its final state and on-device
reductions are read back.

Each junction's kernel variant comes from its own features and its state is
saved and restored exactly between ticks, so a request's results are the
same bits alone or in any mix, at any tick length.

FP64 plain-form requests (Junction objects) run through
cmtj_run_simulation_f64 on a small pool of their own streams, overlapping
the FP32 ticks and one another; their inputs go up asynchronously from
pinned memory, so admitting one never waits for another's kernel.
"""
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import _abi, autotune, batch, engine
from .core import SolverMode


@dataclass
class Request:
    """A batch of independent solves.  FP32: `spec` (BatchSpec) and
    `n_steps` ([n] or scalar); FP64 plain: `junctions` (Junction objects,
    one plan for all)."""
    spec: object = None
    n_steps: object = None
    solver: SolverMode = SolverMode.RK4
    precision: str = "f32"
    junctions: list = None
    total_time: float = 0.0
    time_step: float = 1e-13
    red_every: int = 0
    win_start: object = None
    arrival: float = 0.0          # seconds after the trace start
    tag: str = ""
    # filled by the engine
    id: int = -1
    admitted_at: float = None
    done_at: float = None
    state: np.ndarray = None      # F32 state rows (FP32 requests)
    layer_steps: float = 0.0
    n: int = 0

    @property
    def latency(self):
        return None if self.done_at is None else self.done_at - self.arrival


class SlotPool:
    """Device arrays for `capacity` junction slots (4 layer records each)
    and a first-fit allocator of contiguous slot ranges."""

    BYTES_PER_SLOT = (batch.F32_JUNCTION_DTYPE.itemsize + 4 * batch.F32_LAYER_DTYPE.itemsize +
                      batch.F32_STATE_DTYPE.itemsize + 4)

    def __init__(self, hbm_budget_bytes):
        t = engine.torch()
        self.capacity = int(hbm_budget_bytes // self.BYTES_PER_SLOT)
        if self.capacity < 64:
            raise ValueError("HBM budget too small for 64 junction slots")
        C = self.capacity
        self.d_j = t.zeros(C * batch.F32_JUNCTION_DTYPE.itemsize, dtype=t.uint8, device="cuda")
        self.d_l = t.zeros(4 * C * batch.F32_LAYER_DTYPE.itemsize, dtype=t.uint8, device="cuda")
        self.d_s = t.zeros(C * batch.F32_STATE_DTYPE.itemsize, dtype=t.uint8, device="cuda")
        self.d_log = t.zeros(4, dtype=t.float32, device="cuda")
        self.free = [(0, C)]  # sorted (start, length)

    def alloc(self, n):
        for k, (a, ln) in enumerate(self.free):
            if ln >= n:
                if ln == n:
                    self.free.pop(k)
                else:
                    self.free[k] = (a + n, ln - n)
                return a
        return None

    def release(self, a, n):
        self.free.append((a, n))
        self.free.sort()
        merged = []
        for s, ln in self.free:
            if merged and merged[-1][0] + merged[-1][1] == s:
                merged[-1] = (merged[-1][0], merged[-1][1] + ln)
            else:
                merged.append((s, ln))
        self.free = merged


class ServingEngine:
    """Admission by HBM budget, device-resident state, tick-level continuous
    batching.  `run(requests)` replays a trace (arrival times relative to
    the start) and returns the completed requests."""

    def __init__(self, hbm_budget_bytes=8 << 30, chunk_steps=2000, time_step=1e-13, max_active_solves=None,
                 n_streams=8, policy="sjf"):
        self.lib = engine.require_gpu()
        self.t = engine.torch()
        self.pool = SlotPool(hbm_budget_bytes)
        self.chunk = int(chunk_steps)
        self.dt = float(time_step)
        # Working set: enough junctions to fill every SM twice over; later
        # requests wait, so requests complete roughly in arrival order
        # instead of all sharing the GPU until the end of the trace.
        if max_active_solves is None:
            import ctypes
            sms = ctypes.c_int32()
            self.lib.cmtj_device_info(self.t.cuda.current_device(), ctypes.byref(sms), None, None)
            max_active_solves = 2 * sms.value * 5 * 128
        self.max_active = int(max_active_solves)
        # admission order among requests that have arrived: "fifo", or "sjf"
        # (smallest layer-steps first, ties by arrival), which cuts the
        # median latency of a saturated loop without changing any result
        if policy not in ("fifo", "sjf"):
            raise ValueError("policy must be 'fifo' or 'sjf'")
        self.policy = policy
        self.stream = self.t.cuda.Stream()
        self.streams = [self.t.cuda.Stream() for _ in range(max(1, n_streams))]
        # FP64 plain requests: a few streams so that they overlap one another
        # and the FP32 ticks, taken in turn
        self.streams64 = [self.t.cuda.Stream() for _ in range(4)]
        self._next64 = 0
        # one 64-byte work ticket per launch group of a tick
        self.tickets = self.t.zeros(256 * 16, dtype=self.t.int32, device="cuda")
        self.active = []     # FP32 requests on the device: (req, slot, meta)
        self.active64 = []   # (req, lowered, layers, log, status, event, plan, buffers kept alive)
        self._next_id = 0
        self.params = np.zeros(1, dtype=batch.F32_PARAMS_DTYPE)
        self.stats = {"ticks": 0, "host_s": 0.0, "device_wait_s": 0.0, "admit_s": 0.0}
        # launch groups (device order arrays) are rebuilt only when the set
        # of running requests changes; the host runs at most `ahead` ticks
        # in front of the device and synchronises only to retire requests
        self._groups = None
        self._tick_events = []
        self.ahead = 2

    # ------------------------------------------------------------ admission
    def _pinned(self, arr):
        """The bytes of a numpy array in pinned host memory, for an
        asynchronous copy (PyTorch's pinned allocator keeps the block until
        the copy that reads it is done)."""
        return self.t.from_numpy(np.ascontiguousarray(arr).view(np.uint8).reshape(-1).copy()).pin_memory()

    def _admit(self, req, now):
        if req.precision == "f64":
            return self._admit_f64(req, now)
        n = req.spec.n
        active = sum(r.n for r, _ in self.active)
        if active and active + n > self.max_active:
            return False
        slot = self.pool.alloc(n)
        if slot is None:
            return False
        low = batch.lower(req.spec, self.dt, req.n_steps, win_start=req.win_start)
        jr = low.junctions.copy()
        jr["layer_offset"] = 4 * (slot + np.arange(n))
        jr["log_offset"] = 0
        lay = np.zeros(4 * n, dtype=batch.F32_LAYER_DTYPE)
        L = low.junctions["n_layers"].astype(np.int64)
        src_off = low.junctions["layer_offset"].astype(np.int64)
        for l in range(4):
            has = L > l
            lay[4 * np.nonzero(has)[0] + l] = low.layers[src_off[has] + l]
        st = np.zeros(n, dtype=batch.F32_STATE_DTYPE)
        own = low.features | (np.where(low.n_waves > 1, 4, np.where(low.n_waves > 0, 1, 0)) << 16)
        variant = np.zeros(n, dtype=np.int64)
        for key in np.unique(L * (1 << 24) + own):
            nl, code = int(key >> 24), int(key & ((1 << 24) - 1))
            v = self.lib.cmtj_batch_variant_f32(nl, int(req.solver), code)
            if v < 0:
                raise ValueError("no FP32 kernel variant for layers=%d features=0x%x" % (nl, code))
            variant[(L * (1 << 24) + own) == key] = v
        # asynchronous copies from pinned memory, in stream order after the
        # ticks in flight (the slots are free) and before the next tick
        # (which waits for the group rebuild recorded after them)
        with self.t.cuda.stream(self.stream):
            JB, LB, SB = (batch.F32_JUNCTION_DTYPE.itemsize, batch.F32_LAYER_DTYPE.itemsize,
                          batch.F32_STATE_DTYPE.itemsize)
            self.pool.d_j[slot * JB:(slot + n) * JB].copy_(self._pinned(jr), non_blocking=True)
            self.pool.d_l[4 * slot * LB:4 * (slot + n) * LB].copy_(self._pinned(lay), non_blocking=True)
            self.pool.d_s[slot * SB:(slot + n) * SB].copy_(self._pinned(st), non_blocking=True)
        req.id = self._next_id
        self._next_id += 1
        req.admitted_at = now
        req.n = n
        req.layer_steps = float(np.sum(low.n_steps * L))
        ids = slot + np.arange(n)
        parts = {}
        for key in np.unique(L * (1 << 32) + variant):
            sel = (L * (1 << 32) + variant) == key
            parts[(int(key >> 32), int(req.solver), int(key & ((1 << 32) - 1)), int(req.red_every))] = \
                ids[sel].astype(np.int32)
        meta = {"slot": slot, "parts": parts, "steps_max": int(low.n_steps.max()), "done": 0}
        self.active.append((req, meta))
        return True

    def _admit_f64(self, req, now):
        """Lower the request's junctions and launch their FP64 plain run on
        the next FP64 stream.  The host copies are pinned and asynchronous:
        the loop never waits for an earlier FP64 request's kernel."""
        plan = engine.plan_run(req.total_time, req.time_step, req.total_time if req.total_time > 0 else 1.0)
        solver = req.junctions[0].getSolver(req.solver)
        from ._lower import lower
        low = lower(req.junctions, plan, solver, False)
        stream = self.streams64[self._next64 % len(self.streams64)]
        self._next64 += 1
        pinned = []

        def up(arr):
            h = self._pinned(arr)
            pinned.append(h)
            return h.to("cuda", non_blocking=True)

        alpha = None
        larr = low.layers
        if low.alpha_specs is not None:
            # buffered alpha noise: this run's buffers, filled on the stream
            from ._lower import with_alpha_buffers
            from .noise import device_buffers
            alpha = device_buffers(low.alpha_specs, int(larr[low.alpha_layers[0]]["alpha_len"]), stream=stream)
            larr = with_alpha_buffers(low, alpha.data_ptr())
        with self.t.cuda.stream(stream):
            d_j, d_l = up(low.junctions), up(larr)
            d_tab = up(low.tables) if low.tables is not None else None
            n = len(req.junctions)
            d_log = self.t.empty((n, max(plan.n_log, 1), low.log_width), dtype=self.t.float64, device="cuda")
            d_st = self.t.zeros(2 * n, dtype=self.t.int32, device="cuda")
            rc = self.lib.cmtj_run_simulation_f64(engine.ptr(d_j), n, engine.ptr(d_l), engine.ptr(d_tab),
                                                  low.params.ctypes.data, engine.ptr(d_log), engine.ptr(d_st),
                                                  engine.stream_ptr(stream))
            _abi.check(rc, self.lib)
            ev = self.t.cuda.Event()
            ev.record(stream)
        req.id = self._next_id
        self._next_id += 1
        req.admitted_at = now
        req.n = n
        req.layer_steps = float(n * plan.total_iterations * np.mean([j.layerNo for j in req.junctions]))
        # the device and pinned buffers stay referenced until the event
        self.active64.append((req, low, d_l, d_log, d_st, ev, plan, (d_j, d_tab, pinned, alpha)))
        return True

    # ------------------------------------------------------------ ticks
    def _build_groups(self):
        """(layer count, solver, variant, reduction cadence) -> junction ids
        of the running requests, one launch each per tick: a junction always
        runs the same code whatever its neighbours in the pool."""
        groups = {}
        for req, meta in self.active:
            if meta["done"] >= meta["steps_max"]:
                continue
            for key, ids in meta["parts"].items():
                groups.setdefault(key, []).append(ids)
        built = []
        with self.t.cuda.stream(self.stream):
            for key, parts in sorted(groups.items()):
                order = np.concatenate(parts).astype(np.int32)
                built.append((key, self._pinned(order).to("cuda", non_blocking=True).view(self.t.int32),
                              int(order.size)))
        ev = self.t.cuda.Event()
        ev.record(self.stream)  # admission copies and the order uploads
        self._groups = (built, ev)

    def _tick(self):
        """Advance every running FP32 junction by up to chunk_steps, without
        waiting for the device (at most `ahead` ticks in flight)."""
        while len(self._tick_events) >= self.ahead:
            t_dev = time.perf_counter()
            self._tick_events.pop(0).synchronize()
            self.stats["device_wait_s"] += time.perf_counter() - t_dev
        t_host = time.perf_counter()
        if self._groups is None:
            self._build_groups()
        built, ready = self._groups
        # partitions of one tick run concurrently, one stream (and one ticket)
        # each, so their launch tails overlap; junction sets are disjoint.
        # A stream's next tick follows its previous one in stream order, and
        # every stream waits for the previous tick's end on all streams.
        prev = self._tick_events[-1] if self._tick_events else None
        if len(built) > 256:
            raise RuntimeError("more than 256 launch groups in one tick")
        ends = []
        for q, ((nl, solver, v, red), d_order, cnt) in enumerate(built):
            s = self.streams[q % len(self.streams)]
            s.wait_event(ready)
            if prev is not None:
                s.wait_event(prev)
            p = np.zeros(1, dtype=batch.F32_PARAMS_DTYPE)
            p["dt"] = self.dt
            p["chunk_steps"] = self.chunk
            p["log_mode"] = batch.LOG_NONE
            p["solver"] = solver
            p["red_every"] = red
            if autotune.enabled():
                # the resident-CTA bound the autotuner chose for this kind of
                # partition, when it has met one (no trial launches here)
                c = autotune.lookup(autotune.f32_key(nl, solver, v, 0, False, cnt))
                if c is not None:
                    v = (v & 0xffffff) | (int(c["bound"]) << 24)
            ticket = self.tickets[q * 16:]
            d_order.record_stream(s)  # kept alive for s when the groups are rebuilt
            rc = self.lib.cmtj_batch_run_f32(engine.ptr(self.pool.d_j), engine.ptr(self.pool.d_l),
                                             engine.ptr(self.pool.d_s), engine.ptr(d_order), cnt, nl, v,
                                             p.ctypes.data, engine.ptr(self.pool.d_log), engine.ptr(ticket), 0,
                                             engine.stream_ptr(s))
            _abi.check(rc, self.lib)
            e = self.t.cuda.Event()
            e.record(s)
            ends.append(e)
        done = self.t.cuda.Event()
        for e in ends:
            self.stream.wait_event(e)
        done.record(self.stream)
        self._tick_events.append(done)
        self.stats["host_s"] += time.perf_counter() - t_host
        self.stats["ticks"] += 1
        finished = False
        for req, meta in self.active:
            if meta["done"] < meta["steps_max"]:
                meta["done"] += self.chunk
                if meta["done"] >= meta["steps_max"]:
                    meta["end_event"] = done
                    finished = True
        if finished:
            self._groups = None

    def _retire(self, now):
        keep = []
        SB = batch.F32_STATE_DTYPE.itemsize
        for req, meta in self.active:
            ev = meta.get("end_event")
            if ev is not None and ev.query():
                a = meta["slot"]
                st = self.pool.d_s[a * SB:(a + req.n) * SB].cpu().numpy().view(batch.F32_STATE_DTYPE).copy()
                req.state = st
                req.done_at = now()
                self.pool.release(a, req.n)
            else:
                keep.append((req, meta))
        self.active = keep
        keep64 = []
        for item in self.active64:
            req, low, d_l, d_log, d_st, ev, plan, _ = item
            if ev.query():
                low.layers = d_l.cpu().numpy().view(_abi.LAYER_DTYPE).copy()
                from ._lower import apply_results
                apply_results(req.junctions, low, d_log.cpu().numpy(), d_st.cpu().numpy().view(np.uint32), plan)
                req.done_at = now()
            else:
                keep64.append(item)
        self.active64 = keep64

    # ------------------------------------------------------------ replay
    def run(self, requests, realtime=True):
        """Replay requests (sorted by arrival).  With realtime, arrivals are
        wall-clock offsets from the start; latencies are wall-clock."""
        pending = sorted(requests, key=lambda r: r.arrival)
        t0 = time.perf_counter()
        now = (lambda: time.perf_counter() - t0) if realtime else (lambda: float("inf"))
        qi = 0
        waiting = []  # arrived, not yet admitted
        while qi < len(pending) or waiting or self.active or self.active64:
            tnow = now()
            ta = time.perf_counter()
            while qi < len(pending) and pending[qi].arrival <= tnow:
                waiting.append(pending[qi])
                qi += 1
            if self.policy == "sjf":
                waiting.sort(key=lambda r: (_work_estimate(r), r.arrival))
            while waiting:
                if not self._admit(waiting[0], tnow):
                    break  # the head waits for slots to free up
                if waiting[0].precision != "f64":
                    self._groups = None
                waiting.pop(0)
            self.stats["admit_s"] += time.perf_counter() - ta
            if any(meta["done"] < meta["steps_max"] for _, meta in self.active):
                self._tick()
                self._retire(now)
            elif self.active:
                # everything launched: wait for the oldest tick, then retire
                t_dev = time.perf_counter()
                if self._tick_events:
                    self._tick_events.pop(0).synchronize()
                self.stats["device_wait_s"] += time.perf_counter() - t_dev
                self._retire(now)
            elif self.active64:
                time.sleep(0.0005)
                self._retire(now)
            elif qi < len(pending) and not waiting:
                wait = pending[qi].arrival - now()
                if wait > 0:
                    time.sleep(min(wait, 0.01))
        for st in self.streams64:
            st.synchronize()
        return pending


def _work_estimate(req):
    """Layer-steps a request asks for, from its description alone."""
    if req.precision == "f64":
        return float(len(req.junctions)) * req.total_time / req.time_step * np.mean(
            [j.layerNo for j in req.junctions])
    steps = np.broadcast_to(np.asarray(req.n_steps, dtype=np.float64), (req.spec.n,))
    return float(np.sum(steps * req.spec.n_layers))


# --------------------------------------------------------------------------
# Traces
# --------------------------------------------------------------------------
def make_trace(n_requests, rate_hz=200.0, seed=7, min_solves=64, max_solves=16384, t_min=2e-9, t_max=40e-9,
               dt=1e-13, f64_fraction=0.0):
    """Poisson arrivals at rate_hz; each request holds log-uniform
    64..16,384 solves of one kind: PIMM-style 2-layer RK4 (T = 0), p-bit
    1-layer Euler-Heun at 300 K, or uneven 1-4-layer spin-diode RK4
    (sweeps.pimm_config / pbit_config / vsd_config), with one duration in
    [t_min, t_max] per solve.  A fraction of requests is FP64 plain (64
    solves, 2 ns, 2-layer RK4 Junction objects)."""
    from . import sweeps
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate_hz, size=n_requests))
    reqs = []
    for k in range(n_requests):
        if rng.random() < f64_fraction:
            reqs.append(_f64_request(rng, t[k], k))
            continue
        n = int(np.exp(rng.uniform(np.log(min_solves), np.log(max_solves))))
        kind = int(rng.integers(0, 3))
        if kind == 0:
            sp, _ = sweeps.pimm_config(n_h=n, n_draw=1, seed=int(rng.integers(1 << 30)), dt=dt)
            solver = SolverMode.RK4
        elif kind == 1:
            sp, _, _ = sweeps.pbit_config(n_j=1, n_per=n, seed=int(rng.integers(1 << 30)), dt=dt)
            solver = SolverMode.EulerHeun
        else:
            sp, _ = sweeps.vsd_config(n_f=1, n_h=n, seed=int(rng.integers(1 << 30)), dt=dt)
            solver = SolverMode.RK4
        steps = (rng.uniform(t_min, t_max, size=n) / dt).astype(np.int64)
        reqs.append(Request(spec=sp, n_steps=steps, solver=solver, arrival=float(t[k]),
                            tag=["pimm", "pbit", "vsd"][kind], red_every=10 if kind == 2 else 0))
    return reqs


def _f64_request(rng, arrival, k):
    import cmtj_gb300 as cm
    from .sweeps import MTJ_DEMAG
    js = []
    for q in range(64):
        d = [cm.CVector(*MTJ_DEMAG[0:3]), cm.CVector(*MTJ_DEMAG[3:6]), cm.CVector(*MTJ_DEMAG[6:9])]
        a = cm.Layer("free", cm.CVector(0, 0, 1), cm.CVector(0, 0, 1), 1.2, 1.5e-9, 1e-16, d, 0.01)
        b = cm.Layer("ref", cm.CVector(0, 0, 1), cm.CVector(0, 0, 1), 1.5, 2e-9, 1e-16, d, 0.01)
        j = cm.Junction([a, b], 100, 200)
        j.setLayerAnisotropyDriver("free", cm.constantDriver(float(rng.uniform(1e5, 6e5))))
        j.setLayerAnisotropyDriver("ref", cm.constantDriver(1e6))
        j.setLayerExternalFieldDriver("all", cm.AxialDriver(float(rng.uniform(-6e5, 6e5)), 0, 0))
        js.append(j)
    return Request(precision="f64", junctions=js, total_time=2e-9, arrival=float(arrival), tag="f64")


def summary(reqs, wall_s):
    lat = np.array([r.latency for r in reqs if r.latency is not None])
    solves = sum(r.n for r in reqs)
    ls = sum(r.layer_steps for r in reqs)
    return {"requests": len(reqs), "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "solves_per_s": solves / wall_s,
            "layer_steps_per_s": ls / wall_s, "wall_s": wall_s}

"""Buffered 1/f^alpha noise: the `noise` submodule of the reference
(python/cmtj.cpp:448-462, core/noise.hpp:138-308).

A buffer of n samples is n white Gaussian draws coloured by the 1/f^alpha
filter of BufferedAlphaNoise::fillBuffer (noise.hpp:186-225); it is filled
on the GPU by cmtj_alpha_noise_f32 (csrc/alpha_noise.cu), which follows the
reference's algorithm exactly, including its float filter weights and the
two halved and dropped spectral bins.  The white draws come from a Philox
stream keyed by `seed` (the reference draws from an unseeded mt19937), so
buffers agree with the reference's in distribution, and given the same
white draws they agree sample by sample.

Layers that call setAlphaNoise get one such buffer per axis per run,
generated on the device before the run (junction.hpp:1912-1916) and read
by the Euler-Heun and Heun runners as getOneFVector (1130-1136).
"""
import numpy as np

from . import _abi
from .core import Axis, CVector, _new_seed

# scratch held by one generator call (rows are processed as many at a time
# as fit)
SCRATCH_BUDGET = 1 << 30


def specs_array(rows):
    """cmtj_alpha_noise_t records from (alpha, std, seed, counter,
    component) tuples."""
    a = np.zeros(len(rows), dtype=_abi.ALPHA_NOISE_DTYPE)
    for k, (alpha, std, seed, counter, comp) in enumerate(rows):
        a[k]["alpha"] = alpha
        a[k]["std"] = std
        a[k]["seed_lo"] = seed & 0xFFFFFFFF
        a[k]["seed_hi"] = (seed >> 32) & 0xFFFFFFFF
        a[k]["counter"] = counter
        a[k]["component"] = comp
    return a


def device_buffers(specs, n, white=None, stream=None):
    """Fill len(specs) buffers of n samples on the GPU; returns the device
    tensor [rows, n] (float32).  `white` (host [rows, n] float32) replaces
    the Philox white draws."""
    from . import engine
    t = engine.torch()
    lib = engine.require_gpu()
    rows = len(specs)
    out = t.empty((max(rows, 1), n), dtype=t.float32, device="cuda")
    if rows == 0:
        return out[:0]
    per_row = int(lib.cmtj_alpha_noise_scratch_bytes(n))
    if per_row == 0:
        raise ValueError("alpha-noise buffer of %d samples is outside [1, %d]" % (n, _abi.ALPHA_MAX_LEN))
    chunk = max(1, min(rows, SCRATCH_BUDGET // per_row))
    scratch = t.empty(chunk * per_row, dtype=t.uint8, device="cuda")
    d_specs = engine.to_device(specs)
    d_white = None
    if white is not None:
        d_white = t.from_numpy(np.ascontiguousarray(white, dtype=np.float32).reshape(rows, n)).cuda()
    rc = lib.cmtj_alpha_noise_f32(engine.ptr(d_specs), rows, n, engine.ptr(d_white), engine.ptr(out),
                                  engine.ptr(scratch), chunk * per_row, engine.stream_ptr(stream))
    _abi.check(rc, lib)
    if stream is not None:
        # the temporaries were allocated on the current stream: keep them
        # until the generator has run on `stream`
        stream.synchronize()
    return out


def fill_buffers(specs, n, white=None):
    """As device_buffers, copied to the host ([rows, n] float32)."""
    return device_buffers(specs, n, white).cpu().numpy()


class BufferedAlphaNoise:
    """BufferedAlphaNoise(bufferSize, alpha, std, scale) (noise.hpp:138-260):
    tick() returns scale times the next buffered sample, refilling the
    buffer (new white draws) each time it wraps."""

    def __init__(self, bufferSize, alpha, std, scale, _seed=None, _component=0):
        self.bufferSize = int(bufferSize)
        self.alpha = float(alpha)
        self.std = float(std)
        self.scale = float(scale)
        self.seed = _new_seed() if _seed is None else int(_seed)
        self.component = int(_component)
        self._counter = 0
        self._index = 0
        self._result = None

    def fillBuffer(self):
        spec = specs_array([(self.alpha, self.std, self.seed, self._counter, self.component)])
        self._result = fill_buffers(spec, self.bufferSize)[0]
        self._counter += self.bufferSize

    def getFullBuffer(self):
        return None if self._result is None else self._result.copy()

    def tick(self):
        if self._index == 0:
            self.fillBuffer()
        ret = float(self._result[self._index])
        self._index = (self._index + 1) % self.bufferSize
        return self.scale * ret


class _NullTicker:
    def tick(self):
        return 0.0


class VectorAlphaNoise:
    """VectorAlphaNoise(bufferSize, alpha, std, scale, axis=Axis.all)
    (noise.hpp:262-308): one buffered component per axis (all three for
    Axis.all, whose sample vector is normalised), times `scale`.  The
    components share one seed and take normals 0, 1, 2 of each Philox draw,
    as the solver's per-layer buffers do; each advances on its own ticks."""

    def __init__(self, bufferSize, alpha, std, scale, axis=Axis.all):
        axis = Axis(int(axis))
        if axis == Axis.none:
            raise RuntimeError("Invalid axis specified: %d" % int(axis))
        self.scale = float(scale)
        self.axis = axis
        self.normalized = axis == Axis.all
        self.seed = _new_seed()
        active = (0, 1, 2) if axis == Axis.all else (int(axis),)
        self.components = [BufferedAlphaNoise(bufferSize, alpha, std, 1.0, self.seed, c) if c in active
                           else _NullTicker() for c in (0, 1, 2)]
        self.prevSample = CVector()
        self.currentSample = CVector()

    def tickVector(self):
        self.prevSample = self.currentSample
        self.currentSample = CVector(*[c.tick() for c in self.components])
        if self.normalized:
            self.currentSample.normalize()
        return self.currentSample * self.scale

    def tick(self):
        return self.components[0].tick() * self.scale

    def getPrevSample(self):
        return self.prevSample

    def getScale(self):
        return self.scale

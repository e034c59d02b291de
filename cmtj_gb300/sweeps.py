"""Vectorised batch builders for parameter sweeps (the work of
cmtj/utils/procedures.py PIMM_procedure and VSD_procedure, and of the
reference's process-pool `distribute`, expressed as one device batch).

Each builder returns a BatchSpec filled with numpy arrays (no per-junction
Python objects) plus its step count(s)."""
import numpy as np

from .batch import (FEAT_WAVES, MAX_WAVES, TGT_HX, TGT_HY, TGT_HZ, TGT_I, WAVE_DTYPE, BatchSpec, F32_STT,
                    q64_frac, step_window)
from .core import MR_CLASSIC

MTJ_DEMAG = np.array([0.0024, 0, 0, 0, 0.0024, 0, 0, 0, 0.9952])


def mtj_2layer(n, K_free, J, H, seed=0):
    """n copies of the 2-layer MTJ of the R(H) sweep: free Ms 1.2 T,
    t 1.5 nm, reference Ms 1.5 T, Ku 1e6 J/m^3, t 2 nm, both along z,
    alpha 0.01, demag diag(0.0024, 0.0024, 0.9952), surface 1e-16 m^2,
    classic MR Rp 100, Rap 200.  K_free [n], J [n] (IEC, J/m^2), H [n,3]
    (both layers)."""
    sp = BatchSpec.empty(n)
    sp.n_layers[:] = 2
    sp.Ms[:, 0], sp.Ms[:, 1] = 1.2, 1.5
    sp.thickness[:, 0], sp.thickness[:, 1] = 1.5e-9, 2e-9
    sp.surface[:, :2] = 1e-16
    sp.alpha[:, :2] = 0.01
    sp.demag[:, :2] = MTJ_DEMAG
    sp.K[:, 0] = K_free
    sp.K[:, 1] = 1e6
    # setIECDriver("free", "ref"): free gets the top coupling, ref the bottom
    sp.Jt[:, 0] = J
    sp.Jb[:, 1] = J
    sp.Hc[:, 0] = H
    sp.Hc[:, 1] = H
    sp.mr_mode[:] = MR_CLASSIC
    sp.Rp[:], sp.Rap[:] = 100.0, 200.0
    mst = sp.Ms[:, :2] * sp.thickness[:, :2]
    sp.mix_w[:, :2] = mst / mst.sum(axis=1, keepdims=True)
    sp.seed[:, :2] = np.random.default_rng(seed).integers(0, 2 ** 63, size=(n, 2), dtype=np.uint64)
    return sp


def pimm_config(n_h=512, n_draw=512, seed=1, dt=1e-13, total=5e-9, h_max=600e3, pulse=1e3, pulse_len=1e-12):
    """Batched PIMM: n_h x n_draw 2-layer junctions, Ku(free) ~ U[1e5, 6e5],
    J ~ U[-1e-4, 1e-4] (seeded), H on an n_h-point grid over +-h_max along x,
    a pulse_len Oersted step of `pulse` A/m along x on both layers
    (PIMM_procedure's excitation, procedures.py:93-111), then free ringing;
    total time `total` at step dt.  Returns (spec, n_steps)."""
    rng = np.random.default_rng(seed)
    n = n_h * n_draw
    Hgrid = np.linspace(-h_max, h_max, n_h)
    H = np.zeros((n, 3))
    H[:, 0] = np.repeat(Hgrid, n_draw)
    K = rng.uniform(1e5, 6e5, size=n)
    J = rng.uniform(-1e-4, 1e-4, size=n)
    sp = mtj_2layer(n, K, J, H, seed=seed)
    w = np.zeros((n, MAX_WAVES), dtype=WAVE_DTYPE)
    w["target"][:, 0] = TGT_HX
    w["kind"][:, 0] = 3  # step
    w["amp"][:, 0] = pulse
    on, off = step_window(0.0, pulse_len, dt, None)
    w["on"][:, 0] = on
    w["off"][:, 0] = off
    w["layer_mask"][:, 0] = 0b11
    sp.wave_table = w
    sp.wave_count = np.ones(n, dtype=np.int64)
    return sp, int(total / dt)


def vsd_config(n_f=128, n_h=1024, seed=3, dt=1e-13, t_min=5e-9, t_max=50e-9, amp=500.0, h_max=500e3):
    """Uneven spin-diode scan: n_f frequencies (1-20 GHz) x n_h fields over
    +-h_max along x; 1-4 layer stacks in a 1:2:2:1 ratio with Ms ~ U[0.8, 1.6]
    T, Ku ~ U[1e5, 8e5] along random in-plane or +-z axes, alpha ~ U[0.005,
    0.03]; a sine Oersted field `amp` A/m along y at the scan frequency on
    every layer (VSD_procedure, procedures.py:241-258); durations U[t_min,
    t_max].  R: classic for 1-2 layers (1-layer reference along x), series Rx
    for 3-4 layers.  I(t) = sin(2 pi f t) drives the on-device <I R>.
    Returns (spec, n_steps[n])."""
    from .batch import MR_SERIES
    rng = np.random.default_rng(seed)
    n = n_f * n_h
    freqs = np.linspace(1e9, 20e9, n_f)
    f = np.tile(freqs, n_h)
    Hx = np.repeat(np.linspace(-h_max, h_max, n_h), n_f)
    L = rng.choice(np.array([1, 2, 2, 3, 3, 4]), size=n)
    sp = BatchSpec.empty(n)
    sp.n_layers[:] = L
    sp.Ms[:] = rng.uniform(0.8, 1.6, size=(n, 4))
    sp.thickness[:] = rng.uniform(1e-9, 2e-9, size=(n, 4))
    sp.surface[:] = 1e-16
    sp.alpha[:] = rng.uniform(0.005, 0.03, size=(n, 4))
    sp.K[:] = rng.uniform(1e5, 8e5, size=(n, 4))
    inplane = rng.random((n, 4)) < 0.5
    phi = rng.uniform(0, 2 * np.pi, size=(n, 4))
    sgn = np.where(rng.random((n, 4)) < 0.5, -1.0, 1.0)
    sp.anis[:] = np.where(inplane[..., None], np.stack([np.cos(phi), np.sin(phi), 0 * phi], -1),
                          np.stack([0 * phi, 0 * phi, sgn], -1))
    sp.m0[:] = sp.anis
    sp.demag[:] = [0.0, 0, 0, 0, 0.0, 0, 0, 0, 1.0]
    J = rng.uniform(-1e-4, 1e-4, size=(n, 3))
    sp.Jt[:, :3] = J
    sp.Jb[:, 1:4] = J
    sp.Hc[:, :, 0] = Hx[:, None]
    sp.mr_mode[:] = np.where(L <= 2, MR_CLASSIC, MR_SERIES)
    sp.Rp[:], sp.Rap[:] = 100.0, 200.0
    sp.ref[:, 0] = [1.0, 0, 0]
    sp.strip[:, 0, :] = 100.0   # Rx0
    sp.strip[:, 2, :] = -0.24   # AMR_X
    sp.strip[:, 4, :] = -0.46   # SMR_X
    sp.vsd_freq[:] = f
    w = np.zeros((n, MAX_WAVES), dtype=WAVE_DTYPE)
    w["target"][:, 0] = TGT_HY
    w["kind"][:, 0] = 2  # sine
    w["amp"][:, 0] = amp
    w["dph"][:, 0] = q64_frac(f * dt)
    w["dph_half"][:, 0] = q64_frac(f * dt * 0.5)
    w["layer_mask"][:, 0] = (1 << L) - 1
    sp.wave_table = w
    sp.wave_count = np.ones(n, dtype=np.int64)
    sp.seed[:] = rng.integers(0, 2 ** 63, size=(n, 4), dtype=np.uint64)
    n_steps = (rng.uniform(t_min, t_max, size=n) / dt).astype(np.int64)
    return sp, n_steps


def pbit_config(n_j=64, n_per=16384, seed=2, dt=1e-13, t_min=5e-9, t_max=20e-9, j_max=5e11, T=300.0,
                polarisation=0.6, pulse_len=1e-9):
    """Stochastic p-bit: n_j current densities (0..j_max A/m^2) x n_per
    single-layer STT junctions: Ms 1.0 T, Ku 2.5e5 J/m^3 along z, t 1.2 nm,
    surface 7e-17 m^2, alpha 0.02, T = 300 K, Slonczewski STT with
    polarisation 0.6, lambda 1, beta 0, reference -z, zero demag; a 1 ns
    current step from t = 0; m from +z; durations U[t_min, t_max].
    Returns (spec, n_steps[n])."""
    rng = np.random.default_rng(seed)
    n = n_j * n_per
    jd = np.repeat(np.linspace(0, j_max, n_j), n_per)
    sp = BatchSpec.empty(n)
    sp.n_layers[:] = 1
    sp.Ms[:, 0] = 1.0
    sp.thickness[:, 0] = 1.2e-9
    sp.surface[:, 0] = 7e-17
    sp.alpha[:, 0] = 0.02
    sp.K[:, 0] = 2.5e5
    sp.T[:, 0] = T
    sp.temperature[:, 0] = True
    sp.flags[:, 0] = F32_STT
    sp.stt_p[:, 0] = polarisation
    sp.stt_l[:, 0] = 1.0
    sp.ref[:, 0] = [0, 0, -1.0]
    sp.ref_type[:, 0] = 1
    sp.mr_mode[:] = MR_CLASSIC
    sp.Rp[:], sp.Rap[:] = 100.0, 200.0
    w = np.zeros((n, MAX_WAVES), dtype=WAVE_DTYPE)
    w["target"][:, 0] = TGT_I
    w["kind"][:, 0] = 3
    w["amp"][:, 0] = jd
    on, off = step_window(0.0, pulse_len, dt, None)
    w["on"][:, 0] = on
    w["off"][:, 0] = off
    w["layer_mask"][:, 0] = 1
    sp.wave_table = w
    sp.wave_count = np.ones(n, dtype=np.int64)
    sp.seed[:, 0] = rng.integers(0, 2 ** 63, size=n, dtype=np.uint64)
    n_steps = (rng.uniform(t_min, t_max, size=n) / dt).astype(np.int64)
    return sp, n_steps, jd

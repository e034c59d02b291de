// FP64 plain form, fixed-step solvers (RK4, Euler-Heun, Heun): one lane per
// layer.
//
// The fixed-step runners of Junction::runSimulation (core/junction.hpp:
// 1668-1815) step every layer of a junction from the magnetisations its
// neighbours had at the start of the step (Heun's corrector: from their
// predictions), so the layers of one step are independent of each other.
// Here each layer runs on its own lane of a G-lane group (G = 1, 2, 4 or 8,
// at least the junction's layer count); the neighbours come from the
// adjacent lanes by warp shuffle, and every lane evaluates the expressions
// of plain_f64.cuh in the same order as the one-thread Dormand-Prince
// kernel does, so the results do not depend on the layout.  The serial
// chain of a step is one layer's instead of n layers'.
//
// The chain is latency-bound (one warp per SM issues far below the FP64
// pipe's rate), so a block is one warp of 32/G junctions and blocks spread
// over the SMs.  Driver slots whose driver is constant are read directly
// (slot mask per lane), and the four RK4 stages run as a rolled loop so the
// field code is compiled once per kernel.
//
// This unit is compiled with --fmad=false like plain_f64.cu.
#include "plain_f64.cuh"
#include "plain_lanes.h"

using namespace cmtjd;

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ D3 shfl3(const D3 &v, int src) {
  return d3(__shfl_sync(kFull, v.x, src), __shfl_sync(kFull, v.y, src), __shfl_sync(kFull, v.z, src));
}

// The columns of one layer in a log row (logLayerParams, junction.hpp:
// 1580-1636): the energy-log side values, then m.
__device__ __forceinline__ void layer_cols(double *r, const Side &s, const D3 &m, bool energies) {
  int col = 0;
  if (energies) {
    r[col++] = s.K;
    r[col++] = s.K2;
    r[col++] = s.Jb;
    r[col++] = s.Jt;
    r[col++] = s.I;
    const D3 v[7] = {s.Hext, s.Hiec, s.Hanis, s.Hdemag, zero3(), s.Hfl, s.Hdl};
#pragma unroll
    for (int q = 0; q < 7; ++q) {
      r[col++] = v[q].x;
      r[col++] = v[q].y;
      r[col++] = v[q].z;
    }
  }
  r[col++] = m.x;
  r[col++] = m.y;
  r[col] = m.z;
}

template <int SOLVER>
__global__ void __launch_bounds__(32)
    k_plain_lanes(const cmtj_junction_t *__restrict__ junctions, int32_t n_junctions,
                  const cmtj_layer_t *__restrict__ params, cmtj_layer_t *layers, const double *__restrict__ tables,
                  cmtj_sim_params_t p, int G, double *__restrict__ log, uint32_t *__restrict__ status) {
  // `params` and `layers` address the same records: every field but mag is
  // read through `params`, mag is read and written through `layers` only.
  const int lane = threadIdx.x;
  const int l = lane & (G - 1);
  const int lead = lane - l;
  const int j = blockIdx.x * (32 / G) + lane / G;
  const bool have = j < n_junctions;
  int n = 0;
  int64_t off = 0;
  uint32_t code = CMTJ_STATUS_OK;
  int mr_mode = CMTJ_MR_NONE;
  if (have) {
    n = junctions[j].n_layers;
    off = junctions[j].layer_offset;
    mr_mode = junctions[j].mr_mode;
    if (n < 1 || n > G) {
      code = CMTJ_STATUS_BAD_INPUT;
      n = 0;
    }
  }
  bool run = n > 0;  // the same on every lane of a junction
  const bool mine = run && l < n;
  const cmtj_layer_t &L = params[mine ? off + l : 0];
  const double dt = p.time_step;
  const bool energies = p.calculate_energies != 0;
  const cmtj_constants_t c = p.c;
  const int width = energies ? CMTJ_ENERGY_COLS : 3;
  D3 mag = zero3();
  uint32_t dyn = 0;
  Side side;
  side.K = side.K2 = side.Jb = side.Jt = side.I = 0.0;
  side.Hext = side.Hiec = side.Hanis = side.Hdemag = side.Hfl = side.Hdl = zero3();
  if (mine) {
    mag = load3(layers[off + l].mag);
    dyn = dynamic_slots(L);
  }
  const int below_src = lead + (l > 0 ? l - 1 : 0);
  const int above_src = lead + (l + 1 < G ? l + 1 : l);
  double *out = have ? log + (size_t)j * p.n_log * p.log_width : nullptr;
  uint32_t row = 0;

  for (uint32_t i = 0; i < p.total_iterations; ++i) {
    if (!__any_sync(kFull, run)) break;
    const double t = (double)i * dt;
    const bool step = mine && run;
    // neighbours at the start of the step; zero beyond the stack's ends
    D3 below = shfl3(mag, below_src), above = shfl3(mag, above_src);
    if (l == 0) below = zero3();
    if (l >= n - 1) above = zero3();

    if (SOLVER == CMTJ_RK4) {
      // Layer::rk4_step (1017-1041); neighbours frozen for all four stages
      // (runMultiLayerSolver, 1680-1707)
      D3 next = mag;
      bool nan = false;
      if (step) {
        D3 k = zero3(), acc = zero3();
#pragma unroll 1
        for (int s = 0; s < 4; ++s) {
          const double ts = s == 0 ? t : (s == 3 ? t + dt : t + 0.5 * dt);
          const D3 mi = s == 0 ? mag : (s == 3 ? mag + k : mag + k * 0.5);
          const DriverCtx dc = {tables, i, s == 0 ? 0 : (s == 3 ? 2 : 1)};
          k = rhs(L, c, ts, mi, below, above, dc, (s == 3 && energies) ? &side : nullptr, nullptr, dyn) * dt;
          acc = s == 0 ? k : acc + (s == 3 ? k : k * 2.0);
        }
        next = normalized(mag + acc / 6.0);
        nan = isnan(next.x);
      }
      // rk4_step throws at the first layer whose m is NaN: the layers below
      // it keep this step's update, the layers above it do not
      const unsigned group = (G == 32 ? kFull : ((1u << G) - 1u)) << lead;
      const unsigned bad = __ballot_sync(kFull, nan) & group;
      if (bad) {
        const int first = __ffs(bad) - 1 - lead;
        if (step && l <= first) mag = next;
        if (run) code = CMTJ_STATUS_NAN;
        run = false;
      } else if (step) {
        mag = next;
      }
    } else if (SOLVER == CMTJ_EULER_HEUN) {
      // eulerHeunSolverStep (1709-1754)
      if (step) {
        const DriverCtx d0 = {tables, i, 0};
        const D3 dW = langevin(L, c, t, i, d0, dyn);
        const D3 f = rhs(L, c, t, mag, below, above, d0, energies ? &side : nullptr, nullptr, dyn);
        const D3 g = stoch_torque(L, c, mag, dW);
        const D3 mNext = mag + g * sqrt(dt);
        const D3 g2 = stoch_torque(L, c, mNext, dW);
        mag = normalized(mag + f * dt + smul(0.5, g + g2) * sqrt(dt));
      }
    } else {
      // heunSolverStep (1756-1815): the corrector sees the neighbours'
      // predictions
      D3 fn = zero3(), gn = zero3(), dW = zero3(), pred = zero3();
      if (step) {
        const DriverCtx d0 = {tables, i, 0};
        fn = rhs(L, c, t, mag, below, above, d0, nullptr, nullptr, dyn);
        dW = langevin(L, c, t, i, d0, dyn);
        gn = stoch_torque(L, c, mag, dW);
        pred = mag + fn * dt + gn * sqrt(dt);
      }
      D3 pb = shfl3(pred, below_src), pa = shfl3(pred, above_src);
      if (l == 0) pb = zero3();
      if (l >= n - 1) pa = zero3();
      if (step) {
        const DriverCtx d2 = {tables, i, 2};
        const D3 f2 = rhs(L, c, t + dt, pred, pb, pa, d2, energies ? &side : nullptr, nullptr, dyn);
        const D3 g2 = stoch_torque(L, c, pred, dW);
        mag = mag + smul(0.5 * dt, fn + f2) + smul(0.5, gn + g2) * sqrt(dt);
        mag = normalized(mag);
      }
    }

    if (!(i % p.write_every)) {
      // magnetoresistance (calculateMagnetoresistance 1865-1867,
      // stripMagnetoResistance 1835-1857) from the layer lanes
      const D3 m1 = shfl3(mag, lead + (G > 1 ? 1 : 0));
      double inv_x = 0.0, inv_y = 0.0;
      if (mine && mr_mode == CMTJ_MR_STRIP) {
        const cmtj_junction_t &J = junctions[j];
        const double Rx = J.Rx0[l] + J.AMR_X[l] * (mag.x * mag.x) + J.SMR_X[l] * (mag.y * mag.y);
        const double Ry = J.Ry0[l] + 0.5 * J.AHE[l] * mag.z + (J.AMR_Y[l] + J.SMR_Y[l]) * mag.x * mag.y;
        inv_x = 1. / Rx;
        inv_y = 1. / Ry;
      }
      double Rx_acc = 0.0, Ry_acc = 0.0;
      for (int q = 0; q < G; ++q) {
        const double a = __shfl_sync(kFull, inv_x, lead + q), b = __shfl_sync(kFull, inv_y, lead + q);
        if (q < n) {
          Rx_acc = Rx_acc + a;
          Ry_acc = Ry_acc + b;
        }
      }
      if (run) {
        double *r = out + (size_t)row * p.log_width;
        if (mine) layer_cols(r + l * width, side, mag, energies);
        if (l == 0) {
          const cmtj_junction_t &J = junctions[j];
          double r0 = 0.0, r1 = 0.0;
          if (mr_mode == CMTJ_MR_CLASSIC) {
            const double cosT = n == 1 ? dot(mag, load3(L.ref)) : dot(mag, m1);
            r0 = J.Rp + (((J.Rap - J.Rp) / 2.0) * (1.0 - cosT));
          } else if (mr_mode == CMTJ_MR_STRIP) {
            r0 = 1 / Rx_acc;
            r1 = 1 / Ry_acc;
          }
          double *rr = r + n * width;
          rr[0] = r0;
          rr[1] = r1;
          rr[2] = 0.0;
          rr[3] = t;
        }
        ++row;
      }
    }
  }
  if (mine) {
    layers[off + l].mag[0] = mag.x;
    layers[off + l].mag[1] = mag.y;
    layers[off + l].mag[2] = mag.z;
  }
  if (have && l == 0) {
    status[2 * j] = code;
    status[2 * j + 1] = row;
  }
}

}  // namespace

namespace cmtjd {

int plain_lanes_group(int max_layers) {
  if (max_layers <= 1) return max_layers == 1 ? 1 : CMTJ_MAX_LAYERS;
  if (max_layers <= 2) return 2;
  if (max_layers <= 4) return 4;
  return CMTJ_MAX_LAYERS;
}

cudaError_t plain_lanes_launch(const cmtj_junction_t *d_junctions, int32_t n_junctions, cmtj_layer_t *d_layers,
                               const double *d_tables, const cmtj_sim_params_t &p, double *d_log, uint32_t *d_status,
                               cudaStream_t stream) {
  const int G = plain_lanes_group(p.max_layers);
  const int per_block = 32 / G;
  const int blocks = (n_junctions + per_block - 1) / per_block;
  if (p.solver == CMTJ_RK4)
    k_plain_lanes<CMTJ_RK4><<<blocks, 32, 0, stream>>>(d_junctions, n_junctions, d_layers, d_layers, d_tables, p, G,
                                                       d_log, d_status);
  else if (p.solver == CMTJ_EULER_HEUN)
    k_plain_lanes<CMTJ_EULER_HEUN><<<blocks, 32, 0, stream>>>(d_junctions, n_junctions, d_layers, d_layers, d_tables,
                                                              p, G, d_log, d_status);
  else
    k_plain_lanes<CMTJ_HEUN><<<blocks, 32, 0, stream>>>(d_junctions, n_junctions, d_layers, d_layers, d_tables, p, G,
                                                        d_log, d_status);
  return cudaGetLastError();
}

}  // namespace cmtjd

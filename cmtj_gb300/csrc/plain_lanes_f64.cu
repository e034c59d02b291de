// FP64 plain form, fixed-step solvers (RK4, Euler-Heun, Heun): layers
// side by side on lanes.
//
// The fixed-step runners of Junction::runSimulation (core/junction.hpp:
// 1668-1815) step every layer of a junction from the magnetisations its
// neighbours had at the start of the step (Heun's corrector: from their
// predictions), so the layers of one step are independent of each other.
// Here each layer runs on its own lane (V = D3) or on its own quad of lanes,
// one vector component per lane (V = C3, lane3.cuh), within a group of
// G layer slots (G = 1, 2, 4 or 8, at least the junction's layer count).
// The neighbours come from the adjacent layer slots by warp shuffle, and
// every lane evaluates the expressions of plain_f64.cuh in the same order
// as the one-thread Dormand-Prince kernel does, so the results do not
// depend on the layout.  The serial chain of a step is one layer's instead
// of n layers'.
//
// The chain is latency-bound: a warp FP64 instruction occupies the SM
// sub-partition's FP64 unit for the same time with one active lane or 32,
// so idle lanes cost nothing and the quad layout, with about 2.5x fewer
// instructions per step, is the faster one until the batch fills the GPU.
// A block is one warp; blocks spread over the SMs.  Driver slots whose
// driver is constant are read directly (slot mask per lane), and the four
// RK4 stages run as a rolled loop so the field code is compiled once per
// kernel.
//
// This unit is compiled with --fmad=false like plain_f64.cu.
#include "lane3.cuh"
#include "plain_f64.cuh"
#include "plain_lanes.h"

using namespace cmtjd;

namespace {

constexpr unsigned kFull = 0xffffffffu;

// The columns of one layer in a log row (logLayerParams, junction.hpp:
// 1580-1636): the energy-log side values, then m.
template <class V>
__device__ __forceinline__ void layer_cols(double *r, const SideT<V> &s, const V &m, bool energies) {
  double *mcol = r;
  if (energies) {
    if (scalar_owner(m)) {
      r[0] = s.K;
      r[1] = s.K2;
      r[2] = s.Jb;
      r[3] = s.Jt;
      r[4] = s.I;
    }
    store3(r + 5, s.Hext);
    store3(r + 8, s.Hiec);
    store3(r + 11, s.Hanis);
    store3(r + 14, s.Hdemag);
    store3(r + 17, V::zero());
    store3(r + 20, s.Hfl);
    store3(r + 23, s.Hdl);
    mcol = r + 26;
  }
  store3(mcol, m);
}

// The whole run of the warp's junctions.  DYN = false when no layer of the
// warp has a time-dependent driver slot: every slot then reads its
// constantValue, a loop invariant.
template <int SOLVER, class V, bool DYN>
__device__ __forceinline__ void run_lanes(const cmtj_junction_t *__restrict__ junctions, int32_t n_junctions,
                                          const cmtj_layer_t *__restrict__ params, cmtj_layer_t *layers,
                                          const double *__restrict__ tables, const cmtj_sim_params_t &p, int G,
                                          double *__restrict__ log, uint32_t *__restrict__ status) {
  constexpr int P = V::kLanes;  // lanes per layer
  const int span = G * P;       // lanes per junction (<= 32)
  const int lane = threadIdx.x;
  const int jl = lane % span;
  const int l = jl / P;  // layer slot of this lane
  const int lead = lane - jl;
  const int j = blockIdx.x * (32 / span) + lane / span;
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
  V mag = V::zero();
  uint32_t dyn = 0;
  SideT<V> side;
  side.K = side.K2 = side.Jb = side.Jt = side.I = 0.0;
  side.Hext = side.Hiec = side.Hanis = side.Hdemag = side.Hfl = side.Hdl = V::zero();
  if (mine) {
    mag = V::load(layers[off + l].mag);
    if (DYN) dyn = dynamic_slots(L);
  }
  const int below_src = l > 0 ? lane - P : lane;
  const int above_src = l + 1 < G ? lane + P : lane;
  double *out = have ? log + (size_t)j * p.n_log * p.log_width : nullptr;
  uint32_t row = 0;

  for (uint32_t i = 0; i < p.total_iterations; ++i) {
    if (!__any_sync(kFull, run)) break;
    const double t = (double)i * dt;
    const bool step = mine && run;
    // neighbours at the start of the step; zero beyond the stack's ends
    V below = shfl_vec(mag, below_src), above = shfl_vec(mag, above_src);
    if (l == 0) below = V::zero();
    if (l >= n - 1) above = V::zero();

    if (SOLVER == CMTJ_RK4) {
      // Layer::rk4_step (1017-1041); neighbours frozen for all four stages
      // (runMultiLayerSolver, 1680-1707)
      V next = mag;
      bool nan = false;
      if (step) {
        V k = V::zero(), acc = V::zero();
#pragma unroll 1
        for (int s = 0; s < 4; ++s) {
          const double ts = s == 0 ? t : (s == 3 ? t + dt : t + 0.5 * dt);
          const V mi = s == 0 ? mag : (s == 3 ? mag + k : mag + k * 0.5);
          const DriverCtx dc = {tables, i, s == 0 ? 0 : (s == 3 ? 2 : 1)};
          k = rhs(L, c, ts, mi, below, above, dc, (s == 3 && energies) ? &side : nullptr, nullptr, dyn) * dt;
          acc = s == 0 ? k : acc + (s == 3 ? k : k * 2.0);
        }
        next = normalized(mag + acc / 6.0);
        nan = x_is_nan(next);
      }
      // rk4_step throws at the first layer whose m is NaN: the layers below
      // it keep this step's update, the layers above it do not
      const unsigned group = (span == 32 ? kFull : ((1u << span) - 1u)) << lead;
      const unsigned bad = __ballot_sync(kFull, nan) & group;
      if (bad) {
        const int first = (__ffs(bad) - 1 - lead) / P;
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
        const V dW = langevin<V>(L, c, t, i, d0, dyn);
        const V f = rhs(L, c, t, mag, below, above, d0, energies ? &side : nullptr, nullptr, dyn);
        const V g = stoch_torque(L, c, mag, dW);
        const V mNext = mag + g * sqrt(dt);
        const V g2 = stoch_torque(L, c, mNext, dW);
        mag = normalized(mag + f * dt + smul(0.5, g + g2) * sqrt(dt));
      }
    } else {
      // heunSolverStep (1756-1815): the corrector sees the neighbours'
      // predictions
      V fn = V::zero(), gn = V::zero(), dW = V::zero(), pred = V::zero();
      if (step) {
        const DriverCtx d0 = {tables, i, 0};
        fn = rhs(L, c, t, mag, below, above, d0, nullptr, nullptr, dyn);
        dW = langevin<V>(L, c, t, i, d0, dyn);
        gn = stoch_torque(L, c, mag, dW);
        pred = mag + fn * dt + gn * sqrt(dt);
      }
      V pb = shfl_vec(pred, below_src), pa = shfl_vec(pred, above_src);
      if (l == 0) pb = V::zero();
      if (l >= n - 1) pa = V::zero();
      if (step) {
        const DriverCtx d2 = {tables, i, 2};
        const V f2 = rhs(L, c, t + dt, pred, pb, pa, d2, energies ? &side : nullptr, nullptr, dyn);
        const V g2 = stoch_torque(L, c, pred, dW);
        mag = mag + smul(0.5 * dt, fn + f2) + smul(0.5, gn + g2) * sqrt(dt);
        mag = normalized(mag);
      }
    }

    if (!(i % p.write_every)) {
      // magnetoresistance (calculateMagnetoresistance 1865-1867,
      // stripMagnetoResistance 1835-1857) from the layer lanes; every lane
      // takes part in the shuffles
      const V m1 = shfl_vec(mag, l == 0 && G > 1 ? lane + P : lane);
      const double cos01 = dot(mag, m1);
      const double mx = comp_of(mag, 0), my = comp_of(mag, 1), mz = comp_of(mag, 2);
      double inv_x = 0.0, inv_y = 0.0;
      if (mine && mr_mode == CMTJ_MR_STRIP) {
        const cmtj_junction_t &J = junctions[j];
        const double Rx = J.Rx0[l] + J.AMR_X[l] * (mx * mx) + J.SMR_X[l] * (my * my);
        const double Ry = J.Ry0[l] + 0.5 * J.AHE[l] * mz + (J.AMR_Y[l] + J.SMR_Y[l]) * mx * my;
        inv_x = 1. / Rx;
        inv_y = 1. / Ry;
      }
      double Rx_acc = 0.0, Ry_acc = 0.0;
      for (int q = 0; q < G; ++q) {
        const double a = __shfl_sync(kFull, inv_x, lead + q * P), b = __shfl_sync(kFull, inv_y, lead + q * P);
        if (q < n) {
          Rx_acc = Rx_acc + a;
          Ry_acc = Ry_acc + b;
        }
      }
      const double cos_ref = (run && l == 0 && n == 1) ? dot(mag, V::load(L.ref)) : 0.0;
      if (run) {
        double *r = out + (size_t)row * p.log_width;
        if (mine) layer_cols(r + l * width, side, mag, energies);
        if (l == 0 && scalar_owner(mag)) {
          const cmtj_junction_t &J = junctions[j];
          double r0 = 0.0, r1 = 0.0;
          if (mr_mode == CMTJ_MR_CLASSIC) {
            const double cosT = n == 1 ? cos_ref : cos01;
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
  if (mine) store3(layers[off + l].mag, mag);
  if (have && jl == 0) {
    status[2 * j] = code;
    status[2 * j + 1] = row;
  }
}

template <int SOLVER, class V>
__global__ void __launch_bounds__(32)
    k_plain_lanes(const cmtj_junction_t *__restrict__ junctions, int32_t n_junctions,
                  const cmtj_layer_t *__restrict__ params, cmtj_layer_t *layers, const double *__restrict__ tables,
                  cmtj_sim_params_t p, int G, double *__restrict__ log, uint32_t *__restrict__ status) {
  // `params` and `layers` address the same records: every field but mag is
  // read through `params`, mag is read and written through `layers` only.
  const int span = G * V::kLanes;
  const int lane = threadIdx.x;
  const int l = (lane % span) / V::kLanes;
  const int j = blockIdx.x * (32 / span) + lane / span;
  bool varying = false;
  if (j < n_junctions) {
    const int n = junctions[j].n_layers;
    if (l < n && n <= G) varying = dynamic_slots(params[junctions[j].layer_offset + l]) != 0u;
  }
  if (__any_sync(kFull, varying))
    run_lanes<SOLVER, V, true>(junctions, n_junctions, params, layers, tables, p, G, log, status);
  else
    run_lanes<SOLVER, V, false>(junctions, n_junctions, params, layers, tables, p, G, log, status);
}

}  // namespace

namespace cmtjd {

int plain_lanes_group(int max_layers) {
  if (max_layers <= 1) return max_layers == 1 ? 1 : CMTJ_MAX_LAYERS;
  if (max_layers <= 2) return 2;
  if (max_layers <= 4) return 4;
  return CMTJ_MAX_LAYERS;
}

int plain_lanes_per_layer(const cmtj_sim_params_t &p, int32_t n_junctions, int sm_count) {
  if (p.lanes_per_layer == 1 || p.lanes_per_layer == 4) return p.lanes_per_layer;
  // quads while the batch holds at most two quad warps per SM sub-partition
  const long long quad_warps = ((long long)n_junctions * plain_lanes_group(p.max_layers) * 4 + 31) / 32;
  return quad_warps <= 2LL * 4 * sm_count ? 4 : 1;
}

template <class V>
static void launch_solver(int solver, int blocks, cudaStream_t stream, const cmtj_junction_t *d_junctions,
                          int32_t n_junctions, cmtj_layer_t *d_layers, const double *d_tables,
                          const cmtj_sim_params_t &p, int G, double *d_log, uint32_t *d_status) {
  if (solver == CMTJ_RK4)
    k_plain_lanes<CMTJ_RK4, V><<<blocks, 32, 0, stream>>>(d_junctions, n_junctions, d_layers, d_layers, d_tables, p,
                                                          G, d_log, d_status);
  else if (solver == CMTJ_EULER_HEUN)
    k_plain_lanes<CMTJ_EULER_HEUN, V><<<blocks, 32, 0, stream>>>(d_junctions, n_junctions, d_layers, d_layers,
                                                                 d_tables, p, G, d_log, d_status);
  else
    k_plain_lanes<CMTJ_HEUN, V><<<blocks, 32, 0, stream>>>(d_junctions, n_junctions, d_layers, d_layers, d_tables, p,
                                                           G, d_log, d_status);
}

cudaError_t plain_lanes_launch(const cmtj_junction_t *d_junctions, int32_t n_junctions, cmtj_layer_t *d_layers,
                               const double *d_tables, const cmtj_sim_params_t &p, double *d_log, uint32_t *d_status,
                               cudaStream_t stream) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int G = plain_lanes_group(p.max_layers);
  const int P = plain_lanes_per_layer(p, n_junctions, sms);
  const int per_block = 32 / (G * P);
  const int blocks = (n_junctions + per_block - 1) / per_block;
  if (P == 4)
    launch_solver<C3>(p.solver, blocks, stream, d_junctions, n_junctions, d_layers, d_tables, p, G, d_log, d_status);
  else
    launch_solver<D3>(p.solver, blocks, stream, d_junctions, n_junctions, d_layers, d_tables, p, G, d_log, d_status);
  return cudaGetLastError();
}

}  // namespace cmtjd

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
// A step is bound by its warp's FP64 instructions: on GB300 each holds the
// SM sub-partition's FP64 pipe for about 64 cycles whatever the lane mask,
// and a warp's independent FP64 instructions do not overlap.  Idle lanes
// therefore cost nothing, and the quad layout, with about 2.5x fewer FP64
// instructions per step, is the faster one until the batch fills the GPU.
// A block is one warp; blocks spread over the SMs.  Driver slots whose
// driver is constant are read directly (slot mask per lane), and the four
// RK4 stages run as a rolled loop so the field code is compiled once per
// kernel.  A warp whose layers are all field-only (RK4) runs a variant
// without the per-term branches, with the layer constants in registers and
// the IEC term formed once per step; its field and anisotropy drivers may
// be time-dependent.  Under CMTJ_ARITH_FUSED such a warp, if its
// anisotropy and IEC drivers are constant, runs lane_step_fused instead
// (plain_lanes.cuh): not the reference's bits, about a sixth of the FP64
// instructions.
//
// This unit is compiled with --fmad=false like plain_f64.cu; the fused step
// calls fma() explicitly.
#include "plain_lanes.cuh"
#include "plain_lanes.h"

using namespace cmtjd;

namespace {

// The whole run of the warp's junctions.  DYN = false when no layer of the
// warp has a time-dependent driver slot: every slot then reads its
// constantValue, a loop invariant.  FIELD (RK4): every layer of the warp is
// field-only (FieldOnly), with its constants in registers; with DYN, its
// field and anisotropy drivers may be time-dependent.  FUSED (with FIELD):
// the CMTJ_ARITH_FUSED step (lane_step_fused); only the field drivers may
// then be time-dependent.
template <int SOLVER, class V, bool DYN, bool FIELD, bool FUSED = false>
__device__ __forceinline__ void run_lanes(const cmtj_junction_t *__restrict__ junctions, int32_t n_junctions,
                                          const cmtj_layer_t *params, cmtj_layer_t *layers,
                                          const double *__restrict__ tables, const cmtj_sim_params_t &p, int G,
                                          double *__restrict__ log, uint32_t *__restrict__ status) {
  const LaneGeo g = lane_geo<V>(G);
  const int j = blockIdx.x * (32 / g.span) + g.lane / g.span;
  const bool have = j < n_junctions;
  int n = 0;
  int64_t off = 0;
  uint32_t code = CMTJ_STATUS_OK;
  int mr_mode = CMTJ_MR_NONE;
  double half_span = 0.0;
  if (have) {
    n = junctions[j].n_layers;
    off = junctions[j].layer_offset;
    mr_mode = junctions[j].mr_mode;
    half_span = classic_half_span(junctions[j]);
    if (n < 1 || n > G) {
      code = CMTJ_STATUS_BAD_INPUT;
      n = 0;
    }
  }
  bool run = n > 0;  // the same on every lane of a junction
  const bool mine = run && g.l < n;
  const cmtj_layer_t &L = params[mine ? off + g.l : 0];
  const double dt = p.time_step;
  const bool energies = p.calculate_energies != 0;
  const cmtj_constants_t c = p.c;
  V mag = V::zero();
  uint32_t dyn = 0;
  SideT<V> side;
  side.K = side.K2 = side.Jb = side.Jt = side.I = 0.0;
  side.Hext = side.Hiec = side.Hanis = side.Hdemag = side.Hfl = side.Hdl = V::zero();
  if (mine) {
    mag = V::load(layers[off + g.l].mag);
    if (DYN) dyn = dynamic_slots(L);
  }
  FieldOnly<V> fo;
  if constexpr (FIELD) {
    fo = field_only_load<V>(L, c);
    field_only_flags<V>(fo, dyn);
  }
  const bool edge_only = !__any_sync(kWarpAll, n >= 3);
  // a constant temperature gives the same thermal sigma at every step
  double sigma_run = -1.0;
  if constexpr (SOLVER != CMTJ_RK4) {
    if (mine && L.temperatureSet && !(dyn & (1u << CMTJ_SLOT_TEMPERATURE)))
      sigma_run = langevin_sigma(L, c, L.drv[CMTJ_SLOT_TEMPERATURE].constantValue);
  }
  Fused<V> fu;
  if (FUSED) fu = fused_load<V>(fo, dt);
  double *out = have ? log + (size_t)j * p.n_log * p.log_width : nullptr;
  uint32_t row = 0;

  for (uint32_t i = 0; i < p.total_iterations; ++i) {
    if (!__any_sync(kWarpAll, run)) break;
    const double t = (double)i * dt;
    int first;
    if constexpr (FUSED)
      first = lane_step_fused<V, DYN>(L, fu, mag, mine && run, g, n, i, t, dt, tables, dyn);
    else if constexpr (SOLVER == CMTJ_RK4)
      first = lane_step<SOLVER, V, DYN && FIELD>(L, c, mag, side, mine && run, g, n, i, t, dt, tables, energies,
                                                 nullptr, dyn, nullptr, FIELD ? &fo : nullptr, edge_only);
    else
      first = lane_step<SOLVER, V, false>(L, c, mag, side, mine && run, g, n, i, t, dt, tables, energies, nullptr,
                                          dyn, nullptr, nullptr, false, sigma_run);
    if (first >= 0) {
      if (run) code = CMTJ_STATUS_NAN;
      run = false;
    }
    if (!(i % p.write_every)) {
      lane_log_row(run ? out + (size_t)row * p.log_width : nullptr, run, mine, junctions, j, L, mag, side, g, n, G,
                   mr_mode, energies, t, half_span);
      if (run) ++row;
    }
  }
  if (mine) store3(layers[off + g.l].mag, mag);
  if (have && g.jl == 0) {
    status[2 * j] = code;
    status[2 * j + 1] = row;
  }
}

template <int SOLVER, class V>
__global__ void __launch_bounds__(32)
    k_plain_lanes(const cmtj_junction_t *__restrict__ junctions, int32_t n_junctions,
                  const cmtj_layer_t *params, cmtj_layer_t *layers, const double *__restrict__ tables,
                  cmtj_sim_params_t p, int G, double *__restrict__ log, uint32_t *__restrict__ status) {
  // `params` and `layers` address the same records, so neither is
  // __restrict__: every field but mag is read through `params`, mag is read
  // and written through `layers` only.
  const int span = G * V::kLanes;
  const int lane = threadIdx.x;
  const int l = (lane % span) / V::kLanes;
  const int j = blockIdx.x * (32 / span) + lane / span;
  bool varying = false, general = false, unfused = false;
  if (j < n_junctions) {
    const int n = junctions[j].n_layers;
    if (l < n && n <= G) {
      const cmtj_layer_t &L = params[junctions[j].layer_offset + l];
      const uint32_t dyn = dynamic_slots(L);
      varying = dyn != 0u;
      general = !field_only(L) || (dyn & kFieldOnlyFixedSlots) != 0u;
      unfused = general || (dyn & (1u << CMTJ_SLOT_ANIS)) != 0u;
    }
  }
  const bool dyn = __any_sync(kWarpAll, varying);
  if constexpr (SOLVER == CMTJ_RK4) {
    if (p.arithmetic == CMTJ_ARITH_FUSED && !p.calculate_energies && !__any_sync(kWarpAll, unfused)) {
      if (dyn)
        run_lanes<SOLVER, V, true, true, true>(junctions, n_junctions, params, layers, tables, p, G, log, status);
      else
        run_lanes<SOLVER, V, false, true, true>(junctions, n_junctions, params, layers, tables, p, G, log, status);
      return;
    }
    if (!__any_sync(kWarpAll, general)) {
      if (dyn)
        run_lanes<SOLVER, V, true, true>(junctions, n_junctions, params, layers, tables, p, G, log, status);
      else
        run_lanes<SOLVER, V, false, true>(junctions, n_junctions, params, layers, tables, p, G, log, status);
      return;
    }
  }
  if (dyn)
    run_lanes<SOLVER, V, true, false>(junctions, n_junctions, params, layers, tables, p, G, log, status);
  else
    run_lanes<SOLVER, V, false, false>(junctions, n_junctions, params, layers, tables, p, G, log, status);
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

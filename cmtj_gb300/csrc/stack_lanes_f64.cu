// Electrically coupled junction stacks, FP64 plain form, with each
// junction's layers on lanes.
//
// Stack::runSimulationKCL / runSimulationNonKCL (core/stack.hpp:317-423)
// as in stack_f64.cu: one CTA per stack, the shared per-step values in
// shared memory, every serial sum formed by one thread in the reference's
// order.  Each junction steps with its layers on lanes (one lane per layer,
// or a layer's x, y, z on a quad of lanes; plain_lanes.cuh), which gives
// the same bits as one thread per junction.  Compiled with --fmad=false.
#include "plain_f64.cuh"
#include "plain_lanes.cuh"
#include "plain_lanes.h"
#include "stack_common.cuh"

using namespace cmtjd;

namespace {

constexpr int kStackLaneThreads = 256;

// Stack::runSimulation with each junction's layers on lanes: junction jj of
// the stack owns lanes [jj * span, (jj + 1) * span) of the CTA.
template <int SOLVER, class V>
__global__ void __launch_bounds__(kStackLaneThreads)
    k_stack_lanes(const cmtj_stack_t *__restrict__ stacks, const double *__restrict__ couplings,
                  const cmtj_junction_t *__restrict__ junctions, const int32_t *__restrict__ top_bottom,
                  const cmtj_layer_t *params, cmtj_layer_t *layers, const double *__restrict__ tables,
                  cmtj_sim_params_t p, int G, double *__restrict__ log, double *__restrict__ stack_log,
                  int32_t stack_width, uint32_t *__restrict__ status) {
  // `params` and `layers` address the same records, so neither is
  // __restrict__: every field but mag is read through `params`, mag is read
  // and written through `layers` only.
  __shared__ double s_m[kMaxStack][3], s_p[kMaxStack][3], s_q[kMaxStack][3];
  __shared__ double s_c[kMaxStack], s_R[kMaxStack], s_I[kMaxStack], s_eff[kMaxStack];
  __shared__ double s_total;
  __shared__ int s_nan;
  const cmtj_stack_t S = stacks[blockIdx.x];
  const int N = S.n_junctions;
  const LaneGeo g = lane_geo<V>(G);
  const int jj = (threadIdx.x >> 5) * (32 / g.span) + g.lane / g.span;  // junction within the stack
  const bool mine_j = jj < N;
  const int gj = S.first_junction + (mine_j ? jj : 0);
  int n = mine_j ? junctions[gj].n_layers : 0;
  const bool bad = mine_j && (n < 1 || n > G);
  if (bad) n = 0;
  const bool mine = mine_j && g.l < n;
  // runSingleLayerSolver: every junction steps its layer 0 alone
  const int n_step = (S.single_layer_runner && SOLVER == CMTJ_RK4) ? (n > 0 ? 1 : 0) : n;
  const bool stepper = mine && g.l < n_step;
  const int64_t off = mine_j ? junctions[gj].layer_offset : 0;
  const cmtj_layer_t &L = params[mine ? off + g.l : 0];
  const int mr_mode = mine_j ? junctions[gj].mr_mode : CMTJ_MR_NONE;
  const double half_span = mine_j ? classic_half_span(junctions[gj]) : 0.0;
  const int top_i = mine_j ? top_bottom[2 * gj] : 0, bot_i = mine_j ? top_bottom[2 * gj + 1] : -1;
  const double *cs = couplings + S.coupling_offset;
  const cmtj_constants_t c = p.c;
  const double dt = p.time_step;
  V mag = V::zero();
  uint32_t dyn = 0;
  SideT<V> side;
  side.K = side.K2 = side.Jb = side.Jt = side.I = 0.0;
  side.Hext = side.Hiec = side.Hanis = side.Hdemag = side.Hfl = side.Hdl = V::zero();
  if (mine) {
    mag = V::load(layers[off + g.l].mag);
    dyn = dynamic_slots(L);
  }
  const bool lead = mine_j && g.jl == 0;
  if (threadIdx.x == 0) s_nan = 0;
  cmtj_driver_t cur = S.current;  // this junction's current driver for the step
  uint32_t row = 0;
  __syncthreads();
  for (uint32_t i = 0; i < p.total_iterations; ++i) {
    const double t = (double)i * dt;
    const DriverCtx dc0 = {tables, i, 0};
    // storeMagnetisations (stack.hpp:66-77); s_q: the layer the non-delayed
    // coupling reads as this junction's bottom (bottomId, else layer 0)
    if (mine && g.l == top_i) store3(s_m[jj], mag);
    if (mine && bot_i >= 0 && g.l == bot_i) store3(s_p[jj], mag);
    if (lead && bot_i < 0) {
      s_p[jj][0] = S.pol[0], s_p[jj][1] = S.pol[1], s_p[jj][2] = S.pol[2];
    }
    if (mine && g.l == (bot_i >= 0 ? bot_i : 0)) store3(s_q[jj], mag);
    __syncthreads();
    if (S.use_kcl) {
      // runSimulationKCL (381-423): one coupled current for every junction
      if (lead && jj < N - 1)
        s_c[jj] = coupling(S, cs, jj, load3(s_m[jj]), load3(s_m[jj + 1]), load3(s_p[jj]), load3(s_p[jj + 1]));
      __syncthreads();
      if (threadIdx.x == 0) {
        const double I0 = drv(S.current, t, dc0);
        double total = I0;
        for (int k = 0; k < N - 1; ++k) total = total + s_c[k] * I0;
        s_total = total;
      }
      __syncthreads();
      cur.update = CMTJ_DRV_CONSTANT;
      cur.constantValue = s_total;
      cur.phase = 0.0;
      const int first = lane_step<SOLVER, V>(L, c, mag, side, stepper, g, n_step, i, t, dt, tables, false, &cur, dyn);
      const double cosT = classic_cos(L, mag, g, n, G, mine_j && g.l == 0);
      if (lead) {
        if (first >= 0) atomicExch(&s_nan, 1);
        const cmtj_junction_t &J = junctions[gj];
        s_R[jj] = J.Rp + (half_span * (1.0 - cosT));
        s_I[jj] = s_total;
      }
    } else if (S.delayed) {
      // runSimulationNonKCL (317-379), delayed coupling: a running product of
      // (1 + coupling) over the frozen magnetisations
      if (threadIdx.x == 0) {
        double eff = 1;
        s_eff[0] = eff;
        for (int k = 1; k < N; ++k) {
          eff = eff * (1 + coupling(S, cs, k - 1, load3(s_m[k - 1]), load3(s_m[k]), load3(s_p[k - 1]),
                                    load3(s_p[k])));
          s_c[k - 1] = eff;
          s_eff[k] = eff;
        }
      }
      __syncthreads();
      // ScalarDriver operator* scales offset and amplitude (drivers.hpp:313-329)
      cur = S.current;
      if (mine_j) {
        cur.constantValue = S.current.constantValue * s_eff[jj];
        cur.amplitude = S.current.amplitude * s_eff[jj];
        cur.phase = cur.phase + phase_offset(S, jj);
      }
      const int first = lane_step<SOLVER, V>(L, c, mag, side, stepper, g, n_step, i, t, dt, tables, false, &cur, dyn);
      const double cosT = classic_cos(L, mag, g, n, G, mine_j && g.l == 0);
      if (lead) {
        if (first >= 0) atomicExch(&s_nan, 1);
        const cmtj_junction_t &J = junctions[gj];
        s_R[jj] = J.Rp + (half_span * (1.0 - cosT));
        s_I[jj] = drv(cur, t, dc0);
      }
    } else {
      // non-delayed: junction k's coupling sees junction k-1 after its step,
      // so the junctions step one after another
      for (int k = 0; k < N; ++k) {
        const bool me = mine_j && jj == k;
        if (me && g.jl == 0) {
          double eff = 1;
          if (k > 0) {
            eff = s_eff[k - 1] * (1 + coupling(S, cs, k - 1, load3(s_m[k - 1]), load3(s_m[k]), load3(s_p[k - 1]),
                                               load3(s_q[k])));
            s_c[k - 1] = eff;
          }
          s_eff[k] = eff;
        }
        __syncthreads();
        cur = S.current;
        if (me) {
          cur.constantValue = S.current.constantValue * s_eff[k];
          cur.amplitude = S.current.amplitude * s_eff[k];
          cur.phase = cur.phase + phase_offset(S, k);
        }
        const int first =
            lane_step<SOLVER, V>(L, c, mag, side, stepper && me, g, n_step, i, t, dt, tables, false, &cur, dyn);
        const double cosT = classic_cos(L, mag, g, n, G, me && g.l == 0);
        if (me && g.jl == 0) {
          if (first >= 0) atomicExch(&s_nan, 1);
          const cmtj_junction_t &J = junctions[gj];
          s_R[k] = J.Rp + (half_span * (1.0 - cosT));
          s_I[k] = drv(cur, t, dc0);
        }
        // the next junction reads this one's updated top/bottom layers
        if (me && mine && g.l == top_i) store3(s_m[k], mag);
        if (me && mine && bot_i >= 0 && g.l == bot_i) store3(s_p[k], mag);
        __syncthreads();
      }
    }
    __syncthreads();
    if (s_nan) break;
    if (!(i % p.write_every)) {
      // logSimulationStep (stack.hpp:93-103) and logStackData (255-266)
      if (threadIdx.x == 0) {
        double R;
        if (S.kind == CMTJ_STACK_SERIES) {
          R = 0.0;
          for (int k = 0; k < N; ++k) R = R + s_R[k];
        } else {
          double inv = 0.0;
          for (int k = 0; k < N; ++k) inv = inv + 1.0 / s_R[k];
          R = 1. / inv;
        }
        double *sr = stack_log + ((size_t)blockIdx.x * p.n_log + row) * stack_width;
        sr[0] = R;
        for (int k = 0; k < N; ++k) sr[1 + k] = s_I[k];
        for (int k = 0; k < N - 1; ++k) sr[1 + N + k] = s_c[k];
        sr[2 * N] = t;
      }
      lane_log_row(mine_j ? log + ((size_t)gj * p.n_log + row) * p.log_width : nullptr, mine_j && n > 0, mine,
                   junctions, gj, L, mag, side, g, n, G, mr_mode, false, t, half_span);
      ++row;
    }
    __syncthreads();
  }
  if (mine) store3(layers[off + g.l].mag, mag);
  if (lead) {
    status[2 * gj] = bad ? CMTJ_STATUS_BAD_INPUT : (s_nan ? CMTJ_STATUS_NAN : CMTJ_STATUS_OK);
    status[2 * gj + 1] = row;
  }
}

}  // namespace

namespace cmtjd {

cudaError_t stack_lanes_launch(const cmtj_stack_t *d_stacks, int32_t n_stacks, const double *d_couplings,
                               const cmtj_junction_t *d_junctions, const int32_t *d_top_bottom,
                               cmtj_layer_t *d_layers, const double *d_tables, const cmtj_sim_params_t &p,
                               double *d_log, double *d_stack_log, int32_t stack_width, int32_t max_junctions,
                               uint32_t *d_status, cudaStream_t s) {
  // quads first (unless lanes_per_layer asks for 1), else a lane per layer
  const int G = plain_lanes_group(p.max_layers);
  int P = p.lanes_per_layer == 1 ? 1 : 4;
  if (max_junctions * G * P > kStackLaneThreads && p.lanes_per_layer != 4) P = 1;
  if (max_junctions * G * P > kStackLaneThreads) return cudaErrorNotSupported;
  const int span = G * P;
  const int threads = (max_junctions + 32 / span - 1) / (32 / span) * 32;
  if (P == 4 && p.solver == CMTJ_RK4)
    k_stack_lanes<CMTJ_RK4, C3><<<n_stacks, threads, 0, s>>>(d_stacks, d_couplings, d_junctions, d_top_bottom,
                                                             d_layers, d_layers, d_tables, p, G, d_log, d_stack_log,
                                                             stack_width, d_status);
  else if (P == 4)
    k_stack_lanes<CMTJ_EULER_HEUN, C3><<<n_stacks, threads, 0, s>>>(d_stacks, d_couplings, d_junctions,
                                                                    d_top_bottom, d_layers, d_layers, d_tables, p, G,
                                                                    d_log, d_stack_log, stack_width, d_status);
  else if (p.solver == CMTJ_RK4)
    k_stack_lanes<CMTJ_RK4, D3><<<n_stacks, threads, 0, s>>>(d_stacks, d_couplings, d_junctions, d_top_bottom,
                                                             d_layers, d_layers, d_tables, p, G, d_log, d_stack_log,
                                                             stack_width, d_status);
  else
    k_stack_lanes<CMTJ_EULER_HEUN, D3><<<n_stacks, threads, 0, s>>>(d_stacks, d_couplings, d_junctions,
                                                                    d_top_bottom, d_layers, d_layers, d_tables, p, G,
                                                                    d_log, d_stack_log, stack_width, d_status);
  return cudaGetLastError();
}

}  // namespace cmtjd

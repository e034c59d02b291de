// Dipole-coupled junction groups, FP64 plain form, with each junction's
// layers on lanes.
//
// GroupInteraction::runSimulation (core/reservoir.hpp:185-230) with
// stepFunctionalSolver (130-151), as in group_f64.cu: one CTA per group; each
// step the top-layer magnetisations are frozen in shared memory, the lead
// lane of every junction sums the interaction fields from all others in
// index order, and the junction steps with that sum as its top layer's
// reserved interaction field.  Each junction's layers run on lanes (one lane
// per layer, or a layer's x, y, z on a quad; plain_lanes.cuh), with the same
// bits as one thread per junction.  After the run the top layer's HRES
// drivers hold the last sum, as setLayerReservedInteractionField leaves
// them.  Compiled with --fmad=false.
#include "group_common.cuh"
#include "plain_f64.cuh"
#include "plain_lanes.cuh"
#include "plain_lanes.h"

using namespace cmtjd;

namespace {

constexpr int kGroupLaneThreads = 256;

template <int SOLVER, class V>
__global__ void __launch_bounds__(kGroupLaneThreads)
    k_group_lanes(const cmtj_group_t *__restrict__ groups, const cmtj_pair_t *__restrict__ pairs,
                  const cmtj_junction_t *__restrict__ junctions, const int32_t *__restrict__ top,
                  const cmtj_layer_t *params, cmtj_layer_t *layers, const double *__restrict__ tables,
                  cmtj_sim_params_t p, int G, double *__restrict__ log, uint32_t *__restrict__ status) {
  // `params` and `layers` address the same records, so neither is
  // __restrict__: every field but mag and
  // the HRES drivers is read through `params`; mag is read and written and
  // the HRES drivers are written through `layers` only.
  __shared__ double s_m[kMaxGroup][3], s_h[kMaxGroup][3];
  __shared__ int s_nan;
  const cmtj_group_t Gr = groups[blockIdx.x];
  const int N = Gr.n_junctions;
  const LaneGeo g = lane_geo<V>(G);
  const int jj = (threadIdx.x >> 5) * (32 / g.span) + g.lane / g.span;  // junction within the group
  const bool mine_j = jj < N;
  const int gj = Gr.first_junction + (mine_j ? jj : 0);
  int n = mine_j ? junctions[gj].n_layers : 0;
  const bool bad = mine_j && (n < 1 || n > G);
  if (bad) n = 0;
  const bool mine = mine_j && g.l < n;
  // runSingleLayerSolver: every junction steps its layer 0 alone
  const int n_step = (Gr.single_layer_runner && SOLVER == CMTJ_RK4) ? (n > 0 ? 1 : 0) : n;
  const bool stepper = mine && g.l < n_step;
  const int64_t off = mine_j ? junctions[gj].layer_offset : 0;
  const cmtj_layer_t &L = params[mine ? off + g.l : 0];
  const int mr_mode = mine_j ? junctions[gj].mr_mode : CMTJ_MR_NONE;
  const double half_span = mine_j ? classic_half_span(junctions[gj]) : 0.0;
  const int ti = mine_j ? top[gj] : 0;
  const bool lead = mine_j && g.jl == 0;
  const cmtj_pair_t *row_pairs = pairs + Gr.pair_offset + (int64_t)(mine_j ? jj : 0) * N;
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
  if (threadIdx.x == 0) s_nan = 0;
  uint32_t row = 0, steps = 0;
  __syncthreads();
  for (uint32_t i = 0; i < p.total_iterations; ++i) {
    const double t = (double)i * dt;
    if (mine && g.l == ti) store3(s_m[jj], mag);
    __syncthreads();
    if (lead) {
      const D3 H = interaction_field(Gr.interaction, row_pairs, s_m, N, jj);
      s_h[jj][0] = H.x, s_h[jj][1] = H.y, s_h[jj][2] = H.z;
    }
    __syncthreads();
    const double *hres = (mine && g.l == ti) ? s_h[jj] : nullptr;
    const int first =
        lane_step<SOLVER, V>(L, c, mag, side, stepper, g, n_step, i, t, dt, tables, false, nullptr, dyn, hres);
    if (lead && first >= 0) atomicExch(&s_nan, 1);
    ++steps;
    __syncthreads();
    if (s_nan) break;
    if (!(i % p.write_every)) {
      lane_log_row(mine_j ? log + ((size_t)gj * p.n_log + row) * p.log_width : nullptr, mine_j && n > 0, mine,
                   junctions, gj, L, mag, side, g, n, G, mr_mode, false, t, half_span);
      ++row;
    }
  }
  if (mine) store3(layers[off + g.l].mag, mag);
  if (lead) {
    // the reserved interaction field is a constant axial driver holding the
    // last step's sum
    for (int k = 0; k < 3; ++k) {
      layers[off + ti].drv[CMTJ_SLOT_HRES + k].update = CMTJ_DRV_CONSTANT;
      if (steps) layers[off + ti].drv[CMTJ_SLOT_HRES + k].constantValue = s_h[jj][k];
    }
    status[2 * gj] = bad ? CMTJ_STATUS_BAD_INPUT : (s_nan ? CMTJ_STATUS_NAN : CMTJ_STATUS_OK);
    status[2 * gj + 1] = row;
  }
}

template <class V>
void launch(int solver, int blocks, int threads, cudaStream_t s, const cmtj_group_t *d_groups,
            const cmtj_pair_t *d_pairs, const cmtj_junction_t *d_junctions, const int32_t *d_top,
            cmtj_layer_t *d_layers, const double *d_tables, const cmtj_sim_params_t &p, int G, double *d_log,
            uint32_t *d_status) {
  if (solver == CMTJ_RK4)
    k_group_lanes<CMTJ_RK4, V><<<blocks, threads, 0, s>>>(d_groups, d_pairs, d_junctions, d_top, d_layers, d_layers,
                                                          d_tables, p, G, d_log, d_status);
  else if (solver == CMTJ_EULER_HEUN)
    k_group_lanes<CMTJ_EULER_HEUN, V><<<blocks, threads, 0, s>>>(d_groups, d_pairs, d_junctions, d_top, d_layers,
                                                                 d_layers, d_tables, p, G, d_log, d_status);
  else
    k_group_lanes<CMTJ_HEUN, V><<<blocks, threads, 0, s>>>(d_groups, d_pairs, d_junctions, d_top, d_layers, d_layers,
                                                           d_tables, p, G, d_log, d_status);
}

}  // namespace

namespace cmtjd {

cudaError_t group_lanes_launch(const cmtj_group_t *d_groups, int32_t n_groups, const cmtj_pair_t *d_pairs,
                               const cmtj_junction_t *d_junctions, const int32_t *d_top, cmtj_layer_t *d_layers,
                               const double *d_tables, const cmtj_sim_params_t &p, double *d_log,
                               int32_t max_junctions, uint32_t *d_status, cudaStream_t s) {
  // quads first (unless lanes_per_layer asks for 1), else a lane per layer
  const int G = plain_lanes_group(p.max_layers);
  int P = p.lanes_per_layer == 1 ? 1 : 4;
  if (max_junctions * G * P > kGroupLaneThreads && p.lanes_per_layer != 4) P = 1;
  if (max_junctions * G * P > kGroupLaneThreads) return cudaErrorNotSupported;
  const int span = G * P;
  const int threads = (max_junctions + 32 / span - 1) / (32 / span) * 32;
  if (P == 4)
    launch<C3>(p.solver, n_groups, threads, s, d_groups, d_pairs, d_junctions, d_top, d_layers, d_tables, p, G, d_log,
               d_status);
  else
    launch<D3>(p.solver, n_groups, threads, s, d_groups, d_pairs, d_junctions, d_top, d_layers, d_tables, p, G, d_log,
               d_status);
  return cudaGetLastError();
}

}  // namespace cmtjd

// Dipole-coupled junction groups, FP64 plain form.
//
// GroupInteraction::runSimulation (core/reservoir.hpp:185-230) with
// stepFunctionalSolver (130-151): one CTA runs one group.  This kernel runs
// one thread per junction, for groups too wide for k_group_lanes
// (group_lanes_f64.cu), which steps each junction with its layers on lanes.  Each step the top-layer magnetisations are frozen in shared
// memory; every junction sums the interaction fields from all others in
// index order, sets the sum as its top layer's reserved interaction field
// (the HRES driver slots, as setLayerReservedInteractionField does) and
// steps.  The pair geometry (separations, their 3rd and 5th powers, or the
// dipole tensors) is fixed and comes from the host, formed with the
// reference's own libm; only the m-dependent part is evaluated here, in the
// reference's operand order.  Compiled with --fmad=false like plain_f64.cu.
#include "group_common.cuh"
#include "plain_f64.cuh"

using namespace cmtjd;

namespace {

__global__ void __launch_bounds__(kMaxGroup) k_group_f64(const cmtj_group_t *__restrict__ groups,
                                                         const cmtj_pair_t *__restrict__ pairs,
                                                         const cmtj_junction_t *__restrict__ junctions,
                                                         const int32_t *__restrict__ top, cmtj_layer_t *layers,
                                                         const double *__restrict__ tables, cmtj_sim_params_t p,
                                                         double *__restrict__ log, uint32_t *__restrict__ status) {
  __shared__ double s_m[kMaxGroup][3];
  __shared__ int s_nan;
  const cmtj_group_t G = groups[blockIdx.x];
  const int N = G.n_junctions;
  const int j = threadIdx.x;
  const bool mine = j < N;
  const int gj = G.first_junction + (mine ? j : 0);
  const cmtj_junction_t &J = junctions[gj];
  const int n = J.n_layers;
  cmtj_layer_t *Ls = layers + J.layer_offset;
  const int ti = top[gj];
  const cmtj_pair_t *row_pairs = pairs + G.pair_offset + (int64_t)(mine ? j : 0) * N;
  D3 mag[CMTJ_MAX_LAYERS];
  D3 work[CMTJ_MAX_LAYERS + 2];
  Side side[CMTJ_MAX_LAYERS];
  if (mine) {
    for (int l = 0; l < n; ++l) {
      mag[l] = load3(Ls[l].mag);
      side[l].K = side[l].K2 = side[l].Jb = side[l].Jt = side[l].I = 0.0;
      side[l].Hext = side[l].Hiec = side[l].Hanis = side[l].Hdemag = side[l].Hfl = side[l].Hdl = zero3();
    }
    // the reserved interaction field is a constant axial driver
    for (int k = 0; k < 3; ++k) Ls[ti].drv[CMTJ_SLOT_HRES + k].update = CMTJ_DRV_CONSTANT;
  }
  if (j == 0) s_nan = 0;
  uint32_t row = 0;
  __syncthreads();
  for (uint32_t i = 0; i < p.total_iterations; ++i) {
    const double t = (double)i * p.time_step;
    if (mine) {
      const D3 m = mag[ti];
      s_m[j][0] = m.x, s_m[j][1] = m.y, s_m[j][2] = m.z;
    }
    __syncthreads();
    if (mine) {
      const D3 H = interaction_field(G.interaction, row_pairs, s_m, N, j);
      Ls[ti].drv[CMTJ_SLOT_HRES + 0].constantValue = H.x;
      Ls[ti].drv[CMTJ_SLOT_HRES + 1].constantValue = H.y;
      Ls[ti].drv[CMTJ_SLOT_HRES + 2].constantValue = H.z;
      const bool ok = junction_step(n, Ls, mag, work, side, i, t, p, tables, nullptr, G.single_layer_runner != 0);
      if (!ok) atomicExch(&s_nan, 1);
    }
    __syncthreads();
    if (s_nan) break;
    if (!(i % p.write_every)) {
      if (mine) log_row(log + ((size_t)gj * p.n_log + row) * p.log_width, J, n, Ls, mag, side, t, false);
      ++row;
    }
  }
  if (mine) {
    for (int l = 0; l < n; ++l) {
      Ls[l].mag[0] = mag[l].x;
      Ls[l].mag[1] = mag[l].y;
      Ls[l].mag[2] = mag[l].z;
    }
    status[2 * gj] = s_nan ? CMTJ_STATUS_NAN : CMTJ_STATUS_OK;
    status[2 * gj + 1] = row;
  }
}

}  // namespace

extern "C" int cmtj_run_group_f64(const cmtj_group_t *d_groups, int32_t n_groups, const cmtj_pair_t *d_pairs,
                                  const cmtj_junction_t *d_junctions, const int32_t *d_top, cmtj_layer_t *d_layers,
                                  const double *d_tables, const cmtj_sim_params_t *p, double *d_log,
                                  int32_t max_junctions, uint32_t *d_status, void *stream) {
  if (!p || n_groups < 0 || max_junctions < 1 || max_junctions > kMaxGroup) {
    cmtj_set_error("cmtj_run_group_f64: bad arguments (groups=%d, max_junctions=%d in [1, %d])", n_groups,
                   max_junctions, kMaxGroup);
    return CMTJ_ERR_ARG;
  }
  if (n_groups == 0) return CMTJ_OK;
  if (!d_groups || !d_pairs || !d_junctions || !d_top || !d_layers || !d_status || (p->n_log > 0 && !d_log)) {
    cmtj_set_error("cmtj_run_group_f64: null device buffer");
    return CMTJ_ERR_ARG;
  }
  if (p->write_every == 0 || (p->solver != CMTJ_RK4 && p->solver != CMTJ_EULER_HEUN && p->solver != CMTJ_HEUN)) {
    cmtj_set_error("cmtj_run_group_f64: write_every must be >= 1 and the solver RK4, Euler-Heun or Heun");
    return CMTJ_ERR_ARG;
  }
  // layers on lanes when the widest group fits a CTA of lanes
  const cudaError_t e = cmtjd::group_lanes_launch(d_groups, n_groups, d_pairs, d_junctions, d_top, d_layers, d_tables,
                                                  *p, d_log, max_junctions, d_status, cmtj_stream(stream));
  if (e == cudaSuccess) return CMTJ_OK;
  if (e != cudaErrorNotSupported) {
    cmtj_set_error("launch of k_group_lanes failed: %s", cudaGetErrorString(e));
    return CMTJ_ERR_CUDA;
  }
  const int threads = (max_junctions + 31) / 32 * 32;
  k_group_f64<<<n_groups, threads, 0, cmtj_stream(stream)>>>(d_groups, d_pairs, d_junctions, d_top, d_layers,
                                                              d_tables, *p, d_log, d_status);
  CMTJ_LAUNCH_CHECK("k_group_f64");
  return CMTJ_OK;
}

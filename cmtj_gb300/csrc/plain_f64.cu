// FP64 plain form of the macrospin time loop.
//
// Every floating-point expression keeps the reference's operand order, and
// the units of this form are compiled with --fmad=false, so a*b+c is never
// contracted into an FMA: additions, multiplications, divisions and square
// roots round exactly as the reference's x86-64 build does, and
// deterministic trajectories agree with it bit for bit except where CUDA's
// sin/exp/erf/log differ from glibc's by an ulp.  pow(x, 3) is evaluated as
// a correctly rounded cube (see cube_rn).
//
// The fixed-step solvers run one lane per layer (plain_lanes_f64.cu).  The
// Dormand-Prince loop (core/junction.hpp:1982-2045) runs here, one thread
// per junction, for large batches, and with a layer's x, y, z on a quad of
// lanes for the rest (dp_quads_f64.cu): each layer's step sees the step
// size the previous layer's step chose, so its layers cannot run side by
// side.  The state of a
// junction lives in the thread's registers / local memory; layer parameters
// and drivers are read from the caller's cmtj_layer_t array through L1.
#include "plain_f64.cuh"
#include "plain_lanes.h"

using namespace cmtjd;

namespace {

__global__ void __launch_bounds__(64) k_dormand_prince_f64(const cmtj_junction_t *__restrict__ junctions,
                                                           int32_t n_junctions, cmtj_layer_t *layers,
                                                           const double *__restrict__ tables, cmtj_sim_params_t p,
                                                           double *__restrict__ log, uint32_t *__restrict__ status) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_junctions) return;
  const cmtj_junction_t &J = junctions[j];
  const int n = J.n_layers;
  if (n < 1 || n > CMTJ_MAX_LAYERS) {
    status[2 * j] = CMTJ_STATUS_BAD_INPUT;
    status[2 * j + 1] = 0;
    return;
  }
  cmtj_layer_t *Ls = layers + J.layer_offset;
  const double dt = p.time_step;

  D3 mag[CMTJ_MAX_LAYERS];
  D3 work[CMTJ_MAX_LAYERS + 2];
  Side side[CMTJ_MAX_LAYERS];
  for (int l = 0; l < n; ++l) {
    mag[l] = load3(Ls[l].mag);
    side[l].K = side[l].K2 = side[l].Jb = side[l].Jt = side[l].I = 0.0;
    side[l].Hext = side[l].Hiec = side[l].Hanis = side[l].Hdemag = side[l].Hfl = side[l].Hdl = zero3();
  }
  const bool energies = p.calculate_energies != 0;
  uint32_t row = 0, code = CMTJ_STATUS_OK;
  double *out = log + (size_t)j * p.n_log * p.log_width;
  // runSimulation's adaptive loop (junction.hpp:1982-2045).  Each layer's
  // step sees the step size the previous layer's step chose (one shared
  // timeStep reference in runMultiLayerSolver, 1680-1707), and t advances
  // by the size chosen for the next step, both as in the reference.  A
  // rejection with several layers stops with CMTJ_STATUS_DP_STALL where
  // the reference continues from hopt = -1 without end.
  double t = 0.0, next_write = 0.0, cur = dt;
  uint64_t attempts = 0;
  while (t < p.total_time) {
    if (++attempts > p.max_attempts) {
      code = CMTJ_STATUS_LIMIT;
      break;
    }
    if (t + cur > p.total_time) cur = p.total_time - t;
    int consecutive = 0;
    if (isnan(cur) || isinf(cur) || cur <= 0) {
      cur = dt;
      consecutive++;
    }
    bool accepted = true, nan = false;
    if (n > 1) {
      work[0] = zero3();
      work[n + 1] = zero3();
      for (int l = 0; l < n; ++l) work[l + 1] = mag[l];
      for (int l = 0; l < n; ++l)
        if (!dp_layer(Ls[l], Ls[l].adaptive, p.c, t, cur, mag[l], work[l], work[l + 2], tables,
                      energies ? &side[l] : nullptr, nan))
          accepted = false;
      if (!accepted) {
        code = CMTJ_STATUS_DP_STALL;
        break;
      }
    } else {
      accepted = dp_layer(Ls[0], Ls[0].adaptive, p.c, t, cur, mag[0], zero3(), zero3(), tables,
                          energies ? &side[0] : nullptr, nan);
    }
    if (nan) {
      code = CMTJ_STATUS_NAN;
      break;
    }
    if (!accepted && (cur < 1e-15 || consecutive >= 10)) accepted = true;
    if (accepted) {
      t += cur;
      if (t >= next_write) {
        if (row >= p.n_log) {
          code = CMTJ_STATUS_LIMIT;
          break;
        }
        log_row(out + (size_t)row * p.log_width, J, n, Ls, mag, side, t, energies);
        ++row;
        next_write = ((double)(uint32_t)(t / p.write_frequency) + 1) * p.write_frequency;
      }
    }
  }
  for (int l = 0; l < n; ++l) {
    Ls[l].mag[0] = mag[l].x;
    Ls[l].mag[1] = mag[l].y;
    Ls[l].mag[2] = mag[l].z;
  }
  status[2 * j] = code;
  status[2 * j + 1] = row;
}

}  // namespace

extern "C" int cmtj_run_simulation_f64(const cmtj_junction_t *d_junctions, int32_t n_junctions,
                                       cmtj_layer_t *d_layers, const double *d_tables,
                                       const cmtj_sim_params_t *p, double *d_log, uint32_t *d_status,
                                       void *stream) {
  if (!p || n_junctions < 0) {
    cmtj_set_error("cmtj_run_simulation_f64: null params or negative junction count");
    return CMTJ_ERR_ARG;
  }
  if (n_junctions == 0) return CMTJ_OK;
  if (!d_junctions || !d_layers || !d_status || (p->n_log > 0 && !d_log)) {
    cmtj_set_error("cmtj_run_simulation_f64: null device buffer");
    return CMTJ_ERR_ARG;
  }
  if (p->write_every == 0) {
    cmtj_set_error("cmtj_run_simulation_f64: write_every must be >= 1");
    return CMTJ_ERR_ARG;
  }
  if (p->solver != CMTJ_RK4 && p->solver != CMTJ_EULER_HEUN && p->solver != CMTJ_HEUN &&
      p->solver != CMTJ_DORMAND_PRINCE) {
    cmtj_set_error("cmtj_run_simulation_f64: unknown solver %d", p->solver);
    return CMTJ_ERR_ARG;
  }
  if (p->arithmetic != CMTJ_ARITH_REFERENCE && p->arithmetic != CMTJ_ARITH_FUSED) {
    cmtj_set_error("cmtj_run_simulation_f64: unknown arithmetic %d", p->arithmetic);
    return CMTJ_ERR_ARG;
  }
  if (p->solver == CMTJ_DORMAND_PRINCE &&
      !(p->write_frequency > 0 && p->time_step > 0 && p->total_time >= 0 && p->max_attempts > 0)) {
    cmtj_set_error("cmtj_run_simulation_f64: Dormand-Prince needs time_step > 0, write_frequency > 0, "
                   "total_time >= 0 and max_attempts > 0");
    return CMTJ_ERR_ARG;
  }
  if (p->solver != CMTJ_DORMAND_PRINCE) {
    const cudaError_t e =
        cmtjd::plain_lanes_launch(d_junctions, n_junctions, d_layers, d_tables, *p, d_log, d_status, cmtj_stream(stream));
    if (e != cudaSuccess) {
      cmtj_set_error("launch of k_plain_lanes failed: %s", cudaGetErrorString(e));
      return CMTJ_ERR_CUDA;
    }
    return CMTJ_OK;
  }
  int dev = 0, sms = 0;
  CMTJ_CUDA_TRY(cudaGetDevice(&dev));
  CMTJ_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  if (cmtjd::dp_quads_pick(*p, n_junctions, sms)) {
    const cudaError_t e =
        cmtjd::dp_quads_launch(d_junctions, n_junctions, d_layers, d_tables, *p, d_log, d_status, cmtj_stream(stream));
    if (e != cudaSuccess) {
      cmtj_set_error("launch of k_dp_quads failed: %s", cudaGetErrorString(e));
      return CMTJ_ERR_CUDA;
    }
    return CMTJ_OK;
  }
  const int threads = 64;
  const int blocks = (n_junctions + threads - 1) / threads;
  k_dormand_prince_f64<<<blocks, threads, 0, cmtj_stream(stream)>>>(d_junctions, n_junctions, d_layers, d_tables,
                                                                     *p, d_log, d_status);
  CMTJ_LAUNCH_CHECK("k_dormand_prince_f64");
  return CMTJ_OK;
}

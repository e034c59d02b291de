// FP64 plain form of the macrospin time loop.
//
// One device thread runs one Junction::runSimulation (core/junction.hpp:
// 1948-1981) from start to end.  Every floating-point expression keeps the
// reference's operand order, and this translation unit is compiled with
// --fmad=false, so a*b+c is never contracted into an FMA: additions,
// multiplications, divisions and square roots round exactly as the
// reference's x86-64 build does, and deterministic trajectories agree with
// it bit for bit except where CUDA's sin/exp/erf/log differ from glibc's by
// an ulp.  pow(x, 3) is evaluated as a correctly rounded cube (see cube_rn).
//
// The state of a junction (m of every layer, side values for the energy
// log) lives in the thread's registers / local memory; layer parameters
// and drivers are read from the caller's cmtj_layer_t array through L1.
#include "plain_f64.cuh"

using namespace cmtjd;

namespace {

__global__ void __launch_bounds__(64) k_run_simulation_f64(const cmtj_junction_t *__restrict__ junctions,
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
  for (uint32_t i = 0; i < p.total_iterations; ++i) {
    const double t = (double)i * dt;
    if (!junction_step(n, Ls, mag, work, side, i, t, p, tables, nullptr, false)) {
      code = CMTJ_STATUS_NAN;
      break;
    }
    if (!(i % p.write_every)) {
      log_row(out + (size_t)row * p.log_width, J, n, Ls, mag, side, t, energies);
      ++row;
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
  if (p->solver != CMTJ_RK4 && p->solver != CMTJ_EULER_HEUN && p->solver != CMTJ_HEUN) {
    cmtj_set_error("cmtj_run_simulation_f64: solver %d is not supported by the FP64 plain form", p->solver);
    return CMTJ_ERR_ARG;
  }
  const int threads = 64;
  const int blocks = (n_junctions + threads - 1) / threads;
  k_run_simulation_f64<<<blocks, threads, 0, cmtj_stream(stream)>>>(d_junctions, n_junctions, d_layers, d_tables,
                                                                     *p, d_log, d_status);
  CMTJ_LAUNCH_CHECK("k_run_simulation_f64");
  return CMTJ_OK;
}

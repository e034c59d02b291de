// FP64 plain form, Dormand-Prince: one junction per quad of lanes.
//
// runSimulation's adaptive loop (core/junction.hpp:1982-2045) as in
// plain_f64.cu's one-thread kernel, with each layer's x, y, z on the three
// lanes of a quad (C3, lane3.cuh).  The layers still step one after another:
// each layer's step sees the step size the previous layer's step chose.
// The junctions of a warp take different numbers of steps, so everything
// here is quad-local: no operation names lanes outside the junction's quad.
// The arithmetic is plain_f64.cuh's, in the same order, so the results are
// the one-thread kernel's bits.  Compiled with --fmad=false.
#include "plain_f64.cuh"
#include "plain_lanes.cuh"
#include "plain_lanes.h"

using namespace cmtjd;

namespace {

// logLayerParams (junction.hpp:1580-1636) and the R columns of
// calculateMagnetoresistance / stripMagnetoResistance (1835-1867), by one
// quad.
__device__ void quad_log_row(double *r, const cmtj_junction_t &J, int n, const cmtj_layer_t *Ls, const C3 *mag,
                             const SideT<C3> *side, double t, bool energies) {
  const int width = energies ? CMTJ_ENERGY_COLS : 3;
  for (int l = 0; l < n; ++l) layer_cols(r + l * width, side[l], mag[l], energies);
  double r0 = 0.0, r1 = 0.0;
  if (J.mr_mode == CMTJ_MR_CLASSIC) {
    const double cosT = n == 1 ? dot(mag[0], C3::load(Ls[0].ref)) : dot(mag[0], mag[1]);
    r0 = J.Rp + (((J.Rap - J.Rp) / 2.0) * (1.0 - cosT));
  } else if (J.mr_mode == CMTJ_MR_STRIP) {
    double Rx_acc = 0.0, Ry_acc = 0.0;
    for (int l = 0; l < n; ++l) {
      const double mx = comp_of(mag[l], 0), my = comp_of(mag[l], 1), mz = comp_of(mag[l], 2);
      const double Rx = J.Rx0[l] + J.AMR_X[l] * (mx * mx) + J.SMR_X[l] * (my * my);
      const double Ry = J.Ry0[l] + 0.5 * J.AHE[l] * mz + (J.AMR_Y[l] + J.SMR_Y[l]) * mx * my;
      Rx_acc = Rx_acc + 1. / Rx;
      Ry_acc = Ry_acc + 1. / Ry;
    }
    r0 = 1 / Rx_acc;
    r1 = 1 / Ry_acc;
  }
  if ((threadIdx.x & 3) == 0) {
    double *rr = r + n * width;
    rr[0] = r0;
    rr[1] = r1;
    rr[2] = 0.0;
    rr[3] = t;
  }
}

__global__ void __launch_bounds__(32) k_dp_quads(const cmtj_junction_t *__restrict__ junctions, int32_t n_junctions,
                                                 cmtj_layer_t *layers, const double *__restrict__ tables,
                                                 cmtj_sim_params_t p, double *__restrict__ log,
                                                 uint32_t *__restrict__ status) {
  const int j = blockIdx.x * 8 + (threadIdx.x >> 2);
  if (j >= n_junctions) return;  // the whole quad
  const bool lead = (threadIdx.x & 3) == 0;
  const cmtj_junction_t &J = junctions[j];
  const int n = J.n_layers;
  if (n < 1 || n > CMTJ_MAX_LAYERS) {
    if (lead) {
      status[2 * j] = CMTJ_STATUS_BAD_INPUT;
      status[2 * j + 1] = 0;
    }
    return;
  }
  cmtj_layer_t *Ls = layers + J.layer_offset;
  const double dt = p.time_step;
  C3 mag[CMTJ_MAX_LAYERS];
  C3 work[CMTJ_MAX_LAYERS + 2];
  SideT<C3> side[CMTJ_MAX_LAYERS];
  cmtj_adaptive_t ap[CMTJ_MAX_LAYERS];  // the PID state, written back at the end
  for (int l = 0; l < n; ++l) {
    mag[l] = C3::load(Ls[l].mag);
    ap[l] = Ls[l].adaptive;
    side[l].K = side[l].K2 = side[l].Jb = side[l].Jt = side[l].I = 0.0;
    side[l].Hext = side[l].Hiec = side[l].Hanis = side[l].Hdemag = side[l].Hfl = side[l].Hdl = C3::zero();
  }
  const bool energies = p.calculate_energies != 0;
  uint32_t row = 0, code = CMTJ_STATUS_OK;
  double *out = log + (size_t)j * p.n_log * p.log_width;
  // the loop of k_dormand_prince_f64: each layer's step sees the step size
  // the previous layer's step chose, t advances by the size chosen for the
  // next step, and a rejection with several layers stops with
  // CMTJ_STATUS_DP_STALL where the reference continues from hopt = -1
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
      work[0] = C3::zero();
      work[n + 1] = C3::zero();
      for (int l = 0; l < n; ++l) work[l + 1] = mag[l];
      for (int l = 0; l < n; ++l)
        if (!dp_layer(Ls[l], ap[l], p.c, t, cur, mag[l], work[l], work[l + 2], tables,
                      energies ? &side[l] : nullptr, nan))
          accepted = false;
      if (!accepted) {
        code = CMTJ_STATUS_DP_STALL;
        break;
      }
    } else {
      accepted = dp_layer(Ls[0], ap[0], p.c, t, cur, mag[0], C3::zero(), C3::zero(), tables,
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
        quad_log_row(out + (size_t)row * p.log_width, J, n, Ls, mag, side, t, energies);
        ++row;
        next_write = ((double)(uint32_t)(t / p.write_frequency) + 1) * p.write_frequency;
      }
    }
  }
  for (int l = 0; l < n; ++l) {
    store3(Ls[l].mag, mag[l]);
    if (lead) Ls[l].adaptive = ap[l];
  }
  if (lead) {
    status[2 * j] = code;
    status[2 * j + 1] = row;
  }
}

}  // namespace

namespace cmtjd {

bool dp_quads_pick(const cmtj_sim_params_t &p, int32_t n_junctions, int sm_count) {
  if (p.lanes_per_layer == 1 || p.lanes_per_layer == 4) return p.lanes_per_layer == 4;
  // quads while the batch holds at most two quad warps per SM sub-partition
  return (n_junctions + 7) / 8 <= 2LL * 4 * sm_count;
}

cudaError_t dp_quads_launch(const cmtj_junction_t *d_junctions, int32_t n_junctions, cmtj_layer_t *d_layers,
                            const double *d_tables, const cmtj_sim_params_t &p, double *d_log, uint32_t *d_status,
                            cudaStream_t stream) {
  k_dp_quads<<<(n_junctions + 7) / 8, 32, 0, stream>>>(d_junctions, n_junctions, d_layers, d_tables, p, d_log,
                                                       d_status);
  return cudaGetLastError();
}

}  // namespace cmtjd

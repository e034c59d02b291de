// Electrically coupled junction stacks, FP64 plain form.
//
// Stack::runSimulationKCL / runSimulationNonKCL (core/stack.hpp:317-423)
// with SeriesStack / ParallelStack coupling and resistance (425-480).  One
// CTA runs one stack.  The shared per-step values (frozen magnetisations,
// coupling strengths, the coupled current) pass through shared memory, and
// every sum the reference forms serially is formed serially by one thread
// in the same order, so results keep the reference's rounding.
//
// k_stack_lanes (stack_lanes_f64.cu) steps each junction with its layers on
// lanes, like the single-junction kernel; k_stack_f64 here, one thread per
// junction, runs the stacks too wide for a CTA of lanes.  Compiled with
// --fmad=false like plain_f64.cu.
#include "plain_f64.cuh"
#include "stack_common.cuh"

using namespace cmtjd;

namespace {

__global__ void __launch_bounds__(kMaxStack) k_stack_f64(const cmtj_stack_t *__restrict__ stacks,
                                                         const double *__restrict__ couplings,
                                                         const cmtj_junction_t *__restrict__ junctions,
                                                         const int32_t *__restrict__ top_bottom, cmtj_layer_t *layers,
                                                         const double *__restrict__ tables, cmtj_sim_params_t p,
                                                         double *__restrict__ log, double *__restrict__ stack_log,
                                                         int32_t stack_width, uint32_t *__restrict__ status) {
  __shared__ double s_m[kMaxStack][3], s_p[kMaxStack][3];
  __shared__ double s_c[kMaxStack], s_R[kMaxStack], s_I[kMaxStack], s_eff[kMaxStack];
  __shared__ double s_total;
  __shared__ int s_nan;
  const cmtj_stack_t S = stacks[blockIdx.x];
  const int N = S.n_junctions;
  const int j = threadIdx.x;
  const bool mine = j < N;
  const int gj = S.first_junction + (mine ? j : 0);
  const cmtj_junction_t &J = junctions[gj];
  const int n = J.n_layers;
  cmtj_layer_t *Ls = layers + J.layer_offset;
  const int top_i = top_bottom[2 * gj], bot_i = top_bottom[2 * gj + 1];
  const double *cs = couplings + S.coupling_offset;
  D3 mag[CMTJ_MAX_LAYERS];
  D3 work[CMTJ_MAX_LAYERS + 2];
  Side side[CMTJ_MAX_LAYERS];
  if (mine) {
    for (int l = 0; l < n; ++l) {
      mag[l] = load3(Ls[l].mag);
      side[l].K = side[l].K2 = side[l].Jb = side[l].Jt = side[l].I = 0.0;
      side[l].Hext = side[l].Hiec = side[l].Hanis = side[l].Hdemag = side[l].Hfl = side[l].Hdl = zero3();
    }
  }
  if (j == 0) s_nan = 0;
  cmtj_driver_t cur = S.current;  // this junction's current driver for the step
  uint32_t row = 0;
  __syncthreads();
  for (uint32_t i = 0; i < p.total_iterations; ++i) {
    const double t = (double)i * p.time_step;
    // storeMagnetisations (stack.hpp:66-77)
    if (mine) {
      const D3 m = mag[top_i];
      const D3 q = bot_i >= 0 ? mag[bot_i] : load3(S.pol);
      s_m[j][0] = m.x, s_m[j][1] = m.y, s_m[j][2] = m.z;
      s_p[j][0] = q.x, s_p[j][1] = q.y, s_p[j][2] = q.z;
    }
    __syncthreads();
    if (S.use_kcl) {
      // runSimulationKCL (381-423): one coupled current for every junction
      if (mine && j < N - 1) {
        s_c[j] = coupling(S, cs, j, load3(s_m[j]), load3(s_m[j + 1]), load3(s_p[j]), load3(s_p[j + 1]));
      }
      __syncthreads();
      if (j == 0) {
        DriverCtx dc = {tables, i, 0};
        const double I0 = drv(S.current, t, dc);
        double total = I0;
        for (int k = 0; k < N - 1; ++k) total = total + s_c[k] * I0;
        s_total = total;
      }
      __syncthreads();
      cur.update = CMTJ_DRV_CONSTANT;
      cur.constantValue = s_total;
      cur.phase = 0.0;
      if (mine) {
        const bool ok = junction_step(n, Ls, mag, work, side, i, t, p, tables, &cur, S.single_layer_runner != 0);
        if (!ok) atomicExch(&s_nan, 1);
        s_R[j] = classic_R(J, n, Ls, mag);
        s_I[j] = s_total;
      }
    } else if (S.delayed) {
      // runSimulationNonKCL (317-379), delayed coupling: a running product of
      // (1 + coupling) over the frozen magnetisations
      if (j == 0) {
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
      if (mine) {
        // ScalarDriver operator* scales offset and amplitude (drivers.hpp:313-329)
        cur = S.current;
        cur.constantValue = S.current.constantValue * s_eff[j];
        cur.amplitude = S.current.amplitude * s_eff[j];
        cur.phase = cur.phase + phase_offset(S, j);
        const bool ok = junction_step(n, Ls, mag, work, side, i, t, p, tables, &cur, S.single_layer_runner != 0);
        if (!ok) atomicExch(&s_nan, 1);
        s_R[j] = classic_R(J, n, Ls, mag);
        DriverCtx dc = {tables, i, 0};
        s_I[j] = drv(cur, t, dc);
      }
    } else {
      // non-delayed: junction k's coupling sees junction k-1 after its step,
      // so the junctions step one after another
      double eff = 1;
      for (int k = 0; k < N; ++k) {
        if (j == k) {
          if (k > 0) {
            const D3 m1 = load3(s_m[k - 1]), p1 = load3(s_p[k - 1]);
            eff = s_eff[k - 1] * (1 + coupling(S, cs, k - 1, m1, mag[top_i], p1, mag[bot_i >= 0 ? bot_i : 0]));
            s_c[k - 1] = eff;
          }
          s_eff[k] = eff;
          cur = S.current;
          cur.constantValue = S.current.constantValue * eff;
          cur.amplitude = S.current.amplitude * eff;
          cur.phase = cur.phase + phase_offset(S, k);
          const bool ok = junction_step(n, Ls, mag, work, side, i, t, p, tables, &cur, S.single_layer_runner != 0);
          if (!ok) atomicExch(&s_nan, 1);
          s_R[k] = classic_R(J, n, Ls, mag);
          DriverCtx dc = {tables, i, 0};
          s_I[k] = drv(cur, t, dc);
          // the next junction reads this one's updated top/bottom layers
          const D3 m = mag[top_i];
          const D3 q = bot_i >= 0 ? mag[bot_i] : load3(S.pol);
          s_m[k][0] = m.x, s_m[k][1] = m.y, s_m[k][2] = m.z;
          s_p[k][0] = q.x, s_p[k][1] = q.y, s_p[k][2] = q.z;
        }
        __syncthreads();
      }
    }
    __syncthreads();
    if (s_nan) break;
    if (!(i % p.write_every)) {
      // logSimulationStep (stack.hpp:93-103) and logStackData (255-266)
      if (j == 0) {
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
      if (mine) log_row(log + ((size_t)gj * p.n_log + row) * p.log_width, J, n, Ls, mag, side, t, false);
      ++row;
    }
    __syncthreads();
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

extern "C" int cmtj_run_stack_f64(const cmtj_stack_t *d_stacks, int32_t n_stacks, const double *d_couplings,
                                  const cmtj_junction_t *d_junctions, const int32_t *d_top_bottom,
                                  cmtj_layer_t *d_layers, const double *d_tables, const cmtj_sim_params_t *p,
                                  double *d_log, double *d_stack_log, int32_t stack_width, int32_t max_junctions,
                                  uint32_t *d_status, void *stream) {
  if (!p || n_stacks < 0 || max_junctions < 2 || max_junctions > kMaxStack || stack_width < 2 * max_junctions + 1) {
    cmtj_set_error("cmtj_run_stack_f64: bad arguments (stacks=%d, max_junctions=%d in [2, %d], stack_width=%d)",
                   n_stacks, max_junctions, kMaxStack, stack_width);
    return CMTJ_ERR_ARG;
  }
  if (n_stacks == 0) return CMTJ_OK;
  if (!d_stacks || !d_couplings || !d_junctions || !d_top_bottom || !d_layers || !d_status ||
      (p->n_log > 0 && (!d_log || !d_stack_log))) {
    cmtj_set_error("cmtj_run_stack_f64: null device buffer");
    return CMTJ_ERR_ARG;
  }
  if (p->write_every == 0 || (p->solver != CMTJ_RK4 && p->solver != CMTJ_EULER_HEUN)) {
    cmtj_set_error("cmtj_run_stack_f64: write_every must be >= 1 and the solver RK4 or Euler-Heun");
    return CMTJ_ERR_ARG;
  }
  // layers on lanes when the widest stack fits a CTA of lanes
  const cudaError_t e = cmtjd::stack_lanes_launch(d_stacks, n_stacks, d_couplings, d_junctions, d_top_bottom,
                                                  d_layers, d_tables, *p, d_log, d_stack_log, stack_width,
                                                  max_junctions, d_status, cmtj_stream(stream));
  if (e == cudaSuccess) return CMTJ_OK;
  if (e != cudaErrorNotSupported) {
    cmtj_set_error("launch of k_stack_lanes failed: %s", cudaGetErrorString(e));
    return CMTJ_ERR_CUDA;
  }
  const int threads = (max_junctions + 31) / 32 * 32;
  k_stack_f64<<<n_stacks, threads, 0, cmtj_stream(stream)>>>(d_stacks, d_couplings, d_junctions, d_top_bottom,
                                                              d_layers, d_tables, *p, d_log, d_stack_log,
                                                              stack_width, d_status);
  CMTJ_LAUNCH_CHECK("k_stack_f64");
  return CMTJ_OK;
}

// Shared parts of the two stack kernels (stack_f64.cu, stack_lanes_f64.cu).
#pragma once
#include <cuda_runtime.h>

#include "plain_f64.cuh"

namespace cmtjd {

constexpr int kMaxStack = 256;

// getEffectiveCouplingStrength (stack.hpp:432-439 series, 461-468 parallel).
static __device__ __forceinline__ double coupling(const cmtj_stack_t &S, const double *cs, int order, const D3 &m1,
                                           const D3 &m2, const D3 &p1, const D3 &p2) {
  const double c = S.n_coupling == 1 ? cs[0] : cs[order];
  const double m1c = dot(m1, p1);
  const double m2c = dot(m2, p2);
  return S.kind == CMTJ_STACK_SERIES ? c * (m1c + m2c) : c * (m1c - m2c);
}

// getPhaseOffset: series phaseOffset * order, parallel phaseOffset.
static __device__ __forceinline__ double phase_offset(const cmtj_stack_t &S, int order) {
  return S.kind == CMTJ_STACK_SERIES ? S.phase_offset * order : S.phase_offset;
}

// Launches k_stack_lanes when every stack fits a CTA of lanes; returns
// cudaErrorNotSupported (and launches nothing) when one does not.
cudaError_t stack_lanes_launch(const cmtj_stack_t *d_stacks, int32_t n_stacks, const double *d_couplings,
                               const cmtj_junction_t *d_junctions, const int32_t *d_top_bottom,
                               cmtj_layer_t *d_layers, const double *d_tables, const cmtj_sim_params_t &p,
                               double *d_log, double *d_stack_log, int32_t stack_width, int32_t max_junctions,
                               uint32_t *d_status, cudaStream_t stream);

}  // namespace cmtjd

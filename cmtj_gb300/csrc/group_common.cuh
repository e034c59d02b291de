// Shared parts of the two group kernels (group_f64.cu, group_lanes_f64.cu).
#pragma once
#include <cuda_runtime.h>

#include "plain_f64.cuh"

namespace cmtjd {

constexpr int kMaxGroup = 256;

// computeDipoleInteraction (reservoir.hpp:77-97) for fixed rij, |rij|^3,
// |rij|^5: prefactor * (3 (m.rij) rij / r5 - m / r3).
static __device__ __forceinline__ D3 dipole_term(const cmtj_pair_t &q, const D3 &m) {
  const D3 rij = d3(q.g[0], q.g[1], q.g[2]);
  const double r3 = q.g[3], r5 = q.g[4];
  const double s = 3 * (m.x * rij.x + m.y * rij.y + m.z * rij.z);
  const D3 a = smul(s, rij) / r5;
  const D3 c = a - m / r3;
  return smul(q.scale, c);
}

// calculate_tensor_interaction (junction.hpp:64-72) with the fixed tensor of
// getDipoleTensorFromRelPositions and Ms V / mu0.
static __device__ __forceinline__ D3 noumra_term(const cmtj_pair_t &q, const D3 &m) {
  const double *t = q.g;
  const D3 r = d3(t[0] * m.x + t[1] * m.y + t[2] * m.z, t[3] * m.x + t[4] * m.y + t[5] * m.z,
                  t[6] * m.x + t[7] * m.y + t[8] * m.z);
  return r * q.scale;
}

// The interaction field on junction j of a group from the frozen top-layer
// magnetisations s_m of its n junctions, summed in index order
// (GroupInteraction::runSimulation, reservoir.hpp:214-228).
static __device__ __forceinline__ D3 interaction_field(int kind, const cmtj_pair_t *row_pairs, const double (*s_m)[3],
                                                       int n, int j) {
  D3 H = zero3();
  if (kind == CMTJ_INTERACTION_NULL) return H;
  for (int k = 0; k < n; ++k) {
    if (k == j) continue;
    const D3 mk = d3(s_m[k][0], s_m[k][1], s_m[k][2]);
    H = H + (kind == CMTJ_INTERACTION_DIPOLE ? dipole_term(row_pairs[k], mk) : noumra_term(row_pairs[k], mk));
  }
  return H;
}

// Launches k_group_lanes when every group fits a CTA of lanes; returns
// cudaErrorNotSupported (and launches nothing) when one does not.
cudaError_t group_lanes_launch(const cmtj_group_t *d_groups, int32_t n_groups, const cmtj_pair_t *d_pairs,
                               const cmtj_junction_t *d_junctions, const int32_t *d_top, cmtj_layer_t *d_layers,
                               const double *d_tables, const cmtj_sim_params_t &p, double *d_log,
                               int32_t max_junctions, uint32_t *d_status, cudaStream_t stream);

}  // namespace cmtjd

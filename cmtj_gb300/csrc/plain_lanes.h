// Launcher of the lane-per-layer FP64 fixed-step kernel (plain_lanes_f64.cu).
#pragma once
#include <cuda_runtime.h>

#include "../../include/cmtj_gpu.h"

namespace cmtjd {

// Lanes per junction for a batch whose junctions have at most max_layers
// layers (0 or out of range: CMTJ_MAX_LAYERS).
int plain_lanes_group(int max_layers);

// Lanes per layer the launcher uses (1 or 4) for this batch on a GPU with
// sm_count SMs.
int plain_lanes_per_layer(const cmtj_sim_params_t &p, int32_t n_junctions, int sm_count);

// RK4, Euler-Heun or Heun over n_junctions junctions (arguments as
// cmtj_run_simulation_f64, already checked).
cudaError_t plain_lanes_launch(const cmtj_junction_t *d_junctions, int32_t n_junctions, cmtj_layer_t *d_layers,
                               const double *d_tables, const cmtj_sim_params_t &p, double *d_log, uint32_t *d_status,
                               cudaStream_t stream);

// Dormand-Prince with one junction per quad of lanes (dp_quads_f64.cu):
// whether the launcher takes it for this batch, and the launch.
bool dp_quads_pick(const cmtj_sim_params_t &p, int32_t n_junctions, int sm_count);
cudaError_t dp_quads_launch(const cmtj_junction_t *d_junctions, int32_t n_junctions, cmtj_layer_t *d_layers,
                            const double *d_tables, const cmtj_sim_params_t &p, double *d_log, uint32_t *d_status,
                            cudaStream_t stream);

}  // namespace cmtjd

// Library-level entry points of libcmtj_gpu.so: version, errors, layout.
#include <cstdarg>
#include <cstdio>

#include "common.cuh"

static thread_local char g_last_error[1024] = "";

void cmtj_set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

extern "C" {

int cmtj_abi_version(void) { return CMTJ_ABI_VERSION; }

const char *cmtj_last_error(void) { return g_last_error; }

int cmtj_log_width(int n_layers, int calculate_energies) {
  return n_layers * (calculate_energies ? CMTJ_ENERGY_COLS : 3) + 4;
}

int cmtj_struct_sizes(int32_t *sizes, int32_t n) {
  const int32_t all[14] = {(int32_t)sizeof(cmtj_driver_t),       (int32_t)sizeof(cmtj_layer_t),
                           (int32_t)sizeof(cmtj_junction_t),     (int32_t)sizeof(cmtj_constants_t),
                           (int32_t)sizeof(cmtj_sim_params_t),   (int32_t)sizeof(cmtj_wave_t),
                           (int32_t)sizeof(cmtj_f32_layer_t),    (int32_t)sizeof(cmtj_f32_junction_t),
                           (int32_t)sizeof(cmtj_f32_state_t),    (int32_t)sizeof(cmtj_f32_params_t),
                           (int32_t)sizeof(cmtj_stack_t),        (int32_t)sizeof(cmtj_group_t),
                           (int32_t)sizeof(cmtj_pair_t),         (int32_t)sizeof(cmtj_alpha_noise_t)};
  if (!sizes || n < 0) {
    cmtj_set_error("cmtj_struct_sizes: null output");
    return CMTJ_ERR_ARG;
  }
  for (int i = 0; i < n && i < 14; ++i) sizes[i] = all[i];
  return CMTJ_OK;
}

int cmtj_device_info(int device, int32_t *sm_count, int32_t *cc_major, int32_t *cc_minor) {
  cudaDeviceProp prop;
  CMTJ_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
  if (sm_count) *sm_count = prop.multiProcessorCount;
  if (cc_major) *cc_major = prop.major;
  if (cc_minor) *cc_minor = prop.minor;
  return CMTJ_OK;
}

}  // extern "C"

// Host side of the FP32 batched form: variant choice, persistent grid size,
// ticket reset and launch.
#include "batch_variants.cuh"

namespace {

int variants_for(int L, const CmtjBatchVariant **v) {
  switch (L) {
  case 1: return cmtj_batch_variants_l1(v);
  case 2: return cmtj_batch_variants_l2(v);
  case 3: return cmtj_batch_variants_l3(v);
  case 4: return cmtj_batch_variants_l4(v);
  default: *v = nullptr; return 0;
  }
}

// Smallest compiled variant whose feature set covers `features`
// (waves beyond one need the four-wave variant).
const CmtjBatchVariant *pick(int L, int solver, int features, int need_nw) {
  const CmtjBatchVariant *v = nullptr;
  const int n = variants_for(L, &v);
  const CmtjBatchVariant *best = nullptr;
  for (int k = 0; k < n; ++k) {
    if (v[k].solver != solver) continue;
    if ((v[k].feat & features) != features) continue;
    if (v[k].nw < need_nw) continue;
    if (!best || __builtin_popcount(v[k].feat) < __builtin_popcount(best->feat)) best = &v[k];
  }
  return best;
}

}  // namespace

extern "C" int cmtj_batch_variant_f32(int32_t n_layers, int32_t solver, int32_t features) {
  const int need_nw = (features >> 16) & 0xff;
  const CmtjBatchVariant *v = pick(n_layers, solver, features & 0xffff, need_nw > 0 ? need_nw : 0);
  return v ? (v->feat | (v->nw << 16)) : CMTJ_ERR_ARG;
}

extern "C" int cmtj_batch_run_f32(const cmtj_f32_junction_t *d_junctions, const cmtj_f32_layer_t *d_layers,
                                  cmtj_f32_state_t *d_state, const int32_t *d_order, int32_t n, int32_t n_layers,
                                  int32_t features, const cmtj_f32_params_t *p, float *d_log, uint32_t *d_ticket,
                                  int32_t grid_blocks, void *stream) {
  if (!p || n < 0 || n_layers < 1 || n_layers > CMTJ_MAX_LAYERS_F32) {
    cmtj_set_error("cmtj_batch_run_f32: bad arguments (n=%d, n_layers=%d)", n, n_layers);
    return CMTJ_ERR_ARG;
  }
  if (n == 0) return CMTJ_OK;
  if (!d_junctions || !d_layers || !d_state || !d_order || !d_ticket) {
    cmtj_set_error("cmtj_batch_run_f32: null device buffer");
    return CMTJ_ERR_ARG;
  }
  if (p->solver != CMTJ_RK4 && p->solver != CMTJ_EULER_HEUN && p->solver != CMTJ_HEUN) {
    cmtj_set_error("cmtj_batch_run_f32: solver %d is not supported", p->solver);
    return CMTJ_ERR_ARG;
  }
  const int channels = p->log_mode == CMTJ_LOG_M ? 3 * n_layers : (p->log_mode == CMTJ_LOG_NONE ? 0 : 1);
  if (channels > 0) {
    if (!d_log || p->log_every == 0 || p->log_tile == 0 || (p->log_tile & 3u)) {
      cmtj_set_error("cmtj_batch_run_f32: logging needs a log buffer, log_every >= 1 and log_tile a multiple of 4");
      return CMTJ_ERR_ARG;
    }
    if (p->log_tile * channels > 96) {
      cmtj_set_error("cmtj_batch_run_f32: log_tile * channels = %u exceeds 96 floats per thread",
                     p->log_tile * channels);
      return CMTJ_ERR_LIMIT;
    }
  }
  const int need_nw = (features >> 16) & 0xff;
  const CmtjBatchVariant *v = pick(n_layers, p->solver, features & 0xffff, need_nw);
  if (!v) {
    cmtj_set_error("cmtj_batch_run_f32: no kernel variant for n_layers=%d solver=%d features=0x%x", n_layers,
                   p->solver, features);
    return CMTJ_ERR_ARG;
  }
  const int threads = 128;
  const size_t smem = (size_t)threads * (channels > 0 ? p->log_tile * channels : 1) * sizeof(float);
  int blocks = grid_blocks;
  if (blocks <= 0) {
    int dev = 0, sms = 0, per_sm = 0;
    CMTJ_CUDA_TRY(cudaGetDevice(&dev));
    CMTJ_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CMTJ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, v->fn, threads, smem));
    if (per_sm < 1) per_sm = 1;
    blocks = sms * per_sm;
    const int needed = (n + threads - 1) / threads;
    if (blocks > needed) blocks = needed;
  }
  cudaStream_t s = cmtj_stream(stream);
  CMTJ_CUDA_TRY(cudaMemsetAsync(d_ticket, 0, sizeof(uint32_t), s));
  cmtjf::Args a;
  a.J = d_junctions;
  a.Ly = d_layers;
  a.S = d_state;
  a.order = d_order;
  a.n = n;
  a.p = *p;
  a.log = d_log;
  a.ticket = d_ticket;
  void *args[] = {&a};
  CMTJ_CUDA_TRY(cudaLaunchKernel(v->fn, dim3(blocks), dim3(threads), args, smem, s));
  return CMTJ_OK;
}

// Host side of the FP32 batched form: variant choice, persistent grid size,
// ticket reset and launch.
#include <cuda.h>

#include <mutex>

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

// Smallest compiled variant whose feature set covers `features` (waves
// beyond one need the four-wave variant); of its instantiations, the one
// with resident-CTA bound `mb` when mb > 0 and one exists, else the
// default one.
const CmtjBatchVariant *pick(int L, int solver, int features, int need_nw, int mb) {
  const CmtjBatchVariant *v = nullptr;
  const int n = variants_for(L, &v);
  const CmtjBatchVariant *best = nullptr;
  for (int k = 0; k < n; ++k) {
    if (v[k].solver != solver || v[k].low) continue;
    if ((v[k].feat & features) != features) continue;
    if (v[k].nw < need_nw) continue;
    if (!best || __builtin_popcount(v[k].feat) < __builtin_popcount(best->feat)) best = &v[k];
  }
  if (best && mb > 0 && best->mb != mb) {
    for (int k = 0; k < n; ++k)
      if (v[k].solver == best->solver && v[k].feat == best->feat && v[k].nw == best->nw && v[k].mb == mb)
        return &v[k];
  }
  return best;
}

inline int variant_code(const CmtjBatchVariant *v) { return v->feat | (v->nw << 16) | (v->mb << 24); }

// Shared-memory words per thread of the cached reduction constants.
int red_words(int L) {
  switch (L) {
  case 1: return cmtjf::red_words<1>();
  case 2: return cmtjf::red_words<2>();
  case 3: return cmtjf::red_words<3>();
  default: return cmtjf::red_words<4>();
  }
}

}  // namespace

extern "C" int cmtj_batch_variant_f32(int32_t n_layers, int32_t solver, int32_t features) {
  const int need_nw = (features >> 16) & 0xff;
  const CmtjBatchVariant *v =
      pick(n_layers, solver, features & 0xffff, need_nw > 0 ? need_nw : 0, (features >> 24) & 0xf);
  return v ? variant_code(v) : CMTJ_ERR_ARG;
}

extern "C" int cmtj_batch_bounds_f32(int32_t n_layers, int32_t solver, int32_t features, int32_t *bounds,
                                     int32_t n) {
  const CmtjBatchVariant *v = nullptr;
  const int count = variants_for(n_layers, &v);
  const CmtjBatchVariant *b = pick(n_layers, solver, features & 0xffff, (features >> 16) & 0xff, 0);
  if (!b || !bounds || n < 1) {
    cmtj_set_error("cmtj_batch_bounds_f32: no variant for n_layers=%d solver=%d features=0x%x", n_layers,
                   solver, features);
    return CMTJ_ERR_ARG;
  }
  int k = 0;
  bounds[k++] = b->mb;
  for (int q = 0; q < count && k < n; ++q)
    if (v[q].low && v[q].solver == b->solver && v[q].feat == b->feat && v[q].nw == b->nw) bounds[k++] = v[q].mb;
  return k;
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
    // A chunk that ends inside a log tile flushes a partial tile, and the
    // next chunk's bulk stores would start off a 16-byte boundary.
    const uint64_t tile_steps = (uint64_t)p->log_every * p->log_tile;
    if (p->chunk_steps != 0xffffffffu && (uint64_t)p->chunk_steps % tile_steps != 0) {
      cmtj_set_error("cmtj_batch_run_f32: chunk_steps %u is not a multiple of log_every * log_tile = %llu",
                     p->chunk_steps, (unsigned long long)tile_steps);
      return CMTJ_ERR_ARG;
    }
  }
  const int need_nw = (features >> 16) & 0xff;
  const CmtjBatchVariant *v = pick(n_layers, p->solver, features & 0xffff, need_nw, (features >> 24) & 0xf);
  if (!v) {
    cmtj_set_error("cmtj_batch_run_f32: no kernel variant for n_layers=%d solver=%d features=0x%x", n_layers,
                   p->solver, features);
    return CMTJ_ERR_ARG;
  }
  const int threads = cmtjf::kRedStride;
  // per thread: its log tile, then (weighted reduction) a compensated sum
  // pair, then (any reduction) the cached reduction constants
  const size_t smem = (size_t)threads *
                      ((channels > 0 ? p->log_tile * channels : 1) + (p->red_weights ? 2 : 0) +
                       (p->red_every ? red_words(n_layers) : 0)) *
                      sizeof(float);
  if (smem > 48u * 1024u)
    CMTJ_CUDA_TRY(cudaFuncSetAttribute(v->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
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

// ---------------------------------------------------------------------------
// Allocation-free variant.
//
// Some callers cannot call cudaMalloc: code that runs while a CUDA graph is
// being captured in relaxed or global mode, real-time or signal-handler
// threads that must not take the driver's allocation locks, and hosts that
// hand a plugin all of its memory up front (a fixed arena) and forbid it any
// allocation of its own.  cmtj_batch_run_f32 needs one uint32 work-stealing
// ticket in global memory, which its caller allocates.  This variant keeps
// its tickets in the library's own device memory instead: the file-scope
// array below, CMTJ_NOALLOC_TICKET_SLOTS (64) tickets of 4 bytes, 256 bytes
// that every GPU which loads the library holds until the process exits.
// ---------------------------------------------------------------------------
static __device__ __align__(256) uint32_t g_noalloc_tickets[CMTJ_NOALLOC_TICKET_SLOTS];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
struct NoallocAddress {
  unsigned long long ctx_id;  // context the address was resolved in (0: unknown)
  uint32_t *ptr;
};
NoallocAddress g_noalloc_addr[kMaxDevices] = {};

// Unique id of the calling thread's current context, through the driver
// entry points the runtime hands out (no link against libcuda, no
// allocation).  0 when the driver does not offer them.
unsigned long long current_context_id() {
  typedef CUresult (*GetCurrentFn)(CUcontext *);
  typedef CUresult (*GetIdFn)(CUcontext, unsigned long long *);
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr, *g = nullptr;
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &g, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
      get_current = reinterpret_cast<GetCurrentFn>(f);
      get_id = reinterpret_cast<GetIdFn>(g);
    }
  });
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of g_noalloc_tickets on the current device, resolved with
// that device current the first time it is used in a context, and again
// whenever the device's context changes (after cudaDeviceReset the module
// is loaded anew and the old address is gone).  In host code the array's
// name is only a host-side stand-in for the symbol, never a device address.
int noalloc_tickets(uint32_t **out) {
  int dev = 0;
  CMTJ_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    cmtj_set_error("cmtj_batch_run_f32_noalloc: device ordinal %d beyond %d", dev, kMaxDevices);
    return CMTJ_ERR_LIMIT;
  }
  // Before the runtime has made a context current this reads 0, and the
  // symbol lookup below creates the primary context; the id is read again
  // after it.  Without the driver entry points every call resolves anew.
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  NoallocAddress &a = g_noalloc_addr[dev];
  if (!a.ptr || ctx == 0 || a.ctx_id != ctx) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_tickets);
    if (e != cudaSuccess || !ptr) {
      cmtj_set_error("cmtj_batch_run_f32_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return CMTJ_ERR_CUDA;
    }
    a.ptr = static_cast<uint32_t *>(ptr);
    a.ctx_id = current_context_id();
  }
  *out = a.ptr;
  return CMTJ_OK;
}
}  // namespace

extern "C" int cmtj_batch_run_f32_noalloc(const cmtj_f32_junction_t *d_junctions, const cmtj_f32_layer_t *d_layers,
                                          cmtj_f32_state_t *d_state, const int32_t *d_order, int32_t n,
                                          int32_t n_layers, int32_t features, const cmtj_f32_params_t *p,
                                          float *d_log, int32_t ticket_slot, int32_t grid_blocks, void *stream) {
  if (ticket_slot < 0 || ticket_slot >= CMTJ_NOALLOC_TICKET_SLOTS) {
    cmtj_set_error("cmtj_batch_run_f32_noalloc: ticket_slot %d is outside [0, %d): the library holds %d "
                   "static tickets",
                   ticket_slot, CMTJ_NOALLOC_TICKET_SLOTS, CMTJ_NOALLOC_TICKET_SLOTS);
    return CMTJ_ERR_LIMIT;
  }
  uint32_t *tickets = nullptr;
  const int rc = noalloc_tickets(&tickets);
  if (rc != CMTJ_OK) return rc;
  // cmtj_batch_run_f32 zeroes the ticket on `stream` before its launch
  // (cudaMemsetAsync, no allocation), so the slot's previous contents never
  // leak into this call.
  return cmtj_batch_run_f32(d_junctions, d_layers, d_state, d_order, n, n_layers, features, p, d_log,
                            tickets + ticket_slot, grid_blocks, stream);
}

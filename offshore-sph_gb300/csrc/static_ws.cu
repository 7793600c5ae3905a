// static_ws.cu -- sph_compute_static: the derivative evaluation with its
// scratch in a device array owned by the library, for callers that cannot
// allocate device memory themselves.
//
// Who needs it: code that drives the step from a context where cudaMalloc is
// not available to it -- a host application whose GPU memory is handed out by
// another component (a framework's caching allocator it cannot reach, a
// fixed memory budget negotiated up front), or a thin foreign-function binding
// that can pass device pointers it was given but has no allocator of its own.
// Such a caller still provides the particle arrays; only the scratch moves
// into the library.
//
// The scratch is one file-scope __device__ array of SPH_STATIC_WS_BYTES.  Every
// GPU that loads the library holds that array until the process exits.  Host
// code never passes the array's host-side symbol to a kernel: the symbol is a
// stand-in, not a device address.  The device address comes from
// cudaGetSymbolAddress, called with the device current, once per CUDA
// context, and is cached under the context's unique id (cuCtxGetId).  A
// context is what owns the loaded module: after cudaDeviceReset, or in a
// caller's own (non-primary) context, the module is loaded again at another
// address, and the new context's id differs from every earlier one, so the
// first call there looks the address up afresh instead of reusing a stale one.
#include <cuda.h>

#include <mutex>

#include "sph_internal.cuh"

namespace {

constexpr size_t kStaticWsBytes = SPH_STATIC_WS_BYTES;
constexpr int kMaxContexts = 64;

__device__ __align__(256) unsigned char g_static_ws[kStaticWsBytes];

// driver entry points, resolved once through the runtime (the library does
// not link libcuda itself)
typedef CUresult (*ctx_get_current_fn)(CUcontext *);
typedef CUresult (*ctx_get_id_fn)(CUcontext, unsigned long long *);
ctx_get_current_fn g_ctx_get_current = nullptr;
ctx_get_id_fn g_ctx_get_id = nullptr;
std::once_flag g_entry_once;

void resolve_entry_points() {
  void *f = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    g_ctx_get_current = (ctx_get_current_fn)f;
  f = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    g_ctx_get_id = (ctx_get_id_fn)f;
}

// unique id of the current context (0 when none is current or the CUDA
// driver does not say)
unsigned long long current_context_id() {
  if (!g_ctx_get_current || !g_ctx_get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  if (g_ctx_get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

struct CachedAddress {
  unsigned long long ctx_id;
  void *ptr;
};
std::mutex g_mutex;
CachedAddress g_cache[kMaxContexts];
int g_cache_used = 0, g_cache_next = 0;

// Device address of g_static_ws in the current context; the first call in a
// context resolves it with cudaGetSymbolAddress (which also makes the
// device's primary context current when no context is) and caches it.
int static_ws_address(void **out) {
  std::call_once(g_entry_once, resolve_entry_points);
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return SPH_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_mutex);
  const unsigned long long id = current_context_id();
  if (id) {
    for (int k = 0; k < g_cache_used; k++)
      if (g_cache[k].ctx_id == id) {
        *out = g_cache[k].ptr;
        return SPH_OK;
      }
  }
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_static_ws) != cudaSuccess || !p) return SPH_ERR_CUDA;
  const unsigned long long id_after = id ? id : current_context_id();
  if (id_after) {  // remember it; the oldest entry gives way when the table is full
    const int slot = g_cache_next;
    g_cache_next = (g_cache_next + 1) % kMaxContexts;
    if (g_cache_used < kMaxContexts) g_cache_used++;
    g_cache[slot].ctx_id = id_after;
    g_cache[slot].ptr = p;
  }
  *out = p;
  return SPH_OK;
}

}  // namespace

extern "C" int sph_compute_static(sph_particles_t *pa, const sph_wcsph_t *w, const sph_config_t *cfg,
                                  uint32_t *status, sph_stream_t stream) {
  if (!pa || pa->n < 0 || !w || !cfg) return SPH_ERR_INVALID_ARGUMENT;
  if (pa->n > SPH_STATIC_MAX_PARTICLES) return SPH_ERR_STATIC_LIMIT;
  sph_workspace_t ws;
  ws.n_cap = SPH_STATIC_MAX_PARTICLES;
  ws.max_cells = SPH_STATIC_MAX_CELLS;
  ws.bytes = kStaticWsBytes;
  if (sph::make_layout(ws.n_cap, ws.max_cells).total > kStaticWsBytes) return SPH_ERR_STATIC_LIMIT;
  int e = static_ws_address(&ws.ptr);
  if (e) return e;
  cudaStream_t st = (cudaStream_t)stream;
  sph::WsPtrs p = sph::ws_ptrs(&ws);
  // the array keeps what the previous call left: counters, grid and control
  // block (reductions, status word) return to a fresh workspace's state
  if (sph::init_workspace(p, st) != cudaSuccess) return SPH_ERR_CUDA;
  e = sph_compute(pa, w, cfg, &ws, stream);
  if (e) return e;
  if (status &&
      cudaMemcpyAsync(status, &p.ctrl->status, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return SPH_ERR_CUDA;
  return SPH_OK;
}

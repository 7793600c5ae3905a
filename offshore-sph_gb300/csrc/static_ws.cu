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
// GPU that loads the library holds that array until the process exits.  Its
// device address is looked up once per device with cudaGetSymbolAddress and
// cached; the host-side symbol itself is only a stand-in and is never passed
// to a kernel.
#include <mutex>

#include "sph_internal.cuh"

namespace {

constexpr size_t kStaticWsBytes = SPH_STATIC_WS_BYTES;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_static_ws[kStaticWsBytes];

std::mutex g_mutex;
void *g_static_ptr[kMaxDevices];

// Device address of g_static_ws on the current device (first use on a device
// resolves and caches it).
int static_ws_address(void **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return SPH_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return SPH_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_static_ptr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_ws) != cudaSuccess || !p) return SPH_ERR_CUDA;
    g_static_ptr[dev] = p;
  }
  *out = g_static_ptr[dev];
  return SPH_OK;
}

// The array keeps whatever the previous call left: return the control block
// (reductions, status word, counters) to its initial state.
__global__ void k_static_ctrl_init(sph::DevCtrl *c) {
  if (threadIdx.x != 0) return;
  memset(c, 0, sizeof(sph::DevCtrl));
  c->xmin = c->ymin = c->hmin_all = c->ts_hmin = c->pd_hmin = sph::kEncMinId;
  c->xmax = c->ymax = c->hmax_new = c->ts_cmax = c->ts_a2max = c->pd_a2max = sph::kEncMaxId;
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
  // counters and control block start from zero on every call
  if (cudaMemsetAsync(p.counts, 0, (size_t)(ws.max_cells + 1) * 4, st) != cudaSuccess) return SPH_ERR_CUDA;
  if (cudaMemsetAsync(p.scan_part, 0, (size_t)p.n_parts * 4, st) != cudaSuccess) return SPH_ERR_CUDA;
  k_static_ctrl_init<<<1, 32, 0, st>>>(p.ctrl);
  if (cudaGetLastError() != cudaSuccess) return SPH_ERR_CUDA;
  e = sph_compute(pa, w, cfg, &ws, stream);
  if (e) return e;
  if (status &&
      cudaMemcpyAsync(status, &p.ctrl->status, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return SPH_ERR_CUDA;
  return SPH_OK;
}

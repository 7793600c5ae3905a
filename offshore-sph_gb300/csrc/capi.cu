// capi.cu -- extern "C" entry points of libsph_gb300 (see include/sph_gb300.h).
#include <string.h>

#include <vector>

#include "sph_internal.cuh"

namespace sph {

static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

WsLayout make_layout(long long n_cap, long long max_cells) {
  WsLayout L;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align256(off + bytes);
    return o;
  };
  size_t n = (size_t)(n_cap > 0 ? n_cap : 1);
  size_t mc = (size_t)max_cells;
  L.n_cap = n_cap;
  L.max_cells = max_cells;
  L.n_parts = (long long)((mc + 1 + kScanTile - 1) / kScanTile);
  L.ctrl = take(sizeof(DevCtrl));
  L.grid = take(sizeof(DevGrid));
  L.keys = take(n * 4);
  L.refcell = take(n * 8);
  L.crank = take(n * 4);
  L.perm_tmp = take(n * 4);
  L.keys_sorted = take(n * 4);
  L.perm = take(n * 4);
  L.meta = take(n * 8);
  L.counts = take((mc + 1) * 4);
  L.cstart = take((mc + 2) * 4);
  L.scan_part = take((size_t)L.n_parts * 4);
  L.rec0 = take(n * 16);
  L.rec1 = take(n * 16);
  L.rec2 = take(n * 16);
  L.rec64a = take(n * 32);
  L.rec64b = take(n * 32);
  // one entry per query slot, per 128-slot chunk and per tile bounds every
  // list the tile pair kernel can write
  L.fb_cap = (long long)(n + n / 128 + mc + 2);
  L.fb = take((size_t)L.fb_cap * 8);
  L.tiles = take((mc + 1) * 4);
  L.tiles_h = take((mc + 1) * 4);
  L.tflag = take((mc + 1 + 31) / 32 * 4);
  L.total = off;
  L.shadow = take(n * 8 * kStateFields);
  L.shadow_label = take(n);
  L.shadow_orig = take(n * 4);
  L.total_shadow = off;
  return L;
}

WsPtrs ws_ptrs(const sph_workspace_t *ws) {
  WsLayout L = make_layout(ws->n_cap, ws->max_cells);
  char *b = (char *)ws->ptr;
  WsPtrs p;
  p.ctrl = (DevCtrl *)(b + L.ctrl);
  p.grid = (DevGrid *)(b + L.grid);
  p.keys = (int *)(b + L.keys);
  p.refcell = (int2 *)(b + L.refcell);
  p.crank = (unsigned int *)(b + L.crank);
  p.perm_tmp = (int *)(b + L.perm_tmp);
  p.keys_sorted = (int *)(b + L.keys_sorted);
  p.perm = (int *)(b + L.perm);
  p.meta = (int2 *)(b + L.meta);
  p.counts = (unsigned int *)(b + L.counts);
  p.cstart = (unsigned int *)(b + L.cstart);
  p.scan_part = (unsigned int *)(b + L.scan_part);
  p.rec0 = (float4 *)(b + L.rec0);
  p.rec1 = (float4 *)(b + L.rec1);
  p.rec2 = (float4 *)(b + L.rec2);
  p.rec64a = (double4_32a *)(b + L.rec64a);
  p.rec64b = (double4_32a *)(b + L.rec64b);
  p.fb = (int2 *)(b + L.fb);
  p.tiles = (int *)(b + L.tiles);
  p.tiles_h = (int *)(b + L.tiles_h);
  p.tflag = (unsigned int *)(b + L.tflag);
  p.fb_cap = L.fb_cap;
  p.n_cap = L.n_cap;
  p.max_cells = L.max_cells;
  p.n_parts = L.n_parts;
  const bool room = ws->bytes >= L.total_shadow;
  p.shadow = room ? (double *)(b + L.shadow) : nullptr;
  p.shadow_label = room ? (int8_t *)(b + L.shadow_label) : nullptr;
  p.shadow_orig = room ? (int *)(b + L.shadow_orig) : nullptr;
  p.orig = nullptr;
  return p;
}

__global__ void k_ctrl_init(DevCtrl *c) {
  if (threadIdx.x != 0) return;
  memset(c, 0, sizeof(DevCtrl));
  c->xmin = c->ymin = c->hmin_all = c->ts_hmin = c->pd_hmin = kEncMinId;
  c->xmax = c->ymax = c->hmax_new = c->ts_cmax = c->ts_a2max = c->pd_a2max = kEncMaxId;
  c->initialised = 0x53504821u;
}

// zero cell counters, zero grid, control block at its identities; returns
// the first error of the four stream operations
cudaError_t init_workspace(const WsPtrs &w, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(w.counts, 0, (size_t)(w.max_cells + 1) * 4, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.scan_part, 0, (size_t)w.n_parts * 4, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.tflag, 0, (size_t)(w.max_cells + 1 + 31) / 32 * 4, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.grid, 0, sizeof(DevGrid), st);
  if (e != cudaSuccess) return e;
  k_ctrl_init<<<1, 32, 0, st>>>(w.ctrl);
  return cudaGetLastError();
}

// Self-test of the bulk-copy primitives: a 64-byte bulk copy completing on
// an mbarrier, and a wait on bytes that never come,
// which must give up after its bound.  result[0] = 1 when the copy landed
// intact, result[1] = 2 when the second wait ran out (1 if it completed).
__global__ void k_selftest_staging(const float4 *src, unsigned int *result) {
  __shared__ float4 buf[4];
  __shared__ unsigned long long bar[2];
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bar[0], 64u);
    bulk_copy_g2s(buf, src, 64u, &bar[0]);
    mbar_arrive_expect_tx(&bar[1], 16u);  // nothing is sent
  }
  bool ok0 = mbar_wait_bounded(&bar[0], 0u);
  if (!ok0) mbar_wait_bounded(&bar[0], 0u, kMbarDrainLimit);  // drain before leaving (bounded)
  const bool ok1 = mbar_wait_bounded(&bar[1], 0u, 256);
  __syncthreads();
  if (threadIdx.x == 0) {
    bool same = ok0;
    for (int q = 0; q < 4 && same; q++)
      same = buf[q].x == src[q].x && buf[q].y == src[q].y && buf[q].z == src[q].z && buf[q].w == src[q].w;
    result[0] = same ? 1u : 0u;
    result[1] = ok1 ? 1u : 2u;
  }
}

// ---------------------------------------------------------------------------
// The sorted copy of the state.  A run of several steps gathers the caller's
// arrays once into the sorted order of a first neighbour build and steps on
// that copy: particles that are neighbours in space are then neighbours in
// memory, so each step's keys, scatter, records and derivative writes touch
// nearly consecutive addresses instead of gathering through the caller's
// order.  The in-cell order still ranks by the caller's index (WsPtrs::orig),
// so the results are those of stepping on the caller's arrays, bit for bit.
// At the end the copy is scattered back.
// ---------------------------------------------------------------------------
StepArgs shadow_args(const WsPtrs &w, long long n) {
  StepArgs b;
  b.n = n;
  b.label = w.shadow_label;
  double *f = w.shadow;
  const long long st = w.n_cap > 0 ? w.n_cap : 1;
  double **dst[kStateFields] = {&b.m, &b.rho, &b.p, &b.c, &b.drho, &b.h, &b.x, &b.y, &b.vx, &b.vy,
                                &b.ax, &b.ay, &b.xsphx, &b.xsphy, &b.x0, &b.y0, &b.vx0, &b.vy0, &b.rho0};
  for (int q = 0; q < kStateFields; q++) *dst[q] = f + q * st;
  return b;
}

__device__ __forceinline__ double *const *state_fields(const StepArgs &a, double *(&f)[kStateFields]) {
  f[0] = a.m; f[1] = a.rho; f[2] = a.p; f[3] = a.c; f[4] = a.drho; f[5] = a.h; f[6] = a.x; f[7] = a.y;
  f[8] = a.vx; f[9] = a.vy; f[10] = a.ax; f[11] = a.ay; f[12] = a.xsphx; f[13] = a.xsphy; f[14] = a.x0;
  f[15] = a.y0; f[16] = a.vx0; f[17] = a.vy0; f[18] = a.rho0;
  return f;
}

// copy slot s = caller particle perm[s]; orig[s] remembers it
__global__ void k_shadow_gather(StepArgs src, StepArgs dst, const int *__restrict__ perm, int *__restrict__ orig) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= src.n) return;
  const int i = perm[s];
  orig[s] = i;
  double *fs[kStateFields], *fd[kStateFields];
  state_fields(src, fs);
  state_fields(dst, fd);
#pragma unroll
  for (int q = 0; q < kStateFields; q++) fd[q][s] = fs[q][i];
  const_cast<int8_t *>(dst.label)[s] = src.label[i];
}

// the copy back to the caller's order (labels do not change)
__global__ void k_shadow_scatter(StepArgs src, StepArgs dst, const int *__restrict__ orig) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= src.n) return;
  const int i = orig[s];
  double *fs[kStateFields], *fd[kStateFields];
  state_fields(src, fs);
  state_fields(dst, fd);
#pragma unroll
  for (int q = 0; q < kStateFields; q++) fd[q][i] = fs[q][s];
}

__global__ void k_fill_dt(double *dt_hist, long long nsteps, double dt) {
  long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsteps) return;
  dt_hist[3 * s] = dt;
  dt_hist[3 * s + 1] = 0.0;
  dt_hist[3 * s + 2] = 0.0;
}

}  // namespace sph

using namespace sph;

static int check_launch() { return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA; }

static bool particles_ok(const sph_particles_t *pa) {
  if (!pa || pa->n < 0) return false;
  if (pa->n == 0) return true;
  const void *ptrs[] = {pa->label, pa->m, pa->rho, pa->p, pa->c, pa->drho, pa->h, pa->x, pa->y, pa->vx,
                        pa->vy, pa->ax, pa->ay, pa->xsphx, pa->xsphy, pa->x0, pa->y0, pa->vx0, pa->vy0,
                        pa->rho0};
  for (const void *p : ptrs)
    if (!p) return false;
  return true;
}

static int ws_ok(const sph_workspace_t *ws, int64_t n) {
  if (!ws || !ws->ptr || ws->max_cells <= 0 || ws->n_cap < 0) return SPH_ERR_INVALID_ARGUMENT;
  if (n > ws->n_cap) return SPH_ERR_WORKSPACE_TOO_SMALL;
  if (n > 0x7fffffffll || ws->max_cells > 0x3fffffffll) return SPH_ERR_INVALID_ARGUMENT;
  if (ws->bytes < make_layout(ws->n_cap, ws->max_cells).total) return SPH_ERR_WORKSPACE_TOO_SMALL;
  return SPH_OK;
}

static bool config_ok(const sph_config_t *c) {
  return c && (c->kernel == SPH_KERNEL_CUBIC || c->kernel == SPH_KERNEL_GAUSSIAN || c->kernel == SPH_KERNEL_WENDLAND) &&
         (c->precision == SPH_PREC_FP64 || c->precision == SPH_PREC_MIXED) &&
         (c->integrator == SPH_INTEGRATOR_PEC || c->integrator == SPH_INTEGRATOR_EULER ||
          c->integrator == SPH_INTEGRATOR_VERLET) &&
         c->nn_scale > 0.0;
}

extern "C" {

int sph_abi_version(void) { return SPH_ABI_VERSION; }

int64_t sph_default_max_cells(int64_t n) {
  int64_t m = 4 * (n > 0 ? n : 1);
  return m < 65536 ? 65536 : m;
}

int sph_workspace_size(int64_t n, int64_t max_cells, size_t *bytes) {
  if (!bytes || n < 0) return SPH_ERR_INVALID_ARGUMENT;
  if (max_cells <= 0) max_cells = sph_default_max_cells(n);
  if (max_cells > 0x3fffffffll) return SPH_ERR_INVALID_ARGUMENT;
  *bytes = make_layout(n, max_cells).total_shadow;
  return SPH_OK;
}

int sph_workspace_init(sph_workspace_t *ws, sph_stream_t stream) {
  if (!ws) return SPH_ERR_INVALID_ARGUMENT;
  if (ws->max_cells <= 0) ws->max_cells = sph_default_max_cells(ws->n_cap);
  int e = ws_ok(ws, 0);
  if (e) return e;
  cudaStream_t st = (cudaStream_t)stream;
  if (init_workspace(ws_ptrs(ws), st) != cudaSuccess) return SPH_ERR_CUDA;
  return cudaStreamSynchronize(st) == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

int sph_get_status(const sph_workspace_t *ws, uint32_t *status, sph_stream_t stream) {
  int e = ws_ok(ws, 0);
  if (e) return e;
  if (!status) return SPH_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  WsPtrs p = ws_ptrs(ws);
  unsigned int v = 0;
  if (cudaMemcpyAsync(&v, &p.ctrl->status, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess) return SPH_ERR_CUDA;
  if (cudaMemsetAsync(&p.ctrl->status, 0, 4, st) != cudaSuccess) return SPH_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return SPH_ERR_CUDA;
  *status = v;
  return SPH_OK;
}

const char *sph_status_string(int code) {
  switch (code) {
    case SPH_OK: return "ok";
    case SPH_ERR_INVALID_ARGUMENT: return "invalid argument";
    case SPH_ERR_WORKSPACE_TOO_SMALL: return "workspace too small";
    case SPH_ERR_CUDA: return "CUDA error";
    case SPH_ERR_NOT_INITIALISED: return "workspace not initialised";
    case SPH_ERR_STATIC_LIMIT: return "more particles than the static scratch of sph_compute_static holds";
    default: return "unknown";
  }
}

int sph_selftest_staging(const void *src64, uint32_t *result, sph_stream_t stream) {
  if (!src64 || !result || ((uintptr_t)src64 & 15u)) return SPH_ERR_INVALID_ARGUMENT;
  k_selftest_staging<<<1, 32, 0, (cudaStream_t)stream>>>((const float4 *)src64, result);
  return check_launch();
}

const char *sph_status_bit_string(uint32_t bit) {
  switch (bit) {
    case SPH_STATUS_CELL_OVERFLOW: return "cell id past the reference grid (reference writes out of bounds)";
    case SPH_STATUS_GRID_COARSENED: return "search grid coarsened to fit the cell capacity";
    case SPH_STATUS_NONFINITE: return "non-finite position or h";
    case SPH_STATUS_GRID_TOO_LARGE: return "reference grid exceeds 2^30 cells per axis";
    case SPH_STATUS_NO_FLUID: return "no fluid particle";
    case SPH_STATUS_SMALL_DT: return "time step below 1e-6";
    case SPH_STATUS_STAGING_TIMEOUT: return "pair kernel staging wait timed out (evaluation incomplete)";
    default: return "unknown";
  }
}

int sph_initialize(sph_particles_t *pa, const sph_wcsph_t *w, const sph_config_t *cfg, sph_stream_t stream) {
  if (!particles_ok(pa) || !w || !cfg) return SPH_ERR_INVALID_ARGUMENT;
  if (pa->n == 0) return SPH_OK;
  launch_initialize(step_args(pa), *w, *cfg, (cudaStream_t)stream);
  return check_launch();
}

int sph_eos(sph_particles_t *pa, const sph_wcsph_t *w, sph_stream_t stream) {
  if (!particles_ok(pa) || !w) return SPH_ERR_INVALID_ARGUMENT;
  if (pa->n == 0) return SPH_OK;
  launch_eos(step_args(pa), *w, (cudaStream_t)stream);
  return check_launch();
}

int sph_kernel_eval(int kernel, int64_t n, const double *r, const double *h, double *out, sph_stream_t stream) {
  if ((kernel != SPH_KERNEL_CUBIC && kernel != SPH_KERNEL_GAUSSIAN && kernel != SPH_KERNEL_WENDLAND) || n < 0 ||
      (n && (!r || !h || !out)))
    return SPH_ERR_INVALID_ARGUMENT;
  if (n == 0) return SPH_OK;
  launch_kernel_map(kernel, 0, n, nullptr, r, h, out, (cudaStream_t)stream);
  return check_launch();
}

int sph_kernel_grad(int kernel, int64_t n, const double *x, const double *r, const double *h, double *out,
                    sph_stream_t stream) {
  if ((kernel != SPH_KERNEL_CUBIC && kernel != SPH_KERNEL_GAUSSIAN && kernel != SPH_KERNEL_WENDLAND) || n < 0 ||
      (n && (!x || !r || !h || !out)))
    return SPH_ERR_INVALID_ARGUMENT;
  if (n == 0) return SPH_OK;
  launch_kernel_map(kernel, 1, n, x, r, h, out, (cudaStream_t)stream);
  return check_launch();
}

int sph_gauss_deriv(int64_t n, const double *r, const double *h, double *out, sph_stream_t stream) {
  if (n < 0 || (n && (!r || !h || !out))) return SPH_ERR_INVALID_ARGUMENT;
  if (n == 0) return SPH_OK;
  launch_kernel_map(SPH_KERNEL_GAUSSIAN, 2, n, nullptr, r, h, out, (cudaStream_t)stream);
  return check_launch();
}

int sph_nn_update(const sph_particles_t *pa, const sph_config_t *cfg, const sph_workspace_t *ws,
                  sph_stream_t stream) {
  if (!particles_ok(pa) || !config_ok(cfg)) return SPH_ERR_INVALID_ARGUMENT;
  int e = ws_ok(ws, pa->n);
  if (e) return e;
  if (pa->n == 0) return SPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  StepArgs a = step_args(pa);
  WsPtrs w = ws_ptrs(ws);
  sph_wcsph_t wc;
  memset(&wc, 0, sizeof(wc));
  launch_bounds(a, w, *cfg, wc, kStageNone, false, nullptr, nullptr, st);
  launch_build(a, w, *cfg, wc, st);
  return check_launch();
}

int sph_nn_count(const sph_particles_t *pa, const sph_config_t *cfg, const sph_workspace_t *ws, int64_t *counts,
                 sph_stream_t stream) {
  if (!particles_ok(pa) || !config_ok(cfg) || (!counts && pa->n)) return SPH_ERR_INVALID_ARGUMENT;
  int e = ws_ok(ws, pa->n);
  if (e) return e;
  if (pa->n == 0) return SPH_OK;
  launch_nn_count(step_args(pa), ws_ptrs(ws), counts, nullptr, nullptr, (cudaStream_t)stream);
  return check_launch();
}

int sph_nn_export(const sph_particles_t *pa, const sph_config_t *cfg, const sph_workspace_t *ws,
                  const int64_t *offsets, int64_t *idx, sph_stream_t stream) {
  if (!particles_ok(pa) || !config_ok(cfg) || (pa->n && (!offsets || !idx))) return SPH_ERR_INVALID_ARGUMENT;
  int e = ws_ok(ws, pa->n);
  if (e) return e;
  if (pa->n == 0) return SPH_OK;
  launch_nn_count(step_args(pa), ws_ptrs(ws), nullptr, offsets, idx, (cudaStream_t)stream);
  return check_launch();
}

int sph_nn_probe_count(const sph_particles_t *pa, const sph_workspace_t *ws, int64_t np, const double *px,
                       const double *py, const double *ph, int64_t *counts, sph_stream_t stream) {
  if (!particles_ok(pa) || np < 0 || (np && (!px || !py || !ph || !counts))) return SPH_ERR_INVALID_ARGUMENT;
  int e = ws_ok(ws, pa->n);
  if (e) return e;
  if (np == 0) return SPH_OK;
  launch_nn_probe(step_args(pa), ws_ptrs(ws), np, px, py, ph, counts, nullptr, nullptr, nullptr, nullptr, nullptr,
                  (cudaStream_t)stream);
  return check_launch();
}

int sph_nn_probe_export(const sph_particles_t *pa, const sph_workspace_t *ws, int64_t np, const double *px,
                        const double *py, const double *ph, const int64_t *offsets, int64_t *idx, double *hij,
                        double *q, double *r, sph_stream_t stream) {
  if (!particles_ok(pa) || np < 0 || (np && (!px || !py || !ph || !offsets || !idx || !hij || !q || !r)))
    return SPH_ERR_INVALID_ARGUMENT;
  int e = ws_ok(ws, pa->n);
  if (e) return e;
  if (np == 0) return SPH_OK;
  launch_nn_probe(step_args(pa), ws_ptrs(ws), np, px, py, ph, nullptr, offsets, idx, hij, q, r, (cudaStream_t)stream);
  return check_launch();
}

int sph_probe_density(const sph_particles_t *pa, const sph_wcsph_t *w, int kernel, const sph_workspace_t *ws,
                      int64_t np, const double *px, const double *py, const double *h_search, const double *h_kernel,
                      double *rho, double *p, sph_stream_t stream) {
  if (!particles_ok(pa) || !w || np < 0 || (np && (!px || !py || !h_search || !h_kernel || !rho || !p)))
    return SPH_ERR_INVALID_ARGUMENT;
  if (kernel != SPH_KERNEL_CUBIC && kernel != SPH_KERNEL_GAUSSIAN && kernel != SPH_KERNEL_WENDLAND)
    return SPH_ERR_INVALID_ARGUMENT;
  int e = ws_ok(ws, pa->n);
  if (e) return e;
  if (np == 0) return SPH_OK;
  launch_probe_density(step_args(pa), ws_ptrs(ws), kernel, np, px, py, h_search, h_kernel, w->rho0, w->B, w->gamma,
                       rho, p, (cudaStream_t)stream);
  return check_launch();
}

static void compute_body(const StepArgs &a, const WsPtrs &w, const sph_wcsph_t &wc, const sph_config_t &cfg,
                         double *dt_out, double *dt_hist, cudaStream_t st, const WallLoad *wall = nullptr,
                         bool write_state = true) {
  const bool do_dt = dt_out != nullptr || dt_hist != nullptr;
  const RecParams rp = rec_params(cfg, wc, write_state, false, do_dt);
  launch_build(a, w, cfg, wc, st, &rp);
  if (wc.use_summation_density) {
    launch_sumdens(a, w, cfg, wc, st);
    launch_records(a, w, cfg, wc, false, true, false, st);
  }
  launch_pair(a, w, cfg, wc, dt_out, dt_hist, st, wall);
}

int sph_compute(sph_particles_t *pa, const sph_wcsph_t *w, const sph_config_t *cfg, const sph_workspace_t *ws,
                sph_stream_t stream) {
  if (!particles_ok(pa) || !w || !config_ok(cfg)) return SPH_ERR_INVALID_ARGUMENT;
  int e = ws_ok(ws, pa->n);
  if (e) return e;
  if (pa->n == 0) return SPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  StepArgs a = step_args(pa);
  WsPtrs wp = ws_ptrs(ws);
  launch_bounds(a, wp, *cfg, *w, kStageNone, true, nullptr, nullptr, st);
  compute_body(a, wp, *w, *cfg, nullptr, nullptr, st);
  return check_launch();
}

int sph_timestep(const sph_particles_t *pa, const sph_wcsph_t *w, const sph_config_t *cfg,
                 const sph_workspace_t *ws, double *dt3, sph_stream_t stream) {
  if (!particles_ok(pa) || !w || !config_ok(cfg) || !dt3) return SPH_ERR_INVALID_ARGUMENT;
  int e = ws_ok(ws, pa->n);
  if (e) return e;
  launch_timestep(step_args(pa), ws_ptrs(ws), *cfg, dt3, nullptr, (cudaStream_t)stream);
  return check_launch();
}

int sph_predict(sph_particles_t *pa, const sph_config_t *cfg, const double *dt, sph_stream_t stream) {
  if (!particles_ok(pa) || !config_ok(cfg) || !dt) return SPH_ERR_INVALID_ARGUMENT;
  if (pa->n == 0) return SPH_OK;
  launch_predict(step_args(pa), *cfg, dt, 0.0, (cudaStream_t)stream);
  return check_launch();
}

int sph_correct(sph_particles_t *pa, const sph_config_t *cfg, const double *dt, sph_stream_t stream) {
  if (!particles_ok(pa) || !config_ok(cfg) || !dt) return SPH_ERR_INVALID_ARGUMENT;
  if (pa->n == 0) return SPH_OK;
  launch_correct(step_args(pa), *cfg, dt, 0.0, (cudaStream_t)stream);
  return check_launch();
}

// Runs of at least this many steps step on the sorted copy of the state
// (when the workspace has room for it): the gather and scatter cost about a
// step's worth of memory traffic.
constexpr int64_t kShadowMinSteps = 4;

// Start of a run on the sorted copy: a neighbour build of the caller's state
// (its order only), then the gather; returns the copy's StepArgs and sets
// wp.orig.  Without room or for short runs, the caller's own arrays.
static StepArgs run_state(const StepArgs &a, WsPtrs &wp, const sph_config_t &cfg, const sph_wcsph_t &wc,
                          int64_t nsteps, cudaStream_t st) {
  if (nsteps < kShadowMinSteps || !wp.shadow) return a;
  launch_bounds(a, wp, cfg, wc, kStageNone, false, nullptr, nullptr, st);
  launch_build(a, wp, cfg, wc, st);
  const StepArgs b = shadow_args(wp, a.n);
  k_shadow_gather<<<nblocks(a.n), kBlock, 0, st>>>(a, b, wp.perm, wp.shadow_orig);
  wp.orig = wp.shadow_orig;
  return b;
}

static void run_finish(const StepArgs &a, const StepArgs &b, const WsPtrs &wp, cudaStream_t st) {
  if (!wp.orig) return;
  k_shadow_scatter<<<nblocks(a.n), kBlock, 0, st>>>(b, a, wp.orig);
}

// Whether step s of a run of nsteps writes p, c and the fluid h back to the
// state.  The first step does: the next bounds pass reads h.  The last does:
// the caller sees the state.  In between, with a fixed h and no summation
// density, no kernel of the run reads p or c (the pair records hold p from
// the EOS, the TimeStep takes c = co), and the values c = co and fluid
// h = h_fixed repeat what the first step wrote, so those steps skip the
// stores; the state after the run is the same.
static bool step_writes_state(const sph_wcsph_t &wc, const sph_config_t &cfg, int64_t s, int64_t nsteps) {
  const bool repeat = cfg.h_fixed > 0.0 && !wc.use_summation_density;
  return !repeat || s == 0 || s + 1 == nsteps;
}

int sph_run(sph_particles_t *pa, const sph_wcsph_t *w, const sph_config_t *cfg, const sph_workspace_t *ws,
            int64_t nsteps, double *dt_hist, sph_stream_t stream) {
  if (!particles_ok(pa) || !w || !config_ok(cfg) || nsteps < 0) return SPH_ERR_INVALID_ARGUMENT;
  int e = ws_ok(ws, pa->n);
  if (e) return e;
  if (pa->n == 0 || nsteps == 0) return SPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const StepArgs caller = step_args(pa);
  WsPtrs wp = ws_ptrs(ws);
  const StepArgs a = run_state(caller, wp, *cfg, *w, nsteps, st);
  const bool fixed = cfg->dt_fixed > 0.0;
  double *ring = &wp.ctrl->dt_ring[0][0];
  if (fixed) {
    if (dt_hist) k_fill_dt<<<nblocks(nsteps), kBlock, 0, st>>>(dt_hist, nsteps, cfg->dt_fixed);
  } else {
    launch_timestep(a, wp, *cfg, ring, dt_hist, st);
  }
  // the corrector of step s-1 and the predictor of step s run as one pass
  // in front of step s's neighbour build; the last corrector runs alone
  for (int64_t s = 0; s < nsteps; s++) {
    double *prev = ring + 3 * ((s + 1) & 1);
    double *cur = ring + 3 * (s & 1);
    double *nxt = ring + 3 * ((s + 1) & 1);
    launch_bounds(a, wp, *cfg, *w, s == 0 ? kStagePredict : kStageCorrectPredict, true, prev, cur, st);
    double *hist_next = (dt_hist && !fixed && s + 1 < nsteps) ? dt_hist + 3 * (s + 1) : nullptr;
    compute_body(a, wp, *w, *cfg, fixed ? nullptr : nxt, hist_next, st, nullptr,
                 step_writes_state(*w, *cfg, s, nsteps));
  }
  launch_correct(a, *cfg, ring + 3 * ((nsteps - 1) & 1), cfg->dt_fixed, st);
  run_finish(caller, a, wp, st);
  return check_launch();
}

// the differentiation form's constraints: fixed dt and h, PEC, no XSPH or
// summation density; the forward is FP64, the adjoint step FP64 or mixed
static bool adjoint_config_ok(const sph_wcsph_t *w, const sph_config_t *cfg, bool mixed_ok) {
  return cfg->dt_fixed > 0.0 && cfg->h_fixed > 0.0 && cfg->integrator == SPH_INTEGRATOR_PEC &&
         (cfg->precision == SPH_PREC_FP64 || (mixed_ok && cfg->precision == SPH_PREC_MIXED)) && !w->use_xsph &&
         !w->use_summation_density && !cfg->pec_use_xsph && cfg->damping == 0.0;
}

int sph_run_wall_load(sph_particles_t *pa, const sph_wcsph_t *w, const sph_config_t *cfg, const sph_workspace_t *ws,
                      int64_t nsteps, double wall_x, double *fr, double *load_hist, sph_stream_t stream) {
  if (!particles_ok(pa) || !w || !config_ok(cfg) || nsteps < 0 || !fr || !load_hist) return SPH_ERR_INVALID_ARGUMENT;
  if (!adjoint_config_ok(w, cfg, false)) return SPH_ERR_INVALID_ARGUMENT;
  int e = ws_ok(ws, pa->n);
  if (e) return e;
  if (pa->n == 0 || nsteps == 0) return SPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  StepArgs a = step_args(pa);
  WsPtrs wp = ws_ptrs(ws);
  double *ring = &wp.ctrl->dt_ring[0][0];
  WallLoad wall;
  wall.wall_x = wall_x;
  wall.fr = fr;
  if (cudaMemsetAsync(fr, 0, (size_t)pa->n * sizeof(double), st) != cudaSuccess) return SPH_ERR_CUDA;
  for (int64_t s = 0; s < nsteps; s++) {
    double *prev = ring + 3 * ((s + 1) & 1);
    double *cur = ring + 3 * (s & 1);
    launch_bounds(a, wp, *cfg, *w, s == 0 ? kStagePredict : kStageCorrectPredict, true, prev, cur, st);
    compute_body(a, wp, *w, *cfg, nullptr, nullptr, st, &wall);
    launch_sum_fixed(fr, a.n, load_hist + s, st);
  }
  launch_correct(a, *cfg, ring + 3 * ((nsteps - 1) & 1), cfg->dt_fixed, st);
  return check_launch();
}

int sph_adjoint_step(const sph_particles_t *pa, sph_particles_t *half, const sph_wcsph_t *w, const sph_config_t *cfg,
                     const sph_workspace_t *ws, const sph_adjoint_t *adj, sph_stream_t stream) {
  if (!particles_ok(pa) || !particles_ok(half) || half->n != pa->n || !w || !config_ok(cfg) || !adj)
    return SPH_ERR_INVALID_ARGUMENT;
  if (!adjoint_config_ok(w, cfg, true)) return SPH_ERR_INVALID_ARGUMENT;
  const double *need[] = {adj->xb, adj->yb, adj->vxb, adj->vyb, adj->rhob, adj->axb, adj->ayb, adj->drhob,
                          adj->alphab, adj->lax, adj->lay, adj->lad, adj->xhb, adj->yhb, adj->vxhb, adj->vyhb,
                          adj->rhohb, adj->alb};
  for (const double *q : need)
    if (!q) return SPH_ERR_INVALID_ARGUMENT;
  int e = ws_ok(ws, pa->n);
  if (e) return e;
  if (pa->n == 0) return SPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  launch_adjoint_step(step_args(const_cast<sph_particles_t *>(pa)), step_args(half), ws_ptrs(ws), *cfg, *w, *adj, st);
  return check_launch();
}

int sph_run_profiled(sph_particles_t *pa, const sph_wcsph_t *w, const sph_config_t *cfg, const sph_workspace_t *ws,
                     int64_t nsteps, double *stage_ms, sph_stream_t stream) {
  if (!particles_ok(pa) || !w || !config_ok(cfg) || nsteps < 0 || !stage_ms) return SPH_ERR_INVALID_ARGUMENT;
  int e = ws_ok(ws, pa->n);
  if (e) return e;
  for (int k = 0; k < SPH_NSTAGES; k++) stage_ms[k] = 0.0;
  if (pa->n == 0 || nsteps == 0) return SPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const StepArgs caller = step_args(pa);
  WsPtrs wp = ws_ptrs(ws);
  const StepArgs a = run_state(caller, wp, *cfg, *w, nsteps, st);
  const bool fixed = cfg->dt_fixed > 0.0;
  double *ring = &wp.ctrl->dt_ring[0][0];
  // one event after every stage, read after the run: mark[k] closes the
  // interval of stage tag[k] that began at mark[k - 1]
  std::vector<cudaEvent_t> mark;
  std::vector<int> tag;
  mark.reserve((size_t)(4 * nsteps + 3));
  bool ok = true;
  auto lap = [&](int stage) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
      ok = false;
      return;
    }
    cudaEventRecord(e, st);
    mark.push_back(e);
    tag.push_back(stage);
  };
  lap(-1);
  if (!fixed) launch_timestep(a, wp, *cfg, ring, nullptr, st);
  lap(SPH_STAGE_TIMESTEP);
  for (int64_t s = 0; s < nsteps; s++) {
    double *prev = ring + 3 * ((s + 1) & 1);
    double *cur = ring + 3 * (s & 1);
    double *nxt = ring + 3 * ((s + 1) & 1);
    launch_bounds(a, wp, *cfg, *w, s == 0 ? kStagePredict : kStageCorrectPredict, true, prev, cur, st);
    lap(SPH_STAGE_PREDICT);
    const RecParams rp = rec_params(*cfg, *w, step_writes_state(*w, *cfg, s, nsteps), false, !fixed);
    launch_build(a, wp, *cfg, *w, st, &rp);  // the records pass is fused into the build's last kernel
    lap(SPH_STAGE_BUILD);
    if (w->use_summation_density) {
      launch_sumdens(a, wp, *cfg, *w, st);
      launch_records(a, wp, *cfg, *w, false, true, false, st);
    }
    lap(SPH_STAGE_RECORDS);
    launch_pair(a, wp, *cfg, *w, fixed ? nullptr : nxt, nullptr, st);
    lap(SPH_STAGE_PAIR);
  }
  launch_correct(a, *cfg, ring + 3 * ((nsteps - 1) & 1), cfg->dt_fixed, st);
  run_finish(caller, a, wp, st);  // the copy back counts with the last corrector
  lap(SPH_STAGE_CORRECT);
  int rc = (ok && check_launch() == SPH_OK && cudaEventSynchronize(mark.back()) == cudaSuccess) ? SPH_OK : SPH_ERR_CUDA;
  for (size_t k = 1; rc == SPH_OK && k < mark.size(); k++) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, mark[k - 1], mark[k]) != cudaSuccess) rc = SPH_ERR_CUDA;
    stage_ms[tag[k]] += ms;
  }
  for (cudaEvent_t e : mark) cudaEventDestroy(e);
  return rc;
}

}  // extern "C"

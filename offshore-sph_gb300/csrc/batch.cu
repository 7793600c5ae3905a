// batch.cu -- C ABI of the batched form: many independent WCSPH instances
// (tanks of different sizes and resolutions) advanced together, every stage
// one launch over all instances, with per-instance grids, constants and
// Courant dt.  The device work is in nn_build.cu, pair.cu and integrate.cu
// (the k_bt_* kernels).
#include <stdint.h>
#include <string.h>

#include <vector>

#include "sph_internal.cuh"

namespace sph {

void launch_bt_bounds(const StepArgs &a, const WsPtrs &w, const BatchPtrs &B, const sph_config_t &cfg, int stage,
                      int prev, int cur, cudaStream_t st);
void launch_bt_build(const StepArgs &a, const WsPtrs &w, const BatchPtrs &B, cudaStream_t st);
void launch_bt_pair(const StepArgs &a, const WsPtrs &w, const BatchPtrs &B, int kernel, bool xsph, int tile_blocks,
                    cudaStream_t st);
void launch_bt_timestep(const StepArgs &a, const WsPtrs &w, const BatchPtrs &B, int slot, double *dt_hist,
                        cudaStream_t st);
void launch_bt_dt_finish(const WsPtrs &w, const BatchPtrs &B, int slot, double *dt_hist, cudaStream_t st);
void launch_bt_correct(const StepArgs &a, const BatchPtrs &B, const sph_config_t &cfg, int slot, cudaStream_t st);

// per-instance tables after the regular workspace
struct BatchLayout {
  size_t ip, sl, grids, coff, inst, tiles, scan, total;
};

static size_t align256b(size_t v) { return (v + 255) & ~(size_t)255; }

static BatchLayout make_batch_layout(long long n_cap, long long max_cells, long long n_inst) {
  BatchLayout L;
  size_t off = align256b(make_layout(n_cap, max_cells).total);
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align256b(off + bytes);
    return o;
  };
  const size_t ni = (size_t)(n_inst > 0 ? n_inst : 1), n = (size_t)(n_cap > 0 ? n_cap : 1);
  L.ip = take(ni * sizeof(InstParams));
  L.sl = take(ni * sizeof(InstSlots));
  L.grids = take(ni * sizeof(DevGrid));
  L.coff = take((ni + 1) * sizeof(int));
  L.inst = take(n * sizeof(int));
  L.tiles = take(((size_t)max_cells + ni) * sizeof(int2));
  L.scan = take(sizeof(DevGrid));
  L.total = off;
  return L;
}

static BatchPtrs batch_ptrs(const sph_workspace_t *ws, int n_inst) {
  const BatchLayout L = make_batch_layout(ws->n_cap, ws->max_cells, n_inst);
  char *b = (char *)ws->ptr;
  BatchPtrs B;
  B.ip = (InstParams *)(b + L.ip);
  B.sl = (InstSlots *)(b + L.sl);
  B.grids = (DevGrid *)(b + L.grids);
  B.coff = (int *)(b + L.coff);
  B.inst = (int *)(b + L.inst);
  B.tiles = (int2 *)(b + L.tiles);
  B.scan = (DevGrid *)(b + L.scan);
  B.n_inst = n_inst;
  return B;
}

// instance of every particle: the last instance whose range starts at or before it
__global__ void k_bt_inst(BatchPtrs B, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int lo = 0, hi = B.n_inst;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (B.ip[mid].off <= i) lo = mid;
    else hi = mid;
  }
  B.inst[i] = lo;
}

__global__ void k_bt_init_slots(BatchPtrs B) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < B.n_inst; b += gridDim.x * blockDim.x) {
    InstSlots &s = B.sl[b];
    s.xmin = s.ymin = s.hmin_all = s.pd_hmin = kEncMinId;
    s.xmax = s.ymax = s.hmax_new = s.pd_a2max = s.ts_cmax = kEncMaxId;
    s.pd_nfluid = 0;
    s.alias_count = 0;
    s.grid_key.set = 0;  // the instance has no grid yet
    for (int p = 0; p < 2; p++)
      for (int q = 0; q < 3; q++) s.dt_ring[p][q] = 0.0;
  }
}

}  // namespace sph

using namespace sph;

extern "C" {

int sph_batch_workspace_size(int64_t n_total, int64_t n_inst, int64_t max_cells, size_t *bytes) {
  if (!bytes || n_total < 0 || n_inst < 1 || n_inst > (1 << 20)) return SPH_ERR_INVALID_ARGUMENT;
  if (max_cells <= 0) max_cells = 2 * sph_default_max_cells(n_total) + 2 * n_inst;
  if (max_cells < 2 * n_inst || max_cells > 0x3fffffffll) return SPH_ERR_INVALID_ARGUMENT;
  *bytes = make_batch_layout(n_total, max_cells, n_inst).total;
  return SPH_OK;
}

int sph_batch_setup(const sph_workspace_t *ws, int64_t n_inst, const int64_t *offsets, const sph_wcsph_t *w,
                    const double *h_fixed, const sph_config_t *cfg, int32_t tile_shift_max, sph_stream_t stream) {
  if (!ws || !ws->ptr || !offsets || !w || !h_fixed || !cfg || n_inst < 1 || n_inst > (1 << 20))
    return SPH_ERR_INVALID_ARGUMENT;
  if (cfg->precision != SPH_PREC_MIXED || cfg->integrator != SPH_INTEGRATOR_PEC || cfg->dt_fixed > 0.0 ||
      cfg->pec_use_xsph || cfg->nn_scale <= 0.0 ||
      (cfg->kernel != SPH_KERNEL_CUBIC && cfg->kernel != SPH_KERNEL_GAUSSIAN && cfg->kernel != SPH_KERNEL_WENDLAND))
    return SPH_ERR_INVALID_ARGUMENT;
  if (ws->max_cells < 2 * n_inst || ws->bytes < make_batch_layout(ws->n_cap, ws->max_cells, n_inst).total)
    return SPH_ERR_WORKSPACE_TOO_SMALL;
  const long long N = offsets[n_inst];
  if (offsets[0] != 0 || N > ws->n_cap || N > 0x7fffffffll) return SPH_ERR_INVALID_ARGUMENT;
  for (int64_t b = 0; b < n_inst; b++) {
    if (offsets[b + 1] <= offsets[b] || !(h_fixed[b] > 0.0)) return SPH_ERR_INVALID_ARGUMENT;
    if (w[b].use_xsph || w[b].use_summation_density) return SPH_ERR_INVALID_ARGUMENT;
  }
  const int ts_own = tile_shift_max >= 0 && tile_shift_max <= 4 ? tile_shift_max : SPH_TILE_SHIFT_OWN;
  std::vector<InstParams> ip((size_t)n_inst);
  for (int64_t b = 0; b < n_inst; b++) {
    InstParams &p = ip[(size_t)b];
    memset(&p, 0, sizeof(p));
    const sph_wcsph_t &wc = w[b];
    p.off = offsets[b];
    p.n = offsets[b + 1] - offsets[b];
    RecParams &rp = p.rp;
    rp.h_fixed = h_fixed[b];
    rp.gamma = wc.gamma; rp.B = wc.B; rp.inv_rho0 = 1.0 / wc.rho0; rp.Pb = wc.Pb; rp.co = wc.co;
    rp.h_fixed_f = (float)h_fixed[b];
    rp.gamma_f = (float)wc.gamma;
    rp.B_f = (float)wc.B;
    rp.inv_rho0_f = (float)(1.0 / wc.rho0);
    rp.rho0_hi = (float)wc.rho0;
    rp.rho0_lo = (float)(wc.rho0 - (double)rp.rho0_hi);
    rp.Pb_f = (float)wc.Pb;
    rp.h_fixed_on = 1;
    rp.Pb_on = wc.Pb != 0.0 ? 1 : 0;
    rp.write_state = 1;
    rp.from_state = 0;
    rp.reduce_h = 1;
    PairParams &pp = p.pp;
    pp.alpha = wc.alpha; pp.beta = wc.beta; pp.co = wc.co; pp.eps = wc.epsilon;
    pp.r0 = wc.r0; pp.D = wc.D; pp.p1 = wc.p1; pp.p2 = wc.p2;
    pp.lj_42 = (wc.p1 == 4.0 && wc.p2 == 2.0) ? 1 : 0;
    pp.cfl_c = cfg->cfl_c; pp.cfl_f = cfg->cfl_f;
    pp.do_dt = 1;
    pp.n = p.n;
    pp.wall_x = 0.0;
    pp.fr = nullptr;
    GridParams &gp = p.gp;
    gp.scale = cfg->nn_scale;
    gp.r0 = wc.r0;
    gp.kernel = cfg->kernel;
    // each instance's share of the cell capacity (its cells + its dump cell)
    gp.max_cells = (ws->max_cells - n_inst) * p.n / N;
    if (gp.max_cells < 1) gp.max_cells = 1;
    gp.ts_ref_max = SPH_TILE_SHIFT_REF;
    gp.ts_own_max = ts_own;
    gp.n = p.n;
    gp.ppc = 0.0;
    p.cfl_c = cfg->cfl_c;
    p.cfl_f = cfg->cfl_f;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const BatchPtrs B = batch_ptrs(ws, (int)n_inst);
  if (init_workspace(ws_ptrs(ws), st) != cudaSuccess) return SPH_ERR_CUDA;
  if (cudaMemcpyAsync(B.ip, ip.data(), ip.size() * sizeof(InstParams), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return SPH_ERR_CUDA;
  k_bt_inst<<<nblocks(N), kBlock, 0, st>>>(B, N);
  k_bt_init_slots<<<(unsigned)((n_inst + 255) / 256), 256, 0, st>>>(B);
  if (cudaStreamSynchronize(st) != cudaSuccess) return SPH_ERR_CUDA;
  return SPH_OK;
}

int64_t sph_batch_instance_cells(const sph_workspace_t *ws, int64_t n_inst, const int64_t *offsets, int64_t b) {
  if (!ws || !offsets || n_inst < 1 || b < 0 || b >= n_inst) return -1;
  const long long N = offsets[n_inst];
  if (N <= 0) return -1;
  long long mc = (ws->max_cells - n_inst) * (offsets[b + 1] - offsets[b]) / N;
  return mc < 1 ? 1 : mc;
}

int sph_batch_run(sph_particles_t *pa, const sph_config_t *cfg, const sph_workspace_t *ws, int64_t n_inst,
                  int64_t nsteps, double *dt_hist, int32_t tile_blocks, sph_stream_t stream) {
  if (!pa || pa->n < 0 || !cfg || !ws || !ws->ptr || n_inst < 1 || nsteps < 0) return SPH_ERR_INVALID_ARGUMENT;
  if (cfg->precision != SPH_PREC_MIXED || cfg->integrator != SPH_INTEGRATOR_PEC) return SPH_ERR_INVALID_ARGUMENT;
  if (pa->n > ws->n_cap) return SPH_ERR_WORKSPACE_TOO_SMALL;
  if (ws->bytes < make_batch_layout(ws->n_cap, ws->max_cells, n_inst).total) return SPH_ERR_WORKSPACE_TOO_SMALL;
  if (pa->n == 0 || nsteps == 0) return SPH_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const StepArgs a = step_args(pa);
  const WsPtrs wp = ws_ptrs(ws);
  const BatchPtrs B = batch_ptrs(ws, (int)n_inst);
  const long long ni = n_inst;
  launch_bt_timestep(a, wp, B, 0, dt_hist, st);
  for (int64_t s = 0; s < nsteps; s++) {
    const int prev = (int)((s + 1) & 1), cur = (int)(s & 1), nxt = (int)((s + 1) & 1);
    launch_bt_bounds(a, wp, B, *cfg, s == 0 ? kStagePredict : kStageCorrectPredict, prev, cur, st);
    launch_bt_build(a, wp, B, st);  // with the records
    launch_bt_pair(a, wp, B, cfg->kernel, false, tile_blocks, st);
    launch_bt_dt_finish(wp, B, nxt, (dt_hist && s + 1 < nsteps) ? dt_hist + 3 * ni * (s + 1) : nullptr, st);
  }
  launch_bt_correct(a, B, *cfg, (int)((nsteps - 1) & 1), st);
  return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

}  // extern "C"

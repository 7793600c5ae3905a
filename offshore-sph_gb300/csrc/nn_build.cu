// nn_build.cu -- neighbour build of the WCSPH step.
//
// Replaces NNLinkedList.update (src/Tools/NNLinkedList.py:37-39, 86-141):
// instead of per-cell linked lists it builds a cell-sorted permutation and a
// cell-start table with a one-digit counting sort over cell ids
// (histogram -> exclusive scan -> scatter -> in-cell rank by particle index,
// which makes the order deterministic).  The reference grid (origin, cell
// size, ncx, ncy, the x-overflow alias) is reproduced exactly; when its cells
// are much wider than the interaction radius the search runs on a finer grid
// of its own and filters candidates by the reference's 3x3 stencil.
#include <math.h>

#include "sph_internal.cuh"

namespace sph {

// ---------------------------------------------------------------------------
// Bounds (and, fused, the PEC predictor of Solver.run's step)
// ---------------------------------------------------------------------------
struct BoundsParams {
  double h_fixed;
  int h_reset;  // 1: hmax over the h the next _compute will set
  int predict;  // 1: PEC.predict the fluid particles first
  double dt_fixed;
  const double *dt;  // device dt when dt_fixed <= 0
  double inv_damp;   // 1 / (1 + 0.5 damping)
  int use_xsph, strict;
};

__global__ void __launch_bounds__(kBlock) k_bounds(StepArgs a, DevCtrl *ctrl, BoundsParams bp) {
  __shared__ unsigned long long red[32];
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long exmin = kEncMinId, exmax = kEncMaxId, eymin = kEncMinId, eymax = kEncMaxId;
  unsigned long long ehmin = kEncMinId, ehmax = kEncMaxId;
  bool bad = false;
  if (i < a.n) {
    int8_t lab = a.label[i];
    double x = a.x[i], y = a.y[i], h = a.h[i];
    double rho = a.rho[i];
    if (bp.predict && is_fluid(lab)) {
      // PEC.predict (src/Integrators/PEC.py:32-59)
      double dt = bp.dt_fixed > 0.0 ? bp.dt_fixed : bp.dt[0];
      double hdt = 0.5 * dt;
      double vx = a.vx[i], vy = a.vy[i];
      a.x0[i] = x;
      a.y0[i] = y;
      a.vx0[i] = vx;
      a.vy0[i] = vy;
      if (bp.use_xsph) {
        x = x + hdt * a.xsphx[i];
        y = y + hdt * a.xsphy[i];
      } else {
        x = x + hdt * vx;
        y = y + hdt * vy;
      }
      a.x[i] = x;
      a.y[i] = y;
      a.vx[i] = (vx + hdt * a.ax[i]) * bp.inv_damp;
      a.vy[i] = (vy + hdt * a.ay[i]) * bp.inv_damp;
      a.rho0[i] = rho;
      rho = rho + hdt * a.drho[i];
      if (bp.strict && rho < 0.0) rho = 0.0;
      a.rho[i] = rho;
    }
    double hn = (bp.h_reset && is_fluid(lab)) ? reset_h(bp.h_fixed, a.m[i], rho) : h;
    bad = !(isfinite(x) && isfinite(y) && isfinite(h));
    exmin = exmax = enc_d(x);
    eymin = eymax = enc_d(y);
    ehmin = enc_d(h);
    ehmax = enc_d(hn);
    if (bad) exmin = eymin = ehmin = kEncMinId, exmax = eymax = ehmax = kEncMaxId;
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&ctrl->status, (unsigned)SPH_STATUS_NONFINITE);
  unsigned long long v;
  v = block_reduce(exmin, MinU64(), kEncMinId, red);
  if (threadIdx.x == 0 && v != kEncMinId) atomicMin(&ctrl->xmin, v);
  v = block_reduce(exmax, MaxU64(), kEncMaxId, red);
  if (threadIdx.x == 0 && v != kEncMaxId) atomicMax(&ctrl->xmax, v);
  v = block_reduce(eymin, MinU64(), kEncMinId, red);
  if (threadIdx.x == 0 && v != kEncMinId) atomicMin(&ctrl->ymin, v);
  v = block_reduce(eymax, MaxU64(), kEncMaxId, red);
  if (threadIdx.x == 0 && v != kEncMaxId) atomicMax(&ctrl->ymax, v);
  v = block_reduce(ehmin, MinU64(), kEncMinId, red);
  if (threadIdx.x == 0 && v != kEncMinId) atomicMin(&ctrl->hmin_all, v);
  v = block_reduce(ehmax, MaxU64(), kEncMaxId, red);
  if (threadIdx.x == 0 && v != kEncMaxId) atomicMax(&ctrl->hmax_new, v);
}

void launch_bounds(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, int mode, const double *dt,
                   double dt_fixed, cudaStream_t st) {
  BoundsParams bp;
  bp.h_fixed = cfg.h_fixed;
  bp.h_reset = mode != kBoundsOnly ? 1 : 0;
  bp.predict = mode == kBoundsPredictPEC ? 1 : 0;
  bp.dt_fixed = dt_fixed;
  bp.dt = dt;
  bp.inv_damp = 1.0 / (1.0 + 0.5 * cfg.damping);
  bp.use_xsph = cfg.pec_use_xsph;
  bp.strict = cfg.pec_strict;
  k_bounds<<<nblocks(a.n), kBlock, 0, st>>>(a, w.ctrl, bp);
}

struct GridParams {
  double scale, r0;
  int kernel;
  long long max_cells;
};

// ---------------------------------------------------------------------------
// Grid: the reference grid (NNLinkedList.py:86-127) and the traversal grid.
// One thread; consumes and resets the bounds slots.
// ---------------------------------------------------------------------------
__global__ void k_grid(DevCtrl *ctrl, DevGrid *g, GridParams gp) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double xmin = dec_d(ctrl->xmin), xmax = dec_d(ctrl->xmax);
  double ymin = dec_d(ctrl->ymin), ymax = dec_d(ctrl->ymax);
  double hmin = dec_d(ctrl->hmin_all), hmax = dec_d(ctrl->hmax_new);
  ctrl->xmin = kEncMinId; ctrl->xmax = kEncMaxId; ctrl->ymin = kEncMinId; ctrl->ymax = kEncMaxId;
  ctrl->hmin_all = kEncMinId; ctrl->hmax_new = kEncMaxId;
  ctrl->alias_count = 0;
  unsigned status = 0;
  bool fin = isfinite(xmin) && isfinite(xmax) && isfinite(ymin) && isfinite(ymax) && isfinite(hmin) &&
             isfinite(hmax);
  if (!fin) {
    status |= SPH_STATUS_NONFINITE;
    xmin = ymin = 0.0; xmax = ymax = 1.0; hmin = hmax = 0.0;
  }
  // cell size (NNLinkedList.py:103-110): scale * min h, 1.0 below 1e-6
  double cs = __dmul_rn(hmin, gp.scale);
  if (cs < 1e-6) cs = 1.0;
  double cs1 = __ddiv_rn(1.0, cs);
  // number of cells (NNLinkedList.py:112-127): ceil(cs1 * (max - min)), at least 1
  double fx = ceil(__dmul_rn(cs1, __dsub_rn(xmax, xmin)));
  double fy = ceil(__dmul_rn(cs1, __dsub_rn(ymax, ymin)));
  if (fx < 1.0) fx = 1.0;
  if (fy < 1.0) fy = 1.0;
  bool huge = fx > (double)(1 << 30) || fy > (double)(1 << 30);
  if (huge) status |= SPH_STATUS_GRID_TOO_LARGE;
  long long ncx = huge ? (1ll << 30) : (long long)fx, ncy = huge ? (1ll << 30) : (long long)fy;
  g->xmin = xmin; g->xmax = xmax; g->ymin = ymin; g->ymax = ymax;
  g->cs = cs; g->inv_cs = cs1;
  g->ncx = ncx; g->ncy = ncy; g->ncells_ref = ncx * ncy;
  g->hmax = hmax;
  // interaction radius the pair kernels need: the kernel support (cubic 2h,
  // Gaussian 3h) and the Lennard-Jones reach min(r0, 3h)
  double kappa = gp.kernel == SPH_KERNEL_CUBIC ? 2.0 : 3.0;
  double R = fmax(kappa * hmax, fmin(gp.r0, 3.0 * hmax)) * (1.0 + 1e-6);
  double ext = fmax(xmax - xmin, ymax - ymin);
  R = fmax(R, fmax(ext * 1e-7, 1e-300));
  g->r_search = R;
  bool fitsA = !huge && (double)ncx * (double)ncy <= (double)gp.max_cells;
  if (fitsA && cs <= 1.5 * R) {
    g->mode = 0;
    g->ntx = (int)ncx;
    g->nty = (int)ncy;
    g->ncells = (int)(ncx * ncy);
    g->ox = xmin; g->oy = ymin; g->ct = cs; g->inv_ct = cs1;
    g->need_filter = 0;
    g->wide = 1;
  } else {
    double ct = R;
    double fnx = 1.0, fny = 1.0;
    bool fits = false;
    for (int it = 0; it < 64 && !fits; it++) {
      fnx = floor((xmax - xmin) / ct) + 1.0;
      fny = floor((ymax - ymin) / ct) + 1.0;
      fits = fnx * fny <= (double)gp.max_cells;
      if (!fits) {
        status |= SPH_STATUS_GRID_COARSENED;
        ct *= sqrt(fnx * fny / (double)gp.max_cells) * 1.05 + 1e-3;
      }
    }
    if (!fits) {  // one cell holding everything: exact, only slower
      ct = fmax(xmax - xmin, ymax - ymin) * 2.0 + R;
      fnx = fny = 1.0;
    }
    long long ntx = (long long)fnx, nty = (long long)fny;
    g->mode = 1;
    g->ntx = (int)ntx;
    g->nty = (int)nty;
    g->ncells = (int)(ntx * nty);
    g->ox = xmin; g->oy = ymin; g->ct = ct; g->inv_ct = 1.0 / ct;
    g->need_filter = (cs >= ct * (1.0 + 1e-9)) ? 0 : 1;
    int wd = (int)ceil(3.0 * hmax * (1.0 + 1e-6) / ct);
    g->wide = wd < 1 ? 1 : (wd > 1024 ? 1024 : wd);
  }
  g->valid = 1;
  if (status) atomicOr(&ctrl->status, status);
}

// ---------------------------------------------------------------------------
// Keys: reference cell, traversal cell, histogram
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_keys(const double *__restrict__ x, const double *__restrict__ y,
                                                 long long n, const DevGrid *__restrict__ gp, DevCtrl *ctrl,
                                                 int *__restrict__ keys, int2 *__restrict__ refcell,
                                                 unsigned int *__restrict__ counts) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool alias = false, overflow = false;
  if (i < n) {
    const DevGrid &g = *gp;
    double xi = x[i], yi = y[i];
    long long cx = ref_floor_div(xi, g.xmin, g.cs, g.inv_cs);
    long long cy = ref_floor_div(yi, g.ymin, g.cs, g.inv_cs);
    long long flat = cx + g.ncx * cy;
    overflow = !(cx >= 0 && cy >= 0 && flat < g.ncells_ref);
    alias = !overflow && cx == g.ncx;
    refcell[i] = make_int2(sat_i32(cx), sat_i32(cy));
    int key;
    if (overflow) {
      key = g.ncells;  // dump cell: never part of a stencil
    } else if (g.mode == 0) {
      key = (int)flat;
    } else {
      long long tx = (long long)floor((xi - g.ox) * g.inv_ct);
      long long ty = (long long)floor((yi - g.oy) * g.inv_ct);
      tx = tx < 0 ? 0 : (tx >= g.ntx ? g.ntx - 1 : tx);
      ty = ty < 0 ? 0 : (ty >= g.nty ? g.nty - 1 : ty);
      key = (int)(tx + (long long)g.ntx * ty);
    }
    keys[i] = key;
    atomicAdd(&counts[key], 1u);
  }
  unsigned am = __ballot_sync(0xffffffffu, alias);
  unsigned om = __ballot_sync(0xffffffffu, overflow);
  if ((threadIdx.x & 31) == 0) {
    if (am) atomicAdd(&ctrl->alias_count, (unsigned)__popc(am));
    if (om) atomicOr(&ctrl->status, (unsigned)SPH_STATUS_CELL_OVERFLOW);
  }
}

// ---------------------------------------------------------------------------
// Exclusive scan of counts[0 .. ncells] (ncells + 1 entries, the last is the
// dump cell) into cstart[0 .. ncells + 1].  Three phases over tiles of
// kScanTile cells; launch sizes depend only on the capacity.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_scan_tiles(const unsigned int *__restrict__ counts,
                                                       const DevGrid *__restrict__ g,
                                                       unsigned int *__restrict__ part) {
  __shared__ unsigned int red[32];
  long long m = (long long)g->ncells + 1;
  long long base = (long long)blockIdx.x * kScanTile;
  unsigned int s = 0;
  if (base < m) {
    for (int t = threadIdx.x; t < kScanTile; t += kBlock) {
      long long c = base + t;
      if (c < m) s += counts[c];
    }
  }
  s = block_reduce(s, AddU32(), 0u, red);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void __launch_bounds__(1024) k_scan_top(unsigned int *part, int nparts) {
  __shared__ unsigned int sh[1024];
  int per = (nparts + 1023) / 1024;
  int b = threadIdx.x * per;
  unsigned int loc = 0;
  for (int t = 0; t < per; t++)
    if (b + t < nparts) loc += part[b + t];
  sh[threadIdx.x] = loc;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    unsigned int v = threadIdx.x >= o ? sh[threadIdx.x - o] : 0u;
    __syncthreads();
    sh[threadIdx.x] += v;
    __syncthreads();
  }
  unsigned int run = sh[threadIdx.x] - loc;  // exclusive
  for (int t = 0; t < per; t++)
    if (b + t < nparts) {
      unsigned int v = part[b + t];
      part[b + t] = run;
      run += v;
    }
}

__global__ void __launch_bounds__(kBlock) k_scan_apply(const unsigned int *__restrict__ counts,
                                                       const DevGrid *__restrict__ g,
                                                       const unsigned int *__restrict__ part,
                                                       unsigned int *__restrict__ cstart) {
  __shared__ unsigned int sh[kBlock];
  constexpr int per = kScanTile / kBlock;  // 16 consecutive cells per thread
  long long m = (long long)g->ncells + 1;
  long long base = (long long)blockIdx.x * kScanTile;
  if (base >= m) return;
  long long c0 = base + (long long)threadIdx.x * per;
  unsigned int v[per];
  unsigned int loc = 0;
#pragma unroll
  for (int t = 0; t < per; t++) {
    v[t] = (c0 + t < m) ? counts[c0 + t] : 0u;
    loc += v[t];
  }
  sh[threadIdx.x] = loc;
  __syncthreads();
  for (int o = 1; o < kBlock; o <<= 1) {
    unsigned int u = threadIdx.x >= o ? sh[threadIdx.x - o] : 0u;
    __syncthreads();
    sh[threadIdx.x] += u;
    __syncthreads();
  }
  unsigned int run = part[blockIdx.x] + sh[threadIdx.x] - loc;
#pragma unroll
  for (int t = 0; t < per; t++) {
    long long c = c0 + t;
    if (c < m) cstart[c] = run;
    run += v[t];
    if (c == m - 1) cstart[m] = run;
  }
}

// ---------------------------------------------------------------------------
// Scatter (counts return to zero) and in-cell rank by particle index
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_scatter(const int *__restrict__ keys, long long n,
                                                    unsigned int *__restrict__ counts,
                                                    const unsigned int *__restrict__ cstart,
                                                    int *__restrict__ perm_tmp, int *__restrict__ keys_sorted) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int key = keys[i];
  unsigned int old = atomicSub(&counts[key], 1u);
  unsigned int slot = cstart[key] + old - 1u;
  perm_tmp[slot] = (int)i;
  keys_sorted[slot] = key;
}

__global__ void __launch_bounds__(kBlock) k_cellsort(const int *__restrict__ perm_tmp,
                                                     const int *__restrict__ keys_sorted,
                                                     const unsigned int *__restrict__ cstart,
                                                     const int2 *__restrict__ refcell, long long n,
                                                     int *__restrict__ perm, int2 *__restrict__ meta) {
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int key = keys_sorted[k];
  unsigned int s = cstart[key], e = cstart[key + 1];
  int v = perm_tmp[k];
  unsigned int rank = 0;
  for (unsigned int t = s; t < e; t++) rank += (unsigned)(perm_tmp[t] < v);
  perm[s + rank] = v;
  meta[s + rank] = refcell[v];
}

void launch_build(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc,
                  cudaStream_t st) {
  GridParams gp;
  gp.scale = cfg.nn_scale;
  gp.r0 = wc.r0;
  gp.kernel = cfg.kernel;
  gp.max_cells = w.max_cells;
  k_grid<<<1, 32, 0, st>>>(w.ctrl, w.grid, gp);
  unsigned nb = nblocks(a.n);
  k_keys<<<nb, kBlock, 0, st>>>(a.x, a.y, a.n, w.grid, w.ctrl, w.keys, w.refcell, w.counts);
  k_scan_tiles<<<(unsigned)w.n_parts, kBlock, 0, st>>>(w.counts, w.grid, w.scan_part);
  k_scan_top<<<1, 1024, 0, st>>>(w.scan_part, (int)w.n_parts);
  k_scan_apply<<<(unsigned)w.n_parts, kBlock, 0, st>>>(w.counts, w.grid, w.scan_part, w.cstart);
  k_scatter<<<nb, kBlock, 0, st>>>(w.keys, a.n, w.counts, w.cstart, w.perm_tmp, w.keys_sorted);
  k_cellsort<<<nb, kBlock, 0, st>>>(w.perm_tmp, w.keys_sorted, w.cstart, w.refcell, a.n, w.perm, w.meta);
}

// ---------------------------------------------------------------------------
// Sorted pair records.  The h reset and the Tait EOS of _loop's first pass
// (SolverTools.py:122-127) are fused here; p, c and the fluid h go back to
// the caller's arrays.  Non-fluid records carry h with the sign bit set.
// ---------------------------------------------------------------------------
struct RecParams {
  double h_fixed, gamma, B, rho0, Pb, co;
  int write_state;  // write p, c, h to the caller's arrays
  int p_from_state; // take p from the caller's array (second pass of summation density)
  int mixed;
};

__device__ __forceinline__ void split_df(double v, float &hi, float &lo) {
  hi = __double2float_rn(v);
  lo = __double2float_rn(v - (double)hi);
}

__global__ void __launch_bounds__(kBlock) k_records(StepArgs a, const int *__restrict__ perm, RecParams rp,
                                                    double4_32a *__restrict__ recA64, double4_32a *__restrict__ recB64,
                                                    float4 *__restrict__ recP, float4 *__restrict__ recV,
                                                    float4 *__restrict__ recS) {
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  int i = perm[k];
  int8_t lab = a.label[i];
  bool fl = is_fluid(lab);
  double m = a.m[i], rho = a.rho[i], h = a.h[i];
  double x = a.x[i], y = a.y[i], vx = a.vx[i], vy = a.vy[i];
  if (fl) h = reset_h(rp.h_fixed, m, rho);
  double p = rp.p_from_state ? a.p[i] : tait_p(rho, lab, rp.gamma, rp.B, rp.rho0, rp.Pb);
  if (rp.write_state) {
    a.p[i] = p;
    a.c[i] = rp.co;
    if (fl) a.h[i] = h;
  }
  double othr = p / (rho * rho);
  double hs = fl ? h : -h;
  if (!fl && h == 0.0) hs = -0.0;
  if (!rp.mixed) {
    recA64[k] = make_double4_32a(x, y, vx, vy);
    recB64[k] = make_double4_32a(m, rho, othr, hs);
  } else {
    float xh, xl, yh, yl, vxh, vxl, vyh, vyl;
    split_df(x, xh, xl);
    split_df(y, yh, yl);
    split_df(vx, vxh, vxl);
    split_df(vy, vyh, vyl);
    recP[k] = make_float4(xh, yh, xl, yl);
    recV[k] = make_float4(vxh, vyh, vxl, vyl);
    recS[k] = make_float4((float)m, (float)rho, (float)othr, (float)hs);
  }
}

void launch_records(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc,
                    bool write_state, const double *rho_override, cudaStream_t st) {
  RecParams rp;
  rp.h_fixed = cfg.h_fixed;
  rp.gamma = wc.gamma; rp.B = wc.B; rp.rho0 = wc.rho0; rp.Pb = wc.Pb; rp.co = wc.co;
  rp.write_state = write_state ? 1 : 0;
  rp.p_from_state = rho_override ? 1 : 0;
  rp.mixed = cfg.precision == SPH_PREC_MIXED ? 1 : 0;
  k_records<<<nblocks(a.n), kBlock, 0, st>>>(a, w.perm, rp, (double4_32a *)w.recA, (double4_32a *)w.recB,
                                             (float4 *)w.recA, (float4 *)w.recB, (float4 *)w.recC);
}

}  // namespace sph

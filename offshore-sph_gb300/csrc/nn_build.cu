// nn_build.cu -- neighbour build of the WCSPH step.
//
// Replaces NNLinkedList.update (src/Tools/NNLinkedList.py:37-39, 86-141):
// instead of per-cell linked lists it builds a cell-sorted permutation and a
// cell-start table with a one-digit counting sort over cell ids
// (histogram -> exclusive scan -> scatter -> in-cell rank by particle index,
// which makes the order deterministic).
//
// The reference grid (origin, cell size, ncx, ncy, the x-overflow alias) is
// reproduced exactly.  Where that grid's 3x3 stencil can truncate pairs that
// contribute (its cells narrower than the interaction radius), the search runs
// on the reference cells themselves (mode 0).  Otherwise it runs on a grid of
// its own with cells of half the interaction radius and a 5x5 stencil
// (mode 1), which visits about 30% fewer candidates; candidates are then
// filtered by the reference's stencil only when the reference could truncate
// (aliased cells, or a grid coarsened to fit the cell capacity).
#include <math.h>

#include <string.h>

#include "sph_internal.cuh"

namespace sph {

// ---------------------------------------------------------------------------
// Bounds (and, fused, the PEC predictor of Solver.run's step)
// ---------------------------------------------------------------------------
struct BoundsParams {
  int stage;      // IntStage
  int h_reset;    // 1: hmax over the h the next _compute will set
  int h_fixed_on; // h_fixed > 0
  int dt_fixed_on;
  int damped;     // damping != 0
  int use_xsph, strict, euler, verlet;
  double h_fixed, dt_fixed;
  double inv_damp;  // 1 / (1 + 0.5 damping)
  double c0;        // 2 inv_damp - 1
  const double *dt_prev, *dt_cur;  // device dt of the previous / current step
};

// The integrator work in front of a neighbour build, on one particle (stored
// only when it is fluid): [the previous step's corrector: PEC.correct
// (src/Integrators/PEC.py:61-89) in its reduced form x0 + dt v, or
// Euler.correct (Euler.py:17-27)] then [this step's PEC.predict
// (PEC.py:32-59)].  Uniform conditions arrive as ints and the half step is
// an exponent decrement, so the FP64 pipe only sees the fused multiply-adds
// of the updates.  Every input is loaded before anything depends on the
// label, so a particle costs one memory round trip.
// The configuration is a compile-time form (integrator, stage, damping,
// XSPH), so that no path that a uniform flag switches off is if-converted
// into every particle's FP64 issue.
template <int INTEG, int STAGE, bool DAMPED, bool XSPH>
__device__ __forceinline__ void integrate_front(const StepArgs &a, long long i, const BoundsParams &bp, bool fl,
                                                double &x, double &y, double &rho) {
  constexpr bool cp = STAGE == kStageCorrectPredict;
  const double hdt = half_exact(bp.dt_fixed_on ? bp.dt_fixed : bp.dt_cur[0]);
  const double dtc = cp ? (bp.dt_fixed_on ? bp.dt_fixed : bp.dt_prev[0]) : 0.0;
  const double vxc = a.vx[i], vyc = a.vy[i];
  if constexpr (INTEG == SPH_INTEGRATOR_VERLET) {
    // [Verlet.correct (src/Integrators/Verlet.py:37-53): kick, second half
    // drift with the new velocity or XSPH] then [Verlet.predict (:28-35):
    // half drift]; the density is not integrated
    double vx = vxc, vy = vyc, nx = x, ny = y;
    if constexpr (cp) {
      const double axv = a.ax[i], ayv = a.ay[i];
      double xs = 0.0, ys = 0.0;
      if constexpr (XSPH) {
        xs = a.xsphx[i];
        ys = a.xsphy[i];
      }
      const double hc = half_exact(dtc);
      vx = fma(dtc, axv, vx);
      vy = fma(dtc, ayv, vy);
      nx = fma(hc, XSPH ? xs : vx, nx);
      ny = fma(hc, XSPH ? ys : vy, ny);
      if (fl) {
        a.vx[i] = vx;
        a.vy[i] = vy;
      }
    }
    nx = fma(hdt, vx, nx);
    ny = fma(hdt, vy, ny);
    if (fl) {
      a.x[i] = nx;
      a.y[i] = ny;
      x = nx;
      y = ny;
    }
    return;
  }
  const double axv = a.ax[i], ayv = a.ay[i], drho = a.drho[i];
  double x0 = 0.0, y0 = 0.0, vx0 = 0.0, vy0 = 0.0, rho0 = 0.0, xs = 0.0, ys = 0.0;
  if constexpr (cp && INTEG != SPH_INTEGRATOR_EULER) {
    x0 = a.x0[i];
    y0 = a.y0[i];
    vx0 = a.vx0[i];
    vy0 = a.vy0[i];
    rho0 = a.rho0[i];
  }
  if constexpr (XSPH && INTEG != SPH_INTEGRATOR_EULER) {
    xs = a.xsphx[i];
    ys = a.xsphy[i];
  }
  double nx = x, ny = y, nrho = rho, vx = vxc, vy = vyc;
  if constexpr (cp) {
    if constexpr (INTEG == SPH_INTEGRATOR_EULER) {
      const double hdt2 = half_exact(dtc * dtc);
      nx = fma(hdt2, axv, fma(dtc, vxc, x));
      ny = fma(hdt2, ayv, fma(dtc, vyc, y));
      vx = fma(dtc, axv, vxc);
      vy = fma(dtc, ayv, vyc);
      nrho = fma(dtc, drho, rho);
      if (fl) {
        a.x[i] = nx;
        a.y[i] = ny;
        a.vx[i] = vx;
        a.vy[i] = vy;
        a.rho[i] = nrho;
        x = nx;
        y = ny;
        rho = nrho;
      }
      return;  // Euler.predict is a no-op
    }
    nx = fma(dtc, XSPH ? xs : vxc, x0);
    ny = fma(dtc, XSPH ? ys : vyc, y0);
    if constexpr (DAMPED) {
      const double c1 = dtc * bp.inv_damp;
      vx = fma(c1, axv, bp.c0 * vx0);
      vy = fma(c1, ayv, bp.c0 * vy0);
    } else {
      vx = fma(dtc, axv, vx0);
      vy = fma(dtc, ayv, vy0);
    }
    nrho = fma(dtc, drho, rho0);
    if (bp.strict && negative_bits(nrho)) nrho = 0.0;
  }
  // PEC.predict with this step's dt
  double px, py;
  if constexpr (XSPH) {
    px = fma(hdt, xs, nx);
    py = fma(hdt, ys, ny);
  } else {
    px = fma(hdt, vx, nx);
    py = fma(hdt, vy, ny);
  }
  double nvx = fma(hdt, axv, vx), nvy = fma(hdt, ayv, vy);
  if constexpr (DAMPED) {
    nvx *= bp.inv_damp;
    nvy *= bp.inv_damp;
  }
  double prho = fma(hdt, drho, nrho);
  if (bp.strict && negative_bits(prho)) prho = 0.0;
  if (fl) {
    a.x0[i] = nx;
    a.y0[i] = ny;
    a.vx0[i] = vx;
    a.vy0[i] = vy;
    a.rho0[i] = nrho;
    a.x[i] = px;
    a.y[i] = py;
    a.vx[i] = nvx;
    a.vy[i] = nvy;
    a.rho[i] = prho;
    x = px;
    y = py;
    rho = prho;
  }
}

// One particle's part of k_bounds: the integrator work in front of the build
// and its six bound values (minima; maxima as minima of the complement),
// folded into v.
template <int INTEG, int STAGE, bool DAMPED, bool XSPH>
__device__ __forceinline__ void bounds_one(const StepArgs &a, long long i, const BoundsParams &bp,
                                           unsigned long long (&v)[6], bool &bad) {
  const int8_t lab = a.label[i];
  double x = a.x[i], y = a.y[i];
  const double h = a.h[i];
  const bool fl = is_fluid(lab);
  constexpr bool front = STAGE != kStageNone;
  const bool hcomp = bp.h_reset && !bp.h_fixed_on;
  double rho = (front || hcomp) ? a.rho[i] : 0.0;
  const double m = hcomp ? a.m[i] : 0.0;
  if constexpr (front) integrate_front<INTEG, STAGE, DAMPED, XSPH>(a, i, bp, fl, x, y, rho);
  double hn = h;
  if (fl && bp.h_reset) hn = bp.h_fixed_on ? bp.h_fixed : compute_h_call(m, rho);
  if (!(finite_bits(x) && finite_bits(y) && finite_bits(h))) {
    bad = true;
    return;
  }
  const unsigned long long ex = enc_d(x), ey = enc_d(y), eh = enc_d(h), en = ~enc_d(hn);
  v[0] = ex < v[0] ? ex : v[0];
  v[1] = ~ex < v[1] ? ~ex : v[1];
  v[2] = ey < v[2] ? ey : v[2];
  v[3] = ~ey < v[3] ? ~ey : v[3];
  v[4] = eh < v[4] ? eh : v[4];
  v[5] = en < v[5] ? en : v[5];
}

__device__ void grid_from_bounds(DevCtrl *ctrl, DevGrid *g, const GridParams &gp);

// Persistent grid-stride blocks (a few per SM), so that the block
// reductions end in few atomics on the shared bound slots.  The last block
// to finish sets the grid of the next build from the reduced bounds.
#ifndef SPH_BOUNDS_BLOCKS
#define SPH_BOUNDS_BLOCKS 4
#endif
constexpr int kBoundsBlocks = SPH_BOUNDS_BLOCKS;  // resident blocks per SM
template <int INTEG, int STAGE, bool DAMPED, bool XSPH>
__global__ void __launch_bounds__(kBlock, kBoundsBlocks) k_bounds(StepArgs a, DevCtrl *ctrl, BoundsParams bp,
                                                                  DevGrid *g, GridParams gp) {
  step_kernel_entry();
  __shared__ unsigned long long red[kBlock / 32][6];
  __shared__ bool last;
  unsigned long long v[6] = {kEncMinId, kEncMinId, kEncMinId, kEncMinId, kEncMinId, kEncMinId};
  bool bad = false;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride)
    bounds_one<INTEG, STAGE, DAMPED, XSPH>(a, i, bp, v, bad);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&ctrl->status, (unsigned)SPH_STATUS_NONFINITE);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 6; q++) {
    const unsigned long long m = warp_min_u64(v[q]);
    if (lane == 0) red[wid][q] = m;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    const int q = threadIdx.x;
    unsigned long long m = kEncMinId;
    for (int w = 0; w < kBlock / 32; w++) m = red[w][q] < m ? red[w][q] : m;
    if (m != kEncMinId) {
      unsigned long long *slot = &ctrl->xmin + q;  // xmin, xmax, ymin, ymax, hmin_all, hmax_new
      if (q & 1) atomicMax(slot, ~m);
      else atomicMin(slot, m);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&ctrl->bounds_done, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    ctrl->bounds_done = 0;
    grid_from_bounds(ctrl, g, gp);
  }
}

// Calls f.template operator()<INTEG, STAGE, DAMPED, XSPH>() for the compile-
// time form of bp (the combinations the integrators use).
template <typename F>
static void front_dispatch(const BoundsParams &bp, F &&f) {
  const bool d = bp.damped != 0, x = bp.use_xsph != 0;
  if (bp.stage == kStageNone) {
    f.template operator()<SPH_INTEGRATOR_PEC, kStageNone, false, false>();
  } else if (bp.euler) {  // Euler.predict is a no-op: only the corrector stage reaches here
    f.template operator()<SPH_INTEGRATOR_EULER, kStageCorrectPredict, false, false>();
  } else if (bp.verlet) {
    if (bp.stage == kStagePredict) {
      if (x) f.template operator()<SPH_INTEGRATOR_VERLET, kStagePredict, false, true>();
      else f.template operator()<SPH_INTEGRATOR_VERLET, kStagePredict, false, false>();
    } else {
      if (x) f.template operator()<SPH_INTEGRATOR_VERLET, kStageCorrectPredict, false, true>();
      else f.template operator()<SPH_INTEGRATOR_VERLET, kStageCorrectPredict, false, false>();
    }
  } else if (bp.stage == kStagePredict) {
    if (d) {
      if (x) f.template operator()<SPH_INTEGRATOR_PEC, kStagePredict, true, true>();
      else f.template operator()<SPH_INTEGRATOR_PEC, kStagePredict, true, false>();
    } else {
      if (x) f.template operator()<SPH_INTEGRATOR_PEC, kStagePredict, false, true>();
      else f.template operator()<SPH_INTEGRATOR_PEC, kStagePredict, false, false>();
    }
  } else {
    if (d) {
      if (x) f.template operator()<SPH_INTEGRATOR_PEC, kStageCorrectPredict, true, true>();
      else f.template operator()<SPH_INTEGRATOR_PEC, kStageCorrectPredict, true, false>();
    } else {
      if (x) f.template operator()<SPH_INTEGRATOR_PEC, kStageCorrectPredict, false, true>();
      else f.template operator()<SPH_INTEGRATOR_PEC, kStageCorrectPredict, false, false>();
    }
  }
}

static GridParams grid_params(const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc) {
  GridParams gp;
  gp.scale = cfg.nn_scale;
  gp.r0 = wc.r0;
  gp.kernel = cfg.kernel;
  gp.max_cells = w.max_cells;
  gp.ts_ref_max = SPH_TILE_SHIFT_REF;
  gp.ts_own_max = SPH_TILE_SHIFT_OWN;
  gp.n = 0;
  gp.ppc = 0.0;
  return gp;
}

void launch_bounds(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc, int stage,
                   bool h_reset, const double *dt_prev, const double *dt_cur, cudaStream_t st) {
  BoundsParams bp;
  bp.stage = stage;
  bp.euler = cfg.integrator == SPH_INTEGRATOR_EULER ? 1 : 0;
  bp.verlet = cfg.integrator == SPH_INTEGRATOR_VERLET ? 1 : 0;
  if (bp.euler && stage == kStagePredict) bp.stage = kStageNone;  // Euler.predict is a no-op
  bp.h_reset = h_reset ? 1 : 0;
  bp.h_fixed = cfg.h_fixed;
  bp.h_fixed_on = cfg.h_fixed > 0.0 ? 1 : 0;
  bp.dt_fixed = cfg.dt_fixed;
  bp.dt_fixed_on = cfg.dt_fixed > 0.0 ? 1 : 0;
  bp.dt_prev = dt_prev;
  bp.dt_cur = dt_cur;
  bp.inv_damp = 1.0 / (1.0 + 0.5 * cfg.damping);
  bp.c0 = 2.0 * bp.inv_damp - 1.0;
  bp.damped = cfg.damping != 0.0 ? 1 : 0;
  bp.use_xsph = cfg.pec_use_xsph;
  bp.strict = cfg.pec_strict;
  GridParams gp = grid_params(w, cfg, wc);
  gp.n = a.n;
  const unsigned nb = persist_blocks(a.n, kBoundsBlocks);
  front_dispatch(bp, [&]<int I, int S, bool D, bool X>() {
    launch_pdl(k_bounds<I, S, D, X>, dim3(nb), dim3(kBlock), 0, st, a, w.ctrl, bp, w.grid, gp);
  });
}


// ---------------------------------------------------------------------------
// Grid: the reference grid (NNLinkedList.py:86-127) and the traversal grid.
// One thread; consumes and resets the bounds slots, and sets the grids only
// when their inputs changed.
// ---------------------------------------------------------------------------
// Tile shift of the reference cells: the largest one whose halo (the 3 x 3
// stencil adds one cell on each side) holds, at the particles per cell the
// previous build saw, at most 85% of the pair kernel's shared-memory halo, so
// that tiles hold enough queries for a tile block without spilling to the
// global path.  Without a previous build on reference cells, 4 x 4 cells.
__device__ int ref_tile_shift(const GridParams &gp) {
  int ts_ref = gp.ts_ref_max < 2 ? gp.ts_ref_max : 2;
  if (gp.ppc > 0.0) {
    ts_ref = 0;
    for (int t = gp.ts_ref_max; t > 0; t--) {
      const double side = (double)((1 << t) + 2);
      if (gp.ppc * side * side <= 0.85 * SPH_HALO_CAP) {
        ts_ref = t;
        break;
      }
    }
  }
  return ts_ref;
}

// Both grids of one build from its bounds and h range, with the reference
// cells numbered in tiles of at most 2^ts_ref; returns status bits.
__device__ unsigned grid_setup(double xmin, double xmax, double ymin, double ymax, double hmin, double hmax,
                               const GridParams &gp, int ts_ref, DevGrid *g) {
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
  g->xminf = (float)xmin; g->yminf = (float)ymin; g->inv_csf = (float)cs1;
  g->hmax = hmax;
  // the mixed records compute h in FP32 (a few ulp from the FP64 value)
  g->hmaxf = __double2float_ru(hmax) * 1.00001f;
  // interaction radius: the kernel support (cubic 2h, Gaussian 3h) and the
  // Lennard-Jones reach min(r0, 3h)
  // support 2h (cubic spline, Wendland C4: zero with zero gradient at q = 2) or 3h (Gaussian)
  const bool cubic = gp.kernel != SPH_KERNEL_GAUSSIAN;
  double R = fmax((cubic ? 2.0 : 3.0) * hmax, fmin(gp.r0, 3.0 * hmax));
  double ext = fmax(xmax - xmin, ymax - ymin);
  R = fmax(R, fmax(ext * 1e-7, 1e-300));
  g->r_search = R;
  // the FP32 hi parts of the positions are truncated to 24 bits: a pair
  // distance formed from them is off by at most 2^-22 sqrt(2) max|coordinate|
  {
    const double amax = fmax(fmax(fabs(xmin), fabs(xmax)), fmax(fabs(ymin), fabs(ymax)));
    g->pad_e = (float)(1.5 * ldexp(amax, -22) + 1e-30);
  }
  // the cubic spline and its gradient vanish at q = 2, so pairs at exactly the
  // support radius contribute nothing; the Gaussian is cut at q <= 3 inclusive
  const bool trunc_free = cubic ? (cs >= R) : (cs >= R * (1.0 + 1e-9));
  // the largest tile shift (up to ts_max) whose padded cell count fits
  // (integer arithmetic: nx, ny are whole numbers below 2^31 here)
  auto tile_fit = [&](double nx, double ny, int ts_max, int &ts_out) {
    const unsigned long long ix = (unsigned long long)nx, iy = (unsigned long long)ny;
    for (int ts = ts_max; ts >= 0; ts--) {
      const unsigned long long T = 1ull << ts;
      const unsigned long long tx = (ix + T - 1) >> ts, ty = (iy + T - 1) >> ts;
      if (tx * ty <= ((unsigned long long)gp.max_cells >> (2 * ts))) {
        ts_out = ts;
        return true;
      }
    }
    return false;
  };
  int tsA = 0;
  const bool fitsA = !huge && tile_fit((double)ncx, (double)ncy, ts_ref, tsA);
  if (!trunc_free && fitsA) {
    g->mode = 0;
    g->ntx = (int)ncx;
    g->nty = (int)ncy;
    g->ts = tsA;
    g->ntlx = (int)((ncx + (1 << tsA) - 1) >> tsA);
    g->ncells = g->ntlx * (int)((ncy + (1 << tsA) - 1) >> tsA) << (2 * tsA);
    g->ct = cs;
    g->oxf = (float)xmin; g->oyf = (float)ymin; g->inv_ctf = (float)cs1;
    g->wt = 1;
    g->need_filter = 0;
    g->wide = 1;
  } else {
    // cells of R/2 with a 5x5 stencil; the margin covers the FP32 binning error
    const double amax = fmax(fmax(fabs(xmin), fabs(xmax)), fmax(fabs(ymin), fabs(ymax)));
    double ct = 0.5 * R;
    for (int it = 0; it < 2; it++) ct = 0.5 * R * (1.0 + 4.0 * (3e-7 * amax / ct) + 1e-5);
    double fnx = 1.0, fny = 1.0;
    bool fits = false;
    int ts = 0;
    for (int it = 0; it < 64 && !fits; it++) {
      fnx = floor((xmax - xmin) / ct) + 1.0;
      fny = floor((ymax - ymin) / ct) + 1.0;
      fits = tile_fit(fnx, fny, gp.ts_own_max, ts);
      if (!fits) {
        status |= SPH_STATUS_GRID_COARSENED;
        ct *= sqrt(fnx * fny / (double)gp.max_cells) * 1.05 + 1e-3;
      }
    }
    if (!fits) {  // one cell holding everything: exact, only slower
      ct = fmax(xmax - xmin, ymax - ymin) * 2.0 + R;
      fnx = fny = 1.0;
      ts = 0;
    }
    g->mode = 1;
    g->ntx = (int)fnx;
    g->nty = (int)fny;
    g->ts = ts;
    g->ntlx = (g->ntx + (1 << ts) - 1) >> ts;
    g->ncells = g->ntlx * ((g->nty + (1 << ts) - 1) >> ts) << (2 * ts);
    g->ct = ct;
    g->oxf = (float)xmin; g->oyf = (float)ymin; g->inv_ctf = (float)(1.0 / ct);
    g->wt = 2;
    g->need_filter = trunc_free ? 0 : 1;
    int wd = (int)ceil(3.0 * hmax * (1.0 + 1e-6) / ct) + 1;
    g->wide = wd < 2 ? 2 : (wd > 1024 ? 1024 : wd);
  }
  g->txmaxf = (float)(g->ntx - 1);
  g->tymaxf = (float)(g->nty - 1);
  g->valid = 1;
  return status;
}

// grid_setup, skipped when its inputs equal, bit for bit, those of the grid
// in use (key): a scene whose walls fix the bounds, at fixed h, keeps its
// grid from build to build.  Returns the status bits of the setup that made
// the grid.
__device__ unsigned grid_setup_keyed(double xmin, double xmax, double ymin, double ymax, double hmin, double hmax,
                                     const GridParams &gp, DevGrid *g, GridKey *key) {
  const int ts_ref = ref_tile_shift(gp);
  const unsigned long long b[6] = {(unsigned long long)__double_as_longlong(xmin),
                                   (unsigned long long)__double_as_longlong(xmax),
                                   (unsigned long long)__double_as_longlong(ymin),
                                   (unsigned long long)__double_as_longlong(ymax),
                                   (unsigned long long)__double_as_longlong(hmin),
                                   (unsigned long long)__double_as_longlong(hmax)};
  const unsigned long long scale = (unsigned long long)__double_as_longlong(gp.scale);
  const unsigned long long r0 = (unsigned long long)__double_as_longlong(gp.r0);
  const GridKey k = *key;  // all loads issued before the comparison
  bool same = (k.set == 1) & (k.ts_ref == ts_ref) & (k.kernel == gp.kernel) & (k.ts_own_max == gp.ts_own_max) &
              (k.max_cells == gp.max_cells) & (k.scale == scale) & (k.r0 == r0);
#pragma unroll
  for (int j = 0; j < 6; j++) same &= (k.b[j] == b[j]);
  if (same) return k.status;
  const unsigned status = grid_setup(xmin, xmax, ymin, ymax, hmin, hmax, gp, ts_ref, g);
#pragma unroll
  for (int j = 0; j < 6; j++) key->b[j] = b[j];
  key->scale = scale;
  key->r0 = r0;
  key->max_cells = gp.max_cells;
  key->kernel = gp.kernel;
  key->ts_ref = ts_ref;
  key->ts_own_max = gp.ts_own_max;
  key->status = status;
  key->set = 1;
  return status;
}

// The grid of the next build from the reduced bounds (one thread); the bound
// slots return to their identities.  Runs in the last block of k_bounds.
__device__ void grid_from_bounds(DevCtrl *ctrl, DevGrid *g, const GridParams &gp) {
  const double xmin = dec_d(__ldcg(&ctrl->xmin)), xmax = dec_d(__ldcg(&ctrl->xmax));
  const double ymin = dec_d(__ldcg(&ctrl->ymin)), ymax = dec_d(__ldcg(&ctrl->ymax));
  const double hmin = dec_d(__ldcg(&ctrl->hmin_all)), hmax = dec_d(__ldcg(&ctrl->hmax_new));
  // the previous build's listed tiles and grid, loaded with the bounds
  const unsigned int ntl = __ldcg(&ctrl->tl_count) + __ldcg(&ctrl->tl_back) + __ldcg(&ctrl->tl_heavy);
  const bool prev_ref = g->valid && g->mode == 0;
  const int prev_ts = g->ts;
  ctrl->xmin = kEncMinId; ctrl->xmax = kEncMaxId; ctrl->ymin = kEncMinId; ctrl->ymax = kEncMaxId;
  ctrl->hmin_all = kEncMinId; ctrl->hmax_new = kEncMaxId;
  ctrl->alias_count = 0;
  // particles per cell of the previous build's listed tiles (reference cells)
  GridParams q = gp;
  q.ppc = (prev_ref && ntl > 0u) ? (double)gp.n / ((double)ntl * (double)(1 << (2 * prev_ts))) : 0.0;
  ctrl->tl_count = 0;
  ctrl->tl_back = 0;
  ctrl->tl_heavy = 0;
  const unsigned status = grid_setup_keyed(xmin, xmax, ymin, ymax, hmin, hmax, q, g, &ctrl->grid_key);
  if (status) atomicOr(&ctrl->status, status);
}

// ---------------------------------------------------------------------------
// Keys: reference cell, traversal cell, histogram
// ---------------------------------------------------------------------------
// Traversal cell (tiled id; ncells = the dump cell) and raw reference cell of
// the position (xi, yi) on grid g.
__device__ __forceinline__ int cell_key(const DevGrid &g, double xi, double yi, int2 &ref, bool &alias,
                                        bool &overflow) {
  {
    const long long cx = ref_cell(xi, g.xmin, g.cs, g.inv_cs, g.xminf, g.inv_csf);
    const long long cy = ref_cell(yi, g.ymin, g.cs, g.inv_cs, g.yminf, g.inv_csf);
    const long long flat = cx + g.ncx * cy;
    overflow = !(cx >= 0 && cy >= 0 && flat < g.ncells_ref);
    alias = !overflow && cx == g.ncx;
    ref = make_int2(sat_i32(cx), sat_i32(cy));
    int key;
    if (overflow) {
      key = g.ncells;  // dump cell: never part of a stencil
    } else if (g.mode == 0) {
      int sx, sy;
      storage_cell((int)cx, (int)cy, g.ncx, sx, sy);
      key = tiled_key(sx, sy, g.ts, g.ntlx);
    } else {
      // FP32 binning, monotone in the position (query and candidates agree)
      float ft;
      const float tx = fminf(fmaxf((d2f_trunc(xi) - g.oxf) * g.inv_ctf, 0.f), g.txmaxf);
      const float ty = fminf(fmaxf((d2f_trunc(yi) - g.oyf) * g.inv_ctf, 0.f), g.tymaxf);
      if (g.ntx < (1 << 22) && g.nty < (1 << 22))
        key = tiled_key(floor_small(tx, ft), floor_small(ty, ft), g.ts, g.ntlx);
      else
        key = tiled_key(min(max((int)floorf(tx), 0), g.ntx - 1), min(max((int)floorf(ty), 0), g.nty - 1), g.ts,
                        g.ntlx);
    }
    return key;
  }
}

// Keys of the single-scene build: traversal and reference cells, the
// particle's arrival rank in its cell and the cell totals of the scan tiles.
// Lanes of a warp that share a cell (or a scan tile) take one atomic
// together, so most warps issue a handful.
__global__ void __launch_bounds__(kBlock) k_keys(const double *__restrict__ x, const double *__restrict__ y,
                                                 long long n, const DevGrid *__restrict__ gp, DevCtrl *ctrl,
                                                 int *__restrict__ keys, int2 *__restrict__ refcell,
                                                 unsigned int *__restrict__ crank, unsigned int *__restrict__ counts,
                                                 unsigned int *__restrict__ part, const int8_t *__restrict__ label,
                                                 unsigned int *__restrict__ tflag) {
  step_kernel_entry();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool act = i < n;
  bool alias = false, overflow = false;
  int key = -1 - lane;  // inactive lanes: keys that match no other lane
  if (act) {
    int2 ref;
    key = cell_key(*gp, x[i], y[i], ref, alias, overflow);
    refcell[i] = ref;
    keys[i] = key;
  }
  // A boundary particle marks its tile, which the pair kernel then claims
  // before the tiles of fluid alone (its queries next to the wall cost more).
  // One atomic per tile and warp: a wall's particles sit in few tiles, and
  // one atomic each would queue thousands on the same words.
  const bool wall = act && key < gp->ncells && !is_fluid(label[i]);
  if (__ballot_sync(0xffffffffu, wall)) {
    const int tl = wall ? key >> (2 * gp->ts) : -1;
    const unsigned int tpeers = __match_any_sync(0xffffffffu, tl);
    if (wall && lane == __ffs(tpeers) - 1) atomicOr(&tflag[tl >> 5], 1u << (tl & 31));
  }
  const unsigned int below = (1u << lane) - 1u;
  const unsigned int peers = __match_any_sync(0xffffffffu, key);
  const int leader = __ffs(peers) - 1;
  unsigned int base = 0;
  if (act && lane == leader) base = atomicAdd(&counts[key], (unsigned int)__popc(peers));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (act) crank[i] = base + (unsigned int)__popc(peers & below);
  const int pt = act ? key / kScanTile : -1 - lane;
  const unsigned int tpeers = __match_any_sync(0xffffffffu, pt);
  if (act && lane == __ffs(tpeers) - 1) atomicAdd(&part[pt], (unsigned int)__popc(tpeers));
  const unsigned am = __ballot_sync(0xffffffffu, alias);
  const unsigned om = __ballot_sync(0xffffffffu, overflow);
  if (lane == 0) {
    if (am) atomicAdd(&ctrl->alias_count, (unsigned)__popc(am));
    if (om) atomicOr(&ctrl->status, (unsigned)SPH_STATUS_CELL_OVERFLOW);
  }
}

// ---------------------------------------------------------------------------
// Exclusive scan of counts[0 .. ncells] (ncells + 1 entries, the last is the
// dump cell) into cstart[0 .. ncells + 1], in one pass over tiles of
// kScanTile cells; launch sizes depend only on the capacity.
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanPer = kScanTile / kScanThreads;  // 16 cells (four uint4) per thread
static_assert(kScanPer == 16, "four uint4 of counts per thread");

// The single-scene scan: one block per scan tile, whose offset is the sum of
// the totals of tiles 0 .. t-1 (counted by k_keys), so one pass writes
// cstart.  Small blocks (all of them resident at once on the GPU) with two
// barriers each; a tile that holds no particle skips its counts and writes
// its offset.
__global__ void __launch_bounds__(kScanThreads) k_scan_cells(const unsigned int *__restrict__ counts,
                                                             const DevGrid *__restrict__ g,
                                                             const unsigned int *__restrict__ part,
                                                             unsigned int *__restrict__ cstart) {
  step_kernel_entry();
  __shared__ unsigned int warp_tot[kScanThreads / 32];
  __shared__ unsigned int warp_pre[kScanThreads / 32];
  const long long m = (long long)g->ncells + 1;
  const long long t = blockIdx.x;
  if (t * kScanTile >= m) return;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const long long c0 = t * kScanTile + (long long)threadIdx.x * kScanPer;
  const bool empty = part[t] == 0u;
  unsigned int v[kScanPer];
#pragma unroll
  for (int u = 0; u < kScanPer; u++) v[u] = 0u;
  if (!empty) {
    if (c0 + kScanPer <= m) {
#pragma unroll
      for (int q = 0; q < kScanPer / 4; q++) {
        const uint4 w = *(const uint4 *)(counts + c0 + 4 * q);
        v[4 * q] = w.x; v[4 * q + 1] = w.y; v[4 * q + 2] = w.z; v[4 * q + 3] = w.w;
      }
    } else {
#pragma unroll
      for (int u = 0; u < kScanPer; u++) v[u] = (c0 + u < m) ? counts[c0 + u] : 0u;
    }
  }
  // the totals of the earlier tiles
  unsigned int pre = 0;
  for (long long q = threadIdx.x; q < t; q += kScanThreads) pre += part[q];
  pre = __reduce_add_sync(0xffffffffu, pre);
  unsigned int loc = 0;
#pragma unroll
  for (int u = 0; u < kScanPer; u++) loc += v[u];
  unsigned int inc = loc;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned int x = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += x;
  }
  if (lane == 31) {
    warp_tot[wid] = inc;
    warp_pre[wid] = pre;
  }
  __syncthreads();
  unsigned int run = inc - loc;
#pragma unroll
  for (int w = 0; w < kScanThreads / 32; w++) {
    if (w < wid) run += warp_tot[w];
    run += warp_pre[w];
  }
  unsigned int r[kScanPer + 1];
  r[0] = run;
#pragma unroll
  for (int u = 0; u < kScanPer; u++) r[u + 1] = r[u] + v[u];
  if (c0 + kScanPer <= m) {
#pragma unroll
    for (int q = 0; q < kScanPer / 4; q++)
      *(uint4 *)(cstart + c0 + 4 * q) = make_uint4(r[4 * q], r[4 * q + 1], r[4 * q + 2], r[4 * q + 3]);
  } else {
#pragma unroll
    for (int u = 0; u < kScanPer; u++)
      if (c0 + u < m) cstart[c0 + u] = r[u];
  }
  if (c0 <= m - 1 && m - 1 < c0 + kScanPer) {
#pragma unroll
    for (int u = 0; u < kScanPer; u++)
      if (c0 + u == m - 1) cstart[m] = r[u + 1];  // total
  }
}

// Single-scene scatter: each particle to its cell's range at its arrival
// rank (no atomics); cell counters and scan-tile totals return to zero.
__global__ void __launch_bounds__(kBlock) k_scatter_rank(const int *__restrict__ keys,
                                                         const unsigned int *__restrict__ crank, long long n,
                                                         unsigned int *__restrict__ counts,
                                                         const unsigned int *__restrict__ cstart,
                                                         int *__restrict__ perm_tmp, int *__restrict__ keys_sorted,
                                                         unsigned int *__restrict__ part, long long n_parts) {
  step_kernel_entry();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (long long t = i; t < n_parts; t += (long long)gridDim.x * blockDim.x) part[t] = 0u;
  if (i >= n) return;
  const int key = keys[i];
  const unsigned int slot = cstart[key] + crank[i];
  perm_tmp[slot] = (int)i;
  keys_sorted[slot] = key;
  counts[key] = 0u;
}

// ---------------------------------------------------------------------------
// Pair records and in-cell rank by particle index
// ---------------------------------------------------------------------------
// The mixed form's records of slot k (particle i): FP32 pair records, the h
// reset and the Tait EOS on the relative density (no FP64 arithmetic); p, c
// and the fluid h go back to the caller's arrays when asked.  eh / nf: the
// fluid h for the TimeStep reduction.
// HSRC: where the fluid h and p come from (kHState: the caller's arrays, the
// second summation-density pass; kHFixed: the fixed h; kHCompute: computeH
// in FP32); PB: a nonzero background pressure.  Compile-time, so that the
// paths a run does not take are not if-converted into every particle.
enum { kHState = 0, kHFixed = 1, kHCompute = 2 };
template <int HSRC, bool PB>
__device__ __forceinline__ void record_mixed_t(const StepArgs &a, long long k, int i, const RecParams &rp,
                                               float4 *__restrict__ rec0, float4 *__restrict__ rec1,
                                               float4 *__restrict__ rec2, unsigned long long &eh,
                                               unsigned int &nf) {
  const int8_t lab = a.label[i];
  const bool fl = is_fluid(lab);
  const double m = a.m[i], rho = a.rho[i];
  const double x = a.x[i], y = a.y[i];
  float xh, xl, yh, yl;
  split_df(x, xh, xl);
  split_df(y, yh, yl);
  const float mf = d2f_trunc(m);
  // FP32 pair record; EOS on the relative density (no FP64 arithmetic)
  float rh, rl;
  split_df(rho, rh, rl);
  float hf;
  double hd;
  if (HSRC == kHState || !fl) {
    hd = a.h[i];
    hf = d2f_trunc(hd);
  } else if (HSRC == kHFixed) {
    hd = rp.h_fixed;
    hf = rp.h_fixed_f;
  } else {
    hf = rh > 1e-12f ? 1.3f * sqrtf(mf / rh) : 0.f;  // computeH in FP32
    hd = f2d(hf);
  }
  float pf;  // gauge pressure B ((rho/rho0)^gamma - 1), FP32
  double pd;
  if constexpr (HSRC == kHState) {
    pd = a.p[i];
    pf = d2f_trunc(pd) - rp.Pb_f;
  } else {
    const float d = ((rh - rp.rho0_hi) + (rl - rp.rho0_lo)) * rp.inv_rho0_f;
    pf = fl ? rp.B_f * tait_ratio_m1_f(d, rp.gamma_f) : 0.f;
    pd = f2d(pf);
    if constexpr (PB) pd += rp.Pb;
  }
  const float ir = rh != 0.f ? __frcp_rn(rh) : 0.f;
  const float othr = (pf + rp.Pb_f) * ir * ir;
  rec0[k] = make_float4(xh, yh, fl ? hf : -hf, mf);
  rec1[k] = make_float4(xl, yl, rh, othr);
  float vxh, vxl, vyh, vyl;
  split_df(a.vx[i], vxh, vxl);
  split_df(a.vy[i], vyh, vyl);
  rec2[k] = make_float4(vxh, vyh, vxl, vyl);
  if (rp.write_state) {
    a.p[i] = pd;
    a.c[i] = rp.co;
    if (fl) a.h[i] = hd;
  }
  if (fl) {
    const unsigned long long e = enc_d(hd);
    eh = e < eh ? e : eh;
    nf++;
  }
}

// record_mixed_t for the flags of rp (runtime form)
__device__ __forceinline__ void record_mixed(const StepArgs &a, long long k, int i, const RecParams &rp,
                                             float4 *__restrict__ rec0, float4 *__restrict__ rec1,
                                             float4 *__restrict__ rec2, unsigned long long &eh, unsigned int &nf) {
  if (rp.from_state) {
    if (rp.Pb_on) record_mixed_t<kHState, true>(a, k, i, rp, rec0, rec1, rec2, eh, nf);
    else record_mixed_t<kHState, false>(a, k, i, rp, rec0, rec1, rec2, eh, nf);
  } else if (rp.h_fixed_on) {
    if (rp.Pb_on) record_mixed_t<kHFixed, true>(a, k, i, rp, rec0, rec1, rec2, eh, nf);
    else record_mixed_t<kHFixed, false>(a, k, i, rp, rec0, rec1, rec2, eh, nf);
  } else {
    if (rp.Pb_on) record_mixed_t<kHCompute, true>(a, k, i, rp, rec0, rec1, rec2, eh, nf);
    else record_mixed_t<kHCompute, false>(a, k, i, rp, rec0, rec1, rec2, eh, nf);
  }
}

// The FP64 form's records of slot k (particle i), the reference's arithmetic.
__device__ __forceinline__ void record_fp64(const StepArgs &a, long long k, int i, const RecParams &rp,
                                            float4 *__restrict__ rec0, double4_32a *__restrict__ r64a,
                                            double4_32a *__restrict__ r64b, unsigned long long &eh,
                                            unsigned int &nf) {
  const int8_t lab = a.label[i];
  const bool fl = is_fluid(lab);
  const double m = a.m[i], rho = a.rho[i];
  const double x = a.x[i], y = a.y[i];
  float xh, xl, yh, yl;
  split_df(x, xh, xl);
  split_df(y, yh, yl);
  const float mf = d2f_trunc(m);
  double h = a.h[i];
  if (fl && !rp.from_state) h = rp.h_fixed_on ? rp.h_fixed : compute_h_call(m, rho);
  const double p = rp.from_state ? a.p[i] : tait_p(rho, lab, rp.gamma, rp.B, rp.inv_rho0, rp.Pb);
  const double othr = p / (rho * rho);
  const double hs = fl ? h : -h;
  r64a[k] = make_double4_32a(x, y, a.vx[i], a.vy[i]);
  r64b[k] = make_double4_32a(m, rho, othr, (!fl && h == 0.0) ? -0.0 : hs);
  const float hf = d2f_trunc(h);
  rec0[k] = make_float4(xh, yh, fl ? hf : -hf, mf);
  if (rp.write_state) {
    a.p[i] = p;
    a.c[i] = rp.co;
    if (fl) a.h[i] = h;
  }
  if (fl) {
    const unsigned long long e = enc_d(h);
    eh = e < eh ? e : eh;
    nf++;
  }
}

// Block minimum of the fluid h and count of fluid particles into the step's
// TimeStep slots (all threads call it).
__device__ __forceinline__ void reduce_h_block(unsigned long long eh, unsigned int nf, unsigned long long *red,
                                               unsigned int *redn, DevCtrl *ctrl) {
  const unsigned long long wm = warp_min_u64(eh);
  const unsigned int wn = __reduce_add_sync(0xffffffffu, nf);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    red[wid] = wm;
    redn[wid] = wn;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long bh = kEncMinId;
    unsigned int bn = 0;
    for (int w = 0; w < kBlock / 32; w++) {
      bh = red[w] < bh ? red[w] : bh;
      bn += redn[w];
    }
    if (bn) {
      atomicMin(&ctrl->pd_hmin, bh);
      atomicAdd(&ctrl->pd_nfluid, bn);
    }
  }
}

// Rank of a slot's particle among the members of its cell, by particle
// index (ov; all lanes call it, inactive lanes with a key that matches no
// other lane), for the batched build.  A cell's members sit in consecutive
// slots, so most cells lie inside one warp: its lanes compare the indices
// they already hold.  outside_cell_rank adds the members of a cell [s, e)
// that lie outside the warp's slots [k0, k0 + 32), loaded again.
__device__ __forceinline__ unsigned int warp_cell_rank(int key, int ov) {
  const unsigned int peers = __match_any_sync(0xffffffffu, key);
  const int first = __ffs(peers) - 1, cnt = __popc(peers);
  const int span = (int)__reduce_max_sync(0xffffffffu, (unsigned)cnt);
  unsigned int rank = 0;
  for (int d = 0; d < span; d++) {
    const int o = __shfl_sync(0xffffffffu, ov, min(first + d, 31));
    rank += (unsigned)(d < cnt && o < ov);
  }
  return rank;
}

__device__ __forceinline__ unsigned int outside_cell_rank(unsigned int s, unsigned int e, unsigned int k0, int ov,
                                                          const int *__restrict__ perm_tmp) {
  unsigned int rank = 0;
  if (s < k0 || e > k0 + 32u) {
    for (unsigned int t = s; t < k0; t++) rank += (unsigned)(perm_tmp[t] < ov);
    for (unsigned int t = k0 + 32u; t < e; t++) rank += (unsigned)(perm_tmp[t] < ov);
  }
  return rank;
}

// In-cell order by particle index (deterministic); the first particle of each
// non-empty tile also lists its tile for the tile pair kernel.  With REC the
// same thread then writes the pair records of its final slot (the records
// pass fused in: kRecMixed FP32 records, kRecFp64 FP64 records).
enum { kRecNone = 0, kRecMixed = 1, kRecFp64 = 2 };
template <int REC, int HSRC = kHFixed, bool PB = false>
__global__ void __launch_bounds__(kBlock) k_cellsort(const int *__restrict__ perm_tmp,
                                                     const int *__restrict__ keys_sorted,
                                                     const unsigned int *__restrict__ cstart,
                                                     const int2 *__restrict__ refcell, long long n,
                                                     const DevGrid *__restrict__ gp, DevCtrl *ctrl,
                                                     int *__restrict__ perm, int2 *__restrict__ meta,
                                                     int *__restrict__ tiles, StepArgs a, RecParams rp,
                                                     float4 *__restrict__ rec0, float4 *__restrict__ rec1,
                                                     float4 *__restrict__ rec2, double4_32a *__restrict__ r64a,
                                                     double4_32a *__restrict__ r64b, const int *__restrict__ orig,
                                                     unsigned int tiles_cap, int *__restrict__ tiles_h,
                                                     unsigned int *__restrict__ tflag) {
  step_kernel_entry();
  __shared__ unsigned long long red[kBlock / 32];
  __shared__ unsigned int redn[kBlock / 32];
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long eh = kEncMinId;
  unsigned int nf = 0;
  if (k < n) {
    const int key = keys_sorted[k];
    const unsigned int s = cstart[key], e = cstart[key + 1];
    const int ts2 = 2 * gp->ts;
    if (key < gp->ncells && (unsigned)k == __ldg(&cstart[(key >> ts2) << ts2])) {
      // The pair kernel claims the tiles list by list, in list order, so
      // that it ends on the cheap ones: first the dense tiles (at least one
      // particle per cell) that hold a boundary particle, whose queries next
      // to the wall cost about twice the others; then the other dense tiles
      // (front of the tile list); then the sparse ones (its back).  The
      // tile's boundary bit (set by k_keys) returns to zero here.
      const int tl = key >> ts2;
      const unsigned int tbit = 1u << (tl & 31);
      const bool wall = (tflag[tl >> 5] & tbit) != 0u;
      if (wall) atomicAnd(&tflag[tl >> 5], ~tbit);
      const unsigned int te = __ldg(&cstart[(tl + 1) << ts2]);
      if (te - (unsigned)k >= (1u << ts2)) {
        if (wall) tiles_h[atomicAdd(&ctrl->tl_heavy, 1u)] = tl;
        else tiles[atomicAdd(&ctrl->tl_count, 1u)] = tl;
      } else {
        tiles[tiles_cap - 1 - atomicAdd(&ctrl->tl_back, 1u)] = tl;
      }
    }
    const int v = perm_tmp[k];
    // rank inside the cell by particle index: the caller's index when the
    // run steps on the sorted copy of the state (orig), so that the order,
    // and with it every sum, is the same as on the caller's arrays.  (The
    // batched form's warp-shuffle rank measured slower here: build stage
    // 70.6 against 69.2 us on the 1M-fluid dam break.)
    unsigned int rank = 0;
    if (orig) {
      const int ov = orig[v];
      for (unsigned int t = s; t < e; t++) rank += (unsigned)(orig[perm_tmp[t]] < ov);
    } else {
      for (unsigned int t = s; t < e; t++) rank += (unsigned)(perm_tmp[t] < v);
    }
    const unsigned int slot = s + rank;
    perm[slot] = v;
    meta[slot] = refcell[v];
    if (REC == kRecMixed) record_mixed_t<HSRC, PB>(a, slot, v, rp, rec0, rec1, rec2, eh, nf);
    if (REC == kRecFp64) record_fp64(a, slot, v, rp, rec0, r64a, r64b, eh, nf);
  }
  if (REC != kRecNone && rp.reduce_h) reduce_h_block(eh, nf, red, redn, ctrl);
}

RecParams rec_params(const sph_config_t &cfg, const sph_wcsph_t &wc, bool write_state, bool p_from_state,
                     bool reduce_h) {
  RecParams rp;
  rp.h_fixed = cfg.h_fixed;
  rp.gamma = wc.gamma; rp.B = wc.B; rp.inv_rho0 = 1.0 / wc.rho0; rp.Pb = wc.Pb; rp.co = wc.co;
  rp.h_fixed_f = (float)cfg.h_fixed;
  rp.gamma_f = (float)wc.gamma;
  rp.B_f = (float)wc.B;
  rp.inv_rho0_f = (float)(1.0 / wc.rho0);
  rp.rho0_hi = (float)wc.rho0;
  rp.rho0_lo = (float)(wc.rho0 - (double)rp.rho0_hi);
  rp.Pb_f = (float)wc.Pb;
  rp.h_fixed_on = cfg.h_fixed > 0.0 ? 1 : 0;
  rp.Pb_on = wc.Pb != 0.0 ? 1 : 0;
  rp.write_state = write_state ? 1 : 0;
  rp.from_state = p_from_state ? 1 : 0;
  rp.reduce_h = reduce_h ? 1 : 0;
  return rp;
}

// The build after k_bounds (which set the grid): keys and ranks, scan,
// scatter, in-cell order.  With rp, the pair records of the form cfg names
// are written by the in-cell-order pass (launch_records' work, fused).
void launch_build(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc,
                  cudaStream_t st, const RecParams *rp) {
  (void)wc;
  const unsigned nb = nblocks(a.n);
  launch_pdl(k_keys, dim3(nb), dim3(kBlock), 0, st, a.x, a.y, a.n, w.grid, w.ctrl, w.keys, w.refcell, w.crank,
             w.counts, w.scan_part, a.label, w.tflag);
  launch_pdl(k_scan_cells, dim3((unsigned)w.n_parts), dim3(kScanThreads), 0, st, w.counts, w.grid, w.scan_part,
             w.cstart);
  launch_pdl(k_scatter_rank, dim3(nb), dim3(kBlock), 0, st, w.keys, w.crank, a.n, w.counts, w.cstart, w.perm_tmp,
             w.keys_sorted, w.scan_part, w.n_parts);
  RecParams none;
  memset(&none, 0, sizeof(none));
#define SPH_CELLSORT(P, ...)                                                                                   \
  launch_pdl(k_cellsort<__VA_ARGS__>, dim3(nb), dim3(kBlock), 0, st, w.perm_tmp, w.keys_sorted, w.cstart,        \
             w.refcell, a.n, w.grid, w.ctrl, w.perm, w.meta, w.tiles, a, P, w.rec0, w.rec1, w.rec2, w.rec64a,      \
             w.rec64b, w.orig, (unsigned)(w.max_cells + 1), w.tiles_h, w.tflag)
  if (!rp) {
    SPH_CELLSORT(none, kRecNone);
  } else if (cfg.precision == SPH_PREC_MIXED) {
    const int hs = rp->from_state ? kHState : (rp->h_fixed_on ? kHFixed : kHCompute);
    const bool pb = rp->Pb_on != 0;
    if (hs == kHState) {
      if (pb) SPH_CELLSORT(*rp, kRecMixed, kHState, true);
      else SPH_CELLSORT(*rp, kRecMixed, kHState, false);
    } else if (hs == kHFixed) {
      if (pb) SPH_CELLSORT(*rp, kRecMixed, kHFixed, true);
      else SPH_CELLSORT(*rp, kRecMixed, kHFixed, false);
    } else {
      if (pb) SPH_CELLSORT(*rp, kRecMixed, kHCompute, true);
      else SPH_CELLSORT(*rp, kRecMixed, kHCompute, false);
    }
  } else {
    SPH_CELLSORT(*rp, kRecFp64);
  }
#undef SPH_CELLSORT
}

// ---------------------------------------------------------------------------
// Sorted pair records as a pass of their own, for the builds whose in-cell
// sort did not write them (the second summation-density pass, the adjoint's
// half state).  The h reset and the Tait EOS of _loop's first pass
// (SolverTools.py:122-127) are done here; p, c and the fluid h go back to the
// caller's arrays.
// ---------------------------------------------------------------------------
template <bool MIXED>
__global__ void __launch_bounds__(kBlock) k_records(StepArgs a, const int *__restrict__ perm, RecParams rp,
                                                    DevCtrl *ctrl, float4 *__restrict__ rec0,
                                                    float4 *__restrict__ rec1, float4 *__restrict__ rec2,
                                                    double4_32a *__restrict__ r64a,
                                                    double4_32a *__restrict__ r64b) {
  __shared__ unsigned long long red[kBlock / 32];
  __shared__ unsigned int redn[kBlock / 32];
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long eh = kEncMinId;
  unsigned int nf = 0;
  if (k < a.n) {
    const int i = perm[k];
    if (MIXED) record_mixed(a, k, i, rp, rec0, rec1, rec2, eh, nf);
    else record_fp64(a, k, i, rp, rec0, r64a, r64b, eh, nf);
  }
  if (rp.reduce_h) reduce_h_block(eh, nf, red, redn, ctrl);
}

void launch_records(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc,
                    bool write_state, bool p_from_state, bool reduce_h, cudaStream_t st) {
  const RecParams rp = rec_params(cfg, wc, write_state, p_from_state, reduce_h);
  if (cfg.precision == SPH_PREC_MIXED)
    k_records<true><<<nblocks(a.n), kBlock, 0, st>>>(a, w.perm, rp, w.ctrl, w.rec0, w.rec1, w.rec2, w.rec64a,
                                                     w.rec64b);
  else
    k_records<false><<<nblocks(a.n), kBlock, 0, st>>>(a, w.perm, rp, w.ctrl, w.rec0, w.rec1, w.rec2, w.rec64a,
                                                      w.rec64b);
}

// ---------------------------------------------------------------------------
// Batched form: many independent instances (tanks) in one particle set, each
// with its own grid, constants, reductions and dt.  Every stage is one launch
// over all instances.  Instance b's cells are the global ids
// [coff[b], coff[b + 1]) (its dump cell last), so one counting sort over the
// global ids sorts every instance at once and keeps each instance's slots in
// its particle range.
// ---------------------------------------------------------------------------
template <int INTEG, int STAGE, bool DAMPED, bool XSPH>
__global__ void __launch_bounds__(kBlock) k_bt_bounds(StepArgs a, BatchPtrs B, BoundsParams bp, int prev, int cur,
                                                      DevCtrl *ctrl) {
  step_kernel_entry();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long v[6] = {kEncMinId, kEncMinId, kEncMinId, kEncMinId, kEncMinId, kEncMinId};
  bool bad = false;
  int b = -1;
  if (i < a.n) {
    b = B.inst[i];
    BoundsParams bi = bp;
    const RecParams &rp = B.ip[b].rp;
    bi.h_fixed = rp.h_fixed;
    bi.h_fixed_on = rp.h_fixed_on;
    bi.dt_prev = B.sl[b].dt_ring[prev];
    bi.dt_cur = B.sl[b].dt_ring[cur];
    bounds_one<INTEG, STAGE, DAMPED, XSPH>(a, i, bi, v, bad);
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(&ctrl->status, (unsigned)SPH_STATUS_NONFINITE);
  InstSlots *sl = B.sl;
  seg_min_u64(v[0], b, [&](int q, unsigned long long m) { atomicMin(&sl[q].xmin, m); });
  seg_min_u64(v[1], b, [&](int q, unsigned long long m) { atomicMax(&sl[q].xmax, ~m); });
  seg_min_u64(v[2], b, [&](int q, unsigned long long m) { atomicMin(&sl[q].ymin, m); });
  seg_min_u64(v[3], b, [&](int q, unsigned long long m) { atomicMax(&sl[q].ymax, ~m); });
  seg_min_u64(v[4], b, [&](int q, unsigned long long m) { atomicMin(&sl[q].hmin_all, m); });
  seg_min_u64(v[5], b, [&](int q, unsigned long long m) { atomicMax(&sl[q].hmax_new, ~m); });
}

// every instance's grids (one thread each), then the cell offsets
__global__ void k_bt_grid(BatchPtrs B, DevCtrl *ctrl) {
  step_kernel_entry();
  unsigned status = 0;
  for (int b = threadIdx.x; b < B.n_inst; b += blockDim.x) {
    InstSlots &s = B.sl[b];
    const double xmin = dec_d(s.xmin), xmax = dec_d(s.xmax), ymin = dec_d(s.ymin), ymax = dec_d(s.ymax);
    const double hmin = dec_d(s.hmin_all), hmax = dec_d(s.hmax_new);
    s.xmin = kEncMinId; s.xmax = kEncMaxId; s.ymin = kEncMinId; s.ymax = kEncMaxId;
    s.hmin_all = kEncMinId; s.hmax_new = kEncMaxId;
    s.alias_count = 0;
    status |= grid_setup_keyed(xmin, xmax, ymin, ymax, hmin, hmax, B.ip[b].gp, &B.grids[b], &s.grid_key);
    B.coff[b] = B.grids[b].ncells + 1;  // its cells and its dump cell
  }
  if (status) atomicOr(&ctrl->status, status);
  __syncthreads();
  // exclusive prefix of the instances' cell counts: each thread a contiguous
  // run of instances, then a block scan of the run totals
  __shared__ int wsum[32];
  const int per = (B.n_inst + (int)blockDim.x - 1) / (int)blockDim.x;
  const int b0 = (int)threadIdx.x * per, b1 = min(b0 + per, B.n_inst);
  int loc = 0;
  for (int b = b0; b < b1; b++) loc += B.coff[b];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = ((int)blockDim.x + 31) >> 5;
  int inc = loc;
  for (int d = 1; d < 32; d <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += v;
  }
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  int run = inc - loc;
  for (int w = 0; w < wid; w++) run += wsum[w];
  __syncthreads();  // every thread has read the counts of its run
  for (int b = b0; b < b1; b++) {
    const int c = B.coff[b];
    B.coff[b] = run;
    run += c;
  }
  if (threadIdx.x == blockDim.x - 1) {
    int total = 0;
    for (int w = 0; w < nw; w++) total += wsum[w];
    B.coff[B.n_inst] = total;
    B.scan->ncells = total - 1;  // the scan kernels cover ids 0 .. run - 1
    ctrl->tl_count = 0;
  }
}

// k_keys over every instance: cell ids offset by the instance's first cell;
// arrival ranks and scan-tile totals as in k_keys.
__global__ void __launch_bounds__(kBlock) k_bt_keys(const double *__restrict__ x, const double *__restrict__ y,
                                                    long long n, BatchPtrs B, DevCtrl *ctrl, int *__restrict__ keys,
                                                    int2 *__restrict__ refcell, unsigned int *__restrict__ crank,
                                                    unsigned int *__restrict__ counts,
                                                    unsigned int *__restrict__ part) {
  step_kernel_entry();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const bool act = i < n;
  bool alias = false, overflow = false;
  int key = -1 - lane;
  if (act) {
    const int b = B.inst[i];
    int2 ref;
    key = B.coff[b] + cell_key(B.grids[b], x[i], y[i], ref, alias, overflow);
    refcell[i] = ref;
    keys[i] = key;
    if (alias) atomicAdd(&B.sl[b].alias_count, 1u);
  }
  const unsigned int below = (1u << lane) - 1u;
  const unsigned int peers = __match_any_sync(0xffffffffu, key);
  const int leader = __ffs(peers) - 1;
  unsigned int base = 0;
  if (act && lane == leader) base = atomicAdd(&counts[key], (unsigned int)__popc(peers));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (act) crank[i] = base + (unsigned int)__popc(peers & below);
  const int pt = act ? key / kScanTile : -1 - lane;
  const unsigned int tpeers = __match_any_sync(0xffffffffu, pt);
  if (act && lane == __ffs(tpeers) - 1) atomicAdd(&part[pt], (unsigned int)__popc(tpeers));
  const unsigned om = __ballot_sync(0xffffffffu, overflow);
  if (lane == 0 && om) atomicOr(&ctrl->status, (unsigned)SPH_STATUS_CELL_OVERFLOW);
}

// k_cellsort with the tile list of every instance (entries (instance, tile))
// and the mixed-form records of each final slot with its instance's
// constants; the TimeStep's min h and fluid count per instance.
__global__ void __launch_bounds__(kBlock) k_bt_cellsort(const int *__restrict__ perm_tmp,
                                                        const int *__restrict__ keys_sorted,
                                                        const unsigned int *__restrict__ cstart,
                                                        const int2 *__restrict__ refcell, long long n, BatchPtrs B,
                                                        DevCtrl *ctrl, int *__restrict__ perm,
                                                        int2 *__restrict__ meta, StepArgs a,
                                                        float4 *__restrict__ rec0, float4 *__restrict__ rec1,
                                                        float4 *__restrict__ rec2) {
  step_kernel_entry();
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long eh = kEncMinId;
  unsigned int nf = 0;
  int b = -1;
  const int lane = threadIdx.x & 31;
  const bool act = k < n;
  const int key = act ? keys_sorted[k] : -1 - lane;  // inactive lanes match no other lane
  const int v = act ? perm_tmp[k] : 0;
  unsigned int rank = warp_cell_rank(key, v);
  if (act) {
    const unsigned int s = cstart[key], e = cstart[key + 1];
    rank += outside_cell_rank(s, e, (unsigned int)(k - lane), v, perm_tmp);
    const unsigned int slot = s + rank;
    perm[slot] = v;
    meta[slot] = refcell[v];
    b = B.inst[v];
    const int c0 = B.coff[b], lk = key - c0;
    const DevGrid &g = B.grids[b];
    const int ts2 = 2 * g.ts;
    if (lk < g.ncells && (unsigned)k == __ldg(&cstart[c0 + ((lk >> ts2) << ts2)]))
      B.tiles[atomicAdd(&ctrl->tl_count, 1u)] = make_int2(b, lk >> ts2);
    record_mixed(a, slot, v, B.ip[b].rp, rec0, rec1, rec2, eh, nf);
  }
  InstSlots *sl = B.sl;
  seg_min_u64(eh, b, [&](int q, unsigned long long m) { atomicMin(&sl[q].pd_hmin, m); });
  seg_add_u32(nf, b, [&](int q, unsigned int c) { atomicAdd(&sl[q].pd_nfluid, c); });
}

void launch_bt_bounds(const StepArgs &a, const WsPtrs &w, const BatchPtrs &B, const sph_config_t &cfg, int stage,
                      int prev, int cur, cudaStream_t st) {
  BoundsParams bp;
  bp.stage = stage;
  bp.euler = cfg.integrator == SPH_INTEGRATOR_EULER ? 1 : 0;
  bp.verlet = cfg.integrator == SPH_INTEGRATOR_VERLET ? 1 : 0;
  if (bp.euler && stage == kStagePredict) bp.stage = kStageNone;
  bp.h_reset = 1;
  bp.h_fixed = 0.0;
  bp.h_fixed_on = 0;
  bp.dt_fixed = 0.0;
  bp.dt_fixed_on = 0;
  bp.dt_prev = nullptr;
  bp.dt_cur = nullptr;
  bp.inv_damp = 1.0 / (1.0 + 0.5 * cfg.damping);
  bp.c0 = 2.0 * bp.inv_damp - 1.0;
  bp.damped = cfg.damping != 0.0 ? 1 : 0;
  bp.use_xsph = cfg.pec_use_xsph;
  bp.strict = cfg.pec_strict;
  front_dispatch(bp, [&]<int I, int S, bool D, bool X>() {
    launch_pdl(k_bt_bounds<I, S, D, X>, dim3(nblocks(a.n)), dim3(kBlock), 0, st, a, B, bp, prev, cur, w.ctrl);
  });
}

// the batched build with the records fused into the in-cell sort
void launch_bt_build(const StepArgs &a, const WsPtrs &w, const BatchPtrs &B, cudaStream_t st) {
  const unsigned nb = nblocks(a.n);
  launch_pdl(k_bt_grid, dim3(1), dim3(256), 0, st, B, w.ctrl);
  launch_pdl(k_bt_keys, dim3(nb), dim3(kBlock), 0, st, a.x, a.y, a.n, B, w.ctrl, w.keys, w.refcell, w.crank,
             w.counts, w.scan_part);
  launch_pdl(k_scan_cells, dim3((unsigned)w.n_parts), dim3(kScanThreads), 0, st, w.counts, B.scan, w.scan_part,
             w.cstart);
  launch_pdl(k_scatter_rank, dim3(nb), dim3(kBlock), 0, st, w.keys, w.crank, a.n, w.counts, w.cstart, w.perm_tmp,
             w.keys_sorted, w.scan_part, w.n_parts);
  launch_pdl(k_bt_cellsort, dim3(nb), dim3(kBlock), 0, st, w.perm_tmp, w.keys_sorted, w.cstart, w.refcell, a.n, B,
             w.ctrl, w.perm, w.meta, a, w.rec0, w.rec1, w.rec2);
}

}  // namespace sph

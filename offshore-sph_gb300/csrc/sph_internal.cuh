// sph_internal.cuh -- device-side structures and math shared by the kernels
// of the WCSPH step (neighbour build, fused pair interaction, integrators).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "sph_gb300.h"

namespace sph {

constexpr int kBlock = 256;
constexpr int kScanTile = 4096;  // cells per scan tile (256 threads x 16)

// ---------------------------------------------------------------------------
// Order-preserving encoding of doubles for unsigned 64-bit atomicMin/Max.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long enc_d(double v) {
  unsigned long long u = (unsigned long long)__double_as_longlong(v);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double dec_d(unsigned long long e) {
  unsigned long long u = (e & 0x8000000000000000ull) ? (e & 0x7fffffffffffffffull) : ~e;
  return __longlong_as_double((long long)u);
}
constexpr unsigned long long kEncMinId = 0xffffffffffffffffull;  // identity of min
constexpr unsigned long long kEncMaxId = 0ull;                   // identity of max

// ---------------------------------------------------------------------------
// Workspace-resident control block: reductions, status, dt ring.
// Every reduction slot is returned to its identity by the kernel that
// consumes it, so no memset is needed between evaluations.
// ---------------------------------------------------------------------------
struct DevCtrl {
  // bounds of the next neighbour build (all active particles)
  unsigned long long xmin, xmax, ymin, ymax;
  unsigned long long hmin_all;  // h before the h reset (reference cell size)
  unsigned long long hmax_new;  // h after the h reset (search radius)
  // TimeStep reductions over fluid
  unsigned long long ts_hmin, ts_cmax, ts_a2max;
  unsigned int ts_nfluid;
  unsigned int done_pair;  // last-block counters
  unsigned int done_ts;
  unsigned int status;     // sticky SPH_STATUS_* bits
  unsigned int alias_count;
  unsigned int initialised;
  unsigned int pad[2];
  double dt_ring[2][3];  // {dt, dt_c, dt_f} of the step with that parity
};

// Search grid, written by the grid kernel of each neighbour build.
struct DevGrid {
  // reference grid (src/Tools/NNLinkedList.py:86-127)
  double xmin, xmax, ymin, ymax, cs, inv_cs;
  long long ncx, ncy, ncells_ref;
  // traversal grid
  int mode;         // 0: the reference cells themselves, 1: own grid + reference-stencil filter
  int ntx, nty;     // traversal cells per axis
  int ncells;       // traversal cells in use (cell ncells is the dump cell)
  double ox, oy;    // traversal origin (mode 1)
  double ct, inv_ct;  // traversal cell size (mode 1)
  int need_filter;  // mode 1: candidates must pass the reference-stencil test
  int wide;         // mode 1: stencil half-width (cells) covering q <= 3 at hmax
  double hmax;      // max h after the h reset
  double r_search;  // interaction radius the traversal covers
  int valid;
  int pad;
};

// Byte offsets of the workspace regions (computed on the host).
struct WsLayout {
  size_t ctrl, grid, keys, refcell, perm_tmp, keys_sorted, perm, meta, counts, cstart, scan_part, recA,
      recB, recC, rho_sd, total;
  long long n_cap, max_cells, n_parts;
};

WsLayout make_layout(long long n_cap, long long max_cells);

struct WsPtrs {
  DevCtrl *ctrl;
  DevGrid *grid;
  int *keys;          // traversal cell of particle i (caller order)
  int2 *refcell;      // raw reference cell (cx, cy) of particle i
  int *perm_tmp;      // unsorted-within-cell permutation
  int *keys_sorted;   // traversal cell of sorted slot k
  int *perm;          // sorted slot -> particle index
  int2 *meta;         // raw reference cell of sorted slot k
  unsigned int *counts;  // per cell counters (zero between builds)
  unsigned int *cstart;  // exclusive prefix of counts, cstart[ncells] = n
  unsigned int *scan_part;
  void *recA, *recB, *recC;  // sorted pair records
  double *rho_sd;            // summation-density result (caller order)
  long long n_cap, max_cells, n_parts;
};

WsPtrs ws_ptrs(const sph_workspace_t *ws);

// ---------------------------------------------------------------------------
// Small device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool is_fluid(int8_t l) { return l == SPH_FLUID; }

// Exact floor((a - o) / s) of the reference (NNLinkedList.py:164-176), using
// the reciprocal and falling back to the correctly rounded division only
// when the quotient is near an integer.
__device__ __forceinline__ long long ref_floor_div(double a, double o, double s, double inv_s) {
  double d = a - o;
  double t = d * inv_s;
  double f = floor(t);
  double fr = t - f;
  if (fr < 1e-9 || fr > 1.0 - 1e-9) f = floor(__ddiv_rn(d, s));
  return (long long)f;
}

// 32-bit signed saturation for cell coordinates
__device__ __forceinline__ int sat_i32(long long v) {
  return v > (1ll << 30) ? (1 << 30) : (v < -(1ll << 30) ? -(1 << 30) : (int)v);
}

// Storage (flat-id) cell of a raw reference cell: the x-overflow cx == ncx
// aliases into (0, cy + 1) (NNLinkedList.py:200-208).
__device__ __forceinline__ void storage_cell(int cx, int cy, long long ncx, int &sx, int &sy) {
  if (cx >= ncx) {
    sx = 0;
    sy = cy + 1;
  } else {
    sx = cx;
    sy = cy;
  }
}

// Tait EOS of one particle (TaitEOS.py:6-31) plus the background pressure
// (WCSPH.py:131-149).  gamma == 7 uses repeated products.
__device__ __forceinline__ double tait_p(double rho, int8_t label, double gamma, double B, double rho0,
                                         double Pb) {
  if (!is_fluid(label)) return 0.0 + Pb;
  double r = rho / rho0;
  double ratio;
  if (gamma == 7.0) {
    double r2 = r * r;
    double r4 = r2 * r2;
    ratio = r4 * r2 * r;
  } else {
    ratio = pow(r, gamma);
  }
  return (ratio - 1.0) * B + Pb;
}

// computeH (SolverTools.py:106-118)
__device__ __forceinline__ double compute_h(double m, double rho) {
  return rho > 1e-12 ? 1.3 * sqrt(m / rho) : 0.0;
}

// The fluid h of the h reset (Solver.py:242-246)
__device__ __forceinline__ double reset_h(double h_fixed, double m, double rho) {
  return h_fixed > 0.0 ? h_fixed : compute_h(m, rho);
}

// ---------------------------------------------------------------------------
// Smoothing kernels in FP64, as the reference writes them
// ---------------------------------------------------------------------------
constexpr double kCubicFac = 10.0 / (7.0 * M_PI);  // CubicSpline.py:24
constexpr double kInvPi = 1.0 / M_PI;              // Gaussian.py:18

// CubicSpline.evaluate (CubicSpline.py:12-36)
__device__ __forceinline__ double cubic_w(double r, double h) {
  const double alpha = kCubicFac / (h * h);
  const double q = r / h;
  if (q > 2.0) return 0.0;
  if (q > 1.0) {
    const double t = 2.0 - q;
    return alpha * 0.25 * (t * t * t);
  }
  return alpha * (1.0 - 1.5 * (q * q) * (1.0 - 0.5 * q));
}
// CubicSpline.gradient (CubicSpline.py:40-70): the factor multiplying x
__device__ __forceinline__ double cubic_gcoef(double r, double h) {
  const double alpha = kCubicFac / (h * h);
  const double q = r / h;
  if ((q > 2.0) || (r < 1e-10)) return 0.0;
  double g;
  if (q > 1.0) {
    const double t = 2.0 - q;
    g = -0.75 * (t * t);
  } else {
    g = -3.0 * q * (1.0 - 0.75 * q);
  }
  return alpha * g / (h * r);
}
// Gaussian.evaluate (Gaussian.py:16-24)
__device__ __forceinline__ double gauss_w(double r, double h) {
  const double q = r / h;
  if (q <= 3.0) return kInvPi / (h * h) * exp(-q * q);
  return 0.0;
}
// Gaussian.derivative (Gaussian.py:26-35)
__device__ __forceinline__ double gauss_dwdq(double r, double h) {
  const double q = r / h;
  if (q <= 3.0) return -2.0 * q * (kInvPi / (h * h)) * exp(-q * q);
  return 0.0;
}
// Gaussian.gradient (Gaussian.py:37-59): the factor multiplying x
__device__ __forceinline__ double gauss_gcoef(double r, double h) {
  const double tmp = r * h;
  if (tmp > 1e-12) {
    const double q = r / h;
    if (q <= 3.0) return (-2.0 * q * (kInvPi / (h * h)) * exp(-q * q)) / tmp;
  }
  return 0.0;
}

// ---------------------------------------------------------------------------
// Block reductions (256 threads)
// ---------------------------------------------------------------------------
template <typename T, typename Op>
__device__ __forceinline__ T warp_reduce(T v, Op op) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

struct MinU64 {
  __device__ unsigned long long operator()(unsigned long long a, unsigned long long b) const {
    return a < b ? a : b;
  }
};
struct MaxU64 {
  __device__ unsigned long long operator()(unsigned long long a, unsigned long long b) const {
    return a > b ? a : b;
  }
};
struct AddU32 {
  __device__ unsigned int operator()(unsigned int a, unsigned int b) const { return a + b; }
};

// Reduce one value per thread over the block; the result is valid in thread 0.
template <typename T, typename Op>
__device__ __forceinline__ T block_reduce(T v, Op op, T ident, T *smem /* 32 */) {
  v = warp_reduce(v, op);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) smem[wid] = v;
  __syncthreads();
  int nw = (blockDim.x + 31) >> 5;
  v = (threadIdx.x < nw) ? smem[threadIdx.x] : ident;
  if (wid == 0) v = warp_reduce(v, op);
  return v;
}

// ---------------------------------------------------------------------------
// Kernel launch helpers (defined in the .cu files)
// ---------------------------------------------------------------------------
inline unsigned int nblocks(long long n, int bs = kBlock) {
  long long b = (n + bs - 1) / bs;
  return (unsigned int)(b < 1 ? 1 : b);
}

struct StepArgs {
  // state (caller order)
  long long n;
  const int8_t *label;
  double *m, *rho, *p, *c, *drho, *h, *x, *y, *vx, *vy, *ax, *ay, *xsphx, *xsphy;
  double *x0, *y0, *vx0, *vy0, *rho0;
};

inline StepArgs step_args(const sph_particles_t *pa) {
  StepArgs a;
  a.n = pa->n;
  a.label = pa->label;
  a.m = pa->m; a.rho = pa->rho; a.p = pa->p; a.c = pa->c; a.drho = pa->drho; a.h = pa->h;
  a.x = pa->x; a.y = pa->y; a.vx = pa->vx; a.vy = pa->vy; a.ax = pa->ax; a.ay = pa->ay;
  a.xsphx = pa->xsphx; a.xsphy = pa->xsphy;
  a.x0 = pa->x0; a.y0 = pa->y0; a.vx0 = pa->vx0; a.vy0 = pa->vy0; a.rho0 = pa->rho0;
  return a;
}

// Neighbour build: bounds (+ optional fused integrator predict), grid,
// keys, counting sort, sorted pair records.
enum BoundsMode { kBoundsOnly = 0, kBoundsPredictPEC = 1, kBoundsReset = 2 };
void launch_bounds(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, int mode, const double *dt,
                   double dt_fixed, cudaStream_t st);
void launch_build(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc,
                  cudaStream_t st);
// gather the sorted pair records (EOS, h reset); rho_override replaces rho
// (summation density) when not null
void launch_records(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc,
                    bool write_state, const double *rho_override, cudaStream_t st);
// fused pair interaction; dt_out (ring slot) receives the next TimeStep
void launch_pair(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc,
                 double *dt_out, double *dt_hist, cudaStream_t st);
void launch_sumdens(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc,
                    cudaStream_t st);
void launch_nn_count(const StepArgs &a, const WsPtrs &w, int64_t *counts, const int64_t *offsets, int64_t *idx,
                     cudaStream_t st);
// integrators and per-particle stages
void launch_predict(const StepArgs &a, const sph_config_t &cfg, const double *dt, double dt_fixed,
                    cudaStream_t st);
void launch_correct(const StepArgs &a, const sph_config_t &cfg, const double *dt, double dt_fixed,
                    cudaStream_t st);
void launch_timestep(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, double *dt3, double *dt_hist,
                     cudaStream_t st);
void launch_initialize(const StepArgs &a, const sph_wcsph_t &wc, const sph_config_t &cfg, cudaStream_t st);
void launch_eos(const StepArgs &a, const sph_wcsph_t &wc, cudaStream_t st);
// elementwise kernel maps: what 0 = W, 1 = gradient factor * x, 2 = Gaussian dW/dq
void launch_kernel_map(int kernel, int what, long long n, const double *x, const double *r, const double *h,
                       double *out, cudaStream_t st);

}  // namespace sph

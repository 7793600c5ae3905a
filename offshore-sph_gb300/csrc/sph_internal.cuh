// sph_internal.cuh -- device-side structures and math shared by the kernels
// of the WCSPH step (neighbour build, fused pair interaction, integrators).
//
// A note on arithmetic: on GB300 the FP64 pipe issues a small fraction of the
// FP32/INT rate, so even per-particle stages become FP64-issue-bound long
// before they reach HBM bandwidth.  The mixed form therefore moves every
// conversion it can to the integer pipe (bit-level double<->float splits) and
// keeps FP64 arithmetic for the state updates only.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#include "sph_gb300.h"

namespace sph {

constexpr int kBlock = 256;
constexpr int kScanTile = 4096;  // cells per scan tile (1024 threads x 4, one uint4 each)
// largest tile shift of the cell numbering: tiles of 2^s x 2^s cells over the
// reference grid and over the own grid (0 = plain row-major cells).  The
// reference grid's shift adapts to the particles per cell (grid_setup).
#ifndef SPH_TILE_SHIFT_REF
#define SPH_TILE_SHIFT_REF 3
#endif
#ifndef SPH_TILE_SHIFT_OWN
#define SPH_TILE_SHIFT_OWN 4
#endif
// particles of one tile's halo that the pair tile kernel stages in shared
// memory (a larger halo takes the global-memory path)
#ifndef SPH_HALO_CAP
#define SPH_HALO_CAP 1024
#endif

// ---------------------------------------------------------------------------
// Order-preserving encoding of doubles for unsigned 64-bit atomicMin/Max
// (integer operations only).
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

// finite test on the bit pattern (no FP64 instruction)
__device__ __forceinline__ bool finite_bits(double v) {
  return ((unsigned long long)__double_as_longlong(v) & 0x7ff0000000000000ull) != 0x7ff0000000000000ull;
}

// ---------------------------------------------------------------------------
// double <-> float on the integer pipe
// ---------------------------------------------------------------------------
// float -> double, exact; denormals through an out-of-line conversion, so
// that the compiler cannot if-convert it into every thread's path
static __device__ __noinline__ double f2d_slow(float f) { return (double)f; }
__device__ __forceinline__ double f2d(float f) {
  unsigned u = __float_as_uint(f);
  unsigned s = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  unsigned long long r;
  if (e == 0u) {
    if (m != 0u) return f2d_slow(f);  // denormal (never in practice)
    r = (unsigned long long)s << 32;
  } else if (e == 0xffu) {
    r = ((unsigned long long)(s | 0x7ff00000u | (m >> 3)) << 32) | ((unsigned long long)(m & 7u) << 29);
  } else {
    r = ((unsigned long long)(s | ((e + 896u) << 20) | (m >> 3)) << 32) | ((unsigned long long)(m & 7u) << 29);
  }
  return __longlong_as_double((long long)r);
}

// The rare out-of-float-range cases go through out-of-line FP64 conversions,
// so that the compiler cannot if-convert them into every thread's path.
static __device__ __noinline__ float d2f_slow(double d) { return __double2float_rn(d); }
static __device__ __noinline__ float2 split_slow(double d) {
  const float hi = __double2float_rn(d);
  return make_float2(hi, __double2float_rn(d - (double)hi));
}

// double -> float by truncating the mantissa (relative error < 2^-23)
__device__ __forceinline__ float d2f_trunc(double d) {
  unsigned long long u = (unsigned long long)__double_as_longlong(d);
  unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
  unsigned s = hi & 0x80000000u;
  if ((u << 1) == 0ull) return __uint_as_float(s);
  int e = (int)((hi >> 20) & 0x7ffu) - 896;
  if (e <= 0 || e >= 255) return d2f_slow(d);  // out of float range, inf, nan: rare
  return __uint_as_float(s | ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
}

// double -> (hi, lo) floats with d = hi + lo to 2^-47 relative: hi is d's
// mantissa truncated to 24 bits, lo the remaining 29 bits rounded to 24.
__device__ __forceinline__ void split_df(double d, float &hi, float &lo) {
  unsigned long long u = (unsigned long long)__double_as_longlong(d);
  unsigned h32 = (unsigned)(u >> 32), l32 = (unsigned)u;
  unsigned s = h32 & 0x80000000u;
  if ((u << 1) == 0ull) {
    hi = __uint_as_float(s);
    lo = 0.f;
    return;
  }
  int eb = (int)((h32 >> 20) & 0x7ffu);
  int e = eb - 896;
  if (e <= 0 || e >= 255) {
    const float2 r = split_slow(d);
    hi = r.x;
    lo = r.y;
    return;
  }
  hi = __uint_as_float(s | ((unsigned)e << 23) | ((h32 & 0xfffffu) << 3) | (l32 >> 29));
  // low 29 mantissa bits m, weight 2^(eb - 1075), converted without the
  // conversion unit: 2^23 + k is exact in FP32 for k < 2^23, so m = mh 2^23 + ml
  // becomes two exact subtractions and one correctly rounded FMA
  const unsigned m = l32 & 0x1fffffffu;
  const float fl = __uint_as_float(0x4B000000u | (m & 0x7fffffu)) - 8388608.0f;
  const float fh = __uint_as_float(0x4B000000u | (m >> 23)) - 8388608.0f;
  const float mf = fmaf(fh, 8388608.0f, fl);
  const int se = eb - 948;  // biased float exponent of 2^(eb - 1075)
  const float scale = se > 0 ? __uint_as_float((unsigned)se << 23) : 0.f;
  lo = __uint_as_float(__float_as_uint(mf * scale) | s);
}

// floor(t) for 0 <= t < 2^23 as an int and as a float, on the FMA pipe:
// t + 2^23 rounded down is 2^23 + floor(t)
__device__ __forceinline__ int floor_small(float t, float &ft) {
  const float b = __fadd_rd(t, 8388608.0f);
  ft = b - 8388608.0f;
  return (int)(__float_as_uint(b) - 0x4B000000u);
}

// ---------------------------------------------------------------------------
// Workspace-resident control block: reductions, status, dt ring.  Every
// reduction slot is returned to its identity by the kernel that consumes it.
// ---------------------------------------------------------------------------
// Inputs of the last grid setup on a grid, with the status bits it returned.
// The setup is a pure function of them, so a build whose inputs match bit for
// bit keeps the grid as it is.  set = 0 (zeroed workspace): no grid yet.
struct GridKey {
  unsigned long long b[6];  // xmin, xmax, ymin, ymax, hmin, hmax (raw bits)
  unsigned long long scale, r0;  // raw bits
  long long max_cells;
  int kernel, ts_ref, ts_own_max;
  unsigned int status;
  int set;
};

struct DevCtrl {
  // bounds of the next neighbour build (all active particles)
  unsigned long long xmin, xmax, ymin, ymax;
  unsigned long long hmin_all;  // h before the h reset (reference cell size)
  unsigned long long hmax_new;  // h after the h reset (search radius)
  // TimeStep reductions over fluid: standalone TimeStep kernel ...
  unsigned long long ts_hmin, ts_cmax, ts_a2max;
  unsigned int ts_nfluid;
  unsigned int done_ts;
  // ... and the one fused into the step (h from the records pass, a^2 from the pair pass)
  unsigned long long pd_hmin, pd_a2max;
  unsigned int pd_nfluid;
  unsigned int done_pair;
  unsigned int status;  // sticky SPH_STATUS_* bits
  unsigned int alias_count;
  unsigned int initialised;
  // pair-kernel scheduling: next tile chunk and finished blocks of the tile
  // kernel; entries and finished blocks of the fallback list
  unsigned int tile_next, tile_done;
  unsigned int fb_count, fb_done;
  // non-empty tiles listed by the build (single-scene build): tl_heavy dense
  // tiles holding a boundary particle in their own list, tl_count other dense
  // ones from the front of the tile list, tl_back sparse ones from its back
  unsigned int tl_count, tl_back, tl_heavy;
  unsigned int bounds_done;  // finished blocks of the bounds pass (its last block sets the grid)
  double dt_ring[2][3];  // {dt, dt_c, dt_f} of the step with that parity
  GridKey grid_key;      // inputs of the grid in use
};

// the bound slots are consecutive (k_bounds indexes them from xmin)
static_assert(offsetof(DevCtrl, xmax) == offsetof(DevCtrl, xmin) + 8 &&
                  offsetof(DevCtrl, ymin) == offsetof(DevCtrl, xmin) + 16 &&
                  offsetof(DevCtrl, ymax) == offsetof(DevCtrl, xmin) + 24 &&
                  offsetof(DevCtrl, hmin_all) == offsetof(DevCtrl, xmin) + 32 &&
                  offsetof(DevCtrl, hmax_new) == offsetof(DevCtrl, xmin) + 40,
              "bound slots of DevCtrl");

// Search grid, written by the last block of the bounds pass of each
// neighbour build (the batched form: by its grid kernel, per instance).
struct DevGrid {
  // reference grid (src/Tools/NNLinkedList.py:86-127)
  double xmin, xmax, ymin, ymax, cs, inv_cs;
  long long ncx, ncy, ncells_ref;
  float xminf, yminf, inv_csf;  // FP32 fast path of the reference binning
  float hmaxf;  // FP32 bound on every record's |h| (hmax rounded up, with margin)
  // traversal grid
  int mode;    // 0: the reference cells with their 3x3 stencil; 1: own grid
  int ntx, nty;  // traversal cells per axis
  int ncells;  // cell ids in use, tiles padded (id ncells is the dump cell)
  int ts;      // cells are numbered in tiles of 2^ts x 2^ts, row-major inside a tile
  int ntlx;    // tiles per row
  float oxf, oyf, inv_ctf;  // mode 1 binning (FP32, monotone)
  float txmaxf, tymaxf;     // ntx - 1, nty - 1 in FP32 (the binning's clamps)
  int wt;           // stencil half-width of the pair kernels
  int need_filter;  // mode 1: candidates must pass the reference-stencil test
  int wide;         // mode 1: half-width covering q <= 3 at hmax (export, aliased queries)
  double ct;        // traversal cell size
  double hmax;      // max h after the h reset
  double r_search;  // interaction radius the pair kernels need
  float pad_e;      // bound on |x_hi - x| + |x_j,hi - x_j| over the domain (prefilter padding)
  int valid;
};

// Byte offsets of the workspace regions (computed on the host).
// total: what every entry point needs; total_shadow adds the sorted copy of
// the state that sph_run steps on when the workspace has room for it.
struct WsLayout {
  size_t ctrl, grid, keys, refcell, crank, perm_tmp, keys_sorted, perm, meta, counts, cstart, scan_part, rec0,
      rec1, rec2, rec64a, rec64b, fb, tiles, tiles_h, tflag, total;
  size_t shadow, shadow_label, shadow_orig, total_shadow;
  long long n_cap, max_cells, n_parts, fb_cap;
};
constexpr int kStateFields = 19;  // the FP64 fields of particle_dtype

WsLayout make_layout(long long n_cap, long long max_cells);

// ---------------------------------------------------------------------------
// Per-call parameter blocks of the stages (one per instance in the batched
// form).
// ---------------------------------------------------------------------------
struct GridParams {
  double scale, r0;
  int kernel;
  long long max_cells;
  int ts_ref_max, ts_own_max;  // largest tile shifts of the cell numbering
  long long n;                 // particles of the build
  // particles per cell of the previous build's listed tiles, when that build
  // used the reference cells (0: unknown); sets the next reference tile shift
  double ppc;
};
// grid_setup_keyed skips the setup when the GridKey of the grid in use holds
// the same inputs: a field added here that grid_setup reads must join the key
static_assert(sizeof(GridParams) == 56, "a new GridParams field must be compared by grid_setup_keyed");

struct RecParams {
  double h_fixed, gamma, B, inv_rho0, Pb, co;
  float h_fixed_f, gamma_f, B_f, inv_rho0_f, rho0_hi, rho0_lo, Pb_f;
  int h_fixed_on, Pb_on;
  int write_state;   // write p, c, h to the caller's arrays
  int from_state;    // p and h from the caller's arrays (second summation-density pass)
  int reduce_h;      // min h over fluid for the step's TimeStep
};

struct PairParams {
  double alpha, beta, co, eps, r0, D, p1, p2;
  int lj_42;  // p1 == 4 and p2 == 2
  double cfl_c, cfl_f;
  int do_dt;
  long long n;
  // wall load (FP64 form): fr[i] = -m_i x (x part of the Lennard-Jones
  // acceleration from boundary neighbours at x >= wall_x), when fr != nullptr
  double wall_x;
  double *fr;
};

// One instance of the batched form: its particle range, its stage
// parameters, and its reductions and dt ring.
struct InstParams {
  long long off, n;
  RecParams rp;
  PairParams pp;
  GridParams gp;
  double cfl_c, cfl_f;
};
struct InstSlots {
  unsigned long long xmin, xmax, ymin, ymax, hmin_all, hmax_new;  // bounds of the next build
  unsigned long long pd_hmin, pd_a2max;                            // TimeStep of the next step
  unsigned long long ts_cmax;                                      // initial TimeStep: max c
  unsigned int pd_nfluid, alias_count;
  double dt_ring[2][3];
  GridKey grid_key;  // inputs of the instance's grid in use
};
struct BatchPtrs {
  InstParams *ip;
  InstSlots *sl;
  DevGrid *grids;    // per instance
  int *coff;         // first global cell id of each instance, then the total
  int *inst;         // instance of each particle (caller order)
  int2 *tiles;       // (instance, tile) of the non-empty tiles of the build
  DevGrid *scan;     // ncells = total cells - 1, for the scan kernels
  int n_inst;
};

// Reductions over a warp whose lanes may belong to different instances of
// the batched form; lanes of one instance are contiguous (instance-major
// order), b < 0 for lanes without a particle.  commit(b, value) applies the
// atomic to instance b's slot.  Every lane of the warp must call.
template <class F>
__device__ __forceinline__ void seg_min_u64(unsigned long long v, int b, F &&commit) {
  const int b0 = __shfl_sync(0xffffffffu, b, 0);
  if (__all_sync(0xffffffffu, b == b0)) {
    unsigned long long m = v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
      m = t < m ? t : m;
    }
    if ((threadIdx.x & 31) == 0 && b0 >= 0 && m != kEncMinId) commit(b0, m);
  } else if (b >= 0 && v != kEncMinId) {
    commit(b, v);
  }
}
template <class F>
__device__ __forceinline__ void seg_add_u32(unsigned int v, int b, F &&commit) {
  const int b0 = __shfl_sync(0xffffffffu, b, 0);
  if (__all_sync(0xffffffffu, b == b0)) {
    const unsigned int s = __reduce_add_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0 && b0 >= 0 && s) commit(b0, s);
  } else if (b >= 0 && v) {
    commit(b, v);
  }
}

// Sorted pair records (slot k = k-th particle in cell order):
//   rec0  float4 (x_hi, y_hi, h, m)  x_hi, y_hi: FP64 position with its mantissa
//                                    truncated to 24 bits; h with the sign bit
//                                    set for non-fluid particles
//   rec1  float4 (x_lo, y_lo, rho, p / rho^2)    mixed form: x = x_hi + x_lo
//   rec2  float4 (vx_hi, vy_hi, vx_lo, vy_lo)    mixed form
//   rec64a double4 (x, y, vx, vy)                FP64 form
//   rec64b double4 (m, rho, p / rho^2, h signed)
struct WsPtrs {
  DevCtrl *ctrl;
  DevGrid *grid;
  int *keys;          // traversal cell of particle i (caller order)
  int2 *refcell;      // raw reference cell (cx, cy) of particle i
  unsigned int *crank;  // arrival rank of particle i in its cell (current neighbour build)
  int *perm_tmp;      // unsorted-within-cell permutation
  int *keys_sorted;   // traversal cell of sorted slot k
  int *perm;          // sorted slot -> particle index
  int2 *meta;         // raw reference cell of sorted slot k
  unsigned int *counts;  // per cell counters (zero between builds)
  unsigned int *cstart;  // exclusive prefix of counts, cstart[ncells + 1] = n
  unsigned int *scan_part;  // cell total of each scan tile (zero between builds)
  float4 *rec0, *rec1, *rec2;
  double4_32a *rec64a, *rec64b;
  int2 *fb;  // fallback list of the tile pair kernel: (first slot, count <= 128)
  int *tiles;    // non-empty tiles of the current build (dense from the front, sparse from the back)
  int *tiles_h;  // its dense tiles that hold a boundary particle
  unsigned int *tflag;  // one bit per tile: it holds a boundary particle (zero between builds)
  long long n_cap, max_cells, n_parts, fb_cap;
  // The sorted copy of the state (when the workspace has room): kStateFields
  // arrays of n_cap doubles, the labels, and each copy index's caller index.
  double *shadow;
  int8_t *shadow_label;
  int *shadow_orig;
  // set while a run steps on the copy: the in-cell order ranks particles by
  // their caller index orig[i] instead of their index i (null: by i)
  const int *orig;
};

WsPtrs ws_ptrs(const sph_workspace_t *ws);

// A workspace's initial state: zero cell counters, scan-tile totals and grid,
// the control block at its identities (capi.cu); asynchronous on st, returns
// the first CUDA error.
cudaError_t init_workspace(const WsPtrs &w, cudaStream_t st);

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
  // with a power-of-two cell size (the 1.0 of a scene whose smallest h is
  // 0) the product by the reciprocal is the exact quotient already
  const bool pow2 = (__double_as_longlong(s) & 0x000fffffffffffffll) == 0;
  if (!pow2) {
    double fr = t - f;
    if (fr < 1e-9 || fr > 1.0 - 1e-9) f = floor(__ddiv_rn(d, s));
  }
  return (long long)f;
}
static __device__ __noinline__ long long ref_floor_div_slow(double a, double o, double s, double inv_s) {
  return ref_floor_div(a, o, s, inv_s);
}

// The same binning with an FP32 fast path: the FP32 estimate decides unless
// it lands within its error bound of a cell edge (then the exact FP64 test
// does).  With af = a truncated to FP32 (relative error 2^-23), of = o and
// inv_sf = 1/s rounded (2^-24 each) and two rounded FP32 operations, the
// estimate t is within ((|af| + |of|) inv_sf + t) 2^-22 of the exact
// (a - o) / s; the margin doubles that, and the FP64 quotient of the
// reference is within 2^-52 t of the exact one, far inside it.  So the few
// particles in the margin are the only ones that take the FP64 division (a
// lane or two of a warp, each costing the warp the slow FP64 pipe).
__device__ __forceinline__ long long ref_cell(double a, double o, double s, double inv_s, float of, float inv_sf) {
  const float af = d2f_trunc(a);
  const float t = (af - of) * inv_sf;
  const float span = (fabsf(af) + fabsf(of)) * inv_sf;
  const bool range = t >= 0.f && t < 1e6f && span < 4000.f;
  float f;
  const int c = floor_small(range ? t : 0.f, f);
  const float fr = t - f;
  const float mg = (span + t) * 4.76837158e-7f + 9.5367432e-7f;  // 2^-21 (span + t) + 2^-20
  if (range && fr > mg && fr < 1.0f - mg) return c;
  return ref_floor_div_slow(a, o, s, inv_s);
}

// exact halving of a positive normal double on the integer pipe
static __device__ __noinline__ double half_slow(double v) { return 0.5 * v; }
__device__ __forceinline__ double half_exact(double v) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
  if (e > 1u && e < 0x7ffu) return __longlong_as_double((long long)(u - (1ull << 52)));
  return half_slow(v);
}

// v < 0.0 on the bit pattern: sign set, not -0.0, not NaN
__device__ __forceinline__ bool negative_bits(double v) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const unsigned long long mag = u & 0x7fffffffffffffffull;
  return (u >> 63) != 0ull && mag != 0ull && mag <= 0x7ff0000000000000ull;
}

// 64-bit min / max over a warp with two 32-bit REDUX steps
__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
  const unsigned hi = (unsigned)(v >> 32), lo = (unsigned)v;
  const unsigned mh = __reduce_min_sync(0xffffffffu, hi);
  const unsigned ml = __reduce_min_sync(0xffffffffu, hi == mh ? lo : 0xffffffffu);
  return ((unsigned long long)mh << 32) | ml;
}
__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
  const unsigned hi = (unsigned)(v >> 32), lo = (unsigned)v;
  const unsigned mh = __reduce_max_sync(0xffffffffu, hi);
  const unsigned ml = __reduce_max_sync(0xffffffffu, hi == mh ? lo : 0u);
  return ((unsigned long long)mh << 32) | ml;
}

// ---------------------------------------------------------------------------
// Bulk asynchronous copies global -> shared (cp.async.bulk, the TMA engine's
// 1D form) completing on a shared-memory mbarrier.  Addresses 16-byte
// aligned, sizes multiples of 16 bytes.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// orders this thread's earlier generic-proxy shared-memory accesses before
// its later async-proxy (bulk copy) ones
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, unsigned long long *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Per-thread asynchronous copies global -> shared (cp.async, 16 bytes each,
// through L2 only): a thread issues any number of them without holding the
// data in registers, then waits for all of its own; a block barrier after the
// wait makes every thread's copies visible to the block.  Addresses 16-byte
// aligned.
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Bounded wait for phase `parity` of bar; false when the limit ran out.
// kMbarWaitLimit polls take milliseconds, far longer than any staging copy of
// a few tens of KB.  After a wait ran out, a block drains with the 16x longer
// kMbarDrainLimit before it leaves, so that it does not exit with copies
// still writing into its shared memory.  Should the drain run out as well,
// the block leaves anyway (every wait stays bounded): the copies in flight
// can then only write shared memory that a later block of the same launch
// may reuse, and that launch has already set SPH_STATUS_STAGING_TIMEOUT,
// which marks the whole evaluation as failed.
constexpr int kMbarWaitLimit = 1 << 22;
constexpr int kMbarDrainLimit = 1 << 26;
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, uint32_t parity,
                                                  int limit = kMbarWaitLimit) {
  for (int it = 0; it < limit; it++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// 32-bit signed saturation for cell coordinates
__device__ __forceinline__ int sat_i32(long long v) {
  return v > (1ll << 30) ? (1 << 30) : (v < -(1ll << 30) ? -(1 << 30) : (int)v);
}

// Cell id of traversal cell (cx, cy): tiles of 2^ts x 2^ts cells in
// row-major order, cells row-major inside a tile, so that consecutive ids
// cover compact patches of the domain.
__device__ __forceinline__ int tiled_key(int cx, int cy, int ts, int ntlx) {
  const int m = (1 << ts) - 1;
  return ((((cy >> ts) * ntlx + (cx >> ts)) << ts) + (cy & m)) * (1 << ts) + (cx & m);
}
__device__ __forceinline__ void tiled_cell(int key, int ts, int ntlx, int &cx, int &cy) {
  const int m = (1 << ts) - 1;
  const int tile = key >> (2 * ts), local = key & ((1 << (2 * ts)) - 1);
  cx = (tile % ntlx) * (1 << ts) + (local & m);
  cy = (tile / ntlx) * (1 << ts) + (local >> ts);
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

// Stencil of one query.  Mode 0: the reference's 3x3 cells around the
// query's raw cell (validity as NNLinkedList._get_valid_cell_index); mode 1:
// the own grid.  Cell ids are tiled (tiled_key), so the cells of one stencil
// row are one contiguous range of sorted slots per tile they touch.  The key
// of (x, y) splits into a row part and a column part; the column parts of the
// segment bounds are the same for every row and are computed once.
struct Stencil {
  int y0, y1;          // rows, clipped (empty when y0 > y1)
  int x0, x1;          // columns, clipped
  int ca, cb, cc, cd;  // column parts: first segment [ca, cb), second [cc, cd)
  int ts, ntlx;
  bool multi;          // columns span more than two tiles
  __device__ __forceinline__ static int colpart(int x, int ts) {
    return ((x >> ts) << (2 * ts)) + (x & ((1 << ts) - 1));
  }
  __device__ __forceinline__ int rowpart(int y) const {
    return (((y >> ts) * ntlx) << (2 * ts)) + ((y & ((1 << ts) - 1)) << ts);
  }
  __device__ __forceinline__ Stencil(const DevGrid &g, int2 qref, int qkey, int W) {
    ts = g.ts;
    ntlx = g.ntlx;
    int cx, cy;
    bool ok = true;
    if (g.mode == 0) {
      cx = qref.x;
      cy = qref.y;
    } else {
      ok = qkey < g.ncells;
      tiled_cell(qkey, ts, ntlx, cx, cy);
    }
    x0 = max(cx - W, 0);
    x1 = min(cx + W, g.ntx - 1);
    y0 = max(cy - W, 0);
    y1 = min(cy + W, g.nty - 1);
    if (!ok || x0 > x1) y1 = y0 - 1;
    multi = (x1 >> ts) - (x0 >> ts) > 1;
    const int xs = ((x0 >> ts) + 1) << ts;  // first column of the next tile
    ca = colpart(x0, ts);
    if (xs <= x1) {
      cb = colpart(xs - 1, ts) + 1;
      cc = colpart(xs, ts);
      cd = colpart(x1, ts) + 1;
    } else {
      cb = colpart(x1, ts) + 1;
      cc = cd = cb;
    }
  }
};

// visit(j) for every slot j of the stencil.  Each row is one loop over its
// (at most two) segments, with the four bounds loaded up front, so that the
// threads of a warp -- whose split points differ -- stay converged.  Columns
// spanning more than two tiles (tiles narrower than the stencil) walk the
// tiles one by one.
template <class F>
__device__ __forceinline__ void for_stencil(const Stencil &sten, const unsigned int *__restrict__ cstart,
                                            F &&visit) {
  if (!sten.multi) {
    for (int yy = sten.y0; yy <= sten.y1; yy++) {
      const unsigned int *c = cstart + sten.rowpart(yy);
      const unsigned int s0 = __ldg(c + sten.ca), e0 = __ldg(c + sten.cb);
      const unsigned int s1 = __ldg(c + sten.cc), e1 = __ldg(c + sten.cd);
      // slots [s0, e0) then [s1, e1) as one uniform index range
      const unsigned int jump = s1 - e0, jend = e0 + (e1 - s1);
      for (unsigned int j = s0; j < jend; j++) visit(j >= e0 ? j + jump : j);
    }
  } else {
    const int m = (1 << sten.ts) - 1;
    for (int yy = sten.y0; yy <= sten.y1; yy++) {
      const unsigned int *c = cstart + sten.rowpart(yy);
      for (int xs = sten.x0; xs <= sten.x1; xs = (xs | m) + 1) {
        const int xe = min(sten.x1, xs | m);
        const unsigned int e = __ldg(c + Stencil::colpart(xe, sten.ts) + 1);
        for (unsigned int j = __ldg(c + Stencil::colpart(xs, sten.ts)); j < e; j++) visit(j);
      }
    }
  }
}

__device__ __forceinline__ bool in_ref_stencil(const int2 *__restrict__ meta, unsigned int j, const DevGrid &g,
                                               int2 qref) {
  const int2 mj = __ldg(&meta[j]);
  int sx, sy;
  storage_cell(mj.x, mj.y, g.ncx, sx, sy);
  return abs(sx - qref.x) <= 1 && abs(sy - qref.y) <= 1;
}

// Tait EOS of one particle (TaitEOS.py:6-31) plus the background pressure
// (WCSPH.py:131-149), FP64.  gamma == 7 uses repeated products.
__device__ __forceinline__ double tait_p(double rho, int8_t label, double gamma, double B, double inv_rho0,
                                         double Pb) {
  if (!is_fluid(label)) return 0.0 + Pb;
  double r = rho * inv_rho0;
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

// (1 + d)^gamma - 1 in FP32 for the relative density d = rho / rho0 - 1
// (exact binomial expansion for gamma == 7; keeps full relative accuracy as
// d -> 0, where the FP64 form cancels)
__device__ __forceinline__ float tait_ratio_m1_f(float d, float gamma) {
  if (gamma == 7.0f) return d * (7.f + d * (21.f + d * (35.f + d * (35.f + d * (21.f + d * (7.f + d))))));
  return expm1f(gamma * log1pf(d));
}

// computeH (SolverTools.py:106-118)
__device__ __forceinline__ double compute_h(double m, double rho) {
  return rho > 1e-12 ? 1.3 * sqrt(m / rho) : 0.0;
}

// computeH out of line: a path that selects it by a uniform flag calls it
// only when taken (inlined, the compiler evaluates both sides of the select,
// and its division and square root then cost every particle FP64 issue)
static __device__ __noinline__ double compute_h_call(double m, double rho) { return compute_h(m, rho); }

// The fluid h of the h reset (Solver.py:242-246)
__device__ __forceinline__ double reset_h(double h_fixed, double m, double rho) {
  return h_fixed > 0.0 ? h_fixed : compute_h_call(m, rho);
}

// ---------------------------------------------------------------------------
// Smoothing kernels in FP64, as the reference writes them
// ---------------------------------------------------------------------------
constexpr double kCubicFac = 10.0 / (7.0 * M_PI);  // CubicSpline.py:24
constexpr double kInvPi = 1.0 / M_PI;              // Gaussian.py:18
constexpr double kWendFac = 9.0 / (4.0 * M_PI);    // Wendland.py:22

// support of a kernel in units of h: 3 for the Gaussian (cut at q <= 3), 2
// for the cubic spline and Wendland C4, which vanish with a zero gradient at
// q = 2
template <int KERNEL>
struct Support {
  static constexpr int q = KERNEL == SPH_KERNEL_GAUSSIAN ? 3 : 2;
};

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
// Wendland.evaluate (Wendland.py:10-34)
__device__ __forceinline__ double wendland_w(double r, double h) {
  const double alpha = kWendFac / (h * h);
  const double q = r / h;
  if (q >= 2.0) return 0.0;
  const double inner = 1.0 - 0.5 * q;
  return alpha * (pow(inner, 6.0) * (35.0 / 12.0 * q * q + 3.0 * q + 1.0));
}
// Wendland.gradient (Wendland.py:36-64): the factor multiplying x
__device__ __forceinline__ double wendland_gcoef(double r, double h) {
  const double alpha = kWendFac / (h * h);
  const double q = r / h;
  if ((q >= 2.0) || (r < 1e-10)) return 0.0;
  const double inner = 1.0 - 0.5 * q;
  const double grad = pow(inner, 5.0) * (-14.0 / 3.0) * q * (1 + 2.5 * q);
  return alpha * grad / (h * r);
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
// Block reductions
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

// SMs of the current device (cached per device; pair.cu)
int sm_count();

// Blocks of a persistent grid-stride launch over n items: per_sm blocks of
// bs threads on every SM, fewer when n is small.
inline unsigned int persist_blocks(long long n, int per_sm = 8, int bs = kBlock) {
  const unsigned int nb = nblocks(n, bs), cap = (unsigned int)(sm_count() * per_sm);
  return nb < cap ? nb : cap;
}

// Programmatic dependent launch between the kernels of a step.  A kernel
// launched with launch_pdl has its launch prepared while the stream's
// previous kernel runs; it begins with step_kernel_entry(), whose wait holds
// every thread until that kernel has completed and its writes are visible,
// so no read or write of shared data moves ahead of it.  No kernel triggers
// its dependent early (griddepcontrol.launch_dependents): the dependent's
// blocks would then sit waiting on SMs the running grid still uses, which
// measured slower than the implicit trigger at completion.  Launched without
// the attribute, the wait returns at once.  Under stream capture the
// dependency becomes a programmatic graph edge.
__device__ __forceinline__ void step_kernel_entry() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
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

// Neighbour build: bounds of the positions the next evaluation sees, with
// the integrator work that precedes it fused in front: none, the predictor
// of the first step, or the previous step's corrector followed by this
// step's predictor.  h_reset: take hmax over the h the evaluation will set.
enum IntStage { kStageNone = 0, kStagePredict = 1, kStageCorrectPredict = 2 };
void launch_bounds(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc, int stage,
                   bool h_reset, const double *dt_prev, const double *dt_cur, cudaStream_t st);
RecParams rec_params(const sph_config_t &cfg, const sph_wcsph_t &wc, bool write_state, bool p_from_state,
                     bool reduce_h);
// neighbour build after launch_bounds; with rp the records pass is fused in
void launch_build(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc,
                  cudaStream_t st, const RecParams *rp = nullptr);
// Sorted pair records (h reset + Tait EOS fused).  write_state: write p, c
// and the fluid h back; p_from_state: take p from the caller's array (second
// records pass of summation density); reduce_h: feed the step's TimeStep.
void launch_records(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc,
                    bool write_state, bool p_from_state, bool reduce_h, cudaStream_t st);
// fused pair interaction; dt_out (ring slot) receives the next TimeStep
// optional per-particle wall load of the FP64 pair kernel
struct WallLoad {
  double wall_x;  // boundary particles at x >= wall_x form the wall
  double *fr;     // fr[i] = -m_i (Lennard-Jones acceleration of i from the wall).x
};
void launch_pair(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc,
                 double *dt_out, double *dt_hist, cudaStream_t st,
                 const WallLoad *wall = nullptr);
void launch_sum_fixed(const double *v, long long n, double *out, cudaStream_t st);
void launch_adjoint_step(const StepArgs &s, const StepArgs &h, const WsPtrs &w, const sph_config_t &cfg,
                         const sph_wcsph_t &wc, const sph_adjoint_t &adj, cudaStream_t st);
void launch_nn_probe(const StepArgs &a, const WsPtrs &w, long long np, const double *px, const double *py,
                     const double *ph, int64_t *counts, const int64_t *offsets, int64_t *idx, double *hij, double *q,
                     double *r, cudaStream_t st);
void launch_probe_density(const StepArgs &a, const WsPtrs &w, int kernel, long long np, const double *px,
                          const double *py, const double *ph, const double *hk, double rho0, double B, double gamma,
                          double *rho, double *p, cudaStream_t st);
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

// pair.cu -- the fused pair interaction of the WCSPH step.
//
// One thread per cell-sorted fluid particle i evaluates in one pass
// everything _loop computes per particle (src/Tools/SolverTools.py:143-173):
// the kernel value and gradient (src/Kernels/CubicSpline.py,
// src/Kernels/Gaussian.py), continuity (src/Equations/Continuity.py),
// momentum with artificial viscosity and gravity (src/Equations/Momentum.py,
// src/Methods/WCSPH.py:151-169), the Lennard-Jones boundary force
// (src/Equations/BoundaryForce.py) and XSPH (src/Equations/XSPH.py).  The
// TimeStep of the next step (src/Equations/TimeStep.py:7-91) is fused into
// the epilogue.
//
// Each thread alternates two phases so that the expensive physics runs over
// dense lists instead of sparse, divergent candidate loops:
//   1. walk the stencil rows with one 16-byte load and a conservative FP32
//      radius test per candidate (hi parts of the positions, padded by their
//      truncation bound) and append the survivors to a per-thread list in
//      shared memory;
//   2. evaluate the pair physics over the list, after the exact test.
// FP64 form: phase 2 redoes the reference's neighbour test exactly
// (q = r / h_ij <= 3 with correctly rounded operations) and its arithmetic.
// Mixed form: phase 2 runs in FP32 on double-float differences of the FP64
// state.
#include <math.h>

#include <type_traits>

#include "sph_internal.cuh"

namespace sph {

constexpr int kPairBlock = 128;
// per-thread neighbour-list capacity: above the typical number of pairs inside
// the support (about 21 for the cubic spline at h = 1.3 dx, 43 for the
// Gaussian cut at 3h), so that the mid-walk flush -- which runs divergently --
// stays rare
template <int KERNEL>
struct ListCap {
  static constexpr int value = Support<KERNEL>::q == 2 ? 32 : 64;
};
#ifndef SPH_PAIR_MIXED_BLOCKS
#define SPH_PAIR_MIXED_BLOCKS 8
#endif


// Exact size of the reference's neighbour set of a query whose own cell is
// not in its stencil (x-overflow alias) or whose h is not positive; those are
// the only queries that can have an empty set (src/Tools/SolverTools.py:150-153).
__device__ int exact_count(const StepArgs &a, const int *__restrict__ perm, const DevGrid &g, int2 qref, int qkey,
                           int W, bool filter, const int2 *__restrict__ meta, const unsigned int *__restrict__ cstart,
                           double xi, double yi, double hi) {
  const Stencil sten(g, qref, qkey, W);
  int cnt = 0;
  for_stencil(sten, cstart, [&](unsigned int j) {
    if (filter && !in_ref_stencil(meta, j, g, qref)) return;
    const int pj = perm[j];
    const double dx = xi - a.x[pj], dy = yi - a.y[pj];
    const double r = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    const double q = __ddiv_rn(r, __dmul_rn(0.5, __dadd_rn(hi, a.h[pj])));
    if (q <= 3.0) cnt++;
  });
  return cnt;
}

// TimeStep epilogue: the block's max a^2 over fluid; the last block computes
// {dt, dt_courant, dt_force} (TimeStep.py:7-56) from the min h the records
// pass gathered, and resets the slots.
__device__ __forceinline__ void timestep_epilogue(DevCtrl *ctrl, unsigned long long ea, double co, double cfl_c,
                                                  double cfl_f, double *dt_out, double *dt_hist,
                                                  unsigned int *zero_on_last = nullptr,
                                                  unsigned int nblocks = 0 /* 0: every block of the grid */) {
  __shared__ unsigned long long red[kPairBlock / 32];
  __shared__ bool last;
  const unsigned int nb = nblocks ? nblocks : gridDim.x;
  const unsigned long long wm = warp_max_u64(ea);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = wm;
  __syncthreads();
  unsigned long long ba = kEncMaxId;
  if (threadIdx.x == 0) {
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) ba = red[w] > ba ? red[w] : ba;
    if (nb == 1) {
      last = true;
    } else {
      if (ba != kEncMaxId) atomicMax(&ctrl->pd_a2max, ba);
      __threadfence();
      last = atomicAdd(&ctrl->done_pair, 1u) == nb - 1;
    }
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    unsigned long long eh, ea2;
    unsigned int cnt;
    if (nb == 1) {
      // the only block: the other contributions came from kernels that
      // completed before this one started, so plain loads see them (one
      // round trip instead of a fence and a chain of returning atomics)
      eh = __ldcg(&ctrl->pd_hmin);
      ea2 = __ldcg(&ctrl->pd_a2max);
      cnt = __ldcg(&ctrl->pd_nfluid);
      ea2 = ba > ea2 ? ba : ea2;
      ctrl->pd_hmin = kEncMinId;
      ctrl->pd_a2max = kEncMaxId;
      ctrl->pd_nfluid = 0u;
    } else {
      __threadfence();
      eh = atomicExch(&ctrl->pd_hmin, kEncMinId);
      ea2 = atomicExch(&ctrl->pd_a2max, kEncMaxId);
      cnt = atomicExch(&ctrl->pd_nfluid, 0u);
      atomicExch(&ctrl->done_pair, 0u);
    }
    if (zero_on_last) *zero_on_last = 0u;
    const double min_h = dec_d(eh);
    const double max_a2 = dec_d(ea2);
    const double max_c = co;  // compute_speed_of_sound gives co to every particle (WCSPH.py:110-129)
    double dc = __ddiv_rn(__dmul_rn(cfl_c, min_h), max_c);
    double df = max_a2 < 1e-12 ? 1e10 : __dmul_rn(cfl_f, __dsqrt_rn(__ddiv_rn(min_h, max_a2)));
    double dt = (df < dc) ? df : dc;  // Python min(c, f) keeps c on ties
    unsigned st = 0;
    if (cnt == 0) {
      st |= SPH_STATUS_NO_FLUID;
      dt = dc = df = nan("");
    }
    if (dt < 1e-6) st |= SPH_STATUS_SMALL_DT;
    if (st) atomicOr(&ctrl->status, st);
    if (dt_out) {
      dt_out[0] = dt;
      dt_out[1] = dc;
      dt_out[2] = df;
    }
    if (dt_hist) {
      dt_hist[0] = dt;
      dt_hist[1] = dc;
      dt_hist[2] = df;
    }
  }
}

// a^2 as TimeStep.computeVars forms it (no contraction)
__device__ __forceinline__ double accel2(double ax, double ay) {
  return __dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay));
}

// ---------------------------------------------------------------------------
// Mixed-form pair physics, shared by the tile kernel and the global-path
// kernel so that both give bit-identical sums for the same candidate order.
// ---------------------------------------------------------------------------
struct MixedAcc {
  float fd = 0.f, fax = 0.f, fay = 0.f, fbx = 0.f, fby = 0.f, fsx = 0.f, fsy = 0.f;
};

struct MixedConsts {
  float KC, r02f, co, alpha, beta, eps, D;
  float avc;  // alpha c_ij with c_ij = co / 2 (Momentum.py's averaged c, the neighbour's c being 0)
};

template <int KERNEL>
__device__ __forceinline__ MixedConsts mixed_consts(const PairParams &pp) {
  MixedConsts c;
  c.KC = (float)(Support<KERNEL>::q * Support<KERNEL>::q);  // (support / h)^2
  const float r0f = (float)pp.r0;
  c.r02f = r0f * r0f;
  c.co = (float)pp.co;
  c.alpha = (float)pp.alpha;
  c.beta = (float)pp.beta;
  c.eps = (float)pp.eps;
  c.D = (float)pp.D;
  c.avc = c.alpha * 0.5f * c.co;
  return c;
}

// Uniform fluid h (the run has a fixed h, Solver(h=...)) and beta = 0 (the
// reference's WCSPH default): every fluid record carries the same FP32 h, so
// for a fluid query i and a fluid neighbour j, h_ij = 0.5 (h_i + h_j) = h_i
// exactly, and the averaged h of the viscosity term is h_i as well.  The
// kernel, gradient and viscosity constants are then per query, computed once,
// and with beta = 0 the viscosity
//   Pi_ij = mu (beta mu - alpha c_ij) / rho_ij,  mu = h v.r / (r^2 + 0.01 h^2)
// is (-2 alpha c_ij h) v.r / ((r^2 + 0.01 h^2)(rho_i + rho_j)): one
// reciprocal per pair.
struct UniformQ {
  float lim;     // (support h)^2
  float inv_h;   // 1 / h
  float al;      // the kernel's normalisation at h
  float g0, g1, g2;  // kernel-gradient polynomial coefficients with al / h folded in
  float hb2;     // 0.01 h^2 (viscosity denominator)
  float pic;     // -2 alpha c_ij h (viscosity numerator)
};

template <int KERNEL>
__device__ __forceinline__ UniformQ uniform_q(const MixedConsts &c, float h) {
  UniformQ u;
  u.lim = c.KC * (h * h);
  u.inv_h = __fdividef(1.0f, h);
  const float fac = KERNEL == SPH_KERNEL_CUBIC ? (float)kCubicFac
                                               : (KERNEL == SPH_KERNEL_WENDLAND ? (float)kWendFac : (float)kInvPi);
  u.al = fac * u.inv_h * u.inv_h;
  const float alh = u.al * u.inv_h;
  if (KERNEL == SPH_KERNEL_CUBIC) {
    // dW/dr / r = al/h (-0.75 (2 - q)^2) / r (q > 1), al/h q (2.25 q - 3) / r (q <= 1)
    u.g0 = -0.75f * alh;
    u.g1 = 2.25f * alh;
    u.g2 = -3.0f * alh;
  } else if (KERNEL == SPH_KERNEL_WENDLAND) {
    // dW/dr / r = al/h (1 - q/2)^5 q (-14/3 - 35/3 q) / r
    u.g0 = (-14.0f / 3.0f) * alh;
    u.g1 = (-35.0f / 3.0f) * alh;
    u.g2 = 0.f;
  } else {
    // dW/dr / r = -2 al / h^2 exp(-q^2)
    u.g0 = -2.0f * alh * u.inv_h;
    u.g1 = u.g2 = 0.f;
  }
  u.hb2 = 0.01f * (h * h);
  u.pic = -2.0f * c.avc * h;
  return u;
}

// One FLUID neighbour j of fluid query i under a uniform fluid h and beta = 0
// (see UniformQ): the same equations as mixed_pair's fluid branch with the
// per-pair h arithmetic taken out.
template <int KERNEL, bool XSPH, bool SUMDENS>
__device__ __forceinline__ void mixed_fluid_uh(MixedAcc &acc, const MixedConsts &c, const UniformQ &u, float hq,
                                               float4 Qi, float4 Ri, float4 Vi, float4 qj, float4 rj,
                                               const float4 *vjp) {
  const float dx = (Qi.x - qj.x) + (Ri.x - rj.x);
  const float dy = (Qi.y - qj.y) + (Ri.y - rj.y);
  const float d2 = dx * dx + dy * dy;
  if (d2 > u.lim) return;
  const float4 vj = *vjp;
  // 1/r, and 0 below r = 1e-10 (d2 = 1e-20), where the kernel gradient of
  // the 2h kernels is taken as 0: the guard on the gradient folds into it
  const bool g2h = KERNEL == SPH_KERNEL_CUBIC || KERNEL == SPH_KERNEL_WENDLAND;
  const float inv_r = d2 >= (g2h ? 1e-20f : 0.f) && d2 > 0.f ? rsqrtf(d2) : 0.f;
  const float r = d2 * inv_r;
  const float q = r * u.inv_h;
  const float vxij = (Vi.x - vj.x) + (Vi.z - vj.z);
  const float vyij = (Vi.y - vj.y) + (Vi.w - vj.w);
  float w = 0.f, coef;
  if (KERNEL == SPH_KERNEL_CUBIC) {
    const float t2 = fmaxf(2.0f - q, 0.f);
    const bool outer = q > 1.0f;
    if (XSPH) w = outer ? u.al * 0.25f * (t2 * t2 * t2) : u.al * (1.0f - 1.5f * (q * q) * (1.0f - 0.5f * q));
    const float g = outer ? u.g0 * (t2 * t2) : q * fmaf(u.g1, q, u.g2);
    coef = g * inv_r;
  } else if (KERNEL == SPH_KERNEL_WENDLAND) {
    const float inner = fmaxf(1.0f - 0.5f * q, 0.f);
    const float i2 = inner * inner, i5 = i2 * i2 * inner;
    if (XSPH) w = u.al * (i5 * inner) * ((35.0f / 12.0f) * q * q + 3.0f * q + 1.0f);
    coef = i5 * q * fmaf(u.g1, q, u.g0) * inv_r;
  } else {
    const float e = __expf(-q * q);
    if (XSPH) w = u.al * e;
    coef = r * hq > 1e-12f ? u.g0 * e : 0.f;
  }
  const float dwx = coef * dx, dwy = coef * dy;
  const float mj = qj.w;
  if (!SUMDENS) acc.fd = fmaf(mj, vxij * dwx + vyij * dwy, acc.fd);
  const float dot = vxij * dx + vyij * dy;
  const float rs = Ri.z + rj.z;  // 2 rho_ij
  const float PI = dot < 0.f ? u.pic * dot * __fdividef(1.0f, (d2 + u.hb2) * rs) : 0.f;
  const float fac = mj * (Ri.w + rj.w + PI);
  acc.fax = fmaf(-fac, dwx, acc.fax);
  acc.fay = fmaf(-fac, dwy, acc.fay);
  if (XSPH) {
    const float fx = -c.eps * mj * w * __fdividef(2.0f, rs);
    acc.fsx = fmaf(fx, vxij, acc.fsx);
    acc.fsy = fmaf(fx, vyij, acc.fsy);
  }
}

// One candidate j of query i: the exact support test, then continuity,
// momentum with artificial viscosity, the Lennard-Jones boundary force and
// XSPH.  Qi/qj: x_hi, y_hi, h (sign bit: non-fluid), m; Ri/rj: x_lo, y_lo,
// rho, p / rho^2; Vi and *vjp: vx_hi, vy_hi, vx_lo, vy_lo (read only when the
// pair is inside the support).
template <int KERNEL, bool XSPH, bool SUMDENS>
__device__ __forceinline__ void mixed_pair(MixedAcc &acc, const MixedConsts &c, float4 Qi, float4 Ri, float4 Vi,
                                           float4 qj, float4 rj, const float4 *vjp) {
  const float hif = Qi.z;
  const float dx = (Qi.x - qj.x) + (Ri.x - rj.x);
  const float dy = (Qi.y - qj.y) + (Ri.y - rj.y);
  const float d2 = dx * dx + dy * dy;
  const float hij = 0.5f * (hif + fabsf(qj.z));
  const float h2 = hij * hij;
  const bool jf = !signbit(qj.z);
  float lim = c.KC * h2;
  if (!jf) lim = fmaxf(lim, fminf(c.r02f, 9.0f * h2));
  if (d2 > lim) return;
  const float4 vj = *vjp;
  const float inv_h = __fdividef(1.0f, hij);
  const float inv_r = d2 > 0.f ? rsqrtf(d2) : 0.f;
  const float r = d2 * inv_r;
  const float q = r * inv_h;
  const float vxij = (Vi.x - vj.x) + (Vi.z - vj.z);
  const float vyij = (Vi.y - vj.y) + (Vi.w - vj.w);
  float w, coef;
  if (KERNEL == SPH_KERNEL_CUBIC) {
    const float al = (float)kCubicFac * inv_h * inv_h;
    const float t2 = fmaxf(2.0f - q, 0.f);
    const bool outer = q > 1.0f;
    w = outer ? al * 0.25f * (t2 * t2 * t2) : al * (1.0f - 1.5f * (q * q) * (1.0f - 0.5f * q));
    const float gq = outer ? -0.75f * (t2 * t2) : -3.0f * q * (1.0f - 0.75f * q);
    coef = r >= 1e-10f ? al * gq * inv_h * inv_r : 0.f;
  } else if (KERNEL == SPH_KERNEL_WENDLAND) {
    const float al = (float)kWendFac * inv_h * inv_h;
    const float inner = fmaxf(1.0f - 0.5f * q, 0.f);
    const float i2 = inner * inner, i5 = i2 * i2 * inner;
    w = al * (i5 * inner) * ((35.0f / 12.0f) * q * q + 3.0f * q + 1.0f);
    const float gq = i5 * (-14.0f / 3.0f) * q * (1.0f + 2.5f * q);
    coef = r >= 1e-10f ? al * gq * inv_h * inv_r : 0.f;
  } else {
    const float ac = (float)kInvPi * inv_h * inv_h;
    const float e = __expf(-q * q);
    w = ac * e;
    coef = r * hij > 1e-12f ? -2.0f * ac * e * inv_h * inv_h : 0.f;
  }
  const float dwx = coef * dx, dwy = coef * dy;
  const float mj = qj.w;
  if (jf) {
    if (!SUMDENS) acc.fd = fmaf(mj, vxij * dwx + vyij * dwy, acc.fd);
    const float dot = vxij * dx + vyij * dy;
    const float hb = 0.5f * (hif + hij);
    const float mu = hb * dot * __fdividef(1.0f, d2 + 0.01f * hb * hb);
    const float PI = dot < 0.f ? mu * (c.beta * mu - c.alpha * 0.5f * c.co) * __fdividef(2.0f, Ri.z + rj.z) : 0.f;
    const float fac = mj * (Ri.w + rj.w + PI);
    acc.fax = fmaf(-fac, dwx, acc.fax);
    acc.fay = fmaf(-fac, dwy, acc.fay);
  } else if (d2 <= c.r02f && d2 > 1e-24f) {
    const float ir2 = __fdividef(1.0f, d2);
    const float f2 = c.r02f * ir2;
    const float fac = c.D * (f2 * f2 - f2) * ir2;
    acc.fbx = fmaf(fac, dx, acc.fbx);
    acc.fby = fmaf(fac, dy, acc.fby);
  }
  if (XSPH) {
    const float fac = -c.eps * mj * w * __fdividef(2.0f, Ri.z + rj.z);
    acc.fsx = fmaf(fac, vxij, acc.fsx);
    acc.fsy = fmaf(fac, vyij, acc.fsy);
  }
}

// One list entry j of query i: with a uniform fluid h and beta = 0 (UH), fluid
// neighbours take the fast path and the rest (boundary particles) the general
// one.
template <int KERNEL, bool XSPH, bool SUMDENS, bool UH>
__device__ __forceinline__ void mixed_entry(MixedAcc &acc, const MixedConsts &c, const UniformQ &u, float4 Qi,
                                            float4 Ri, float4 Vi, float4 qj, float4 rj, const float4 *vjp) {
  if (UH && !signbit(qj.z))
    mixed_fluid_uh<KERNEL, XSPH, SUMDENS>(acc, c, u, Qi.z, Qi, Ri, Vi, qj, rj, vjp);
  else
    mixed_pair<KERNEL, XSPH, SUMDENS>(acc, c, Qi, Ri, Vi, qj, rj, vjp);
}

// Writes the derivatives of particle i (gravity on y) and returns its encoded
// a^2 for the TimeStep reduction.
template <bool XSPH, bool SUMDENS>
__device__ __forceinline__ unsigned long long mixed_store(const MixedAcc &acc, const StepArgs &a, int i) {
  const float axs = acc.fax + acc.fbx, ays = acc.fay + acc.fby;
  a.ax[i] = f2d(axs);
  a.ay[i] = f2d(ays) - 9.81;
  a.drho[i] = SUMDENS ? 0.0 : f2d(acc.fd);
  if (XSPH) {
    a.xsphx[i] = a.vx[i] + f2d(acc.fsx);
    a.xsphy[i] = a.vy[i] + f2d(acc.fsy);
  } else {
    a.xsphx[i] = 0.0;
    a.xsphy[i] = 0.0;
  }
  const float ayg = ays - 9.81f;
  return enc_d(f2d(axs * axs + ayg * ayg));
}

struct PairPtrs {
  const float4 *rec0, *rec1, *rec2;
  const double4_32a *r64a, *r64b;
  const int *perm, *keys_sorted;
  const int2 *meta;
  const unsigned int *cstart;
  const DevGrid *grid;
  DevCtrl *ctrl;
};

// resident blocks per SM the register allocation targets: the mixed form is
// latency-bound and wants occupancy; the FP64 form is FP64-issue-bound
template <bool MIXED>
struct PairOcc {
  static constexpr int blocks = MIXED ? SPH_PAIR_MIXED_BLOCKS : 4;
};

// Global-path evaluation of query slot k (all candidate records read from
// global memory); returns the encoded a^2 of a fluid query, else the max
// identity.  lists: the block's per-thread candidate lists.
template <int KERNEL, bool XSPH, bool SUMDENS, bool MIXED, bool UH = false>
__device__ __forceinline__ unsigned long long pair_query(const StepArgs &a, const PairPtrs &P, const PairParams &pp,
                                                         const DevGrid &g, bool filter, long long k,
                                                         unsigned int (*lists)[kPairBlock], int cell0 = 0) {
  // cell0: global id of grid g's first cell (batched form)
  const unsigned int *cst = P.cstart + cell0;
  constexpr int kListCap = ListCap<KERNEL>::value;
  const int tid = threadIdx.x;
  unsigned long long ea = kEncMaxId;
  const float SK = (float)Support<KERNEL>::q * 1.000002f;  // support / h, padded
  const float r0f = (float)pp.r0;
  const float pad = g.pad_e;
  {
    const float4 Qi = P.rec0[k];  // x_hi, y_hi, h (signed), m
    const float hif = Qi.z;
    if (!signbit(hif)) {
      const int i = P.perm[k];
      const int2 qref = P.meta[k];
      const int qkey = P.keys_sorted[k] - cell0;
      const bool slow = qref.x >= g.ncx || !(hif > 0.f);
      const int W = g.mode == 0 ? 1 : (slow ? g.wide : g.wt);
      // query state
      double xi = 0, yi = 0, vxi = 0, vyi = 0, rhoi = 0, slf = 0, hi = 0;
      float4 Ri = make_float4(0, 0, 0, 0), Vi = make_float4(0, 0, 0, 0);
      if (MIXED) {
        Ri = P.rec1[k];  // x_lo, y_lo, rho, p / rho^2
        Vi = P.rec2[k];
      } else {
        const double4_32a A = P.r64a[k], B = P.r64b[k];
        xi = A.x; yi = A.y; vxi = A.z; vyi = A.w;
        rhoi = B.y; slf = B.z; hi = B.w;
      }
      // accumulators: FP32 (mixed) or FP64
      MixedAcc acc;
      const MixedConsts mc = mixed_consts<KERNEL>(pp);
      const UniformQ uq = uniform_q<KERNEL>(mc, hif);
      double dd = 0.0, dax = 0.0, day = 0.0, dbx = 0.0, dby = 0.0, dsx = 0.0, dsy = 0.0, dfr = 0.0;

      // ---- phase 2: pair physics over the list
      auto physics = [&](int cnt) {
        for (int t = 0; t < cnt; t++) {
          const unsigned int j = lists[t][tid];
          if (MIXED) {
            mixed_entry<KERNEL, XSPH, SUMDENS, UH>(acc, mc, uq, Qi, Ri, Vi, P.rec0[j], P.rec1[j], P.rec2 + j);
          } else {
            const double4_32a A = P.r64a[j], B = P.r64b[j];
            const double dx = xi - A.x, dy = yi - A.y;
            const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
            const double hij = __dmul_rn(0.5, __dadd_rn(hi, fabs(B.w)));
            const double r = __dsqrt_rn(d2);
            const double q = __ddiv_rn(r, hij);
            if (!(q <= 3.0)) continue;  // NNLinkedList.py:74
            const bool jf = !signbit(B.w);
            const double mj = B.x, rhoj = B.y;
            const double vxij = vxi - A.z, vyij = vyi - A.w;
            double w = 0.0, coef = 0.0;
            if (KERNEL == SPH_KERNEL_CUBIC) {
              if (q <= 2.0) {
                const double al = kCubicFac / (hij * hij);
                if (q > 1.0) {
                  const double t2 = 2.0 - q;
                  w = al * 0.25 * (t2 * t2 * t2);
                  if (r >= 1e-10) coef = al * (-0.75 * (t2 * t2)) / (hij * r);
                } else {
                  w = al * (1.0 - 1.5 * (q * q) * (1.0 - 0.5 * q));
                  if (r >= 1e-10) coef = al * (-3.0 * q * (1.0 - 0.75 * q)) / (hij * r);
                }
              }
            } else if (KERNEL == SPH_KERNEL_WENDLAND) {
              w = wendland_w(r, hij);
              coef = wendland_gcoef(r, hij);
            } else {
              const double ac = kInvPi / (hij * hij);
              const double e = exp(-q * q);
              w = ac * e;
              const double tmp = r * hij;
              if (tmp > 1e-12) coef = (-2.0 * q * ac * e) / tmp;
            }
            const double dwx = coef * dx, dwy = coef * dy;
            if (jf) {
              if (!SUMDENS) dd += mj * (vxij * dwx + vyij * dwy);
              const double dot = vxij * dx + vyij * dy;
              double PI = 0.0;
              if (dot < 0.0) {
                const double hb = 0.5 * (hi + hij);
                const double mu = hb * dot / (r * r + 0.01 * hb * hb);
                PI = mu * (pp.beta * mu - pp.alpha * (0.5 * pp.co)) / (0.5 * (rhoi + rhoj));
              }
              const double fac = slf + B.z + PI;
              dax += -mj * fac * dwx;
              day += -mj * fac * dwy;
            } else if (r <= pp.r0 && r > 1e-12) {
              const double frac = pp.r0 / r;
              double tmp;
              if (pp.lj_42) {
                const double f2 = frac * frac;
                tmp = f2 * f2 - f2;
              } else {
                tmp = pow(frac, pp.p1) - pow(frac, pp.p2);
              }
              const double fac = pp.D * tmp;
              const double r2 = r * r;
              dbx += fac * dx / r2;
              dby += fac * dy / r2;
              if (pp.fr && A.x >= pp.wall_x) dfr += fac * dx / r2;
            }
            if (XSPH) {
              const double fac = -pp.eps * mj * w / (0.5 * (rhoi + rhoj));
              dsx += fac * vxij;
              dsy += fac * vyij;
            }
          }
        }
      };

      // ---- phase 1: padded FP32 radius test, append to this thread's list
      const Stencil sten(g, qref, qkey, W);
      int nl = 0;
      for_stencil(sten, cst, [&](unsigned int j) {
        if (j == (unsigned int)k) return;  // the particle itself contributes zero
        if (filter && !in_ref_stencil(P.meta, j, g, qref)) return;
        const float4 qj = P.rec0[j];
        const float dx = Qi.x - qj.x, dy = Qi.y - qj.y;
        const float d2 = dx * dx + dy * dy;
        const float hij = 0.5f * (hif + fabsf(qj.z));
        float reach = SK * hij;
        if (signbit(qj.z)) reach = fmaxf(reach, fminf(r0f, 3.0f * hij) * 1.000002f);
        const float rp = reach + pad;
        if (d2 <= rp * rp) {
          lists[nl][tid] = j;
          if (++nl == kListCap) {
            physics(nl);
            nl = 0;
          }
        }
      });
      physics(nl);

      // the reference's set always holds the particle itself, except for the
      // slow queries, whose set size is counted exactly
      bool any = true;
      if (slow) {
        if (MIXED) {
          xi = a.x[i];
          yi = a.y[i];
          hi = a.h[i];
        }
        any = exact_count(a, P.perm, g, qref, qkey, W, g.mode == 1, P.meta, cst, xi, yi, hi) > 0;
      }
      if (any) {
        if (MIXED) {
          ea = mixed_store<XSPH, SUMDENS>(acc, a, i);
        } else {
          const double axf = dax + dbx;
          const double ayf = (day - 9.81) + dby;
          a.drho[i] = SUMDENS ? 0.0 : dd;
          a.xsphx[i] = XSPH ? vxi + dsx : 0.0;
          a.xsphy[i] = XSPH ? vyi + dsy : 0.0;
          ea = enc_d(accel2(axf, ayf));
          a.ax[i] = axf;
          a.ay[i] = ayf;
          if (pp.fr) pp.fr[i] = -P.r64b[k].x * dfr;
        }
      } else {
        ea = enc_d(accel2(a.ax[i], a.ay[i]));  // keeps its previous values (SolverTools.py:150-153)
        if (!MIXED && pp.fr) pp.fr[i] = 0.0;
      }
    }
  }
  return ea;
}

template <int KERNEL, bool XSPH, bool SUMDENS, bool MIXED>
__global__ void __launch_bounds__(kPairBlock, PairOcc<MIXED>::blocks)
    k_pair(StepArgs a, PairPtrs P, PairParams pp, double *dt_out, double *dt_hist) {
  __shared__ unsigned int lists[ListCap<KERNEL>::value][kPairBlock];
  const DevGrid g = *P.grid;
  const bool filter = g.mode == 1 && (g.need_filter || P.ctrl->alias_count > 0);
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long ea = kEncMaxId;
  if (k < pp.n) ea = pair_query<KERNEL, XSPH, SUMDENS, MIXED>(a, P, pp, g, filter, k, lists);
  if (pp.do_dt) timestep_epilogue(P.ctrl, ea, pp.co, pp.cfl_c, pp.cfl_f, dt_out, dt_hist);
}

// The queries the tile kernel left over (slot ranges of at most kPairBlock
// slots), on the global path; the last block resets the list and, when asked,
// finishes the TimeStep reduction.
constexpr int kListBlocks = 6;
template <int KERNEL, bool XSPH, bool SUMDENS, bool UH>
__global__ void __launch_bounds__(kPairBlock, kListBlocks)
    k_pair_list(StepArgs a, PairPtrs P, PairParams pp, const int2 *__restrict__ fb, double *dt_out,
                double *dt_hist) {
  step_kernel_entry();
  __shared__ unsigned int lists[ListCap<KERNEL>::value][kPairBlock];
  const unsigned int cnt = *(volatile unsigned int *)&P.ctrl->fb_count;
  // only the blocks that have entries take part (at least block 0, which
  // finishes the TimeStep when the list is empty); the rest leave at once.
  // A block that starts after the last participant emptied the list reads
  // 0 and leaves too: the list is emptied only once every participant,
  // itself included, has read the count.
  const unsigned int parts = cnt < gridDim.x ? (cnt > 0u ? cnt : 1u) : gridDim.x;
  if (blockIdx.x >= parts) return;
  unsigned long long ea = kEncMaxId;
  if (blockIdx.x < cnt) {
    const DevGrid g = *P.grid;
    const bool filter = g.mode == 1 && (g.need_filter || P.ctrl->alias_count > 0);
    for (unsigned int e = blockIdx.x; e < cnt; e += gridDim.x) {
      const int2 r = fb[e];
      if ((int)threadIdx.x < r.y) {
        const unsigned long long q =
            pair_query<KERNEL, XSPH, SUMDENS, true, UH>(a, P, pp, g, filter, r.x + threadIdx.x, lists);
        ea = q > ea ? q : ea;
      }
    }
  }
  __syncthreads();
  // the last participant empties the fallback list (with the TimeStep
  // epilogue when there is one)
  if (pp.do_dt) {
    timestep_epilogue(P.ctrl, ea, pp.co, pp.cfl_c, pp.cfl_f, dt_out, dt_hist, &P.ctrl->fb_count, parts);
  } else if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&P.ctrl->fb_done, 1u) == parts - 1) {
      P.ctrl->fb_count = 0;
      P.ctrl->fb_done = 0;
    }
  }
}

// ---------------------------------------------------------------------------
// Summation density (SolverTools.py:129-140, SummationDensity.py:5-13):
// rho_i = sum over fluid neighbours (itself included) of m_j W(r, h_ij).
// ---------------------------------------------------------------------------
template <int KERNEL, bool MIXED>
__global__ void __launch_bounds__(kPairBlock) k_sumdens(StepArgs a, PairPtrs P, long long n) {
  const DevGrid g = *P.grid;
  const bool filter = g.mode == 1 && (g.need_filter || P.ctrl->alias_count > 0);
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float4 Qi = P.rec0[k];
  const float hif = Qi.z;
  if (signbit(hif)) return;
  const int2 qref = P.meta[k];
  const int qkey = P.keys_sorted[k];
  const bool slow = qref.x >= g.ncx || !(hif > 0.f);
  const int W = g.mode == 0 ? 1 : (slow ? g.wide : g.wt);
  double xi = 0, yi = 0, hi = 0;
  float4 Ri = make_float4(0, 0, 0, 0);
  if (MIXED) {
    Ri = P.rec1[k];
  } else {
    const double4_32a A = P.r64a[k], B = P.r64b[k];
    xi = A.x; yi = A.y; hi = B.w;
  }
  const float KC = (float)(Support<KERNEL>::q * Support<KERNEL>::q);
  const float SK = (float)Support<KERNEL>::q * 1.000002f;
  double rho = 0.0;
  float rhof = 0.f;
  const Stencil sten(g, qref, qkey, W);
  for_stencil(sten, P.cstart, [&](unsigned int j) {
      if (filter && !in_ref_stencil(P.meta, j, g, qref)) return;
      const float4 qj = P.rec0[j];
      if (signbit(qj.z)) return;  // SummationDensity.py: fluid neighbours only
      const float hij = 0.5f * (hif + fabsf(qj.z));
      if (MIXED) {
        const float4 rj = P.rec1[j];
        const float dx = (Qi.x - qj.x) + (Ri.x - rj.x);
        const float dy = (Qi.y - qj.y) + (Ri.y - rj.y);
        const float d2 = dx * dx + dy * dy;
        if (d2 > KC * hij * hij) return;
        const float q = sqrtf(d2) / hij;
        float w;
        if (KERNEL == SPH_KERNEL_CUBIC) {
          const float al = (float)kCubicFac / (hij * hij);
          const float t = fmaxf(2.0f - q, 0.f);
          w = q > 1.0f ? al * 0.25f * t * t * t : al * (1.0f - 1.5f * q * q * (1.0f - 0.5f * q));
        } else if (KERNEL == SPH_KERNEL_WENDLAND) {
          const float inner = fmaxf(1.0f - 0.5f * q, 0.f), i2 = inner * inner;
          w = (float)kWendFac / (hij * hij) * (i2 * i2 * i2) * ((35.0f / 12.0f) * q * q + 3.0f * q + 1.0f);
        } else {
          w = (float)kInvPi / (hij * hij) * __expf(-q * q);
        }
        rhof += qj.w * w;
      } else {
        const float dx = Qi.x - qj.x, dy = Qi.y - qj.y;
        const float rp = SK * hij + g.pad_e;
        if (dx * dx + dy * dy > rp * rp) return;
        const double4_32a A = P.r64a[j], B = P.r64b[j];
        const double ddx = xi - A.x, ddy = yi - A.y;
        const double r = __dsqrt_rn(__dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)));
        const double h = __dmul_rn(0.5, __dadd_rn(hi, fabs(B.w)));
        if (__ddiv_rn(r, h) <= 3.0)
          rho += B.x * (KERNEL == SPH_KERNEL_CUBIC ? cubic_w(r, h)
                                                   : (KERNEL == SPH_KERNEL_WENDLAND ? wendland_w(r, h) : gauss_w(r, h)));
      }
   });
  a.rho[P.perm[k]] = MIXED ? f2d(rhof) : rho;
}

// ---------------------------------------------------------------------------
// Neighbour-set export (NNLinkedList.near for every particle, FP64 exact):
// count pass (idx == nullptr) or fill pass.  Reads the caller's arrays.
// Each list comes out in the reference's order (NNLinkedList.py:50-78): the
// 3x3 stencil cells with the x shift outer and the y shift inner, and inside
// a cell its linked list, head-insert order, i.e. descending index.
// ---------------------------------------------------------------------------
// Sort key of member j in the list of a query whose raw reference cell is
// qref: the stencil position of j's storage cell (an x-overflow particle is
// stored in the aliased cell), then descending index.  Smaller comes first.
__device__ __forceinline__ unsigned long long ref_order_key(const int2 *__restrict__ refcell, long long ncx,
                                                            int2 qref, long long j) {
  const int2 rc = refcell[j];
  int sx, sy;
  storage_cell(rc.x, rc.y, ncx, sx, sy);
  const unsigned p = (unsigned)((sx - qref.x + 1) * 3 + (sy - qref.y + 1));  // 0..8 for members
  return ((unsigned long long)p << 32) | (unsigned long long)(0xffffffffu - (unsigned)j);
}

// insertion sort of idx[0..cnt) (and the parallel arrays, when given) into
// the reference's order
__device__ void sort_ref_order(int64_t *idx, double *a0, double *a1, double *a2, long long cnt,
                               const int2 *__restrict__ refcell, long long ncx, int2 qref) {
  for (long long s = 1; s < cnt; s++) {
    const int64_t v = idx[s];
    const unsigned long long kv = ref_order_key(refcell, ncx, qref, v);
    double b0 = 0, b1 = 0, b2 = 0;
    if (a0) {
      b0 = a0[s];
      b1 = a1[s];
      b2 = a2[s];
    }
    long long t = s - 1;
    while (t >= 0 && ref_order_key(refcell, ncx, qref, idx[t]) > kv) {
      idx[t + 1] = idx[t];
      if (a0) {
        a0[t + 1] = a0[t];
        a1[t + 1] = a1[t];
        a2[t + 1] = a2[t];
      }
      t--;
    }
    idx[t + 1] = v;
    if (a0) {
      a0[t + 1] = b0;
      a1[t + 1] = b1;
      a2[t + 1] = b2;
    }
  }
}

__global__ void __launch_bounds__(kPairBlock)
    k_nn_export(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ h,
                long long n, const int *__restrict__ perm, const int *__restrict__ keys_sorted,
                const int2 *__restrict__ meta, const int2 *__restrict__ refcell,
                const unsigned int *__restrict__ cstart, const DevGrid *__restrict__ gp, int64_t *counts,
                const int64_t *offsets, int64_t *idx) {
  const DevGrid g = *gp;
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int i = perm[k];
  const double xi = x[i], yi = y[i], hi = h[i];
  const int2 qref = meta[k];
  const int qkey = keys_sorted[k];
  const int W = g.mode == 1 ? g.wide : 1;
  const bool filter = g.mode == 1;
  long long cnt = 0;
  const long long base = idx ? offsets[i] : 0;
  const Stencil sten(g, qref, qkey, W);
  for_stencil(sten, cstart, [&](unsigned int j) {
      if (filter && !in_ref_stencil(meta, j, g, qref)) return;
      const int pj = perm[j];
      const double dx = xi - x[pj], dy = yi - y[pj];
      const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
      const double r = __dsqrt_rn(d2);
      const double hij = __dmul_rn(0.5, __dadd_rn(hi, h[pj]));
      const double q = __ddiv_rn(r, hij);
      if (q <= 3.0) {
        if (idx) idx[base + cnt] = pj;
        cnt++;
      }
   });
  if (!idx) {
    counts[i] = cnt;
    return;
  }
  sort_ref_order(idx + base, nullptr, nullptr, nullptr, cnt, refcell, g.ncx, qref);
}

// ---------------------------------------------------------------------------
// Tile kernel (mixed form).  A block takes one tile of 2^ts x 2^ts cells at a
// time and stages the records of the tile and its W-cell halo in shared
// memory: a table of the (2^ts + 2W)^2 halo cells (counts -> exclusive scan ->
// shared-memory offsets, cells row-major, so each stencil row of a query is
// one contiguous shared-memory range), then the records row by row.  Its
// queries walk their stencils in shared memory, with 16-bit list entries.
// The candidate order (rows, then cells by x, then slot) is the global
// path's, so both give the same sums.
// Left to the global path, through the fallback list: tiles whose halo does
// not fit, queries whose own cell is not in their stencil or whose h is not
// positive, and every query when candidates need the reference-stencil filter
// or the halo table does not fit (wide stencils).
// Blocks are persistent and claim one tile at a time from the list of
// non-empty tiles the neighbour build writes, the next claim overlapping the
// current tile.
// ---------------------------------------------------------------------------
constexpr int kTileThreads = 256;   // threads of a tile block (8 warps)
static_assert(kTileThreads >= 16 * 16, "a sparse unit's slots fit one per thread");
constexpr int kHaloCellsMax = 400;  // (16 + 2 * 2)^2: 16x16 tiles with a 5x5 stencil
constexpr int kHaloScanPer = (kHaloCellsMax + 31) / 32;
#ifndef SPH_TILE_UNROLL_PAIRS
#define SPH_TILE_UNROLL_PAIRS 1
#endif
#ifndef SPH_TILE_UNROLL_CANDS
#define SPH_TILE_UNROLL_CANDS 2
#endif
// resident tile blocks per SM (registers and shared memory allow three for
// the 32-entry lists of the 2h kernels, two for the Gaussian's 64)
template <int KERNEL>
struct TileBlocks {
  static constexpr int value = ListCap<KERNEL>::value == 32 ? 3 : 2;
};
constexpr bool kSplitTail = true;  // the last tiles of a launch as half-tile units
constexpr int kTileUnrollPairs = SPH_TILE_UNROLL_PAIRS;  // ILP over list entries
constexpr int kTileUnrollCands = SPH_TILE_UNROLL_CANDS;  // ILP over stencil candidates
constexpr int kHaloCap = SPH_HALO_CAP;  // particles of one halo in shared memory
static_assert(kHaloCap <= 65535, "list entries are 16-bit");
static_assert(kHaloCellsMax <= 65535, "query map entries are 16-bit halo cells");

__device__ __forceinline__ void fb_push(DevCtrl *ctrl, int2 *fb, unsigned int fb_cap, unsigned int s,
                                        unsigned int len) {
  const unsigned int e = atomicAdd(&ctrl->fb_count, 1u);
  if (e < fb_cap) fb[e] = make_int2((int)s, (int)len);
}

// Geometry and constants of the grid a tile belongs to.
struct TileGeom {
  int ts, ntlx, ntx, nty, W, T, HW, HC;
  int cell0;  // global id of the grid's first cell (batched form; 0 otherwise)
  long long ncx;
  float r0f, pad, hmaxf;
};

__device__ __forceinline__ TileGeom tile_geom(const DevGrid &g, double r0, int cell0) {
  TileGeom tg;
  tg.ts = g.ts;
  tg.ntlx = g.ntlx;
  tg.ntx = g.ntx;
  tg.nty = g.nty;
  tg.W = g.mode == 0 ? 1 : g.wt;
  tg.T = 1 << g.ts;
  tg.HW = tg.T + 2 * tg.W;
  tg.HC = tg.HW * tg.HW;
  tg.cell0 = cell0;
  tg.ncx = g.ncx;
  tg.r0f = (float)r0;
  tg.pad = g.pad_e;
  tg.hmaxf = g.hmaxf;
  return tg;
}

// shared memory of the tile kernels (dynamic: above the 48 KB static limit)
template <int KERNEL>
struct TileShared {
  float4 h0[kHaloCap], h1[kHaloCap], h2[kHaloCap];  // rec0, rec1, rec2 of the halo
  unsigned short lists[ListCap<KERNEL>::value][kTileThreads];
  unsigned int hoff[kHaloCellsMax + 1];  // shared-memory offset of each halo cell, then the total
  unsigned int hgs[kHaloCellsMax];       // its first sorted slot
  unsigned short qmap[kHaloCap];         // halo cell of each query of the tile
  int s_tile[2];                         // this and the next claimed work unit (-1: none left)
  int s_inst[2];                         // their instances (batched form)
  unsigned long long red[kTileThreads / 32];
};

// One tile: stage its halo, run its queries.  Returns this thread's largest
// encoded a^2 over its queries.  All threads of the block call it together.
//   1. halo table: every halo cell's first sorted slot and count;
//   2. warp 0: exclusive scan of the counts (shared-memory offsets); then
//      every warp copies halo rows into shared memory (a row is at most three
//      runs of consecutive slots) and the threads map each query of the tile
//      to its halo cell;
//   3. each query walks its stencil rows.
// TSC / WC: the tile shift and stencil half-width as compile-time constants
// (the own grid's 16x16 tiles with a 5x5 stencil), so that the halo
// coordinate arithmetic has no integer division; 0 takes them from tg.
// UH: every fluid particle has the same h (UniformQ).
// part: 0 the whole tile; 1 and 2 its first and second half of cell rows;
// 3 to 6 its four quarters (the kernel's last tiles are split so that its
// final round of work is short).
template <int KERNEL, bool XSPH, bool SUMDENS, bool UH, int TSC, int WC>
__device__ __forceinline__ unsigned long long tile_process(const StepArgs &a, const PairPtrs &P, const TileGeom &tg,
                                                           const MixedConsts &mc, int t, int part,
                                                           TileShared<KERNEL> &sm, DevCtrl *ctrl, int2 *fb,
                                                           unsigned int fb_cap, bool skip_dry) {
  constexpr int kListCap = ListCap<KERNEL>::value;
  const int tid = threadIdx.x;
  const int ts = TSC ? TSC : tg.ts;
  const int W = TSC ? WC : tg.W;
  const int T = 1 << ts, HW = T + 2 * W;
  const int rows = part == 0 ? T : (part <= 2 ? T >> 1 : T >> 2);
  const int row0 = part == 2 ? T >> 1 : (part >= 3 ? (part - 3) * (T >> 2) : 0);
  const int HWy = rows + 2 * W, HC = HW * HWy;
  const int ntlx = tg.ntlx;
  float4 *h0 = sm.h0, *h1 = sm.h1, *h2 = sm.h2;
  unsigned int *hoff = sm.hoff, *hgs = sm.hgs;
  const unsigned int *cst = P.cstart + tg.cell0;  // this grid's cells
  unsigned long long ea = kEncMaxId;
  const unsigned int tb = (unsigned int)t << (2 * ts);  // the tile's first cell (row-major inside)
  const unsigned int qs = __ldg(&cst[tb + row0 * T]), qe = __ldg(&cst[tb + (row0 + rows) * T]);
  const int ox = (t % ntlx) * T - W, oy = (t / ntlx) * T + row0 - W;
  // 1. halo table: counts and first slots.  With skip_dry (the batched form,
  // whose small tanks hold many tiles of wall particles alone), alongside,
  // for a sparse unit (less than one particle per cell), whether its own
  // slots hold a fluid particle (the sign bit of a record's h marks the
  // others): a unit of boundary particles alone has no query and stages
  // nothing.  A sparse unit has fewer slots than the block has threads: one
  // load per thread, issued before the table's loads and used only at the
  // barrier.  (On the single-scene dam break the test cost more than the
  // few dry tiles it saves.)
  const bool dense = !skip_dry || qe - qs >= (unsigned int)(T * rows);
  float hq0 = -1.f;  // sign bit set: no fluid
  if (!dense && qs + tid < qe) hq0 = __ldg(&P.rec0[qs + tid].z);
  for (int c = tid; c < HC; c += kTileThreads) {
    const int x = ox + c % HW, y = oy + c / HW;
    unsigned int gs = 0, cnt = 0;
    if (x >= 0 && x < tg.ntx && y >= 0 && y < tg.nty) {
      const int key = tiled_key(x, y, ts, ntlx);
      gs = __ldg(&cst[key]);
      cnt = __ldg(&cst[key + 1]) - gs;
    }
    hgs[c] = gs;
    hoff[c] = cnt;
  }
  if (!__syncthreads_or(dense || !signbit(hq0))) return ea;
  if (tid < 32) {  // 2. exclusive scan of the counts, kHaloScanPer cells per lane
    const int c0 = tid * kHaloScanPer;
    unsigned int v[kHaloScanPer], sum = 0;
#pragma unroll
    for (int u = 0; u < kHaloScanPer; u++) {
      v[u] = c0 + u < HC ? hoff[c0 + u] : 0u;
      sum += v[u];
    }
    unsigned int inc = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned int o = __shfl_up_sync(0xffffffffu, inc, d);
      if (tid >= d) inc += o;
    }
    unsigned int run = inc - sum;
#pragma unroll
    for (int u = 0; u < kHaloScanPer; u++) {
      if (c0 + u < HC) hoff[c0 + u] = run;
      run += v[u];
    }
    if (tid == 31) hoff[HC] = inc;
  }
  __syncthreads();
  const unsigned int total = hoff[HC];
  if (total == 0) {  // nothing to stage (a listed tile holds particles)
    __syncthreads();
    return ea;
  }
  if (total > (unsigned)kHaloCap) {  // halo does not fit: global path
    if (tid == 0)
      for (unsigned int s = qs; s < qe; s += kPairBlock) fb_push(ctrl, fb, fb_cap, s, min((unsigned)kPairBlock, qe - s));
    __syncthreads();
    return ea;
  }
  // 2b. the halo's records, row by row: warp w copies halo rows w, w + 8,
  // ...; a row's cells are one shared-memory range, and in global memory at
  // most three runs (the cells of one row inside one tile are consecutive
  // ids).  Each lane issues 16-byte asynchronous copies of particles of the
  // row, so that all copies of the halo are in flight together and the block
  // waits once.  (One bulk copy per run and record array would be ~180 small
  // copies per tile, whose per-copy cost dominates.)
  {
    const int warp = tid >> 5, lane = tid & 31;
    const int xa = ox > 0 ? ox : 0;
    const int xe = ox + HW < tg.ntx ? ox + HW : tg.ntx;
    for (int y = warp; y < HWy; y += kTileThreads / 32) {
      const int gy = oy + y;
      if (gy < 0 || gy >= tg.nty || xa >= xe) continue;
      const int cb = y * HW - ox;  // halo cell of grid column x: cb + x
      if (T >= W) {
        // runs [xa, x1), [x1, x2), [x2, xe) (empty when their bounds meet)
        const int x1 = min(((xa >> ts) + 1) << ts, xe);
        const int x2 = min(((x1 >> ts) + 1) << ts, xe);
        const unsigned int sA = hoff[cb + xa], sB = hoff[cb + x1], sC = hoff[cb + x2], sE = hoff[cb + xe];
        const unsigned int gA = hgs[cb + xa], gB = x1 < xe ? hgs[cb + x1] : 0u, gC = x2 < xe ? hgs[cb + x2] : 0u;
        for (unsigned int k = sA + lane; k < sE; k += 32) {
          const unsigned int src = k < sB ? gA + (k - sA) : (k < sC ? gB + (k - sB) : gC + (k - sC));
          cp_async16(h0 + k, P.rec0 + src);
          cp_async16(h1 + k, P.rec1 + src);
          cp_async16(h2 + k, P.rec2 + src);
        }
      } else {
        // tiles narrower than the stencil: the row's runs one by one
        for (int x = xa; x < xe;) {
          const int re = min(((x >> ts) + 1) << ts, xe);
          const unsigned int s0 = hoff[cb + x], e0 = hoff[cb + re], g0 = hgs[cb + x];
          for (unsigned int k = s0 + lane; k < e0; k += 32) {
            cp_async16(h0 + k, P.rec0 + g0 + (k - s0));
            cp_async16(h1 + k, P.rec1 + g0 + (k - s0));
            cp_async16(h2 + k, P.rec2 + g0 + (k - s0));
          }
          x = re;
        }
      }
    }
  }
  // query -> halo cell, for the tile's own cells (their sorted slots are the
  // tile's query range, in cell order)
  for (int c = tid; c < T * rows; c += kTileThreads) {
    const int hc = (W + (c >> ts)) * HW + W + (c & (T - 1));
    const unsigned int cnt = hoff[hc + 1] - hoff[hc], base = hgs[hc] - qs;
    for (unsigned int u = 0; u < cnt; u++) sm.qmap[base + u] = (unsigned short)hc;
  }
  cp_async_wait_all();
  __syncthreads();
  // 3. queries.  Candidate radius: the padded reach of the largest pair h
  // (every |h| <= hmaxf), so that one compare per candidate suffices
  const float SK = (float)Support<KERNEL>::q * 1.000002f;  // support / h, padded
  const unsigned int nq = qe - qs;
  for (unsigned int q = tid; q < nq; q += kTileThreads) {
    const int hc = sm.qmap[q];
    const int hx = hc % HW, hy = hc / HW;
    const unsigned int k = qs + q;
    const unsigned int sq = hoff[hc] + (k - hgs[hc]);  // the query's own shared-memory slot
    const float4 Qi = h0[sq];
    const float hif = Qi.z;
    if (signbit(hif)) continue;  // queries are fluid
    // an x-overflow alias (reference cells only) or h <= 0: global path
    if ((W == 1 && P.meta[k].x >= tg.ncx) || !(hif > 0.f)) {
      fb_push(ctrl, fb, fb_cap, k, 1u);
      continue;
    }
    const float4 Ri = h1[sq], Vi = h2[sq];
    const int i = P.perm[k];
    const UniformQ uq = uniform_q<KERNEL>(mc, hif);
    MixedAcc acc;
    auto physics = [&](int cnt) {
#pragma unroll kTileUnrollPairs
      for (int u = 0; u < cnt; u++) {
        const unsigned int j = sm.lists[u][tid];
        mixed_entry<KERNEL, XSPH, SUMDENS, UH>(acc, mc, uq, Qi, Ri, Vi, h0[j], h1[j], h2 + j);
      }
    };
    const float hq = 0.5f * (hif + tg.hmaxf);
    const float rq = fmaxf(SK * hq, fminf(tg.r0f, 3.0f * hq) * 1.000002f) + tg.pad;
    const float rq2 = rq * rq;
    int nl = 0;
    // the stencil rows' slot ranges, the query's own row as the two ranges
    // either side of its own slot (the particle itself is no candidate)
    for (int r = -W, seg = 0; r <= W; seg = 0, r++) {
      const unsigned int *row = hoff + (hy + r) * HW + hx;
      unsigned int j = row[-W];
      const unsigned int e = row[W + 1];
      unsigned int se = r == 0 ? sq : e;
      for (;;) {
        while (j < se) {
          if (nl == kListCap) {
            physics(nl);
            nl = 0;
          }
          // a chunk that cannot overflow the list: every candidate is
          // written, and kept (counted) when inside the radius
          const unsigned int ce = min(se, j + (unsigned int)(kListCap - nl));
#pragma unroll kTileUnrollCands
          for (; j < ce; j++) {
            const float2 p = *reinterpret_cast<const float2 *>(h0 + j);
            const float dx = Qi.x - p.x, dy = Qi.y - p.y;
            sm.lists[nl][tid] = (unsigned short)j;
            nl += fmaf(dx, dx, dy * dy) <= rq2 ? 1 : 0;
          }
        }
        if (r != 0 || seg) break;
        seg = 1;
        j = sq + 1;
        se = e;
      }
    }
    physics(nl);
    const unsigned long long qa = mixed_store<XSPH, SUMDENS>(acc, a, i);
    ea = qa > ea ? qa : ea;
  }
  __syncthreads();
  return ea;
}

// block-wide max of v in thread 0 (all threads call it)
template <int NT>
__device__ __forceinline__ unsigned long long block_max_u64(unsigned long long v, unsigned long long *red) {
  const unsigned long long wm = warp_max_u64(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = wm;
  __syncthreads();
  unsigned long long b = kEncMaxId;
  if (threadIdx.x == 0)
    for (int w = 0; w < NT / 32; w++) b = red[w] > b ? red[w] : b;
  __syncthreads();
  return b;
}

// the tile of a single-scene grid with the shape the grid has
template <int KERNEL, bool XSPH, bool SUMDENS, bool UH>
__device__ __forceinline__ unsigned long long tile_any(const StepArgs &a, const PairPtrs &P, const TileGeom &tg,
                                                       const MixedConsts &mc, int t, int part,
                                                       TileShared<KERNEL> &sm, DevCtrl *ctrl, int2 *fb,
                                                       unsigned int fb_cap, bool skip_dry) {
  if (tg.ts == 4 && tg.W == 2)
    return tile_process<KERNEL, XSPH, SUMDENS, UH, 4, 2>(a, P, tg, mc, t, part, sm, ctrl, fb, fb_cap, skip_dry);
  if (tg.ts == 3 && tg.W == 2)
    return tile_process<KERNEL, XSPH, SUMDENS, UH, 3, 2>(a, P, tg, mc, t, part, sm, ctrl, fb, fb_cap, skip_dry);
  return tile_process<KERNEL, XSPH, SUMDENS, UH, 0, 0>(a, P, tg, mc, t, part, sm, ctrl, fb, fb_cap, skip_dry);
}

template <int KERNEL, bool XSPH, bool SUMDENS, bool UH>
__global__ void __launch_bounds__(kTileThreads, TileBlocks<KERNEL>::value)
    k_pair_tiles(StepArgs a, PairPtrs P, PairParams pp, const int *__restrict__ tiles,
                 const int *__restrict__ tiles_h, unsigned int tiles_cap,
                 int2 *__restrict__ fb, unsigned int fb_cap) {
  step_kernel_entry();
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TileShared<KERNEL> &sm = *reinterpret_cast<TileShared<KERNEL> *>(smem_raw);
  const int tid = threadIdx.x;
  DevCtrl *ctrl = P.ctrl;
  const DevGrid *gp = P.grid;
  const TileGeom tg = tile_geom(*gp, pp.r0, 0);
  const bool filter = gp->mode == 1 && (gp->need_filter || ctrl->alias_count > 0);
  const MixedConsts mc = mixed_consts<KERNEL>(pp);
  unsigned long long ea = kEncMaxId;

  if (filter || tg.HC > kHaloCellsMax) {
    // everything on the global path, in 128-slot chunks
    if (tid == 0) {
      const long long nch = (pp.n + kPairBlock - 1) / kPairBlock;
      for (long long c = blockIdx.x; c < nch; c += gridDim.x)
        fb_push(ctrl, fb, fb_cap, (unsigned)(c * kPairBlock), (unsigned)min((long long)kPairBlock, pp.n - c * kPairBlock));
    }
  } else {
    // Work units in claim order: dense tiles with a wall along a side (their
    // own list), the other dense tiles (listed from the front of the tile
    // list), then the sparse ones (listed from its back).  Of that order, the
    // last `sq` tiles come as four quarter-tile units each and the `sh`
    // before them as two half-tile units each, so that the kernel's final
    // rounds of work are short.  A unit is encoded as 8 tile + part (part 0:
    // whole tile; 1, 2: halves; 3 to 6: quarters), -1 when none is left.
    const unsigned int nh = ctrl->tl_heavy, ntl = nh + ctrl->tl_count, nall = ntl + ctrl->tl_back;
    const unsigned int sq = (kSplitTail && tg.ts >= 2) ? min(nall, gridDim.x / 4u) : 0u;
    const unsigned int sh = (kSplitTail && tg.ts >= 1) ? min(nall - sq, gridDim.x) : 0u;
    const unsigned int nw = nall - sq - sh;  // whole-tile units
    auto tile_at = [&](unsigned int p) {
      return p < nh ? tiles_h[p] : (p < ntl ? tiles[p - nh] : tiles[tiles_cap - 1 - (p - ntl)]);
    };
    auto claim = [&](unsigned int c) {
      if (c < nw) return 8 * tile_at(c);
      c -= nw;
      if (c < 2 * sh) return 8 * tile_at(nw + (c >> 1)) + 1 + (int)(c & 1u);
      c -= 2 * sh;
      return c < 4 * sq ? 8 * tile_at(nw + sh + (c >> 2)) + 3 + (int)(c & 3u) : -1;
    };
    if (tid == 0) {
      if (blockIdx.x == 0) {  // the dump cell (reference-OOB particles) is in no tile
        const unsigned int d0 = __ldg(&P.cstart[gp->ncells]), d1 = __ldg(&P.cstart[gp->ncells + 1]);
        for (unsigned int s = d0; s < d1; s += kPairBlock) fb_push(ctrl, fb, fb_cap, s, min((unsigned)kPairBlock, d1 - s));
      }
      sm.s_tile[0] = claim(atomicAdd(&ctrl->tile_next, 1u));
    }
    __syncthreads();
    for (int it = 0;; it++) {
      const int u = sm.s_tile[it & 1];
      if (u < 0) break;
      if (tid == 0)  // claim the next unit while this one runs
        sm.s_tile[(it + 1) & 1] = claim(atomicAdd(&ctrl->tile_next, 1u));
      const unsigned long long q =
          tile_any<KERNEL, XSPH, SUMDENS, UH>(a, P, tg, mc, u >> 3, u & 7, sm, ctrl, fb, fb_cap, false);
      ea = q > ea ? q : ea;
    }
  }
  // this block's max a^2 (the list kernel finishes the TimeStep reduction);
  // the last block resets the tile counter
  if (pp.do_dt) {
    const unsigned long long ba = block_max_u64<kTileThreads>(ea, sm.red);
    if (tid == 0 && ba != kEncMaxId) atomicMax(&ctrl->pd_a2max, ba);
  }
  if (tid == 0) {
    __threadfence();
    if (atomicAdd(&ctrl->tile_done, 1u) == gridDim.x - 1) {
      ctrl->tile_next = 0;
      ctrl->tile_done = 0;
    }
  }
}

// ---------------------------------------------------------------------------
// Batched form: the tile kernel over the (instance, tile) list of all
// instances, each tile with its instance's grid and constants, and the
// fallback list with each entry's instance (see nn_build.cu).  Every instance
// has a fixed h, so the uniform-h form applies to the instances whose
// viscosity beta is 0; the others take the general per-pair form.
// ---------------------------------------------------------------------------
template <int KERNEL, bool XSPH, bool SUMDENS>
__global__ void __launch_bounds__(kTileThreads, TileBlocks<KERNEL>::value)
    k_bt_pair_tiles(StepArgs a, PairPtrs P, BatchPtrs B, int2 *__restrict__ fb, unsigned int fb_cap) {
  step_kernel_entry();
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TileShared<KERNEL> &sm = *reinterpret_cast<TileShared<KERNEL> *>(smem_raw);
  const int tid = threadIdx.x;
  DevCtrl *ctrl = P.ctrl;
  const unsigned int ntl = ctrl->tl_count;
  if (tid == 0) {
    if (blockIdx.x == 0)  // every instance's dump cell (reference-OOB particles) is in no tile
      for (int b = 0; b < B.n_inst; b++) {
        const int c = B.coff[b] + B.grids[b].ncells;
        const unsigned int d0 = __ldg(&P.cstart[c]), d1 = __ldg(&P.cstart[c + 1]);
        for (unsigned int s = d0; s < d1; s += kPairBlock) fb_push(ctrl, fb, fb_cap, s, min((unsigned)kPairBlock, d1 - s));
      }
    const unsigned int c = atomicAdd(&ctrl->tile_next, 1u);
    const int2 e = c < ntl ? B.tiles[c] : make_int2(-1, -1);
    sm.s_inst[0] = e.x;
    sm.s_tile[0] = e.y;
  }
  __syncthreads();
  for (int it = 0;; it++) {
    const int t = sm.s_tile[it & 1], b = sm.s_inst[it & 1];
    if (t < 0) break;
    if (tid == 0) {  // claim the next tile while this one runs
      const unsigned int c = atomicAdd(&ctrl->tile_next, 1u);
      const int2 e = c < ntl ? B.tiles[c] : make_int2(-1, -1);
      sm.s_inst[(it + 1) & 1] = e.x;
      sm.s_tile[(it + 1) & 1] = e.y;
    }
    const DevGrid &g = B.grids[b];
    const PairParams &pp = B.ip[b].pp;
    const TileGeom tg = tile_geom(g, pp.r0, B.coff[b]);
    const bool filter = g.mode == 1 && (g.need_filter || B.sl[b].alias_count > 0);
    if (filter || tg.HC > kHaloCellsMax) {  // this instance's tiles go to the global path
      if (tid == 0) {
        const unsigned int *cst = P.cstart + tg.cell0;
        const unsigned int qs = __ldg(&cst[t << (2 * tg.ts)]), qe = __ldg(&cst[(t + 1) << (2 * tg.ts)]);
        for (unsigned int s = qs; s < qe; s += kPairBlock) fb_push(ctrl, fb, fb_cap, s, min((unsigned)kPairBlock, qe - s));
      }
      __syncthreads();
      continue;
    }
    const MixedConsts mc = mixed_consts<KERNEL>(pp);
    const unsigned long long ea =
        pp.beta == 0.0 ? tile_any<KERNEL, XSPH, SUMDENS, true>(a, P, tg, mc, t, 0, sm, ctrl, fb, fb_cap, true)
                       : tile_any<KERNEL, XSPH, SUMDENS, false>(a, P, tg, mc, t, 0, sm, ctrl, fb, fb_cap, true);
    const unsigned long long ba = block_max_u64<kTileThreads>(ea, sm.red);
    if (tid == 0 && ba != kEncMaxId) atomicMax(&B.sl[b].pd_a2max, ba);
  }
  if (tid == 0) {
    __threadfence();
    if (atomicAdd(&ctrl->tile_done, 1u) == gridDim.x - 1) {
      ctrl->tile_next = 0;
      ctrl->tile_done = 0;
    }
  }
}

template <int KERNEL, bool XSPH, bool SUMDENS>
__global__ void __launch_bounds__(kPairBlock, kListBlocks)
    k_bt_pair_list(StepArgs a, PairPtrs P, BatchPtrs B, const int2 *__restrict__ fb) {
  step_kernel_entry();
  __shared__ unsigned int lists[ListCap<KERNEL>::value][kPairBlock];
  __shared__ unsigned long long red[kPairBlock / 32];
  const unsigned int cnt = *(volatile unsigned int *)&P.ctrl->fb_count;
  for (unsigned int e = blockIdx.x; e < cnt; e += gridDim.x) {
    const int2 r = fb[e];
    const int b = B.inst[P.perm[r.x]];  // an entry lies in one instance
    const DevGrid &g = B.grids[b];
    const PairParams &pp = B.ip[b].pp;
    const bool filter = g.mode == 1 && (g.need_filter || B.sl[b].alias_count > 0);
    unsigned long long ea = kEncMaxId;
    if ((int)threadIdx.x < r.y)
      ea = pp.beta == 0.0
               ? pair_query<KERNEL, XSPH, SUMDENS, true, true>(a, P, pp, g, filter, r.x + threadIdx.x, lists, B.coff[b])
               : pair_query<KERNEL, XSPH, SUMDENS, true, false>(a, P, pp, g, filter, r.x + threadIdx.x, lists, B.coff[b]);
    const unsigned long long ba = block_max_u64<kPairBlock>(ea, red);
    if (threadIdx.x == 0 && ba != kEncMaxId) atomicMax(&B.sl[b].pd_a2max, ba);
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&P.ctrl->fb_done, 1u) == gridDim.x - 1) {
      P.ctrl->fb_count = 0;
      P.ctrl->fb_done = 0;
    }
  }
}

// ---------------------------------------------------------------------------
// Probes: NNLinkedList.nearPos (src/Tools/NNLinkedList.py:41-84) at arbitrary
// points, on the table of the last build, and the pressure interpolation the
// reference's ice-coupling example composes from it (Shepard-normalised
// summation density + Tait EOS, examples/IceBreak.py:253-285,
// src/Equations/Shepard.py, src/Equations/SummationDensity.py).
// ---------------------------------------------------------------------------
// Raw reference cell (qref) of point (x, y), its own-grid cell key (clamped
// binning; mode 1) and the stencil half-width W that covers q <= 3 for a
// point with smoothing length h: r <= 1.5 (h + hmax).
__device__ __forceinline__ int probe_cell(const DevGrid &g, double x, double y, double h, int2 &qref, int &W) {
  const long long cx = ref_cell(x, g.xmin, g.cs, g.inv_cs, g.xminf, g.inv_csf);
  const long long cy = ref_cell(y, g.ymin, g.cs, g.inv_cs, g.yminf, g.inv_csf);
  qref = make_int2(sat_i32(cx), sat_i32(cy));
  if (g.mode == 0) {
    W = 1;
    return 0;
  }
  const float tx = fminf(fmaxf((d2f_trunc(x) - g.oxf) * g.inv_ctf, 0.f), g.txmaxf);
  const float ty = fminf(fmaxf((d2f_trunc(y) - g.oyf) * g.inv_ctf, 0.f), g.tymaxf);
  const int kx = min(max((int)floorf(tx), 0), g.ntx - 1), ky = min(max((int)floorf(ty), 0), g.nty - 1);
  const double reach = 1.5 * (h + g.hmax) * (1.0 + 1e-6);
  const double wd = ceil(reach / g.ct) + 1.0;
  W = wd < 1.0 ? 1 : (wd > 1024.0 ? 1024 : (int)wd);
  return tiled_key(kx, ky, g.ts, g.ntlx);
}

__global__ void __launch_bounds__(kPairBlock)
    k_nn_probe(const double *__restrict__ px, const double *__restrict__ py, const double *__restrict__ ph,
               long long np, const double *__restrict__ x, const double *__restrict__ y,
               const double *__restrict__ h, const int *__restrict__ perm, const int2 *__restrict__ meta,
               const int2 *__restrict__ refcell, const unsigned int *__restrict__ cstart,
               const DevGrid *__restrict__ gp, int64_t *counts, const int64_t *offsets, int64_t *idx,
               double *hij_out, double *q_out, double *r_out) {
  const DevGrid g = *gp;
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= np) return;
  const double xi = px[k], yi = py[k], hi = ph[k];
  int2 qref;
  int W;
  const int qkey = probe_cell(g, xi, yi, hi, qref, W);
  const bool filter = g.mode == 1;
  long long cnt = 0;
  const long long base = idx ? offsets[k] : 0;
  const Stencil sten(g, qref, qkey, W);
  for_stencil(sten, cstart, [&](unsigned int j) {
    if (filter && !in_ref_stencil(meta, j, g, qref)) return;
    const int pj = perm[j];
    const double dx = xi - x[pj], dy = yi - y[pj];
    const double r = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    const double hij = __dmul_rn(0.5, __dadd_rn(hi, h[pj]));
    const double q = __ddiv_rn(r, hij);
    if (q <= 3.0) {
      if (idx) {
        idx[base + cnt] = pj;
        hij_out[base + cnt] = hij;
        q_out[base + cnt] = q;
        r_out[base + cnt] = r;
      }
      cnt++;
    }
  });
  if (!idx) {
    counts[k] = cnt;
    return;
  }
  sort_ref_order(idx + base, hij_out + base, q_out + base, r_out + base, cnt, refcell, g.ncx, qref);
}

// rho = sum_fluid m_j W(r_j, hk) / sum_{fluid, rho_j >= 1e-3} W(r_j, hk) m_j / rho_j over
// the nearPos set of (x, y, h_search); p = B ((rho / rho0)^gamma - 1)
template <int KERNEL>
__global__ void __launch_bounds__(kPairBlock)
    k_probe_density(const double *__restrict__ px, const double *__restrict__ py, const double *__restrict__ ph,
                    const double *__restrict__ hk, long long np, StepArgs a, const int *__restrict__ perm,
                    const int2 *__restrict__ meta, const unsigned int *__restrict__ cstart,
                    const DevGrid *__restrict__ gp, double rho0, double B, double gamma, double *rho_out,
                    double *p_out) {
  const DevGrid g = *gp;
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= np) return;
  const double xi = px[k], yi = py[k], hi = ph[k], hw = hk[k];
  int2 qref;
  int W;
  const int qkey = probe_cell(g, xi, yi, hi, qref, W);
  const bool filter = g.mode == 1;
  double shep = 0.0, sum = 0.0;
  int nf = 0;
  const Stencil sten(g, qref, qkey, W);
  for_stencil(sten, cstart, [&](unsigned int j) {
    if (filter && !in_ref_stencil(meta, j, g, qref)) return;
    const int pj = perm[j];
    const double dx = xi - a.x[pj], dy = yi - a.y[pj];
    const double r = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    const double hij = __dmul_rn(0.5, __dadd_rn(hi, a.h[pj]));
    if (!(__ddiv_rn(r, hij) <= 3.0)) return;
    if (!is_fluid(a.label[pj])) return;  // Shepard and SummationDensity take fluid only
    const double w = KERNEL == SPH_KERNEL_CUBIC ? cubic_w(r, hw)
                                                : (KERNEL == SPH_KERNEL_WENDLAND ? wendland_w(r, hw) : gauss_w(r, hw));
    const double m = a.m[pj], rho = a.rho[pj];
    if (!(rho < 1e-3)) shep += w * m / rho;
    sum += m * w;
    nf++;
  });
  const double rho = nf ? sum / shep : 0.0;  // an empty sum without fluid neighbours
  rho_out[k] = rho;
  p_out[k] = (pow(rho / rho0, gamma) - 1.0) * B;
}

void launch_nn_probe(const StepArgs &a, const WsPtrs &w, long long np, const double *px, const double *py,
                     const double *ph, int64_t *counts, const int64_t *offsets, int64_t *idx, double *hij, double *q,
                     double *r, cudaStream_t st) {
  k_nn_probe<<<nblocks(np, kPairBlock), kPairBlock, 0, st>>>(px, py, ph, np, a.x, a.y, a.h, w.perm, w.meta,
                                                              w.refcell, w.cstart, w.grid, counts, offsets, idx,
                                                              hij, q, r);
}

void launch_probe_density(const StepArgs &a, const WsPtrs &w, int kernel, long long np, const double *px,
                          const double *py, const double *ph, const double *hk, double rho0, double B, double gamma,
                          double *rho, double *p, cudaStream_t st) {
  const unsigned nb = nblocks(np, kPairBlock);
  if (kernel == SPH_KERNEL_CUBIC)
    k_probe_density<SPH_KERNEL_CUBIC><<<nb, kPairBlock, 0, st>>>(px, py, ph, hk, np, a, w.perm, w.meta, w.cstart,
                                                                  w.grid, rho0, B, gamma, rho, p);
  else if (kernel == SPH_KERNEL_WENDLAND)
    k_probe_density<SPH_KERNEL_WENDLAND><<<nb, kPairBlock, 0, st>>>(px, py, ph, hk, np, a, w.perm, w.meta, w.cstart,
                                                                     w.grid, rho0, B, gamma, rho, p);
  else
    k_probe_density<SPH_KERNEL_GAUSSIAN><<<nb, kPairBlock, 0, st>>>(px, py, ph, hk, np, a, w.perm, w.meta, w.cstart,
                                                                     w.grid, rho0, B, gamma, rho, p);
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
static PairPtrs pair_ptrs(const WsPtrs &w) {
  PairPtrs P;
  P.rec0 = w.rec0; P.rec1 = w.rec1; P.rec2 = w.rec2; P.r64a = w.rec64a; P.r64b = w.rec64b;
  P.perm = w.perm; P.keys_sorted = w.keys_sorted; P.meta = w.meta; P.cstart = w.cstart;
  P.grid = w.grid; P.ctrl = w.ctrl;
  return P;
}

static PairParams pair_params(const StepArgs &a, const sph_config_t &cfg, const sph_wcsph_t &wc, bool do_dt) {
  PairParams pp;
  pp.wall_x = 0.0;
  pp.fr = nullptr;
  pp.alpha = wc.alpha; pp.beta = wc.beta; pp.co = wc.co; pp.eps = wc.epsilon;
  pp.r0 = wc.r0; pp.D = wc.D; pp.p1 = wc.p1; pp.p2 = wc.p2;
  pp.lj_42 = (wc.p1 == 4.0 && wc.p2 == 2.0) ? 1 : 0;
  pp.cfl_c = cfg.cfl_c; pp.cfl_f = cfg.cfl_f;
  pp.do_dt = do_dt ? 1 : 0;
  pp.n = a.n;
  return pp;
}

int sm_count() {
  static int cache[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 152;
  if (!cache[dev]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    cache[dev] = v > 0 ? v : 152;
  }
  return cache[dev];
}

// Dynamic shared memory of a tile kernel: allowed above 48 KB once per device
// and kernel (the attribute belongs to the kernel function on a device).
// `done` is the calling launcher's own flag array: every tile kernel
// instantiation has the same function type, so the flag cannot live here.
template <typename K>
static size_t tile_smem(K kern, size_t bytes, bool (&done)[64]) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64 || !done[dev]) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (dev >= 0 && dev < 64) done[dev] = true;
  }
  return bytes;
}

template <int KERNEL, bool XSPH, bool SUMDENS, bool UH>
static void mixed_pair_launch(const StepArgs &a, const WsPtrs &w, const PairParams &pp, double *dt_out,
                              double *dt_hist, cudaStream_t st) {
  // persistent tile kernel, then the global path over what it left
  const int sms = sm_count();
  auto tk = k_pair_tiles<KERNEL, XSPH, SUMDENS, UH>;
  static bool done[64] = {false};  // this instantiation's attribute, per device
  const size_t smem = tile_smem(tk, sizeof(TileShared<KERNEL>), done);
  launch_pdl(tk, dim3(sms * TileBlocks<KERNEL>::value), dim3(kTileThreads), smem, st, a, pair_ptrs(w), pp, w.tiles,
             w.tiles_h, (unsigned)(w.max_cells + 1), w.fb, (unsigned)w.fb_cap);
  launch_pdl(k_pair_list<KERNEL, XSPH, SUMDENS, UH>, dim3(sms * kListBlocks), dim3(kPairBlock), 0, st, a,
             pair_ptrs(w), pp, w.fb, dt_out, dt_hist);
}

template <int KERNEL, bool XSPH, bool SUMDENS>
static void pair_dispatch(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const PairParams &pp,
                          double *dt_out, double *dt_hist, cudaStream_t st) {
  if (cfg.precision == SPH_PREC_MIXED) {
    // a fixed h makes every fluid record's h the same (the uniform-h form,
    // taken when the viscosity's beta is 0)
    if (cfg.h_fixed > 0.0 && pp.beta == 0.0) mixed_pair_launch<KERNEL, XSPH, SUMDENS, true>(a, w, pp, dt_out, dt_hist, st);
    else mixed_pair_launch<KERNEL, XSPH, SUMDENS, false>(a, w, pp, dt_out, dt_hist, st);
  } else {
    // one query per thread; below a few blocks per SM, one-warp blocks so
    // that the FP64-bound work spreads evenly over the SMs
    const int bs = a.n < (long long)sm_count() * kPairBlock * 8 ? 32 : kPairBlock;
    k_pair<KERNEL, XSPH, SUMDENS, false><<<nblocks(a.n, bs), bs, 0, st>>>(a, pair_ptrs(w), pp, dt_out, dt_hist);
  }
}

void launch_pair(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc,
                 double *dt_out, double *dt_hist, cudaStream_t st, const WallLoad *wall) {
  PairParams pp = pair_params(a, cfg, wc, dt_out != nullptr || dt_hist != nullptr);
  if (wall) {
    pp.wall_x = wall->wall_x;
    pp.fr = wall->fr;
  }
  const bool xs = wc.use_xsph != 0, sd = wc.use_summation_density != 0;
  auto go = [&](auto kern) {
    constexpr int K = decltype(kern)::value;
    if (xs) sd ? pair_dispatch<K, true, true>(a, w, cfg, pp, dt_out, dt_hist, st)
               : pair_dispatch<K, true, false>(a, w, cfg, pp, dt_out, dt_hist, st);
    else sd ? pair_dispatch<K, false, true>(a, w, cfg, pp, dt_out, dt_hist, st)
            : pair_dispatch<K, false, false>(a, w, cfg, pp, dt_out, dt_hist, st);
  };
  if (cfg.kernel == SPH_KERNEL_CUBIC) go(std::integral_constant<int, SPH_KERNEL_CUBIC>());
  else if (cfg.kernel == SPH_KERNEL_WENDLAND) go(std::integral_constant<int, SPH_KERNEL_WENDLAND>());
  else go(std::integral_constant<int, SPH_KERNEL_GAUSSIAN>());
}

void launch_sumdens(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc,
                    cudaStream_t st) {
  const unsigned nb = nblocks(a.n, kPairBlock);
  const bool mixed = cfg.precision == SPH_PREC_MIXED;
  const PairPtrs P = pair_ptrs(w);
  auto go = [&](auto kern) {
    constexpr int K = decltype(kern)::value;
    if (mixed) k_sumdens<K, true><<<nb, kPairBlock, 0, st>>>(a, P, a.n);
    else k_sumdens<K, false><<<nb, kPairBlock, 0, st>>>(a, P, a.n);
  };
  if (cfg.kernel == SPH_KERNEL_CUBIC) go(std::integral_constant<int, SPH_KERNEL_CUBIC>());
  else if (cfg.kernel == SPH_KERNEL_WENDLAND) go(std::integral_constant<int, SPH_KERNEL_WENDLAND>());
  else go(std::integral_constant<int, SPH_KERNEL_GAUSSIAN>());
  (void)wc;
}

void launch_nn_count(const StepArgs &a, const WsPtrs &w, int64_t *counts, const int64_t *offsets, int64_t *idx,
                     cudaStream_t st) {
  k_nn_export<<<nblocks(a.n, kPairBlock), kPairBlock, 0, st>>>(a.x, a.y, a.h, a.n, w.perm, w.keys_sorted, w.meta,
                                                               w.refcell, w.cstart, w.grid, counts, offsets, idx);
}

template <int KERNEL, bool XSPH, bool SUMDENS>
static void bt_pair_dispatch(const StepArgs &a, const WsPtrs &w, const BatchPtrs &B, int tile_blocks,
                             cudaStream_t st) {
  const int sms = sm_count();
  if (tile_blocks < 1 || tile_blocks > TileBlocks<KERNEL>::value) tile_blocks = TileBlocks<KERNEL>::value;
  auto tk = k_bt_pair_tiles<KERNEL, XSPH, SUMDENS>;
  static bool done[64] = {false};  // this instantiation's attribute, per device
  const size_t smem = tile_smem(tk, sizeof(TileShared<KERNEL>), done);
  launch_pdl(tk, dim3(sms * tile_blocks), dim3(kTileThreads), smem, st, a, pair_ptrs(w), B, w.fb, (unsigned)w.fb_cap);
  launch_pdl(k_bt_pair_list<KERNEL, XSPH, SUMDENS>, dim3(sms * kListBlocks), dim3(kPairBlock), 0, st, a, pair_ptrs(w),
             B, w.fb);
}

void launch_bt_pair(const StepArgs &a, const WsPtrs &w, const BatchPtrs &B, int kernel, bool xsph, int tile_blocks,
                    cudaStream_t st) {
  (void)xsph;  // the batched form has no XSPH
  if (kernel == SPH_KERNEL_CUBIC) bt_pair_dispatch<SPH_KERNEL_CUBIC, false, false>(a, w, B, tile_blocks, st);
  else if (kernel == SPH_KERNEL_WENDLAND) bt_pair_dispatch<SPH_KERNEL_WENDLAND, false, false>(a, w, B, tile_blocks, st);
  else bt_pair_dispatch<SPH_KERNEL_GAUSSIAN, false, false>(a, w, B, tile_blocks, st);
}

}  // namespace sph

// pair.cu -- the fused pair interaction of the WCSPH step.
//
// One thread per (cell-sorted) fluid particle i gathers its neighbours from
// the cell table and evaluates, in one pass, everything _loop computes per
// particle (src/Tools/SolverTools.py:143-173): the kernel value and gradient
// (src/Kernels/CubicSpline.py, src/Kernels/Gaussian.py), continuity
// (src/Equations/Continuity.py), momentum with artificial viscosity and
// gravity (src/Equations/Momentum.py, src/Methods/WCSPH.py:151-169), the
// Lennard-Jones boundary force (src/Equations/BoundaryForce.py) and XSPH
// (src/Equations/XSPH.py).  The TimeStep reductions of the next step
// (src/Equations/TimeStep.py:58-91) are fused into the epilogue.
//
// FP64 form: the reference's arithmetic, with the neighbour test done with
// explicitly rounded operations so that the accepted set is the reference's.
// Mixed form: FP32 arithmetic on differences formed from double-float
// (hi + lo) copies of the FP64 positions and velocities.
#include <math.h>

#include "sph_internal.cuh"

namespace sph {

constexpr int kPairBlock = 128;

struct PairParams {
  double alpha, beta, co, eps, r0, D, p1, p2;
  int lj_42;  // p1 == 4 and p2 == 2
  double cfl_c, cfl_f;
  int do_dt;
  long long n;
};

// Visit every candidate slot j of query slot k: the 3x3 stencil of the
// reference grid (mode 0, validity as in NNLinkedList._get_valid_cell_index)
// or a (2W+1)^2 stencil of the traversal grid (mode 1) with the
// reference-stencil filter.  Cells of one stencil row are contiguous in the
// sorted order, so each row is one range.
template <typename F>
__device__ __forceinline__ void for_each_candidate(const DevGrid &g, const unsigned int *__restrict__ cstart,
                                                   int2 qref, int qkey, int W, bool filter,
                                                   const int2 *__restrict__ meta, F &&f) {
  int cxq, cyq;
  if (g.mode == 0) {
    cxq = qref.x;
    cyq = qref.y;
  } else {
    if (qkey >= g.ncells) return;
    cxq = qkey % g.ntx;
    cyq = qkey / g.ntx;
  }
  const int nx = g.ntx, ny = g.nty;
  for (int b = -W; b <= W; b++) {
    int yy = cyq + b;
    if (yy < 0 || yy >= ny) continue;
    int x0 = max(cxq - W, 0), x1 = min(cxq + W, nx - 1);
    if (x0 > x1) continue;
    unsigned int s = __ldg(&cstart[x0 + nx * yy]), e = __ldg(&cstart[x1 + nx * yy + 1]);
    for (unsigned int j = s; j < e; j++) {
      if (filter) {
        int2 mj = __ldg(&meta[j]);
        int sx, sy;
        storage_cell(mj.x, mj.y, g.ncx, sx, sy);
        if (abs(sx - qref.x) > 1 || abs(sy - qref.y) > 1) continue;
      }
      f(j);
    }
  }
}

// TimeStep epilogue: block-reduce min h, max a^2 over fluid, the last block
// computes {dt, dt_courant, dt_force} (TimeStep.py:7-56) and resets the slots.
__device__ __forceinline__ void timestep_epilogue(DevCtrl *ctrl, unsigned long long eh, unsigned long long ea,
                                                  unsigned int nf, double co, double cfl_c, double cfl_f,
                                                  double *dt_out, double *dt_hist, unsigned int *done) {
  __shared__ unsigned long long red[32];
  __shared__ unsigned int red32[32];
  __shared__ bool last;
  unsigned long long bh = block_reduce(eh, MinU64(), kEncMinId, red);
  unsigned long long ba = block_reduce(ea, MaxU64(), kEncMaxId, red);
  unsigned int bn = block_reduce(nf, AddU32(), 0u, red32);
  if (threadIdx.x == 0) {
    if (bn) {
      atomicMin(&ctrl->ts_hmin, bh);
      atomicMax(&ctrl->ts_a2max, ba);
      atomicAdd(&ctrl->ts_nfluid, bn);
    }
    __threadfence();
    unsigned int t = atomicAdd(done, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    unsigned long long h = atomicExch(&ctrl->ts_hmin, kEncMinId);
    unsigned long long a2 = atomicExch(&ctrl->ts_a2max, kEncMaxId);
    unsigned int cnt = atomicExch(&ctrl->ts_nfluid, 0u);
    atomicExch(done, 0u);
    double min_h = dec_d(h), max_a2 = dec_d(a2), max_c = co;
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
// FP64 form
// ---------------------------------------------------------------------------
template <int KERNEL, bool XSPH, bool SUMDENS>
__global__ void __launch_bounds__(kPairBlock)
    k_pair64(StepArgs a, const double4_32a *__restrict__ recA, const double4_32a *__restrict__ recB,
             const int *__restrict__ perm, const int *__restrict__ keys_sorted, const int2 *__restrict__ meta,
             const unsigned int *__restrict__ cstart, const DevGrid *__restrict__ gp, DevCtrl *ctrl,
             PairParams pp, double *dt_out, double *dt_hist) {
  const DevGrid g = *gp;
  const bool filter = g.mode == 1 && (g.need_filter || ctrl->alias_count > 0);
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long eh = kEncMinId, ea = kEncMaxId;
  unsigned int nf = 0;
  if (k < pp.n) {
    const double4_32a Ai = recA[k], Bi = recB[k];
    if (!signbit(Bi.w)) {
      const int i = perm[k];
      const double xi = Ai.x, yi = Ai.y, vxi = Ai.z, vyi = Ai.w;
      const double rhoi = Bi.y, slf = Bi.z, hi = Bi.w;
      const int2 qref = meta[k];
      const int qkey = keys_sorted[k];
      int W = 1;
      if (g.mode == 1 && (qref.x == g.ncx || !(hi > 0.0))) W = g.wide;
      double drho = 0.0, axs = 0.0, ays = 0.0, bx = 0.0, by = 0.0, sx = 0.0, sy = 0.0;
      int cnt = 0;
      for_each_candidate(g, cstart, qref, qkey, W, filter, meta, [&](unsigned int j) {
        const double4_32a Aj = recA[j];
        const double4_32a Bj = recB[j];
        const double dx = xi - Aj.x, dy = yi - Aj.y;
        const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
        const double hij = __dmul_rn(0.5, __dadd_rn(hi, fabs(Bj.w)));
        if (d2 > 9.0000001 * hij * hij) return;  // certainly q > 3
        const double r = __dsqrt_rn(d2);
        const double q = __ddiv_rn(r, hij);
        if (!(q <= 3.0)) return;  // NNLinkedList.py:74
        cnt++;
        const bool jf = !signbit(Bj.w);
        const double mj = Bj.x, rhoj = Bj.y;
        const double vxij = vxi - Aj.z, vyij = vyi - Aj.w;
        double w = 0.0, coef = 0.0;
        if (KERNEL == SPH_KERNEL_CUBIC) {
          if (q <= 2.0) {
            const double alpha = kCubicFac / (hij * hij);
            if (q > 1.0) {
              const double t = 2.0 - q;
              w = alpha * 0.25 * (t * t * t);
              if (r >= 1e-10) coef = alpha * (-0.75 * (t * t)) / (hij * r);
            } else {
              w = alpha * (1.0 - 1.5 * (q * q) * (1.0 - 0.5 * q));
              if (r >= 1e-10) coef = alpha * (-3.0 * q * (1.0 - 0.75 * q)) / (hij * r);
            }
          }
        } else {
          const double alpha_c = kInvPi / (hij * hij);
          const double e = exp(-q * q);
          w = alpha_c * e;
          const double tmp = r * hij;
          if (tmp > 1e-12) coef = (-2.0 * q * alpha_c * e) / tmp;
        }
        const double dwx = coef * dx, dwy = coef * dy;
        if (jf) {
          if (!SUMDENS) drho += mj * (vxij * dwx + vyij * dwy);
          const double dot = vxij * dx + vyij * dy;
          double PI = 0.0;
          if (dot < 0.0) {
            const double hb = 0.5 * (hi + hij);
            const double cb = 0.5 * pp.co;
            const double rb = 0.5 * (rhoi + rhoj);
            const double mu = hb * dot / (r * r + 0.01 * hb * hb);
            PI = mu * (pp.beta * mu - pp.alpha * cb) / rb;
          }
          const double fac = slf + Bj.z + PI;
          axs += -mj * fac * dwx;
          ays += -mj * fac * dwy;
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
          bx += fac * dx / r2;
          by += fac * dy / r2;
        }
        if (XSPH) {
          const double fac = -pp.eps * mj * w / (0.5 * (rhoi + rhoj));
          sx += fac * vxij;
          sy += fac * vyij;
        }
      });
      double axf, ayf;
      if (cnt > 0) {
        axf = axs + bx;
        ayf = (ays - 9.81) + by;
        a.drho[i] = SUMDENS ? 0.0 : drho;
        a.ax[i] = axf;
        a.ay[i] = ayf;
        a.xsphx[i] = XSPH ? vxi + sx : 0.0;
        a.xsphy[i] = XSPH ? vyi + sy : 0.0;
      } else {
        axf = a.ax[i];
        ayf = a.ay[i];
      }
      eh = enc_d(hi);
      ea = enc_d(accel2(axf, ayf));
      nf = 1;
    }
  }
  if (pp.do_dt) timestep_epilogue(ctrl, eh, ea, nf, pp.co, pp.cfl_c, pp.cfl_f, dt_out, dt_hist, &ctrl->done_pair);
}

// ---------------------------------------------------------------------------
// Mixed form: FP32 pair arithmetic, FP64 state
// ---------------------------------------------------------------------------
template <int KERNEL, bool XSPH, bool SUMDENS>
__global__ void __launch_bounds__(kPairBlock)
    k_pair32(StepArgs a, const float4 *__restrict__ recP, const float4 *__restrict__ recV,
             const float4 *__restrict__ recS, const int *__restrict__ perm, const int *__restrict__ keys_sorted,
             const int2 *__restrict__ meta, const unsigned int *__restrict__ cstart,
             const DevGrid *__restrict__ gp, DevCtrl *ctrl, PairParams pp, double *dt_out, double *dt_hist) {
  const DevGrid g = *gp;
  const bool filter = g.mode == 1 && (g.need_filter || ctrl->alias_count > 0);
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long eh = kEncMinId, ea = kEncMaxId;
  unsigned int nf = 0;
  const float co = (float)pp.co, alpha = (float)pp.alpha, beta = (float)pp.beta, eps = (float)pp.eps;
  const float r0 = (float)pp.r0, D = (float)pp.D;
  const float r02 = r0 * r0;
  if (k < pp.n) {
    const float4 Si = recS[k];
    if (!signbit(Si.w)) {
      const int i = perm[k];
      const float4 Pi = recP[k], Vi = recV[k];
      const float rhoi = Si.y, slf = Si.z, hi = Si.w;
      const int2 qref = meta[k];
      const int qkey = keys_sorted[k];
      int W = 1;
      if (g.mode == 1 && (qref.x == g.ncx || !(hi > 0.0f))) W = g.wide;
      float drho = 0.f, axs = 0.f, ays = 0.f, bx = 0.f, by = 0.f, sx = 0.f, sy = 0.f;
      int cnt = 0;
      for_each_candidate(g, cstart, qref, qkey, W, filter, meta, [&](unsigned int j) {
        const float4 Pj = __ldg(&recP[j]);
        const float4 Sj = __ldg(&recS[j]);
        const float dx = (Pi.x - Pj.x) + (Pi.z - Pj.z);
        const float dy = (Pi.y - Pj.y) + (Pi.w - Pj.w);
        const float d2 = dx * dx + dy * dy;
        const float hij = 0.5f * (hi + fabsf(Sj.w));
        const float h2 = hij * hij;
        if (!(d2 <= 9.0f * h2)) return;
        cnt++;
        const bool jf = !signbit(Sj.w);
        if (KERNEL == SPH_KERNEL_CUBIC && d2 > 4.0f * h2) {
          // outside the cubic support: only the boundary force can act
          if (!jf && d2 <= r02 && d2 > 1e-24f) {
            const float ir2 = 1.0f / d2;
            const float f2 = r02 * ir2;
            const float fac = D * (f2 * f2 - f2);
            bx += fac * dx * ir2;
            by += fac * dy * ir2;
          }
          return;
        }
        const float4 Vj = __ldg(&recV[j]);
        const float mj = Sj.x, rhoj = Sj.y;
        const float vxij = (Vi.x - Vj.x) + (Vi.z - Vj.z);
        const float vyij = (Vi.y - Vj.y) + (Vi.w - Vj.w);
        const float inv_r = d2 > 0.f ? rsqrtf(d2) : 0.f;
        const float r = d2 * inv_r;
        const float inv_h = __fdividef(1.0f, hij);
        const float q = r * inv_h;
        float w, coef = 0.f;
        if (KERNEL == SPH_KERNEL_CUBIC) {
          const float al = (float)kCubicFac * inv_h * inv_h;
          if (q > 1.0f) {
            const float t = 2.0f - q;
            w = al * 0.25f * (t * t * t);
            if (r >= 1e-10f) coef = al * (-0.75f * (t * t)) * inv_h * inv_r;
          } else {
            w = al * (1.0f - 1.5f * (q * q) * (1.0f - 0.5f * q));
            if (r >= 1e-10f) coef = al * (-3.0f * q * (1.0f - 0.75f * q)) * inv_h * inv_r;
          }
        } else {
          const float ac = (float)kInvPi * inv_h * inv_h;
          const float e = __expf(-q * q);
          w = ac * e;
          if (r * hij > 1e-12f) coef = -2.0f * ac * e * inv_h * inv_h;
        }
        const float dwx = coef * dx, dwy = coef * dy;
        if (jf) {
          if (!SUMDENS) drho += mj * (vxij * dwx + vyij * dwy);
          const float dot = vxij * dx + vyij * dy;
          float PI = 0.f;
          if (dot < 0.f) {
            const float hb = 0.5f * (hi + hij);
            const float mu = hb * dot / (d2 + 0.01f * hb * hb);
            PI = mu * (beta * mu - alpha * 0.5f * co) / (0.5f * (rhoi + rhoj));
          }
          const float fac = slf + Sj.z + PI;
          axs -= mj * fac * dwx;
          ays -= mj * fac * dwy;
        } else if (d2 <= r02 && d2 > 1e-24f) {
          const float ir2 = 1.0f / d2;
          const float f2 = r02 * ir2;
          const float fac = D * (f2 * f2 - f2);
          bx += fac * dx * ir2;
          by += fac * dy * ir2;
        }
        if (XSPH) {
          const float fac = -eps * mj * w / (0.5f * (rhoi + rhoj));
          sx += fac * vxij;
          sy += fac * vyij;
        }
      });
      double axf, ayf;
      if (cnt > 0) {
        axf = (double)axs + (double)bx;
        ayf = ((double)ays - 9.81) + (double)by;
        a.drho[i] = SUMDENS ? 0.0 : (double)drho;
        a.ax[i] = axf;
        a.ay[i] = ayf;
        if (XSPH) {
          a.xsphx[i] = a.vx[i] + (double)sx;
          a.xsphy[i] = a.vy[i] + (double)sy;
        } else {
          a.xsphx[i] = 0.0;
          a.xsphy[i] = 0.0;
        }
      } else {
        axf = a.ax[i];
        ayf = a.ay[i];
      }
      eh = enc_d(a.h[i]);
      ea = enc_d(accel2(axf, ayf));
      nf = 1;
    }
  }
  if (pp.do_dt) timestep_epilogue(ctrl, eh, ea, nf, pp.co, pp.cfl_c, pp.cfl_f, dt_out, dt_hist, &ctrl->done_pair);
}

// ---------------------------------------------------------------------------
// Summation density (SolverTools.py:129-140, SummationDensity.py:5-13):
// rho_i = sum over fluid neighbours of m_j W(r, h_ij), written to rho[i].
// ---------------------------------------------------------------------------
template <int KERNEL, bool MIXED>
__global__ void __launch_bounds__(kPairBlock)
    k_sumdens(StepArgs a, const void *__restrict__ rA, const void *__restrict__ rB, const void *__restrict__ rC,
              const int *__restrict__ perm, const int *__restrict__ keys_sorted, const int2 *__restrict__ meta,
              const unsigned int *__restrict__ cstart, const DevGrid *__restrict__ gp, const DevCtrl *ctrl,
              long long n) {
  const DevGrid g = *gp;
  const bool filter = g.mode == 1 && (g.need_filter || ctrl->alias_count > 0);
  long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double4_32a *recA = (const double4_32a *)rA, *recB = (const double4_32a *)rB;
  const float4 *recP = (const float4 *)rA, *recS = (const float4 *)rC;
  double hi, xi = 0, yi = 0;
  float4 Pi;
  if (MIXED) {
    float4 Si = recS[k];
    if (signbit(Si.w)) return;
    hi = Si.w;
    Pi = recP[k];
  } else {
    double4_32a Bi = recB[k];
    if (signbit(Bi.w)) return;
    hi = Bi.w;
    double4_32a Ai = recA[k];
    xi = Ai.x;
    yi = Ai.y;
  }
  const int2 qref = meta[k];
  const int qkey = keys_sorted[k];
  int W = 1;
  if (g.mode == 1 && (qref.x == g.ncx || !(hi > 0.0))) W = g.wide;
  double rho = 0.0;
  float rhof = 0.f;
  for_each_candidate(g, cstart, qref, qkey, W, filter, meta, [&](unsigned int j) {
    if (MIXED) {
      const float4 Pj = __ldg(&recP[j]);
      const float4 Sj = __ldg(&recS[j]);
      const float dx = (Pi.x - Pj.x) + (Pi.z - Pj.z);
      const float dy = (Pi.y - Pj.y) + (Pi.w - Pj.w);
      const float d2 = dx * dx + dy * dy;
      const float hij = 0.5f * ((float)hi + fabsf(Sj.w));
      if (!(d2 <= 9.0f * hij * hij) || signbit(Sj.w)) return;
      const float q = sqrtf(d2) / hij;
      float w;
      if (KERNEL == SPH_KERNEL_CUBIC) {
        const float al = (float)kCubicFac / (hij * hij);
        if (q > 2.0f) w = 0.f;
        else if (q > 1.0f) { const float t = 2.0f - q; w = al * 0.25f * t * t * t; }
        else w = al * (1.0f - 1.5f * q * q * (1.0f - 0.5f * q));
      } else {
        w = (float)kInvPi / (hij * hij) * __expf(-q * q);
      }
      rhof += Sj.x * w;
    } else {
      const double4_32a Aj = recA[j];
      const double4_32a Bj = recB[j];
      const double dx = xi - Aj.x, dy = yi - Aj.y;
      const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
      const double hij = __dmul_rn(0.5, __dadd_rn(hi, fabs(Bj.w)));
      if (d2 > 9.0000001 * hij * hij) return;
      const double r = __dsqrt_rn(d2);
      const double q = __ddiv_rn(r, hij);
      if (!(q <= 3.0) || signbit(Bj.w)) return;
      double w;
      if (KERNEL == SPH_KERNEL_CUBIC) {
        const double al = kCubicFac / (hij * hij);
        if (q > 2.0) w = 0.0;
        else if (q > 1.0) { const double t = 2.0 - q; w = al * 0.25 * t * t * t; }
        else w = al * (1.0 - 1.5 * q * q * (1.0 - 0.5 * q));
      } else {
        w = kInvPi / (hij * hij) * exp(-q * q);
      }
      rho += Bj.x * w;
    }
  });
  a.rho[perm[k]] = MIXED ? (double)rhof : rho;
}

// ---------------------------------------------------------------------------
// Neighbour-set export (NNLinkedList.near for every particle, FP64 exact):
// count pass (idx == nullptr) or fill pass.  Reads the caller's arrays.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kPairBlock)
    k_nn_export(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ h,
                long long n, const int *__restrict__ perm, const int *__restrict__ keys_sorted,
                const int2 *__restrict__ meta, const unsigned int *__restrict__ cstart,
                const DevGrid *__restrict__ gp, const DevCtrl *ctrl, int64_t *counts, const int64_t *offsets,
                int64_t *idx) {
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
  for_each_candidate(g, cstart, qref, qkey, W, filter, meta, [&](unsigned int j) {
    const int pj = perm[j];
    const double dx = xi - x[pj], dy = yi - y[pj];
    const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    const double r = __dsqrt_rn(d2);
    const double hij = __dmul_rn(0.5, __dadd_rn(hi, h[pj]));
    const double q = __ddiv_rn(r, hij);
    if (!(q <= 3.0)) return;
    if (idx) idx[base + cnt] = pj;
    cnt++;
  });
  if (!idx) {
    counts[i] = cnt;
    return;
  }
  // ascending order within the list
  for (long long s = 1; s < cnt; s++) {
    int64_t v = idx[base + s];
    long long t = s - 1;
    while (t >= 0 && idx[base + t] > v) {
      idx[base + t + 1] = idx[base + t];
      t--;
    }
    idx[base + t + 1] = v;
  }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
static PairParams pair_params(const StepArgs &a, const sph_config_t &cfg, const sph_wcsph_t &wc, bool do_dt) {
  PairParams pp;
  pp.alpha = wc.alpha; pp.beta = wc.beta; pp.co = wc.co; pp.eps = wc.epsilon;
  pp.r0 = wc.r0; pp.D = wc.D; pp.p1 = wc.p1; pp.p2 = wc.p2;
  pp.lj_42 = (wc.p1 == 4.0 && wc.p2 == 2.0) ? 1 : 0;
  pp.cfl_c = cfg.cfl_c; pp.cfl_f = cfg.cfl_f;
  pp.do_dt = do_dt ? 1 : 0;
  pp.n = a.n;
  return pp;
}

template <int KERNEL, bool XSPH, bool SUMDENS>
static void pair_dispatch(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const PairParams &pp,
                          double *dt_out, double *dt_hist, cudaStream_t st) {
  unsigned nb = nblocks(a.n, kPairBlock);
  if (cfg.precision == SPH_PREC_MIXED)
    k_pair32<KERNEL, XSPH, SUMDENS><<<nb, kPairBlock, 0, st>>>(
        a, (const float4 *)w.recA, (const float4 *)w.recB, (const float4 *)w.recC, w.perm, w.keys_sorted, w.meta,
        w.cstart, w.grid, w.ctrl, pp, dt_out, dt_hist);
  else
    k_pair64<KERNEL, XSPH, SUMDENS><<<nb, kPairBlock, 0, st>>>(a, (const double4_32a *)w.recA,
                                                              (const double4_32a *)w.recB, w.perm, w.keys_sorted,
                                                              w.meta, w.cstart, w.grid, w.ctrl, pp, dt_out, dt_hist);
}

void launch_pair(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc,
                 double *dt_out, double *dt_hist, cudaStream_t st) {
  PairParams pp = pair_params(a, cfg, wc, dt_out != nullptr || dt_hist != nullptr);
  const bool xs = wc.use_xsph != 0, sd = wc.use_summation_density != 0;
  if (cfg.kernel == SPH_KERNEL_CUBIC) {
    if (xs) sd ? pair_dispatch<SPH_KERNEL_CUBIC, true, true>(a, w, cfg, pp, dt_out, dt_hist, st)
               : pair_dispatch<SPH_KERNEL_CUBIC, true, false>(a, w, cfg, pp, dt_out, dt_hist, st);
    else sd ? pair_dispatch<SPH_KERNEL_CUBIC, false, true>(a, w, cfg, pp, dt_out, dt_hist, st)
            : pair_dispatch<SPH_KERNEL_CUBIC, false, false>(a, w, cfg, pp, dt_out, dt_hist, st);
  } else {
    if (xs) sd ? pair_dispatch<SPH_KERNEL_GAUSSIAN, true, true>(a, w, cfg, pp, dt_out, dt_hist, st)
               : pair_dispatch<SPH_KERNEL_GAUSSIAN, true, false>(a, w, cfg, pp, dt_out, dt_hist, st);
    else sd ? pair_dispatch<SPH_KERNEL_GAUSSIAN, false, true>(a, w, cfg, pp, dt_out, dt_hist, st)
            : pair_dispatch<SPH_KERNEL_GAUSSIAN, false, false>(a, w, cfg, pp, dt_out, dt_hist, st);
  }
}

void launch_sumdens(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, const sph_wcsph_t &wc,
                    cudaStream_t st) {
  unsigned nb = nblocks(a.n, kPairBlock);
  bool mixed = cfg.precision == SPH_PREC_MIXED;
#define SPH_SD(KN, MX)                                                                                     \
  k_sumdens<KN, MX><<<nb, kPairBlock, 0, st>>>(a, w.recA, w.recB, w.recC, w.perm, w.keys_sorted, w.meta, \
                                               w.cstart, w.grid, w.ctrl, a.n)
  if (cfg.kernel == SPH_KERNEL_CUBIC) {
    if (mixed) SPH_SD(SPH_KERNEL_CUBIC, true);
    else SPH_SD(SPH_KERNEL_CUBIC, false);
  } else {
    if (mixed) SPH_SD(SPH_KERNEL_GAUSSIAN, true);
    else SPH_SD(SPH_KERNEL_GAUSSIAN, false);
  }
#undef SPH_SD
}

void launch_nn_count(const StepArgs &a, const WsPtrs &w, int64_t *counts, const int64_t *offsets, int64_t *idx,
                     cudaStream_t st) {
  k_nn_export<<<nblocks(a.n, kPairBlock), kPairBlock, 0, st>>>(a.x, a.y, a.h, a.n, w.perm, w.keys_sorted, w.meta,
                                                               w.cstart, w.grid, w.ctrl, counts, offsets, idx);
}

}  // namespace sph

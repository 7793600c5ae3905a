// adjoint.cu -- reverse mode of the WCSPH step (FP64 and mixed forms).
//
// The forward step with a fixed dt (src/Solver.py:370-372 timeStep path) and
// the PEC integrator (src/Integrators/PEC.py:32-89, damping 0) maps the state
// S = (x, v, rho, a, drho) of the fluid particles to S':
//   half:    x_h = x + dt/2 v,  v_h = v + dt/2 a,  rho_h = rho + dt/2 drho
//   compute: (A, D) = F(x_h, v_h, rho_h; alpha)   (src/Tools/SolverTools.py:120-175)
//   correct: x' = x + dt v_h,  v' = v + dt A,  rho' = rho + dt D,  a' = A,  drho' = D
// and adds omega * (wall load of the evaluation) to the loss.  The adjoint
// step maps the adjoint of S' back to the adjoint of S:
//   lambda_A = dt vb' + ab',  lambda_D = dt rhob' + drhob'       (k_adj_pre)
//   (xb_h, vb_h, rhob_h, alphab) = VJP of F and of the wall load  (k_pair_adjoint)
//   vb_h += dt xb';  xb = xb' + xb_h;  vb = vb' + dt/2 xb_h + vb_h;
//   ab = dt/2 vb_h;  rhob = rhob' + rhob_h;  drhob = dt/2 rhob_h  (k_adj_post)
//
// k_pair_adjoint is the hand-written vector-Jacobian product of the fused
// pair evaluation: continuity (src/Equations/Continuity.py), momentum with
// artificial viscosity (src/Equations/Momentum.py), the Tait EOS inside
// p/rho^2 (src/Equations/TaitEOS.py) and the Lennard-Jones boundary force
// (src/Equations/BoundaryForce.py).  For a fluid pair (k, j) the outputs of
// both particles enter one scalar
//   phi = lQ . (S dW) + lC (v_kj . dW),
//   lQ = -m_j lambdaA_k + m_k lambdaA_j,  lC = m_j lambdaD_k + m_k lambdaD_j,
//   S = p_k/rho_k^2 + p_j/rho_j^2 + Pi_kj,
// which is the same for (k, j) and (j, k); each thread differentiates it with
// respect to its own position, velocity and density, so the product is a
// gather over the neighbour set with no atomics.  The alpha adjoint takes
// each thread's own outputs only, so each pair counts once.
#include <math.h>

#include "sph_internal.cuh"

namespace sph {

// one-warp blocks: the kernel is FP64-bound and a small case has few warps
// per SM, so small blocks spread them evenly
constexpr int kAdjBlock = 32;
constexpr int kAdjSplit = 1;  // lanes per query

struct AdjParams {
  double alpha, beta, co, r0, D, p1, p2, gamma, B, inv_rho0;
  int lj_42;
  double omega, wall_x, dt;
  long long n;
};

// d(p/rho^2)/drho of a fluid particle from its rho and p/rho^2
// (p = B ((rho/rho0)^gamma - 1) + Pb, src/Equations/TaitEOS.py:6-31)
__device__ __forceinline__ double dothr_drho(double rho, double othr, const AdjParams &ap) {
  if (!(rho > 0.0)) return 0.0;
  const double t = rho * ap.inv_rho0;
  double tg1;  // t^(gamma - 1)
  if (ap.gamma == 7.0) {
    const double t2 = t * t, t3 = t2 * t;
    tg1 = t3 * t3;
  } else {
    tg1 = pow(t, ap.gamma - 1.0);
  }
  const double dp = ap.B * ap.gamma * ap.inv_rho0 * tg1;
  return (dp - 2.0 * othr * rho) / (rho * rho);
}

// The adjoint needs about 1e-12 relative accuracy, not correct rounding, so
// its reciprocals and square roots start from the FP32 hardware estimate
// (reached through the integer-pipe truncating conversion) and take two
// Newton-Raphson steps in FP64, each squaring the relative error:
//   1/x:        y <- y + y (1 - x y)
//   1/sqrt(x):  y <- y + y (1 - x y^2) / 2
// (the FP64 pipe of GB300 issues few instructions per cycle; a correctly
// rounded FP64 division or square root costs several times more).
__device__ __forceinline__ double rcp_nr(double x) {
  double y = f2d(__frcp_rn(d2f_trunc(x)));
  double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  return fma(y, e, y);
}
__device__ __forceinline__ double rsqrt_nr(double x) {
  double y = f2d(rsqrtf(d2f_trunc(x)));
  double e = fma(-x * y, y, 1.0);
  y = fma(0.5 * y, e, y);
  e = fma(-x * y, y, 1.0);
  return fma(0.5 * y, e, y);
}

// kernel gradient factor coef(r) (dW = coef * u) and its r-derivative, with
// the reference's guards (CubicSpline.py:40-70, Gaussian.py:42-59)
// (q = r / h, ih = 1 / h, ir = 1 / r; one reciprocal each per pair)
template <int KERNEL>
__device__ __forceinline__ void grad_coef(double r, double q, double ih, double ir, double &coef, double &dcoef) {
  coef = 0.0;
  dcoef = 0.0;
  const double ih2 = ih * ih;
  if (KERNEL == SPH_KERNEL_CUBIC) {
    if (q > 2.0 || r < 1e-10) return;
    const double al = kCubicFac * ih2;
    double g, gp;
    if (q > 1.0) {
      const double t = 2.0 - q;
      g = -0.75 * t * t;
      gp = 1.5 * t;
    } else {
      g = -3.0 * q * (1.0 - 0.75 * q);
      gp = -3.0 + 4.5 * q;
    }
    const double a = al * ih * ir;
    coef = a * g;
    dcoef = a * (gp * ih - g * ir);
  } else if (KERNEL == SPH_KERNEL_WENDLAND) {
    // g(q) = (1 - q/2)^5 (-14/3) q (1 + 2.5 q) (Wendland.py:58-60)
    if (q >= 2.0 || r < 1e-10) return;
    const double al = kWendFac * ih2;
    const double in = 1.0 - 0.5 * q, in2 = in * in, in4 = in2 * in2;
    const double g = in4 * in * (-14.0 / 3.0) * q * (1.0 + 2.5 * q);
    const double gp = (-14.0 / 3.0) * (in4 * in * (1.0 + 5.0 * q) - 2.5 * in4 * q * (1.0 + 2.5 * q));
    const double a = al * ih * ir;
    coef = a * g;
    dcoef = a * (gp * ih - g * ir);
  } else {
    if (!(q <= 3.0) || !(r > 1e-12 * ih)) return;
    coef = -2.0 * kInvPi * ih2 * exp(-q * q) * ih2;
    dcoef = coef * (-2.0 * r * ih2);
  }
}

struct AdjPtrs {
  const float4 *rec0;  // FP32 positions and signed h (prefilter)
  const double4_32a *r64a, *r64b;
  const int *perm, *keys_sorted;
  const int2 *meta;
  const unsigned int *cstart;
  const DevGrid *grid;
  DevCtrl *ctrl;
  const double *lax, *lay, *lad;                  // lambda_A, lambda_D (caller order)
  double *xhb, *yhb, *vxhb, *vyhb, *rhohb, *alb;  // outputs (caller order)
};

// the candidates of fluid query slot k that fall to lane `part`
template <int KERNEL>
__device__ __forceinline__ void adjoint_query(const AdjPtrs &P, const AdjParams &ap, long long k, int i,
                                              unsigned int part, double &gx, double &gy, double &gvx, double &gvy,
                                              double &grho, double &gal) {
  const DevGrid &g = *P.grid;
  const double4_32a Ak = P.r64a[k], Bk = P.r64b[k];
  const double xk = Ak.x, yk = Ak.y, vxk = Ak.z, vyk = Ak.w;
  const double mk = Bk.x, rhok = Bk.y, othrk = Bk.z, hk = Bk.w;
  const double lAxk = P.lax[i], lAyk = P.lay[i], lDk = P.lad[i];
  const double dothk = dothr_drho(rhok, othrk, ap);
  const double ihk = 1.0 / hk;  // 1 / h_ij of pairs with h_j == h_k
  const double cbar = 0.5 * ap.co;
  const int2 qref = P.meta[k];
  const int qkey = P.keys_sorted[k];
  const bool slow = qref.x >= g.ncx || !(hk > 0.0);
  const int W = g.mode == 0 ? 1 : (slow ? g.wide : g.wt);
  const bool filter = g.mode == 1 && (g.need_filter || P.ctrl->alias_count > 0);
  unsigned int cnt = 0;
  // the forward's padded FP32 reach test: a candidate outside it contributes
  // nothing (kernel support for fluid, min(r0, 3 h_ij) for boundary)
  const float4 Qi = P.rec0[k];
  const float hif = Qi.z, r0f = (float)ap.r0, pad = g.pad_e;
  const float SK = (float)Support<KERNEL>::q * 1.000002f;
  const Stencil sten(g, qref, qkey, W);
  for_stencil(sten, P.cstart, [&](unsigned int j) {
    if ((cnt++ % kAdjSplit) != part) return;
    if (j == (unsigned int)k) return;
    if (filter && !in_ref_stencil(P.meta, j, g, qref)) return;
    {
      const float4 qj = P.rec0[j];
      const float fx = Qi.x - qj.x, fy = Qi.y - qj.y;
      const float hijf = 0.5f * (hif + fabsf(qj.z));
      float reach = SK * hijf;
      if (signbit(qj.z)) reach = fmaxf(reach, fminf(r0f, 3.0f * hijf) * 1.000002f);
      const float rp = reach + pad;
      if (fx * fx + fy * fy > rp * rp) return;
    }
    const double4_32a Aj = P.r64a[j], Bj = P.r64b[j];
    const double dx = xk - Aj.x, dy = yk - Aj.y;
    const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    if (!(d2 > 1e-24)) return;  // coincident: no kernel gradient, no boundary force
    const double ir = rsqrt_nr(d2);
    double r = d2 * ir;
    const double hj = fabs(Bj.w);
    const double hij = __dmul_rn(0.5, __dadd_rn(hk, hj));
    // h_j == h_k (fluid pairs at a fixed h) and h_j == 0 (boundary) are exact
    const double ih = hj == hk ? ihk : (hj == 0.0 ? 2.0 * ihk : rcp_nr(hij));
    double q = r * ih;
    // the forward's neighbour test q = r / h_ij <= 3 (NNLinkedList.py:74),
    // redone with its correctly rounded operations where the estimate could
    // decide differently
    if (fabs(q - 3.0) < 1e-9) {
      r = __dsqrt_rn(d2);
      q = __ddiv_rn(r, hij);
    }
    if (!(q <= 3.0)) return;
    if (!signbit(Bj.w)) {
      // fluid pair: continuity + momentum with artificial viscosity
      const double mj = Bj.x, rhoj = Bj.y, othrj = Bj.z;
      const double vxij = vxk - Aj.z, vyij = vyk - Aj.w;
      double coef, dcoef;
      grad_coef<KERNEL>(r, q, ih, ir, coef, dcoef);
      if (coef == 0.0 && dcoef == 0.0) return;
      const double dWx = coef * dx, dWy = coef * dy;
      const double dot = vxij * dx + vyij * dy;
      const double irbar = 2.0 * rcp_nr(rhok + rhoj);
      double Pi = 0.0, dPi_dmu = 0.0, mu = 0.0, iden = 0.0, hb = 0.0;
      if (dot < 0.0) {
        hb = 0.5 * (hk + hij);
        iden = rcp_nr(d2 + 0.01 * hb * hb);
        mu = hb * dot * iden;
        Pi = mu * (ap.beta * mu - ap.alpha * cbar) * irbar;
        dPi_dmu = (2.0 * ap.beta * mu - ap.alpha * cbar) * irbar;
      }
      const double S = othrk + othrj + Pi;
      const int pj = P.perm[j];
      const double lAxj = P.lax[pj], lAyj = P.lay[pj], lDj = P.lad[pj];
      const double lQx = -mj * lAxk + mk * lAxj, lQy = -mj * lAyk + mk * lAyj;
      const double lC = mj * lDk + mk * lDj;
      const double lQdW = lQx * dWx + lQy * dWy;
      // (d dW / d u)^T z = coef z + dcoef (u . z) u / r
      const double cq = S * dcoef * (dx * lQx + dy * lQy) * ir + lC * dcoef * dot * ir;
      gx += S * coef * lQx + lC * coef * vxij + cq * dx;
      gy += S * coef * lQy + lC * coef * vyij + cq * dy;
      gvx += lC * dWx;
      gvy += lC * dWy;
      if (dot < 0.0) {
        const double f = lQdW * dPi_dmu * hb * iden;
        const double c2 = 2.0 * dot * iden;
        gx += f * (vxij - c2 * dx);
        gy += f * (vyij - c2 * dy);
        gvx += f * dx;
        gvy += f * dy;
        gal += mj * (lAxk * dWx + lAyk * dWy) * (mu * cbar * irbar);
      }
      grho += lQdW * (dothk - 0.5 * Pi * irbar);  // d rbar / d rho_k = 1/2
    } else if (r <= ap.r0 && r > 1e-12) {
      // boundary pair: Lennard-Jones force b = D phi(r) u, phi = ((r0/r)^p1 - (r0/r)^p2) / r^2,
      // and the wall load -m_k b.x when j is on the loaded wall
      const double s = ap.r0 * ir;
      double sp1, sp2;
      if (ap.lj_42) {
        sp2 = s * s;
        sp1 = sp2 * sp2;
      } else {
        sp1 = pow(s, ap.p1);
        sp2 = pow(s, ap.p2);
      }
      const double ir2 = ir * ir;
      const double phi = (sp1 - sp2) * ir2;
      const double dphi = ((-ap.p1 - 2.0) * sp1 + (ap.p2 + 2.0) * sp2) * ir2 * ir;
      const double zx = lAxk - ((ap.omega != 0.0 && Aj.x >= ap.wall_x) ? ap.omega * mk : 0.0), zy = lAyk;
      const double c = dphi * (dx * zx + dy * zy) * ir;
      gx += ap.D * (phi * zx + c * dx);
      gy += ap.D * (phi * zy + c * dy);
    }
  });
}

template <int KERNEL>
__global__ void __launch_bounds__(kAdjBlock, 12) k_pair_adjoint(AdjPtrs P, AdjParams ap) {
  // kAdjSplit adjacent lanes share a query and take every kAdjSplit-th
  // candidate of its stencil; their sums are combined with shuffles
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long k = t / kAdjSplit;
  const unsigned int part = (unsigned int)(t % kAdjSplit);
  double gx = 0.0, gy = 0.0, gvx = 0.0, gvy = 0.0, grho = 0.0, gal = 0.0;
  int i = -1;
  if (k < ap.n) {
    i = P.perm[k];
    if (!signbit(P.r64b[k].w)) adjoint_query<KERNEL>(P, ap, k, i, part, gx, gy, gvx, gvy, grho, gal);
  }
#pragma unroll
  for (int o = 1; o < kAdjSplit; o <<= 1) {
    gx += __shfl_xor_sync(0xffffffffu, gx, o);
    gy += __shfl_xor_sync(0xffffffffu, gy, o);
    gvx += __shfl_xor_sync(0xffffffffu, gvx, o);
    gvy += __shfl_xor_sync(0xffffffffu, gvy, o);
    grho += __shfl_xor_sync(0xffffffffu, grho, o);
    gal += __shfl_xor_sync(0xffffffffu, gal, o);
  }
  if (i >= 0 && part == 0) {  // non-fluid particles get zeros: no outputs, their adjoint is not used
    P.xhb[i] = gx;
    P.yhb[i] = gy;
    P.vxhb[i] = gvx;
    P.vyhb[i] = gvy;
    P.rhohb[i] = grho;
    P.alb[i] = gal;
  }
}

// ---------------------------------------------------------------------------
// Mixed form of the adjoint pair product: the same vector-Jacobian product as
// adjoint_query with the pair arithmetic in FP32 (hardware reciprocals and
// square roots) and the per-particle sums in FP32, over the FP64 records of
// the forward evaluation and the FP64 adjoint vectors.  Differences of FP64
// positions and velocities are formed in FP64 and then rounded, so large
// coordinates lose no accuracy.  The forward's q <= 3 decision is redone
// exactly where FP32 could decide it differently.
// ---------------------------------------------------------------------------
template <int KERNEL>
__device__ __forceinline__ void grad_coef_f(float r, float q, float ih, float ir, float &coef, float &dcoef) {
  coef = 0.f;
  dcoef = 0.f;
  const float ih2 = ih * ih;
  if (KERNEL == SPH_KERNEL_CUBIC) {
    if (q > 2.0f || r < 1e-10f) return;
    const float al = (float)kCubicFac * ih2;
    float g, gp;
    if (q > 1.0f) {
      const float t = 2.0f - q;
      g = -0.75f * t * t;
      gp = 1.5f * t;
    } else {
      g = -3.0f * q * (1.0f - 0.75f * q);
      gp = -3.0f + 4.5f * q;
    }
    const float a = al * ih * ir;
    coef = a * g;
    dcoef = a * (gp * ih - g * ir);
  } else if (KERNEL == SPH_KERNEL_WENDLAND) {
    if (q >= 2.0f || r < 1e-10f) return;
    const float al = (float)kWendFac * ih2;
    const float in = 1.0f - 0.5f * q, in2 = in * in, in4 = in2 * in2;
    const float g = in4 * in * (-14.0f / 3.0f) * q * (1.0f + 2.5f * q);
    const float gp = (-14.0f / 3.0f) * (in4 * in * (1.0f + 5.0f * q) - 2.5f * in4 * q * (1.0f + 2.5f * q));
    const float a = al * ih * ir;
    coef = a * g;
    dcoef = a * (gp * ih - g * ir);
  } else {
    if (!(q <= 3.0f) || !(r > 1e-12f * ih)) return;
    coef = -2.0f * (float)kInvPi * ih2 * __expf(-q * q) * ih2;
    dcoef = coef * (-2.0f * r * ih2);
  }
}

template <int KERNEL>
__device__ __forceinline__ void adjoint_query_mixed(const AdjPtrs &P, const AdjParams &ap, long long k, int i,
                                                    float &gx, float &gy, float &gvx, float &gvy, float &grho,
                                                    float &gal) {
  const DevGrid &g = *P.grid;
  const double4_32a Ak = P.r64a[k], Bk = P.r64b[k];
  const double xk = Ak.x, yk = Ak.y, vxk = Ak.z, vyk = Ak.w;
  const double hk = Bk.w;
  const float mk = d2f_trunc(Bk.x), rhok = d2f_trunc(Bk.y), othrk = d2f_trunc(Bk.z), hkf = d2f_trunc(hk);
  const float lAxk = d2f_trunc(P.lax[i]), lAyk = d2f_trunc(P.lay[i]), lDk = d2f_trunc(P.lad[i]);
  const float dothk = d2f_trunc(dothr_drho(Bk.y, Bk.z, ap));
  const float ihk = __fdividef(1.0f, hkf);
  const float cbar = 0.5f * (float)ap.co, alpha = (float)ap.alpha, beta = (float)ap.beta;
  const float r0 = (float)ap.r0, D = (float)ap.D, p1 = (float)ap.p1, p2 = (float)ap.p2;
  const float omega_m = (float)ap.omega * mk;
  const int2 qref = P.meta[k];
  const int qkey = P.keys_sorted[k];
  const bool slow = qref.x >= g.ncx || !(hk > 0.0);
  const int W = g.mode == 0 ? 1 : (slow ? g.wide : g.wt);
  const bool filter = g.mode == 1 && (g.need_filter || P.ctrl->alias_count > 0);
  const float4 Qi = P.rec0[k];
  const float hif = Qi.z, pad = g.pad_e;
  const float SK = (float)Support<KERNEL>::q * 1.000002f;
  const Stencil sten(g, qref, qkey, W);
  for_stencil(sten, P.cstart, [&](unsigned int j) {
    if (j == (unsigned int)k) return;
    if (filter && !in_ref_stencil(P.meta, j, g, qref)) return;
    {
      const float4 qj = P.rec0[j];
      const float fx = Qi.x - qj.x, fy = Qi.y - qj.y;
      const float hijf = 0.5f * (hif + fabsf(qj.z));
      float reach = SK * hijf;
      if (signbit(qj.z)) reach = fmaxf(reach, fminf(r0, 3.0f * hijf) * 1.000002f);
      const float rp = reach + pad;
      if (fx * fx + fy * fy > rp * rp) return;
    }
    const double4_32a Aj = P.r64a[j], Bj = P.r64b[j];
    const double dxd = xk - Aj.x, dyd = yk - Aj.y;
    const float dx = d2f_trunc(dxd), dy = d2f_trunc(dyd);
    const float d2 = dx * dx + dy * dy;
    if (!(d2 > 1e-24f)) return;  // coincident: no kernel gradient, no boundary force
    const float ir = rsqrtf(d2);
    const float r = d2 * ir;
    const double hj = fabs(Bj.w);
    const float hjf = d2f_trunc(hj);
    const float hij = 0.5f * (hkf + hjf);
    const float ih = hj == hk ? ihk : (hj == 0.0 ? 2.0f * ihk : __fdividef(1.0f, hij));
    const float q = r * ih;
    bool in = q <= 3.0f;
    if (fabsf(q - 3.0f) < 1e-4f) {  // the forward's neighbour test (NNLinkedList.py:74), exactly
      const double rd = __dsqrt_rn(__dadd_rn(__dmul_rn(dxd, dxd), __dmul_rn(dyd, dyd)));
      in = __ddiv_rn(rd, __dmul_rn(0.5, __dadd_rn(hk, hj))) <= 3.0;
    }
    if (!in) return;
    if (!signbit(Bj.w)) {
      // fluid pair: continuity + momentum with artificial viscosity
      const float mj = d2f_trunc(Bj.x), rhoj = d2f_trunc(Bj.y), othrj = d2f_trunc(Bj.z);
      const float vxij = d2f_trunc(vxk - Aj.z), vyij = d2f_trunc(vyk - Aj.w);
      float coef, dcoef;
      grad_coef_f<KERNEL>(r, q, ih, ir, coef, dcoef);
      if (coef == 0.f && dcoef == 0.f) return;
      const float dWx = coef * dx, dWy = coef * dy;
      const float dot = vxij * dx + vyij * dy;
      const float irbar = __fdividef(2.0f, rhok + rhoj);
      float Pi = 0.f, dPi_dmu = 0.f, mu = 0.f, iden = 0.f, hb = 0.f;
      if (dot < 0.f) {
        hb = 0.5f * (hkf + hij);
        iden = __fdividef(1.0f, d2 + 0.01f * hb * hb);
        mu = hb * dot * iden;
        Pi = mu * (beta * mu - alpha * cbar) * irbar;
        dPi_dmu = (2.0f * beta * mu - alpha * cbar) * irbar;
      }
      const float S = othrk + othrj + Pi;
      const int pj = P.perm[j];
      const float lAxj = d2f_trunc(P.lax[pj]), lAyj = d2f_trunc(P.lay[pj]), lDj = d2f_trunc(P.lad[pj]);
      const float lQx = -mj * lAxk + mk * lAxj, lQy = -mj * lAyk + mk * lAyj;
      const float lC = mj * lDk + mk * lDj;
      const float lQdW = lQx * dWx + lQy * dWy;
      // (d dW / d u)^T z = coef z + dcoef (u . z) u / r
      const float cq = S * dcoef * (dx * lQx + dy * lQy) * ir + lC * dcoef * dot * ir;
      gx += S * coef * lQx + lC * coef * vxij + cq * dx;
      gy += S * coef * lQy + lC * coef * vyij + cq * dy;
      gvx += lC * dWx;
      gvy += lC * dWy;
      if (dot < 0.f) {
        const float f = lQdW * dPi_dmu * hb * iden;
        const float c2 = 2.0f * dot * iden;
        gx += f * (vxij - c2 * dx);
        gy += f * (vyij - c2 * dy);
        gvx += f * dx;
        gvy += f * dy;
        gal += mj * (lAxk * dWx + lAyk * dWy) * (mu * cbar * irbar);
      }
      grho += lQdW * (dothk - 0.5f * Pi * irbar);
    } else if (r <= r0 && r > 1e-12f) {
      // boundary pair: Lennard-Jones force and the wall load
      const float s = r0 * ir;
      float sp1, sp2;
      if (ap.lj_42) {
        sp2 = s * s;
        sp1 = sp2 * sp2;
      } else {
        sp1 = __powf(s, p1);
        sp2 = __powf(s, p2);
      }
      const float ir2 = ir * ir;
      const float phi = (sp1 - sp2) * ir2;
      const float dphi = ((-p1 - 2.0f) * sp1 + (p2 + 2.0f) * sp2) * ir2 * ir;
      const float zx = lAxk - ((ap.omega != 0.0 && Aj.x >= ap.wall_x) ? omega_m : 0.f), zy = lAyk;
      const float c = dphi * (dx * zx + dy * zy) * ir;
      gx += D * (phi * zx + c * dx);
      gy += D * (phi * zy + c * dy);
    }
  });
}

template <int KERNEL>
__global__ void __launch_bounds__(kBlock) k_pair_adjoint_mixed(AdjPtrs P, AdjParams ap) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ap.n) return;
  const int i = P.perm[k];
  float gx = 0.f, gy = 0.f, gvx = 0.f, gvy = 0.f, grho = 0.f, gal = 0.f;
  if (!signbit(P.r64b[k].w)) adjoint_query_mixed<KERNEL>(P, ap, k, i, gx, gy, gvx, gvy, grho, gal);
  P.xhb[i] = f2d(gx);
  P.yhb[i] = f2d(gy);
  P.vxhb[i] = f2d(gvx);
  P.vyhb[i] = f2d(gvy);
  P.rhohb[i] = f2d(grho);
  P.alb[i] = f2d(gal);
}

// lambda_A = dt vb' + ab', lambda_D = dt rhob' + drhob' (zero for non-fluid)
__global__ void k_adj_pre(const int8_t *__restrict__ label, long long n, double dt, const double *vxb,
                          const double *vyb, const double *rhob, const double *axb, const double *ayb,
                          const double *drhob, double *lax, double *lay, double *lad) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!is_fluid(label[i])) {
    lax[i] = lay[i] = lad[i] = 0.0;
    return;
  }
  lax[i] = dt * vxb[i] + axb[i];
  lay[i] = dt * vyb[i] + ayb[i];
  lad[i] = dt * rhob[i] + drhob[i];
}

// the half state of step S (PEC.predict's update, src/Integrators/PEC.py:32-60)
// into the scratch particle set; m, h and label are copied
__global__ void k_adj_half(StepArgs s, StepArgs h, double dt) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.n) return;
  const int8_t lab = s.label[i];
  const_cast<int8_t *>(h.label)[i] = lab;  // the scratch set is writable
  h.m[i] = s.m[i];
  h.h[i] = s.h[i];
  const double hdt = 0.5 * dt;
  if (is_fluid(lab)) {
    h.x[i] = s.x[i] + hdt * s.vx[i];
    h.y[i] = s.y[i] + hdt * s.vy[i];
    h.vx[i] = s.vx[i] + hdt * s.ax[i];
    h.vy[i] = s.vy[i] + hdt * s.ay[i];
    double rho = s.rho[i] + hdt * s.drho[i];
    h.rho[i] = rho;
  } else {
    h.x[i] = s.x[i];
    h.y[i] = s.y[i];
    h.vx[i] = s.vx[i];
    h.vy[i] = s.vy[i];
    h.rho[i] = s.rho[i];
  }
}

// state adjoint update of the step (see the top of the file); the *b arrays
// hold the adjoint of S' on entry and that of S on exit; alphab accumulates
__global__ void k_adj_post(const int8_t *__restrict__ label, long long n, double dt, double *xb, double *yb,
                           double *vxb, double *vyb, double *rhob, double *axb, double *ayb, double *drhob,
                           const double *xhb, const double *yhb, const double *vxhb, const double *vyhb,
                           const double *rhohb, const double *alb, double *alphab) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  alphab[i] += alb[i];
  if (!is_fluid(label[i])) return;
  const double hdt = 0.5 * dt;
  const double vhx = vxhb[i] + dt * xb[i], vhy = vyhb[i] + dt * yb[i];
  xb[i] += xhb[i];
  yb[i] += yhb[i];
  vxb[i] += hdt * xhb[i] + vhx;
  vyb[i] += hdt * yhb[i] + vhy;
  axb[i] = hdt * vhx;
  ayb[i] = hdt * vhy;
  rhob[i] += rhohb[i];
  drhob[i] = hdt * rhohb[i];
}

// sum of v[0 .. n) in a fixed order (one block): deterministic
__global__ void k_sum_fixed(const double *__restrict__ v, long long n, double *out) {
  __shared__ double red[1024];
  double s = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) s += v[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

void launch_sum_fixed(const double *v, long long n, double *out, cudaStream_t st) {
  k_sum_fixed<<<1, 1024, 0, st>>>(v, n, out);
}

void launch_adjoint_step(const StepArgs &s, const StepArgs &h, const WsPtrs &w, const sph_config_t &cfg,
                         const sph_wcsph_t &wc, const sph_adjoint_t &adj, cudaStream_t st) {
  const long long n = s.n;
  const double dt = cfg.dt_fixed;
  const unsigned nb = nblocks(n);
  k_adj_pre<<<nb, kBlock, 0, st>>>(s.label, n, dt, adj.vxb, adj.vyb, adj.rhob, adj.axb, adj.ayb, adj.drhob, adj.lax,
                                   adj.lay, adj.lad);
  if (!adj.reuse_build) {
    k_adj_half<<<nb, kBlock, 0, st>>>(s, h, dt);
    // neighbour build and FP64 records of the half state (the forward's own passes)
    launch_bounds(h, w, cfg, wc, kStageNone, true, nullptr, nullptr, st);
    launch_build(h, w, cfg, wc, st);
    sph_config_t c64 = cfg;
    c64.precision = SPH_PREC_FP64;
    launch_records(h, w, c64, wc, true, false, false, st);
  }
  AdjPtrs P;
  P.rec0 = w.rec0;
  P.r64a = w.rec64a;
  P.r64b = w.rec64b;
  P.perm = w.perm;
  P.keys_sorted = w.keys_sorted;
  P.meta = w.meta;
  P.cstart = w.cstart;
  P.grid = w.grid;
  P.ctrl = w.ctrl;
  P.lax = adj.lax;
  P.lay = adj.lay;
  P.lad = adj.lad;
  P.xhb = adj.xhb;
  P.yhb = adj.yhb;
  P.vxhb = adj.vxhb;
  P.vyhb = adj.vyhb;
  P.rhohb = adj.rhohb;
  P.alb = adj.alb;
  AdjParams ap;
  ap.alpha = wc.alpha;
  ap.beta = wc.beta;
  ap.co = wc.co;
  ap.r0 = wc.r0;
  ap.D = wc.D;
  ap.p1 = wc.p1;
  ap.p2 = wc.p2;
  ap.lj_42 = (wc.p1 == 4.0 && wc.p2 == 2.0) ? 1 : 0;
  ap.gamma = wc.gamma;
  ap.B = wc.B;
  ap.inv_rho0 = 1.0 / wc.rho0;
  ap.omega = adj.omega;
  ap.wall_x = adj.wall_x;
  ap.dt = dt;
  ap.n = n;
  if (cfg.precision == SPH_PREC_MIXED) {
    const unsigned nbm = nblocks(n, kBlock);
    if (cfg.kernel == SPH_KERNEL_CUBIC) k_pair_adjoint_mixed<SPH_KERNEL_CUBIC><<<nbm, kBlock, 0, st>>>(P, ap);
    else if (cfg.kernel == SPH_KERNEL_WENDLAND) k_pair_adjoint_mixed<SPH_KERNEL_WENDLAND><<<nbm, kBlock, 0, st>>>(P, ap);
    else k_pair_adjoint_mixed<SPH_KERNEL_GAUSSIAN><<<nbm, kBlock, 0, st>>>(P, ap);
  } else {
    const unsigned nbp = nblocks(n * kAdjSplit, kAdjBlock);
    if (cfg.kernel == SPH_KERNEL_CUBIC) k_pair_adjoint<SPH_KERNEL_CUBIC><<<nbp, kAdjBlock, 0, st>>>(P, ap);
    else if (cfg.kernel == SPH_KERNEL_WENDLAND) k_pair_adjoint<SPH_KERNEL_WENDLAND><<<nbp, kAdjBlock, 0, st>>>(P, ap);
    else k_pair_adjoint<SPH_KERNEL_GAUSSIAN><<<nbp, kAdjBlock, 0, st>>>(P, ap);
  }
  k_adj_post<<<nb, kBlock, 0, st>>>(s.label, n, dt, adj.xb, adj.yb, adj.vxb, adj.vyb, adj.rhob, adj.axb, adj.ayb,
                                    adj.drhob, adj.xhb, adj.yhb, adj.vxhb, adj.vyhb, adj.rhohb, adj.alb, adj.alphab);
}

}  // namespace sph

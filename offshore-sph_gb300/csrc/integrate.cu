// integrate.cu -- per-particle stages of the WCSPH step: PEC / Euler
// integrators, the TimeStep reduction, WCSPH.initialize and the Tait EOS.
#include <math.h>

#include "sph_internal.cuh"

namespace sph {

struct IntParams {
  double dt_fixed;
  const double *dt;
  double inv_damp;
  int damped;
  int use_xsph, strict, integrator;
};

__device__ __forceinline__ double load_dt(const IntParams &ip) { return ip.dt_fixed > 0.0 ? ip.dt_fixed : ip.dt[0]; }

// PEC.predict (src/Integrators/PEC.py:32-59) on the fluid particles
__global__ void __launch_bounds__(kBlock) k_predict(StepArgs a, IntParams ip) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n || !is_fluid(a.label[i])) return;
  const double hdt = 0.5 * load_dt(ip);
  if (ip.integrator == SPH_INTEGRATOR_VERLET) {  // Verlet.predict (src/Integrators/Verlet.py:28-35)
    a.x[i] += hdt * a.vx[i];
    a.y[i] += hdt * a.vy[i];
    return;
  }
  double x = a.x[i], y = a.y[i], vx = a.vx[i], vy = a.vy[i], rho = a.rho[i];
  a.x0[i] = x;
  a.y0[i] = y;
  a.vx0[i] = vx;
  a.vy0[i] = vy;
  if (ip.use_xsph) {
    a.x[i] = x + hdt * a.xsphx[i];
    a.y[i] = y + hdt * a.xsphy[i];
  } else {
    a.x[i] = x + hdt * vx;
    a.y[i] = y + hdt * vy;
  }
  a.vx[i] = (vx + hdt * a.ax[i]) * ip.inv_damp;
  a.vy[i] = (vy + hdt * a.ay[i]) * ip.inv_damp;
  a.rho0[i] = rho;
  rho = rho + hdt * a.drho[i];
  if (ip.strict && rho < 0.0) rho = 0.0;
  a.rho[i] = rho;
}

// PEC.correct (src/Integrators/PEC.py:61-89) or Euler.correct
// (src/Integrators/Euler.py:17-27) on the fluid particles
__device__ __forceinline__ void correct_one(const StepArgs &a, long long i, const IntParams &ip) {
  const double dt = load_dt(ip);
  const double hdt = 0.5 * dt;
  const double ax = a.ax[i], ay = a.ay[i], drho = a.drho[i];
  if (ip.integrator == SPH_INTEGRATOR_VERLET) {  // Verlet.correct (src/Integrators/Verlet.py:37-53)
    const double vx = fma(dt, ax, a.vx[i]), vy = fma(dt, ay, a.vy[i]);
    a.vx[i] = vx;
    a.vy[i] = vy;
    if (ip.use_xsph) {
      a.x[i] = fma(hdt, a.xsphx[i], a.x[i]);
      a.y[i] = fma(hdt, a.xsphy[i], a.y[i]);
    } else {
      a.x[i] = fma(hdt, vx, a.x[i]);
      a.y[i] = fma(hdt, vy, a.y[i]);
    }
    return;
  }
  if (ip.integrator == SPH_INTEGRATOR_EULER) {
    const double vx = a.vx[i], vy = a.vy[i];
    a.x[i] = a.x[i] + dt * vx + 0.5 * dt * dt * ax;
    a.y[i] = a.y[i] + dt * vy + 0.5 * dt * dt * ay;
    a.vx[i] = vx + dt * ax;
    a.vy[i] = vy + dt * ay;
    a.rho[i] = a.rho[i] + dt * drho;
    return;
  }
  // PEC's corrector x = 2 (x0 + dt/2 v) - x0 etc. in its reduced form
  // x0 + dt v: the same value to one rounding, with half the FP64 operations
  const double x0 = a.x0[i], y0 = a.y0[i], vx0 = a.vx0[i], vy0 = a.vy0[i], rho0 = a.rho0[i];
  if (ip.use_xsph) {
    a.x[i] = fma(dt, a.xsphx[i], x0);
    a.y[i] = fma(dt, a.xsphy[i], y0);
  } else {
    a.x[i] = fma(dt, a.vx[i], x0);
    a.y[i] = fma(dt, a.vy[i], y0);
  }
  if (ip.damped) {
    // 2 (v0 + dt/2 a) / (1 + damping/2) - v0
    const double c0 = 2.0 * ip.inv_damp - 1.0, c1 = dt * ip.inv_damp;
    a.vx[i] = fma(c1, ax, c0 * vx0);
    a.vy[i] = fma(c1, ay, c0 * vy0);
  } else {
    a.vx[i] = fma(dt, ax, vx0);
    a.vy[i] = fma(dt, ay, vy0);
  }
  double rho = fma(dt, drho, rho0);
  if (ip.strict && rho < 0.0) rho = 0.0;
  a.rho[i] = rho;
  (void)hdt;
}

__global__ void __launch_bounds__(kBlock) k_correct(StepArgs a, IntParams ip) {
  step_kernel_entry();
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n || !is_fluid(a.label[i])) return;
  correct_one(a, i, ip);
}

static IntParams int_params(const sph_config_t &cfg, const double *dt, double dt_fixed) {
  IntParams ip;
  ip.dt_fixed = dt_fixed;
  ip.dt = dt;
  ip.inv_damp = 1.0 / (1.0 + 0.5 * cfg.damping);
  ip.damped = cfg.damping != 0.0 ? 1 : 0;
  ip.use_xsph = cfg.pec_use_xsph;
  ip.strict = cfg.pec_strict;
  ip.integrator = cfg.integrator;
  return ip;
}

void launch_predict(const StepArgs &a, const sph_config_t &cfg, const double *dt, double dt_fixed,
                    cudaStream_t st) {
  if (cfg.integrator == SPH_INTEGRATOR_EULER) return;  // Euler.predict is a no-op
  k_predict<<<nblocks(a.n), kBlock, 0, st>>>(a, int_params(cfg, dt, dt_fixed));
}

void launch_correct(const StepArgs &a, const sph_config_t &cfg, const double *dt, double dt_fixed,
                    cudaStream_t st) {
  launch_pdl(k_correct, dim3(nblocks(a.n)), dim3(kBlock), 0, st, a, int_params(cfg, dt, dt_fixed));
}

// TimeStep.compute over fluid (src/Equations/TimeStep.py:7-91)
__global__ void __launch_bounds__(kBlock) k_timestep(StepArgs a, DevCtrl *ctrl, double cfl_c, double cfl_f,
                                                     double *dt3, double *dt_hist) {
  step_kernel_entry();
  __shared__ unsigned long long red[32];
  __shared__ unsigned int red32[32];
  __shared__ bool last;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long eh = kEncMinId, ec = kEncMaxId, ea = kEncMaxId;
  unsigned int nf = 0;
  if (i < a.n && is_fluid(a.label[i])) {
    const double ax = a.ax[i], ay = a.ay[i];
    eh = enc_d(a.h[i]);
    ec = enc_d(a.c[i]);
    ea = enc_d(__dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay)));
    nf = 1;
  }
  unsigned long long bh = block_reduce(eh, MinU64(), kEncMinId, red);
  unsigned long long bc = block_reduce(ec, MaxU64(), kEncMaxId, red);
  unsigned long long ba = block_reduce(ea, MaxU64(), kEncMaxId, red);
  unsigned int bn = block_reduce(nf, AddU32(), 0u, red32);
  if (threadIdx.x == 0) {
    if (bn) {
      atomicMin(&ctrl->ts_hmin, bh);
      atomicMax(&ctrl->ts_cmax, bc);
      atomicMax(&ctrl->ts_a2max, ba);
      atomicAdd(&ctrl->ts_nfluid, bn);
    }
    __threadfence();
    last = atomicAdd(&ctrl->done_ts, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    double min_h = dec_d(atomicExch(&ctrl->ts_hmin, kEncMinId));
    double max_c = dec_d(atomicExch(&ctrl->ts_cmax, kEncMaxId));
    double max_a2 = dec_d(atomicExch(&ctrl->ts_a2max, kEncMaxId));
    unsigned int cnt = atomicExch(&ctrl->ts_nfluid, 0u);
    atomicExch(&ctrl->done_ts, 0u);
    double dc = __ddiv_rn(__dmul_rn(cfl_c, min_h), max_c);
    double df = max_a2 < 1e-12 ? 1e10 : __dmul_rn(cfl_f, __dsqrt_rn(__ddiv_rn(min_h, max_a2)));
    double dt = (df < dc) ? df : dc;
    unsigned st = 0;
    if (cnt == 0) {
      st |= SPH_STATUS_NO_FLUID;
      dt = dc = df = nan("");
    }
    if (dt < 1e-6) st |= SPH_STATUS_SMALL_DT;
    if (st) atomicOr(&ctrl->status, st);
    dt3[0] = dt;
    dt3[1] = dc;
    dt3[2] = df;
    if (dt_hist) {
      dt_hist[0] = dt;
      dt_hist[1] = dc;
      dt_hist[2] = df;
    }
  }
}

void launch_timestep(const StepArgs &a, const WsPtrs &w, const sph_config_t &cfg, double *dt3, double *dt_hist,
                     cudaStream_t st) {
  launch_pdl(k_timestep, dim3(nblocks(a.n)), dim3(kBlock), 0, st, a, w.ctrl, cfg.cfl_c, cfg.cfl_f, dt3, dt_hist);
}

// WCSPH.initialize (src/Methods/WCSPH.py:82-108 via TaitEOS_height,
// src/Equations/TaitEOS.py:46-65) and the rest of Solver.setup's fluid
// preparation (src/Solver.py:184-196)
__global__ void __launch_bounds__(kBlock) k_initialize(StepArgs a, double h_fixed, double rho0, double H,
                                                       double B, double gamma, double Pb, double co) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n || !is_fluid(a.label[i])) return;
  a.h[i] = reset_h(h_fixed, a.m[i], a.rho[i]);
  double frac = rho0 * 9.81 * (H - a.y[i]) / B;
  double rho = rho0 * pow(1.0 + frac, 1.0 / gamma);
  a.rho[i] = rho;
  a.p[i] = tait_p(rho, SPH_FLUID, gamma, B, 1.0 / rho0, Pb);
  a.c[i] = co;
}

void launch_initialize(const StepArgs &a, const sph_wcsph_t &wc, const sph_config_t &cfg, cudaStream_t st) {
  k_initialize<<<nblocks(a.n), kBlock, 0, st>>>(a, cfg.h_fixed, wc.rho0, wc.height, wc.B, wc.gamma, wc.Pb, wc.co);
}

// WCSPH.compute_pressure / compute_speed_of_sound for all particles
__global__ void __launch_bounds__(kBlock) k_eos(StepArgs a, double gamma, double B, double rho0, double Pb,
                                                double co) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  a.p[i] = tait_p(a.rho[i], a.label[i], gamma, B, 1.0 / rho0, Pb);
  a.c[i] = co;
}

void launch_eos(const StepArgs &a, const sph_wcsph_t &wc, cudaStream_t st) {
  k_eos<<<nblocks(a.n), kBlock, 0, st>>>(a, wc.gamma, wc.B, wc.rho0, wc.Pb, wc.co);
}

// Kernel.evaluate / gradient / Gaussian.derivative, elementwise
__global__ void __launch_bounds__(kBlock) k_kernel_map(int kernel, int what, long long n, const double *x,
                                                       const double *r, const double *h, double *out) {
  long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double rj = r[j], hj = h[j];
  double v;
  if (what == 2) v = gauss_dwdq(rj, hj);
  else if (what == 0)
    v = kernel == SPH_KERNEL_CUBIC ? cubic_w(rj, hj) : (kernel == SPH_KERNEL_WENDLAND ? wendland_w(rj, hj) : gauss_w(rj, hj));
  else
    v = (kernel == SPH_KERNEL_CUBIC ? cubic_gcoef(rj, hj)
                                    : (kernel == SPH_KERNEL_WENDLAND ? wendland_gcoef(rj, hj) : gauss_gcoef(rj, hj))) *
        x[j];
  out[j] = v;
}

void launch_kernel_map(int kernel, int what, long long n, const double *x, const double *r, const double *h,
                       double *out, cudaStream_t st) {
  k_kernel_map<<<nblocks(n), kBlock, 0, st>>>(kernel, what, n, x, r, h, out);
}

// ---------------------------------------------------------------------------
// Batched form (see nn_build.cu): per-instance TimeStep and corrector.
// ---------------------------------------------------------------------------
// TimeStep's formulas (src/Equations/TimeStep.py:7-56) into dt3 = {dt, dt_c, dt_f};
// returns status bits
__device__ unsigned dt_from(double min_h, double max_c, double max_a2, unsigned int cnt, double cfl_c,
                            double cfl_f, double *dt3) {
  double dc = __ddiv_rn(__dmul_rn(cfl_c, min_h), max_c);
  double df = max_a2 < 1e-12 ? 1e10 : __dmul_rn(cfl_f, __dsqrt_rn(__ddiv_rn(min_h, max_a2)));
  double dt = (df < dc) ? df : dc;
  unsigned st = 0;
  if (cnt == 0) {
    st |= SPH_STATUS_NO_FLUID;
    dt = dc = df = nan("");
  }
  if (dt < 1e-6) st |= SPH_STATUS_SMALL_DT;
  dt3[0] = dt;
  dt3[1] = dc;
  dt3[2] = df;
  return st;
}

// the initial TimeStep's reductions per instance (min h, max c, max a^2 over fluid)
__global__ void __launch_bounds__(kBlock) k_bt_timestep(StepArgs a, BatchPtrs B) {
  step_kernel_entry();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long eh = kEncMinId, ec = kEncMinId, ea = kEncMinId;  // maxima as minima of the complement
  unsigned int nf = 0;
  int b = -1;
  if (i < a.n) {
    b = B.inst[i];
    if (is_fluid(a.label[i])) {
      const double ax = a.ax[i], ay = a.ay[i];
      eh = enc_d(a.h[i]);
      ec = ~enc_d(a.c[i]);
      ea = ~enc_d(__dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay)));
      nf = 1;
    }
  }
  InstSlots *sl = B.sl;
  seg_min_u64(eh, b, [&](int q, unsigned long long m) { atomicMin(&sl[q].pd_hmin, m); });
  seg_min_u64(ec, b, [&](int q, unsigned long long m) { atomicMax(&sl[q].ts_cmax, ~m); });
  seg_min_u64(ea, b, [&](int q, unsigned long long m) { atomicMax(&sl[q].pd_a2max, ~m); });
  seg_add_u32(nf, b, [&](int q, unsigned int c) { atomicAdd(&sl[q].pd_nfluid, c); });
}

// every instance's dt from its reductions into dt_ring[slot] (and dt_hist,
// n_inst x 3, when given); the reductions return to their identities.
// use_c: max c from the reduction (initial TimeStep), else co (the pair
// pass's epilogue, where compute_speed_of_sound gives co to every particle)
__global__ void k_bt_dt_finish(BatchPtrs B, DevCtrl *ctrl, int slot, double *dt_hist, int use_c) {
  step_kernel_entry();
  unsigned st = 0;
  for (int b = threadIdx.x; b < B.n_inst; b += blockDim.x) {
    InstSlots &s = B.sl[b];
    const double min_h = dec_d(s.pd_hmin), max_a2 = dec_d(s.pd_a2max), max_c_r = dec_d(s.ts_cmax);
    const unsigned int cnt = s.pd_nfluid;
    s.pd_hmin = kEncMinId;
    s.pd_a2max = kEncMaxId;
    s.ts_cmax = kEncMaxId;
    s.pd_nfluid = 0;
    const InstParams &p = B.ip[b];
    st |= dt_from(min_h, use_c ? max_c_r : p.pp.co, max_a2, cnt, p.cfl_c, p.cfl_f, s.dt_ring[slot]);
    if (dt_hist) {
      dt_hist[3 * b] = s.dt_ring[slot][0];
      dt_hist[3 * b + 1] = s.dt_ring[slot][1];
      dt_hist[3 * b + 2] = s.dt_ring[slot][2];
    }
  }
  if (st) atomicOr(&ctrl->status, st);
}

__global__ void __launch_bounds__(kBlock) k_bt_correct(StepArgs a, BatchPtrs B, IntParams ip, int slot) {
  step_kernel_entry();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n || !is_fluid(a.label[i])) return;
  IntParams q = ip;
  q.dt = B.sl[B.inst[i]].dt_ring[slot];
  correct_one(a, i, q);
}

void launch_bt_timestep(const StepArgs &a, const WsPtrs &w, const BatchPtrs &B, int slot, double *dt_hist,
                        cudaStream_t st) {
  launch_pdl(k_bt_timestep, dim3(nblocks(a.n)), dim3(kBlock), 0, st, a, B);
  launch_pdl(k_bt_dt_finish, dim3(1), dim3(256), 0, st, B, w.ctrl, slot, dt_hist, 1);
}

void launch_bt_dt_finish(const WsPtrs &w, const BatchPtrs &B, int slot, double *dt_hist, cudaStream_t st) {
  launch_pdl(k_bt_dt_finish, dim3(1), dim3(256), 0, st, B, w.ctrl, slot, dt_hist, 0);
}

void launch_bt_correct(const StepArgs &a, const BatchPtrs &B, const sph_config_t &cfg, int slot, cudaStream_t st) {
  launch_pdl(k_bt_correct, dim3(nblocks(a.n)), dim3(kBlock), 0, st, a, B, int_params(cfg, nullptr, 0.0), slot);
}

}  // namespace sph

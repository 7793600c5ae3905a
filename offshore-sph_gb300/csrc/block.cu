// block.cu -- the per-neighbour-block plugin methods of WCSPH on the device.
//
// The reference's WCSPH exposes compute_density_change, compute_acceleration
// and compute_velocity (src/Methods/WCSPH.py:151-203) on one particle and a
// block of its neighbours in computed_dtype layout (src/Common.py:60-98);
// _loop calls them, plus BoundaryForce, once per particle
// (src/Tools/SolverTools.py:143-173).  The step itself never goes through
// here -- it runs the same equations fused in the pair kernels -- but a user
// of the plugin surface (a custom Method or Solver loop, the reference's own
// formula tests) calls them per block, and this file gives those calls a
// device implementation.
//
// One thread sums the block in its order with no contraction (this file is
// compiled with -fmad=false), the same IEEE operations as the reference's
// loops, so the results agree with the reference to rounding.
#include "sph_internal.cuh"

namespace sph {

struct BlockSelf {
  double p, rho, h, c;
};

__global__ void k_block_equations(sph_block_t b, BlockSelf s, sph_wcsph_t w, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const long long J = b.n;
  // Continuity (src/Equations/Continuity.py:4-16)
  double arho = 0.0;
  for (long long j = 0; j < J; j++) {
    if (b.label[j] != SPH_FLUID) continue;
    const double dot = b.vx[j] * b.dw_x[j] + b.vy[j] * b.dw_y[j];
    arho += b.m[j] * dot;
  }
  // Momentum (src/Equations/Momentum.py:5-57)
  const double slf = s.p / (s.rho * s.rho);
  double a0 = 0.0, a1 = 0.0;
  for (long long j = 0; j < J; j++) {
    if (b.label[j] != SPH_FLUID) continue;
    const double othr = b.p[j] / (b.rho[j] * b.rho[j]);
    const double dot = b.vx[j] * b.x[j] + b.vy[j] * b.y[j];
    double PI = 0.0;
    if (dot < 0) {
      const double hij = 0.5 * (s.h + b.h[j]);
      const double cij = 0.5 * (s.c + b.c[j]);
      const double rhoij = 0.5 * (s.rho + b.rho[j]);
      const double mu = hij * dot / (b.r[j] * b.r[j] + 0.01 * hij * hij);
      const double pp = mu * (w.beta * mu - w.alpha * cij);
      PI = pp / rhoij;
    }
    const double factor = slf + othr + PI;
    a0 += -b.m[j] * factor * b.dw_x[j];
    a1 += -b.m[j] * factor * b.dw_y[j];
  }
  // BoundaryForce (src/Equations/BoundaryForce.py:6-42)
  double f0 = 0.0, f1 = 0.0;
  for (long long j = 0; j < J; j++) {
    if (b.label[j] == SPH_FLUID || b.r[j] > w.r0) continue;
    if (b.r[j] > 1e-12) {
      const double frac = w.r0 / b.r[j];
      const double fac = w.D * (pow(frac, w.p1) - pow(frac, w.p2));
      f0 += fac * b.x[j] / pow(b.r[j], 2.0);
      f1 += fac * b.y[j] / pow(b.r[j], 2.0);
    }
  }
  // XSPH (src/Equations/XSPH.py:5-31)
  double x0 = 0.0, x1 = 0.0;
  for (long long j = 0; j < J; j++) {
    const double rho_ij = 0.5 * (s.rho + b.rho[j]);
    const double fac = -w.epsilon * b.m[j] * b.w[j] / rho_ij;
    x0 += fac * b.vx[j];
    x1 += fac * b.vy[j];
  }
  out[0] = arho;
  out[1] = a0;
  out[2] = a1;
  out[3] = f0;
  out[4] = f1;
  out[5] = x0;
  out[6] = x1;
}

}  // namespace sph

extern "C" int sph_block_equations(const sph_block_t *blk, const double *self4, const sph_wcsph_t *w, double *out,
                                   sph_stream_t stream) {
  if (!blk || blk->n < 0 || !self4 || !w || !out) return SPH_ERR_INVALID_ARGUMENT;
  if (blk->n > 0) {
    const void *need[] = {blk->label, blk->m, blk->p, blk->rho, blk->h, blk->c, blk->r, blk->w,
                          blk->dw_x, blk->dw_y, blk->x, blk->y, blk->vx, blk->vy};
    for (const void *q : need)
      if (!q) return SPH_ERR_INVALID_ARGUMENT;
  }
  sph::BlockSelf s{self4[0], self4[1], self4[2], self4[3]};
  sph::k_block_equations<<<1, 32, 0, (cudaStream_t)stream>>>(*blk, s, *w, out);
  return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

// newmark.cu -- the Newmark-beta integrator of the coupled (structure)
// particles and its acceleration solve (src/Integrators/NewmarkBeta.py), the
// coupling integrator of the ice-sheet example (examples/IceBreak.py:579-586).
//
// predict / correct update the particles labelled SPH_COUPLED, in the
// reference's operation order with no FMA contraction, so that they match it
// bit for bit.  The acceleration solve forms
//   lhs = M + (C gamma) dt + (K beta) dt^2,  rhs = F - K r - C v
// (NewmarkBeta.py:90-91) in LAPACK-style column band storage and solves
// lhs a = rhs by LU with partial pivoting and two triangular solves in one
// block.  The reference inverts lhs (np.linalg.inv) and multiplies; the
// factorisation gives the same a to rounding.  Beam matrices are banded
// (the example's stiffness is pentadiagonal, mass and damping diagonal), so
// the work is O(n (kl + ku) kl); dense matrices (kl = ku = n - 1) run the
// same code in O(n^3).
#include <stdint.h>

#include "sph_internal.cuh"

namespace sph {

constexpr int kSolveBlock = 256;

// NewmarkBeta.predict (NewmarkBeta.py:41-54) / correct (:56-69)
template <bool PREDICT>
__global__ void __launch_bounds__(kBlock) k_newmark(StepArgs a, double beta, double gamma, const double *dtp) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n || a.label[i] != SPH_COUPLED) return;
  const double dt = *dtp;
  const double dt2 = __dmul_rn(dt, dt);
  const double ax = a.ax[i], ay = a.ay[i];
  if (PREDICT) {
    // x + vx dt + ax (0.5 - beta) dt^2 ;  vx + ax (1 - gamma) dt
    const double cb = __dsub_rn(0.5, beta), cg = __dsub_rn(1.0, gamma);
    a.x[i] = __dadd_rn(__dadd_rn(a.x[i], __dmul_rn(a.vx[i], dt)), __dmul_rn(__dmul_rn(ax, cb), dt2));
    a.y[i] = __dadd_rn(__dadd_rn(a.y[i], __dmul_rn(a.vy[i], dt)), __dmul_rn(__dmul_rn(ay, cb), dt2));
    a.vx[i] = __dadd_rn(a.vx[i], __dmul_rn(__dmul_rn(ax, cg), dt));
    a.vy[i] = __dadd_rn(a.vy[i], __dmul_rn(__dmul_rn(ay, cg), dt));
  } else {
    // x + ax beta dt^2 ;  vx + ax gamma dt
    a.x[i] = __dadd_rn(a.x[i], __dmul_rn(__dmul_rn(ax, beta), dt2));
    a.y[i] = __dadd_rn(a.y[i], __dmul_rn(__dmul_rn(ay, beta), dt2));
    a.vx[i] = __dadd_rn(a.vx[i], __dmul_rn(__dmul_rn(ax, gamma), dt));
    a.vy[i] = __dadd_rn(a.vy[i], __dmul_rn(__dmul_rn(ay, gamma), dt));
  }
}

// The band solve.  Inputs M, K, C in row band storage: row i holds columns
// i - kl .. i + ku at [i * (kl + ku + 1) + (j - i + kl)].  The factor works on
// column band storage with room for the pivoting fill-in: element (i, j),
// j - kl - ku <= i <= j + kl, at ab[j * ldab + (kl + ku + i - j)],
// ldab = 2 kl + ku + 1.
struct BandSolve {
  long long n;
  int kl, ku;
  const double *M, *K, *C, *F, *r, *v;
  double beta, gamma, dt;
  double *ab, *rhs, *out;
  int *piv, *info;
};

__device__ __forceinline__ double &band_at(const BandSolve &s, long long i, long long j) {
  const long long ldab = 2 * s.kl + s.ku + 1;
  return s.ab[j * ldab + (s.kl + s.ku + i - j)];
}

__global__ void __launch_bounds__(kSolveBlock) k_newmark_solve(BandSolve s) {
  __shared__ double red_v[kSolveBlock / 32];
  __shared__ int red_i[kSolveBlock / 32];
  __shared__ int s_piv;
  const int tid = threadIdx.x;
  const long long n = s.n;
  const int kl = s.kl, ku = s.ku, w = kl + ku + 1;
  const long long ldab = 2 * kl + ku + 1;
  const double dt2 = __dmul_rn(s.dt, s.dt);
  // lhs (NewmarkBeta.py:91): M + (C gamma) dt + (K beta) dt^2, fill-in rows zero
  for (long long e = tid; e < n * ldab; e += kSolveBlock) s.ab[e] = 0.0;
  __syncthreads();
  for (long long e = tid; e < n * w; e += kSolveBlock) {
    const long long i = e / w, j = i + (e % w) - kl;
    if (j < 0 || j >= n) continue;
    const double m = s.M[e], c = s.C[e], k = s.K[e];
    band_at(s, i, j) = __dadd_rn(__dadd_rn(m, __dmul_rn(__dmul_rn(c, s.gamma), s.dt)), __dmul_rn(__dmul_rn(k, s.beta), dt2));
  }
  // rhs (NewmarkBeta.py:90): F - K r - C v
  for (long long i = tid; i < n; i += kSolveBlock) {
    double kr = 0.0, cv = 0.0;
    const long long j0 = i - kl > 0 ? i - kl : 0, j1 = i + ku < n - 1 ? i + ku : n - 1;
    for (long long j = j0; j <= j1; j++) {
      const long long e = i * w + (j - i + kl);
      kr = fma(s.K[e], s.r[j], kr);
      cv = fma(s.C[e], s.v[j], cv);
    }
    s.rhs[i] = (s.F[i] - kr) - cv;
  }
  if (tid == 0) *s.info = 0;
  __syncthreads();
  // LU with partial pivoting, column by column
  for (long long j = 0; j < n; j++) {
    const int km = (int)(kl < n - 1 - j ? kl : n - 1 - j);
    // pivot: the first largest |a(j + t, j)|, t = 0 .. km
    double bv = -1.0;
    int bi = 0x7fffffff;
    for (int t = tid; t <= km; t += kSolveBlock) {
      const double v = fabs(band_at(s, j + t, j));
      if (v > bv) {
        bv = v;
        bi = t;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi)) {
        bv = ov;
        bi = oi;
      }
    }
    if ((tid & 31) == 0) {
      red_v[tid >> 5] = bv;
      red_i[tid >> 5] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      double v = red_v[0];
      int p = red_i[0];
      for (int q = 1; q < kSolveBlock / 32; q++)
        if (red_v[q] > v || (red_v[q] == v && red_i[q] < p)) {
          v = red_v[q];
          p = red_i[q];
        }
      if (p > km) p = 0;  // no candidate compared (a column of NaNs)
      s_piv = p;
      s.piv[j] = (int)(j + p);
      if (!(v > 0.0) && *s.info == 0) *s.info = (int)(j + 1);  // exactly singular (LAPACK's info)
    }
    __syncthreads();
    const int p = s_piv;
    const long long u = j + kl + ku < n - 1 ? j + kl + ku : n - 1;  // last column the fill-in reaches
    if (p != 0)
      for (long long c = j + tid; c <= u; c += kSolveBlock) {
        double &x = band_at(s, j, c), &y = band_at(s, j + p, c);
        const double t = x;
        x = y;
        y = t;
      }
    __syncthreads();
    const double ajj = band_at(s, j, j);
    if (ajj != 0.0) {
      for (int t = 1 + tid; t <= km; t += kSolveBlock) band_at(s, j + t, j) = band_at(s, j + t, j) / ajj;
      __syncthreads();
      const long long cols = u - j;
      for (long long e = tid; e < (long long)km * cols; e += kSolveBlock) {
        const long long t = 1 + e / cols, c = j + 1 + e % cols;
        band_at(s, j + t, c) = fma(-band_at(s, j + t, j), band_at(s, j, c), band_at(s, j + t, c));
      }
    }
    __syncthreads();
  }
  if (*s.info != 0) return;
  // forward: P and unit-lower L (each column's multipliers below the diagonal)
  for (long long j = 0; j < n; j++) {
    const int km = (int)(kl < n - 1 - j ? kl : n - 1 - j);
    if (tid == 0) {
      const int pj = s.piv[j];
      if (pj != j) {
        const double t = s.rhs[j];
        s.rhs[j] = s.rhs[pj];
        s.rhs[pj] = t;
      }
    }
    __syncthreads();
    const double bj = s.rhs[j];
    for (int t = 1 + tid; t <= km; t += kSolveBlock) s.rhs[j + t] = fma(-band_at(s, j + t, j), bj, s.rhs[j + t]);
    __syncthreads();
  }
  // back: U, kl + ku superdiagonals
  for (long long j = n - 1; j >= 0; j--) {
    if (tid == 0) s.rhs[j] = s.rhs[j] / band_at(s, j, j);
    __syncthreads();
    const double xj = s.rhs[j];
    const long long i0 = j - kl - ku > 0 ? j - kl - ku : 0;
    for (long long i = i0 + tid; i < j; i += kSolveBlock) s.rhs[i] = fma(-band_at(s, i, j), xj, s.rhs[i]);
    __syncthreads();
  }
  for (long long i = tid; i < n; i += kSolveBlock) s.out[i] = s.rhs[i];
}

static size_t align256n(size_t v) { return (v + 255) & ~(size_t)255; }

struct NewmarkWork {
  size_t ab, rhs, piv, info, total;
};

static NewmarkWork newmark_work(long long n, int kl, int ku) {
  NewmarkWork L;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align256n(off + bytes);
    return o;
  };
  L.ab = take((size_t)n * (size_t)(2 * kl + ku + 1) * 8);
  L.rhs = take((size_t)n * 8);
  L.piv = take((size_t)n * 4);
  L.info = take(8);
  L.total = off;
  return L;
}

}  // namespace sph

using namespace sph;

static bool newmark_params_ok(double beta, double gamma) { return beta * 2 >= gamma; }  // NewmarkBeta.py:32

static int newmark_step(sph_particles_t *pa, double beta, double gamma, const double *dt, sph_stream_t stream,
                        bool predict) {
  if (!pa || pa->n < 0 || !dt || !newmark_params_ok(beta, gamma)) return SPH_ERR_INVALID_ARGUMENT;
  if (pa->n == 0) return SPH_OK;
  if (!pa->label || !pa->x || !pa->y || !pa->vx || !pa->vy || !pa->ax || !pa->ay) return SPH_ERR_INVALID_ARGUMENT;
  const StepArgs a = step_args(pa);
  cudaStream_t st = (cudaStream_t)stream;
  if (predict)
    k_newmark<true><<<nblocks(a.n), kBlock, 0, st>>>(a, beta, gamma, dt);
  else
    k_newmark<false><<<nblocks(a.n), kBlock, 0, st>>>(a, beta, gamma, dt);
  return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

extern "C" {

int sph_newmark_predict(sph_particles_t *pa, double beta, double gamma, const double *dt, sph_stream_t stream) {
  return newmark_step(pa, beta, gamma, dt, stream, true);
}

int sph_newmark_correct(sph_particles_t *pa, double beta, double gamma, const double *dt, sph_stream_t stream) {
  return newmark_step(pa, beta, gamma, dt, stream, false);
}

int sph_newmark_work_size(int64_t n, int32_t kl, int32_t ku, size_t *bytes) {
  if (!bytes || n < 0 || kl < 0 || ku < 0 || (n > 0 && (kl > n - 1 || ku > n - 1)) || n > 0x7fffffffll)
    return SPH_ERR_INVALID_ARGUMENT;
  *bytes = newmark_work(n, kl, ku).total;
  return SPH_OK;
}

int sph_newmark_acceleration(int64_t n, int32_t kl, int32_t ku, const double *M, const double *K, const double *C,
                             double beta, double gamma, double dt, const double *F, const double *r, const double *v,
                             double *a, void *work, size_t work_bytes, int32_t *info, sph_stream_t stream) {
  size_t need = 0;
  if (sph_newmark_work_size(n, kl, ku, &need) != SPH_OK || !newmark_params_ok(beta, gamma))
    return SPH_ERR_INVALID_ARGUMENT;
  if (n == 0) return SPH_OK;
  if (!M || !K || !C || !F || !r || !v || !a || !work || !info) return SPH_ERR_INVALID_ARGUMENT;
  if (work_bytes < need) return SPH_ERR_WORKSPACE_TOO_SMALL;
  const NewmarkWork L = newmark_work(n, kl, ku);
  char *b = (char *)work;
  BandSolve s;
  s.n = n;
  s.kl = kl;
  s.ku = ku;
  s.M = M;
  s.K = K;
  s.C = C;
  s.F = F;
  s.r = r;
  s.v = v;
  s.beta = beta;
  s.gamma = gamma;
  s.dt = dt;
  s.ab = (double *)(b + L.ab);
  s.rhs = (double *)(b + L.rhs);
  s.piv = (int *)(b + L.piv);
  s.info = info;
  s.out = a;
  k_newmark_solve<<<1, kSolveBlock, 0, (cudaStream_t)stream>>>(s);
  return cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}

}  // extern "C"

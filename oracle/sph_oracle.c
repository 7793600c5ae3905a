/*
 * sph_oracle.c -- CPU restatement of Offshore-SPH's WCSPH step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA product
 * path: the parity tests, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg load it; the product (offshore-sph_gb300/) never does.
 *
 * It restates the reference's numba code in plain C, in the reference's own
 * traversal and summation order, so that its outputs agree with the reference
 * (run under a pure-Python numba stand-in, see tests/golden/make_golden.py)
 * to round-off.  Compiled with -ffp-contract=off: no FMA contraction, the
 * same IEEE operations the shimmed reference performs.
 *
 * Every function names the reference lines it follows (paths relative to the
 * Offshore-SPH repository root).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define LABEL_FLUID 0 /* src/Common.py:8-12 ParticleType.Fluid */

/* status codes shared with the Python wrapper */
#define OR_OK 0
#define OR_ERR_CELL_OVERFLOW 1 /* flat cell id >= n_cells: out-of-bounds heads[] write in the reference */
#define OR_ERR_ALLOC 2

/* ------------------------------------------------------------------------ */
/* Kernels                                                                   */
/* ------------------------------------------------------------------------ */

/* src/Kernels/CubicSpline.py:12-36 (evaluate), one element */
static double cubic_w(double r, double h) {
  const double fac = 10.0 / (7.0 * M_PI);
  double alpha = fac / (h * h);
  double q = r / h;
  if (q > 2.0) return 0.0;
  if (q > 1.0) return alpha * 0.25 * pow(2.0 - q, 3.0);
  return alpha * (1.0 - 1.5 * pow(q, 2.0) * (1.0 - 0.5 * q));
}

/* src/Kernels/CubicSpline.py:40-70 (gradient), one element */
static double cubic_grad(double x, double r, double h) {
  const double fac = 10.0 / (7.0 * M_PI);
  double alpha = fac / (h * h);
  double q = r / h;
  double grad;
  if ((q > 2.0) || (r < 1e-10)) return 0.0;
  if (q > 1.0) grad = -0.75 * pow(2.0 - q, 2.0);
  else grad = -3.0 * q * (1.0 - 0.75 * q);
  double norm = alpha * grad / (h * r);
  return norm * x;
}

/* src/Kernels/Gaussian.py:16-24 (evaluate) */
static double gauss_w(double r, double h) {
  double alpha = 1.0 / M_PI;
  double q = r / h;
  if (q <= 3.0) {
    double alpha_c = alpha / (h * h);
    return alpha_c * exp(-q * q);
  }
  return 0.0;
}

/* src/Kernels/Gaussian.py:26-35 (derivative) */
static double gauss_dwdq(double r, double h) {
  double alpha = 1.0 / M_PI;
  double q = r / h;
  if (q <= 3.0) {
    double alpha_c = alpha / (h * h);
    return -2.0 * q * alpha_c * exp(-q * q);
  }
  return 0.0;
}

/* src/Kernels/Gaussian.py:37-59 (gradient) */
static double gauss_grad(double x, double r, double h) {
  double alpha = 1.0 / M_PI;
  double tmp = r * h;
  if (tmp > 1e-12) {
    double q = r / h;
    if (q <= 3.0) {
      double alpha_c = alpha / (h * h);
      double dwdq = -2.0 * q * alpha_c * exp(-q * q);
      return dwdq / tmp * x;
    }
    return 0.0;
  }
  return 0.0;
}

/* src/Kernels/Wendland.py:10-34 (evaluate, Wendland C4) */
static double wendland_w(double r, double h) {
  const double fac = 9.0 / (4.0 * M_PI);
  double alpha = fac / (h * h);
  double q = r / h;
  if (q >= 2.0) return 0.0;
  double inner = 1.0 - 0.5 * q;
  return alpha * (pow(inner, 6) * (35.0 / 12.0 * q * q + 3.0 * q + 1.0));
}

/* src/Kernels/Wendland.py:36-64 (gradient) */
static double wendland_grad(double x, double r, double h) {
  const double fac = 9.0 / (4.0 * M_PI);
  double alpha = fac / (h * h);
  double q = r / h;
  if ((q >= 2.0) || (r < 1e-10)) return 0.0;
  double inner = 1.0 - 0.5 * q;
  double grad = pow(inner, 5) * (-14.0 / 3.0) * q * (1 + 2.5 * q);
  double norm = alpha * grad / (h * r);
  return norm * x;
}

/* kernel id: 0 = CubicSpline, 1 = Gaussian, 2 = Wendland */
static double kern_w(int k, double r, double h) {
  return k == 0 ? cubic_w(r, h) : (k == 1 ? gauss_w(r, h) : wendland_w(r, h));
}
static double kern_grad(int k, double x, double r, double h) {
  return k == 0 ? cubic_grad(x, r, h) : (k == 1 ? gauss_grad(x, r, h) : wendland_grad(x, r, h));
}

void or_kernel_eval(int kernel, int64_t n, const double *r, const double *h, double *out) {
  for (int64_t j = 0; j < n; j++) out[j] = kern_w(kernel, r[j], h[j]);
}
void or_kernel_grad(int kernel, int64_t n, const double *x, const double *r, const double *h, double *out) {
  for (int64_t j = 0; j < n; j++) out[j] = kern_grad(kernel, x[j], r[j], h[j]);
}
void or_gauss_deriv(int64_t n, const double *r, const double *h, double *out) {
  for (int64_t j = 0; j < n; j++) out[j] = gauss_dwdq(r[j], h[j]);
}

/* ------------------------------------------------------------------------ */
/* Equations on a "computed" neighbour block (src/Common.py:60-98 layout)    */
/* ------------------------------------------------------------------------ */

/* One neighbour of particle i, the fields of computed_dtype
 * (src/Tools/SolverTools.py:74-104 fills them; c stays 0, line 90). */
typedef struct {
  int8_t label;
  double m, p, rho, h, q, c, r, w, dw_x, dw_y, x, y, vx, vy;
} or_comp;

/* src/Equations/Continuity.py:4-16 */
static double eq_continuity(const or_comp *comp, int64_t J) {
  double arho = 0.0;
  for (int64_t j = 0; j < J; j++) {
    if (comp[j].label != LABEL_FLUID) continue;
    double dot = comp[j].vx * comp[j].dw_x + comp[j].vy * comp[j].dw_y;
    arho += comp[j].m * dot;
  }
  return arho;
}

/* src/Equations/Momentum.py:5-57 (p_* are the fields of the self particle) */
static void eq_momentum(double alpha, double beta, double p_p, double p_rho, double p_h, double p_c,
                        const or_comp *comp, int64_t J, double *ax, double *ay) {
  double slf = p_p / (p_rho * p_rho);
  double a0 = 0.0, a1 = 0.0;
  for (int64_t j = 0; j < J; j++) {
    if (comp[j].label != LABEL_FLUID) continue;
    double othr = comp[j].p / (comp[j].rho * comp[j].rho);
    double dot = comp[j].vx * comp[j].x + comp[j].vy * comp[j].y;
    double PI_ij = 0.0;
    if (dot < 0) {
      double hij = 0.5 * (p_h + comp[j].h);
      double cij = 0.5 * (p_c + comp[j].c);
      double rhoij = 0.5 * (p_rho + comp[j].rho);
      double muij = hij * dot / (comp[j].r * comp[j].r + 0.01 * hij * hij);
      double ppij = muij * (beta * muij - alpha * cij);
      PI_ij = ppij / rhoij;
    }
    double factor = slf + othr + PI_ij;
    a0 += -comp[j].m * factor * comp[j].dw_x;
    a1 += -comp[j].m * factor * comp[j].dw_y;
  }
  *ax = a0;
  *ay = a1;
}

/* src/Equations/BoundaryForce.py:6-42 */
static void eq_boundary(double r0, double D, double p1, double p2, const or_comp *comp, int64_t J,
                        double *fx, double *fy) {
  double f0 = 0.0, f1 = 0.0;
  for (int64_t j = 0; j < J; j++) {
    if ((comp[j].label == LABEL_FLUID) || (comp[j].r > r0)) continue;
    if (comp[j].r > 1e-12) {
      double frac = r0 / comp[j].r;
      double tmp = pow(frac, p1) - pow(frac, p2);
      double fac = D * tmp;
      f0 += fac * comp[j].x / pow(comp[j].r, 2.0);
      f1 += fac * comp[j].y / pow(comp[j].r, 2.0);
    }
  }
  *fx = f0;
  *fy = f1;
}

/* src/Equations/XSPH.py:5-31 */
static void eq_xsph(double epsilon, double p_rho, const or_comp *comp, int64_t J, double *xx, double *xy) {
  double s0 = 0.0, s1 = 0.0;
  for (int64_t j = 0; j < J; j++) {
    double rho_ij = 0.5 * (p_rho + comp[j].rho);
    double fac = -epsilon * comp[j].m * comp[j].w / rho_ij;
    s0 += fac * comp[j].vx;
    s1 += fac * comp[j].vy;
  }
  *xx = s0;
  *xy = s1;
}

/* Flat-array entry points of the four equations, for formula-level parity
 * (the reference's own tests call them on synthetic computed_dtype arrays).
 * Arrays are the computed_dtype fields; out has 1 (continuity) or 2 values. */
static or_comp *pack_comp(int64_t J, const int8_t *label, const double *m, const double *p, const double *rho,
                          const double *h, const double *r, const double *w, const double *dwx,
                          const double *dwy, const double *x, const double *y, const double *vx,
                          const double *vy) {
  or_comp *c = (or_comp *)calloc((size_t)(J > 0 ? J : 1), sizeof(or_comp));
  for (int64_t j = 0; j < J; j++) {
    c[j].label = label[j];
    c[j].m = m[j]; c[j].p = p[j]; c[j].rho = rho[j]; c[j].h = h[j]; c[j].r = r[j];
    c[j].w = w[j]; c[j].dw_x = dwx[j]; c[j].dw_y = dwy[j];
    c[j].x = x[j]; c[j].y = y[j]; c[j].vx = vx[j]; c[j].vy = vy[j];
  }
  return c;
}

void or_equations(int64_t J, const int8_t *label, const double *m, const double *p, const double *rho,
                  const double *h, const double *r, const double *w, const double *dwx, const double *dwy,
                  const double *x, const double *y, const double *vx, const double *vy,
                  const double *self5 /* p, rho, h, c, m of particle i */, const double *par6 /* alpha, beta,
                  r0, D, p1, p2 */, double epsilon, double *out7 /* drho, ax, ay, bx, by, xsx, xsy */) {
  or_comp *c = pack_comp(J, label, m, p, rho, h, r, w, dwx, dwy, x, y, vx, vy);
  out7[0] = eq_continuity(c, J);
  eq_momentum(par6[0], par6[1], self5[0], self5[1], self5[2], self5[3], c, J, &out7[1], &out7[2]);
  eq_boundary(par6[2], par6[3], par6[4], par6[5], c, J, &out7[3], &out7[4]);
  eq_xsph(epsilon, self5[1], c, J, &out7[5], &out7[6]);
  free(c);
}

/* ------------------------------------------------------------------------ */
/* Tait EOS (src/Equations/TaitEOS.py)                                       */
/* ------------------------------------------------------------------------ */

/* TaitEOS.py:6-31 plus WCSPH.compute_pressure's "+ Pb" (WCSPH.py:131-149) */
static double tait(double gamma, double B, double rho0, double rho, int8_t label, double Pb) {
  double v;
  if (label != LABEL_FLUID) v = 0.0;
  else {
    double ratio = pow(rho / rho0, gamma);
    v = (ratio - 1.0) * B;
  }
  return v + Pb;
}

void or_eos(int64_t n, const int8_t *label, const double *rho, double gamma, double B, double rho0, double Pb,
            double *p) {
  for (int64_t i = 0; i < n; i++) p[i] = tait(gamma, B, rho0, rho[i], label[i], Pb);
}

/* TaitEOS.py:46-65 (TaitEOS_height) via WCSPH.initialize (WCSPH.py:82-108) */
void or_tait_height(int64_t n, const double *y, double rho0, double H, double B, double gamma, double *rho) {
  for (int64_t i = 0; i < n; i++) {
    double frac = rho0 * 9.81 * (H - y[i]) / B;
    rho[i] = rho0 * pow(1.0 + frac, 1.0 / gamma);
  }
}

/* ------------------------------------------------------------------------ */
/* Cell linked list (src/Tools/NNLinkedList.py)                              */
/* ------------------------------------------------------------------------ */

typedef struct {
  double scale, xmin, xmax, ymin, ymax, cell_size;
  int64_t ncx, ncy, n_cells, n;
  int64_t *heads, *nexts;
  int status;
} or_nn;

void *or_nn_new(double scale) {
  or_nn *nn = (or_nn *)calloc(1, sizeof(or_nn));
  nn->scale = scale;
  return nn;
}

void or_nn_free(void *p) {
  or_nn *nn = (or_nn *)p;
  if (!nn) return;
  free(nn->heads);
  free(nn->nexts);
  free(nn);
}

/* NNLinkedList._init/_get_cell_size/_get_number_of_cells/_bin
 * (NNLinkedList.py:86-141, 164-208).  Returns OR_ERR_CELL_OVERFLOW when a
 * particle's flat id falls outside heads[] (the reference writes out of
 * bounds there); such particles are not inserted. */
int or_nn_update(void *p, int64_t n, const double *x, const double *y, const double *h) {
  or_nn *nn = (or_nn *)p;
  nn->status = OR_OK;
  nn->n = n;
  double xmin = x[0], xmax = x[0], ymin = y[0], ymax = y[0], hmin = h[0];
  for (int64_t i = 1; i < n; i++) {
    if (x[i] < xmin) xmin = x[i];
    if (x[i] > xmax) xmax = x[i];
    if (y[i] < ymin) ymin = y[i];
    if (y[i] > ymax) ymax = y[i];
    if (h[i] < hmin) hmin = h[i];
  }
  nn->xmin = xmin; nn->xmax = xmax; nn->ymin = ymin; nn->ymax = ymax;
  double cs = hmin * nn->scale;
  if (cs < 1e-6) cs = 1.0;
  nn->cell_size = cs;
  double cs1 = 1. / cs;
  int64_t ncx = (int64_t)ceil(cs1 * (xmax - xmin));
  int64_t ncy = (int64_t)ceil(cs1 * (ymax - ymin));
  if (ncx < 1) ncx = 1;
  if (ncy < 1) ncy = 1;
  nn->ncx = ncx; nn->ncy = ncy; nn->n_cells = ncx * ncy;
  free(nn->heads);
  free(nn->nexts);
  nn->heads = (int64_t *)malloc(sizeof(int64_t) * (size_t)nn->n_cells);
  nn->nexts = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
  if (!nn->heads || !nn->nexts) { nn->status = OR_ERR_ALLOC; return nn->status; }
  for (int64_t c = 0; c < nn->n_cells; c++) nn->heads[c] = -1;
  for (int64_t i = 0; i < n; i++) nn->nexts[i] = -1;
  for (int64_t i = 0; i < n; i++) {
    int64_t cx = (int64_t)floor((x[i] - xmin) / cs);
    int64_t cy = (int64_t)floor((y[i] - ymin) / cs);
    int64_t cid = cx + ncx * cy;
    if (cid < 0 || cid >= nn->n_cells) { nn->status = OR_ERR_CELL_OVERFLOW; continue; }
    nn->nexts[i] = nn->heads[cid];
    nn->heads[cid] = i;
  }
  return nn->status;
}

/* grid of the last update: out_d = {xmin, xmax, ymin, ymax, cell_size},
 * out_i = {ncx, ncy, n_cells} */
void or_nn_grid(void *p, double *out_d, int64_t *out_i) {
  or_nn *nn = (or_nn *)p;
  out_d[0] = nn->xmin; out_d[1] = nn->xmax; out_d[2] = nn->ymin; out_d[3] = nn->ymax; out_d[4] = nn->cell_size;
  out_i[0] = nn->ncx; out_i[1] = nn->ncy; out_i[2] = nn->n_cells;
}

/* heads/nexts of the last update (for tests of the linked-list layout) */
void or_nn_lists(void *p, int64_t *heads, int64_t *nexts) {
  or_nn *nn = (or_nn *)p;
  memcpy(heads, nn->heads, sizeof(int64_t) * (size_t)nn->n_cells);
  memcpy(nexts, nn->nexts, sizeof(int64_t) * (size_t)nn->n);
}

/* NNLinkedList._get_valid_cell_index (NNLinkedList.py:178-198) */
static int64_t valid_cell(const or_nn *nn, int64_t cx, int64_t cy) {
  if (!((nn->ncx > cx && cx > -1) && (nn->ncy > cy && cy > -1))) return -1;
  int64_t ci = cx + nn->ncx * cy;
  if (!(-1 < ci && ci < nn->n_cells)) return -1;
  return ci;
}

/* growable neighbour buffer */
typedef struct {
  int64_t n, cap;
  int64_t *idx;
  double *hij, *q, *r;
} nbuf;

static int nbuf_push(nbuf *b, int64_t j, double hij, double q, double r) {
  if (b->n == b->cap) {
    int64_t nc = b->cap ? 2 * b->cap : 256;
    int64_t *ni = (int64_t *)realloc(b->idx, sizeof(int64_t) * (size_t)nc);
    double *nh = (double *)realloc(b->hij, sizeof(double) * (size_t)nc);
    double *nq = (double *)realloc(b->q, sizeof(double) * (size_t)nc);
    double *nr = (double *)realloc(b->r, sizeof(double) * (size_t)nc);
    if (!ni || !nh || !nq || !nr) return -1;
    b->idx = ni; b->hij = nh; b->q = nq; b->r = nr; b->cap = nc;
  }
  b->idx[b->n] = j; b->hij[b->n] = hij; b->q[b->n] = q; b->r[b->n] = r;
  b->n++;
  return 0;
}

static void nbuf_free(nbuf *b) { free(b->idx); free(b->hij); free(b->q); free(b->r); }

/* NNLinkedList.nearPos (NNLinkedList.py:41-80): shifts -1,0,1 with ix outer
 * and iy inner; each cell's list in head-insert (descending index) order;
 * keep q = r / (0.5 (h + h_j)) <= 3. */
static int near_pos(const or_nn *nn, double x, double y, double h, const double *px, const double *py,
                    const double *ph, nbuf *b) {
  b->n = 0;
  int64_t cx0 = (int64_t)floor((x - nn->xmin) / nn->cell_size);
  int64_t cy0 = (int64_t)floor((y - nn->ymin) / nn->cell_size);
  for (int ix = -1; ix <= 1; ix++) {
    for (int iy = -1; iy <= 1; iy++) {
      int64_t ci = valid_cell(nn, cx0 + ix, cy0 + iy);
      if (ci < 0) continue;
      int64_t nx = nn->heads[ci];
      while (nx != -1) {
        double dx = x - px[nx], dy = y - py[nx];
        double xij2 = dx * dx + dy * dy;
        double r = sqrt(xij2);
        double h_ij = 0.5 * (h + ph[nx]);
        double q_ij = r / h_ij;
        if (q_ij <= 3.0)
          if (nbuf_push(b, nx, h_ij, q_ij, r)) return -1;
        nx = nn->nexts[nx];
      }
    }
  }
  return 0;
}

/* NNLinkedList.nearPos for one point; returns the count (<= cap written) */
int64_t or_nn_near(void *p, double x, double y, double h, const double *px, const double *py, const double *ph,
                   int64_t *idx, double *hij, double *q, double *r, int64_t cap) {
  nbuf b = {0};
  if (near_pos((or_nn *)p, x, y, h, px, py, ph, &b)) { nbuf_free(&b); return -1; }
  for (int64_t k = 0; k < b.n && k < cap; k++) {
    idx[k] = b.idx[k]; hij[k] = b.hij[k]; q[k] = b.q[k]; r[k] = b.r[k];
  }
  int64_t n = b.n;
  nbuf_free(&b);
  return n;
}

/* NNLinkedList.near(i) for every particle with label_filter < 0 or
 * label == label_filter.  CSR output: offsets[n+1]; idx[] in reference
 * order.  Pass idx = NULL to get only offsets (the total is offsets[n]). */
int or_nn_all(void *p, int64_t n, const double *x, const double *y, const double *h, const int8_t *label,
              int label_filter, int64_t *offsets, int64_t *idx) {
  or_nn *nn = (or_nn *)p;
  nbuf b = {0};
  offsets[0] = 0;
  for (int64_t i = 0; i < n; i++) {
    int64_t cnt = 0;
    if (label_filter < 0 || label[i] == label_filter) {
      if (near_pos(nn, x[i], y[i], h[i], x, y, h, &b)) { nbuf_free(&b); return OR_ERR_ALLOC; }
      cnt = b.n;
      if (idx)
        for (int64_t k = 0; k < b.n; k++) idx[offsets[i] + k] = b.idx[k];
    }
    offsets[i + 1] = offsets[i] + cnt;
  }
  nbuf_free(&b);
  return OR_OK;
}

static int cmp_i64(const void *a, const void *b) {
  const int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

/* or_nn_all over nthreads OpenMP threads (the same lists; each particle's
 * query is independent).  sorted != 0 writes every list in ascending index
 * order instead of the reference's traversal order, which makes set
 * comparisons of large cases a plain array comparison. */
int or_nn_all_mt(void *p, int64_t n, const double *x, const double *y, const double *h, const int8_t *label,
                 int label_filter, int64_t *offsets, int64_t *idx, int nthreads, int sorted) {
  or_nn *nn = (or_nn *)p;
  int err = 0;
  if (nthreads < 1) nthreads = 1;
  if (!idx) {
#pragma omp parallel num_threads(nthreads) reduction(| : err)
    {
      nbuf b = {0};
#pragma omp for schedule(dynamic, 256)
      for (int64_t i = 0; i < n; i++) {
        int64_t cnt = 0;
        if (label_filter < 0 || label[i] == label_filter) {
          if (near_pos(nn, x[i], y[i], h[i], x, y, h, &b)) err |= 1;
          cnt = b.n;
        }
        offsets[i + 1] = cnt;
      }
      nbuf_free(&b);
    }
    offsets[0] = 0;
    for (int64_t i = 0; i < n; i++) offsets[i + 1] += offsets[i];
    return err ? OR_ERR_ALLOC : OR_OK;
  }
#pragma omp parallel num_threads(nthreads) reduction(| : err)
  {
    nbuf b = {0};
#pragma omp for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; i++) {
      if (!(label_filter < 0 || label[i] == label_filter)) continue;
      if (near_pos(nn, x[i], y[i], h[i], x, y, h, &b)) { err |= 1; continue; }
      int64_t *dst = idx + offsets[i];
      const int64_t cnt = offsets[i + 1] - offsets[i];
      if (b.n != cnt) { err |= 2; continue; }
      for (int64_t k = 0; k < b.n; k++) dst[k] = b.idx[k];
      if (sorted) qsort(dst, (size_t)cnt, sizeof(int64_t), cmp_i64);
    }
    nbuf_free(&b);
  }
  return err ? OR_ERR_ALLOC : OR_OK;
}

/* ------------------------------------------------------------------------ */
/* The derivative loop (src/Tools/SolverTools.py:120-175)                    */
/* ------------------------------------------------------------------------ */

/* WCSPH constants and switches (src/Methods/WCSPH.py:35-79).  sum_order is
 * not a reference setting: 0 sums each particle's neighbours in the
 * reference's order; 1 sums them in reverse, a control run whose only
 * difference is round-off, used to size how fast round-off differences grow
 * along a trajectory. */
typedef struct {
  double gamma, B, rho0, Pb, co, alpha, beta, epsilon, r0, D, p1, p2;
  int32_t use_xsph, use_summation_density, kernel, sum_order;
} or_wcsph;

/* reverse the order of a neighbour buffer (the sum_order = 1 control) */
static void nbuf_reverse(nbuf *b) {
  for (int64_t a = 0, z = b->n - 1; a < z; a++, z--) {
    int64_t ti = b->idx[a]; b->idx[a] = b->idx[z]; b->idx[z] = ti;
    double t = b->hij[a]; b->hij[a] = b->hij[z]; b->hij[z] = t;
    t = b->q[a]; b->q[a] = b->q[z]; b->q[z] = t;
    t = b->r[a]; b->r[a] = b->r[z]; b->r[z] = t;
  }
}

/* SOA particle view; the arrays are the particle_dtype fields
 * (src/Common.py:26-57) of the active particles, in their order. */
typedef struct {
  int64_t n;
  int8_t *label;
  double *m, *rho, *p, *c, *drho, *h, *x, *y, *vx, *vy, *ax, *ay, *xsphx, *xsphy, *x0, *y0, *vx0, *vy0, *rho0;
} or_particles;

/* One particle i of _loop's regular pass (SolverTools.py:143-173):
 * computeProps (8-44, 74-104), Continuity, Momentum (+gravity, WCSPH.py:151-169),
 * BoundaryForce, XSPH (WCSPH.py:171-189). */
static int loop_one(const or_wcsph *w, const or_nn *nn, or_particles *P, int64_t i, nbuf *b, or_comp **cbuf,
                    int64_t *ccap) {
  if (near_pos(nn, P->x[i], P->y[i], P->h[i], P->x, P->y, P->h, b)) return -1;
  if (w->sum_order == 1) nbuf_reverse(b);
  int64_t J = b->n;
  if (J == 0) return 0; /* keep the previous values (SolverTools.py:150-153) */
  if (J > *ccap) {
    or_comp *nc = (or_comp *)realloc(*cbuf, sizeof(or_comp) * (size_t)J);
    if (!nc) return -1;
    *cbuf = nc;
    *ccap = J;
  }
  or_comp *comp = *cbuf;
  for (int64_t k = 0; k < J; k++) {
    int64_t g = b->idx[k];
    comp[k].label = P->label[g];
    comp[k].p = P->p[g];
    comp[k].m = P->m[g];
    comp[k].c = 0.0; /* SolverTools.py:90 is commented out */
    comp[k].rho = P->rho[g];
    comp[k].h = b->hij[k];
    comp[k].q = b->q[k];
    comp[k].r = b->r[k];
    comp[k].x = P->x[i] - P->x[g];
    comp[k].y = P->y[i] - P->y[g];
    comp[k].vx = P->vx[i] - P->vx[g];
    comp[k].vy = P->vy[i] - P->vy[g];
  }
  for (int64_t k = 0; k < J; k++) {
    comp[k].w = kern_w(w->kernel, comp[k].r, comp[k].h);
    comp[k].dw_x = kern_grad(w->kernel, comp[k].x, comp[k].r, comp[k].h);
    comp[k].dw_y = kern_grad(w->kernel, comp[k].y, comp[k].r, comp[k].h);
  }
  /* WCSPH.compute_density_change (WCSPH.py:191-203) */
  P->drho[i] = w->use_summation_density ? 0.0 : eq_continuity(comp, J);
  double a_x, a_y, b_x, b_y;
  eq_momentum(w->alpha, w->beta, P->p[i], P->rho[i], P->h[i], P->c[i], comp, J, &a_x, &a_y);
  a_y = a_y - 9.81; /* WCSPH.py:169 */
  eq_boundary(w->r0, w->D, w->p1, w->p2, comp, J, &b_x, &b_y);
  P->ax[i] = a_x + b_x;
  P->ay[i] = a_y + b_y;
  if (w->use_xsph) {
    double sx, sy;
    eq_xsph(w->epsilon, P->rho[i], comp, J, &sx, &sy);
    P->xsphx[i] = P->vx[i] + sx;
    P->xsphy[i] = P->vy[i] + sy;
  } else {
    P->xsphx[i] = 0.0;
    P->xsphy[i] = 0.0;
  }
  return 0;
}

/* SolverTools._loop (SolverTools.py:120-175) on an nn built over the same
 * particles.  nthreads > 1 splits the per-particle passes with OpenMP; each
 * particle only writes its own fields, as in the reference's prange loops. */
int or_loop(const or_wcsph *w, void *nnp, or_particles *P, int nthreads) {
  or_nn *nn = (or_nn *)nnp;
  int64_t n = P->n;
  /* p and c for all particles (SolverTools.py:122-127) */
  for (int64_t i = 0; i < n; i++) {
    P->p[i] = tait(w->gamma, w->B, w->rho0, P->rho[i], P->label[i], w->Pb);
    P->c[i] = w->co;
  }
  int err = 0;
  if (nthreads < 1) nthreads = 1;
  if (w->use_summation_density) {
    /* SolverTools.py:129-140: rho_i = sum over fluid j of m_j W(r, h_ij) */
#pragma omp parallel num_threads(nthreads) reduction(| : err)
    {
      nbuf b = {0};
#pragma omp for schedule(dynamic, 64)
      for (int64_t i = 0; i < n; i++) {
        if (P->label[i] != LABEL_FLUID) continue;
        if (near_pos(nn, P->x[i], P->y[i], P->h[i], P->x, P->y, P->h, &b)) { err |= 1; continue; }
        if (w->sum_order == 1) nbuf_reverse(&b);
        double rho = 0.0;
        for (int64_t k = 0; k < b.n; k++) {
          int64_t g = b.idx[k];
          double wv = kern_w(w->kernel, b.r[k], b.hij[k]);
          if (P->label[g] != LABEL_FLUID) continue; /* SummationDensity.py:5-13 */
          rho += P->m[g] * wv;
        }
        P->rho[i] = rho;
      }
      nbuf_free(&b);
    }
  }
#pragma omp parallel num_threads(nthreads) reduction(| : err)
  {
    nbuf b = {0};
    or_comp *cbuf = NULL;
    int64_t ccap = 0;
#pragma omp for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; i++) {
      if (P->label[i] != LABEL_FLUID) continue;
      if (loop_one(w, nn, P, i, &b, &cbuf, &ccap)) err |= 1;
    }
    nbuf_free(&b);
    free(cbuf);
  }
  return err ? OR_ERR_ALLOC : OR_OK;
}

/* The regular pass of _loop (SolverTools.py:143-173) for the fluid particles
 * in [i0, i1) only, on one thread, after the EOS pass over all particles: a
 * bounded sample of an evaluation, for timing the reference's loop at sizes
 * where a whole single-threaded evaluation takes minutes. */
int or_loop_range(const or_wcsph *w, void *nnp, or_particles *P, int64_t i0, int64_t i1) {
  or_nn *nn = (or_nn *)nnp;
  for (int64_t i = 0; i < P->n; i++) {
    P->p[i] = tait(w->gamma, w->B, w->rho0, P->rho[i], P->label[i], w->Pb);
    P->c[i] = w->co;
  }
  nbuf b = {0};
  or_comp *cbuf = NULL;
  int64_t ccap = 0;
  int err = 0;
  if (i0 < 0) i0 = 0;
  if (i1 > P->n) i1 = P->n;
  for (int64_t i = i0; i < i1 && !err; i++) {
    if (P->label[i] != LABEL_FLUID) continue;
    if (loop_one(w, nn, P, i, &b, &cbuf, &ccap)) err = 1;
  }
  nbuf_free(&b);
  free(cbuf);
  return err ? OR_ERR_ALLOC : OR_OK;
}

/* SolverTools.computeH (SolverTools.py:106-118): h = sigma (m/rho)^(1/2) */
static double compute_h(double sigma, double m, double rho) {
  if (rho > 1e-12) return sigma * pow(m / rho, 0.5);
  return 0.0;
}

/* Solver._compute (src/Solver.py:232-256): nn.update over the active
 * particles, then h for fluid (fixed, or computeH(1.3, ...)), then _loop.
 * The "reset accelerations" lines 249-251 assign into a mask copy and have
 * no effect, so they are not restated. */
int or_compute(const or_wcsph *w, void *nnp, or_particles *P, double h_fixed, int nthreads) {
  int st = or_nn_update(nnp, P->n, P->x, P->y, P->h);
  if (st) return st;
  for (int64_t i = 0; i < P->n; i++) {
    if (P->label[i] != LABEL_FLUID) continue;
    P->h[i] = h_fixed > 0 ? h_fixed : compute_h(1.3, P->m[i], P->rho[i]);
  }
  return or_loop(w, nnp, P, nthreads);
}

/* ------------------------------------------------------------------------ */
/* Time step (src/Equations/TimeStep.py:7-91)                                */
/* ------------------------------------------------------------------------ */

/* TimeStep.compute over the fluid particles; out = {dt, dt_courant, dt_force} */
void or_timestep(int64_t n, const int8_t *label, const double *h, const double *c, const double *ax,
                 const double *ay, double gamma_c, double gamma_f, double *out) {
  double min_h = INFINITY, max_c = -INFINITY, max_a2 = -INFINITY;
  int64_t cnt = 0;
  for (int64_t j = 0; j < n; j++) {
    if (label[j] != LABEL_FLUID) continue;
    double a2 = ax[j] * ax[j] + ay[j] * ay[j];
    if (cnt == 0 || h[j] < min_h) min_h = h[j];
    if (cnt == 0 || c[j] > max_c) max_c = c[j];
    if (cnt == 0 || a2 > max_a2) max_a2 = a2;
    cnt++;
  }
  double dc = gamma_c * min_h / max_c;                           /* TimeStep.py:39-41 */
  double df = max_a2 < 1e-12 ? 1e10 : gamma_f * sqrt(min_h / max_a2); /* TimeStep.py:43-48 */
  out[0] = dc < df ? dc : df;
  out[1] = dc;
  out[2] = df;
}

/* ------------------------------------------------------------------------ */
/* Integrators                                                               */
/* ------------------------------------------------------------------------ */

/* PEC.predict (src/Integrators/PEC.py:32-59), over the particles passed
 * (the Solver passes the fluid ones, Solver.py:380) */
void or_pec_predict(or_particles *P, const uint8_t *mask, double dt, double damping, int use_xsph, int strict) {
  for (int64_t j = 0; j < P->n; j++) {
    if (mask && !mask[j]) continue;
    P->x0[j] = P->x[j];
    P->y0[j] = P->y[j];
    P->vx0[j] = P->vx[j];
    P->vy0[j] = P->vy[j];
    if (use_xsph && P->label[j] == LABEL_FLUID) {
      P->x[j] = P->x[j] + 0.5 * dt * P->xsphx[j];
      P->y[j] = P->y[j] + 0.5 * dt * P->xsphy[j];
    } else {
      P->x[j] = P->x[j] + 0.5 * dt * P->vx[j];
      P->y[j] = P->y[j] + 0.5 * dt * P->vy[j];
    }
    P->vx[j] = (P->vx[j] + 0.5 * dt * P->ax[j]) / (1 + 0.5 * damping);
    P->vy[j] = (P->vy[j] + 0.5 * dt * P->ay[j]) / (1 + 0.5 * damping);
    P->rho0[j] = P->rho[j];
    P->rho[j] = P->rho[j] + 0.5 * dt * P->drho[j];
    if (strict && P->rho[j] < 0.0) P->rho[j] = 0.0;
  }
}

/* PEC.correct (src/Integrators/PEC.py:61-89) */
void or_pec_correct(or_particles *P, const uint8_t *mask, double dt, double damping, int use_xsph, int strict) {
  for (int64_t j = 0; j < P->n; j++) {
    if (mask && !mask[j]) continue;
    double mid_x, mid_y;
    if (use_xsph && P->label[j] == LABEL_FLUID) {
      mid_x = P->x0[j] + 0.5 * dt * P->xsphx[j];
      mid_y = P->y0[j] + 0.5 * dt * P->xsphy[j];
    } else {
      mid_x = P->x0[j] + 0.5 * dt * P->vx[j];
      mid_y = P->y0[j] + 0.5 * dt * P->vy[j];
    }
    double mid_vx = (P->vx0[j] + 0.5 * dt * P->ax[j]) / (1 + 0.5 * damping);
    double mid_vy = (P->vy0[j] + 0.5 * dt * P->ay[j]) / (1 + 0.5 * damping);
    P->x[j] = 2 * mid_x - P->x0[j];
    P->y[j] = 2 * mid_y - P->y0[j];
    P->vx[j] = 2 * mid_vx - P->vx0[j];
    P->vy[j] = 2 * mid_vy - P->vy0[j];
    double mid_rho = P->rho0[j] + 0.5 * dt * P->drho[j];
    P->rho[j] = 2 * mid_rho - P->rho0[j];
    if (strict && P->rho[j] < 0.0) P->rho[j] = 0.0;
  }
}

/* Euler.correct (src/Integrators/Euler.py:17-27); Euler.predict is a no-op */
void or_euler_correct(or_particles *P, const uint8_t *mask, double dt) {
  for (int64_t j = 0; j < P->n; j++) {
    if (mask && !mask[j]) continue;
    P->x[j] = P->x[j] + dt * P->vx[j] + 0.5 * dt * dt * P->ax[j];
    P->y[j] = P->y[j] + dt * P->vy[j] + 0.5 * dt * dt * P->ay[j];
    P->vx[j] = P->vx[j] + dt * P->ax[j];
    P->vy[j] = P->vy[j] + dt * P->ay[j];
    P->rho[j] = P->rho[j] + dt * P->drho[j];
  }
}

/* Verlet.predict (src/Integrators/Verlet.py:28-35): drift by half a step */
void or_verlet_predict(or_particles *P, const uint8_t *mask, double dt) {
  for (int64_t j = 0; j < P->n; j++) {
    if (mask && !mask[j]) continue;
    P->x[j] += 0.5 * dt * P->vx[j];
    P->y[j] += 0.5 * dt * P->vy[j];
  }
}

/* Verlet.correct (src/Integrators/Verlet.py:37-53): kick, then the second
 * half drift with the new velocity (or XSPH); the density is not integrated */
void or_verlet_correct(or_particles *P, const uint8_t *mask, double dt, int use_xsph) {
  for (int64_t j = 0; j < P->n; j++) {
    if (mask && !mask[j]) continue;
    P->vx[j] += dt * P->ax[j];
    P->vy[j] += dt * P->ay[j];
    if (use_xsph) {
      P->x[j] += 0.5 * dt * P->xsphx[j];
      P->y[j] += 0.5 * dt * P->xsphy[j];
    } else {
      P->x[j] += 0.5 * dt * P->vx[j];
      P->y[j] += 0.5 * dt * P->vy[j];
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Bare time steps (the body of Solver.run, src/Solver.py:366-410)           */
/* ------------------------------------------------------------------------ */

/* Step options: integrator 0 = PEC, 1 = Euler, 2 = Verlet.  dt_fixed > 0 is the
 * Solver's timeStep (Solver.py:370-372), else TimeStep with gamma_c/gamma_f
 * (Solver.py:210-230).  dt_out (3*nsteps: dt, dt_c, dt_f) may be NULL. */
typedef struct {
  double h_fixed, dt_fixed, gamma_c, gamma_f, damping;
  int32_t integrator, pec_use_xsph, pec_strict, nthreads;
} or_stepopt;

int or_run(const or_wcsph *w, void *nnp, or_particles *P, const or_stepopt *o, int64_t nsteps, double *dt_out) {
  int64_t n = P->n;
  uint8_t *fmask = (uint8_t *)malloc((size_t)(n > 0 ? n : 1));
  if (!fmask) return OR_ERR_ALLOC;
  for (int64_t i = 0; i < n; i++) fmask[i] = P->label[i] == LABEL_FLUID;
  for (int64_t s = 0; s < nsteps; s++) {
    double dts[3];
    if (o->dt_fixed > 0) {
      dts[0] = o->dt_fixed; dts[1] = 0.0; dts[2] = 0.0;
    } else {
      or_timestep(n, P->label, P->h, P->c, P->ax, P->ay, o->gamma_c, o->gamma_f, dts);
    }
    if (dt_out) { dt_out[3 * s] = dts[0]; dt_out[3 * s + 1] = dts[1]; dt_out[3 * s + 2] = dts[2]; }
    double dt = dts[0];
    if (o->integrator == 0) or_pec_predict(P, fmask, dt, o->damping, o->pec_use_xsph, o->pec_strict);
    else if (o->integrator == 2) or_verlet_predict(P, fmask, dt);
    int st = or_compute(w, nnp, P, o->h_fixed, o->nthreads);
    if (st) { free(fmask); return st; }
    if (o->integrator == 0) or_pec_correct(P, fmask, dt, o->damping, o->pec_use_xsph, o->pec_strict);
    else if (o->integrator == 2) or_verlet_correct(P, fmask, dt, o->pec_use_xsph);
    else or_euler_correct(P, fmask, dt);
  }
  free(fmask);
  return OR_OK;
}

int or_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

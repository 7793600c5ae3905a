/*
 * sph_gb300.h -- C ABI of the GB300-native WCSPH step.
 *
 * A drop-in for the hot path of Offshore-SPH's Solver: the cell linked-list
 * neighbour search, the Tait EOS, continuity, momentum with artificial
 * viscosity, the Lennard-Jones boundary force, optional XSPH and summation
 * density, the Courant/force time step and the PEC / Euler integrators.
 * Every entry point names the reference routine it replaces (paths relative
 * to the Offshore-SPH repository root).
 *
 * Conventions
 *  - All particle arrays are DEVICE pointers, structure-of-arrays, one entry
 *    per active particle, in the caller's order (the order of
 *    particleArray[indexes] in the reference).  Results are written back in
 *    that order.
 *  - Nothing here allocates or frees caller memory.  Scratch lives in a
 *    caller-allocated device workspace sized by sph_workspace_size() and
 *    prepared once by sph_workspace_init().
 *  - Every call is asynchronous on the given stream (a cudaStream_t; NULL is
 *    the legacy default stream) and does no host synchronisation, so a
 *    sequence of calls may be captured into a CUDA graph.  The exceptions are
 *    sph_get_status() and sph_workspace_init(), which synchronise.
 *  - Return value: SPH_OK or an SPH_ERR_* code for errors detected on the host
 *    (bad arguments, launch failures).  Conditions detected on the device set
 *    bits in a sticky status word in the workspace, read and cleared with
 *    sph_get_status().
 *  - Not re-entrant per workspace: calls that share a workspace must be
 *    ordered on one stream.  Distinct workspaces are independent.
 */
#ifndef SPH_GB300_H
#define SPH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_ABI_VERSION 1

typedef struct CUstream_st *sph_stream_t; /* identical to cudaStream_t */

/* particle labels (src/Common.py:8-12 ParticleType) */
enum { SPH_FLUID = 0, SPH_BOUNDARY = 1, SPH_TEMP_BOUNDARY = 2, SPH_COUPLED = 3 };

/* smoothing kernels (src/Kernels/CubicSpline.py, src/Kernels/Gaussian.py,
 * src/Kernels/Wendland.py) */
enum { SPH_KERNEL_CUBIC = 0, SPH_KERNEL_GAUSSIAN = 1, SPH_KERNEL_WENDLAND = 2 };

/* arithmetic of the pair interaction: FP64 throughout, or FP32 pair
 * arithmetic over FP64 state (positions, velocities, densities, dt and the
 * integrator stay FP64) */
enum { SPH_PREC_FP64 = 0, SPH_PREC_MIXED = 1 };

/* integrators (src/Integrators/PEC.py, src/Integrators/Euler.py,
 * src/Integrators/Verlet.py) */
enum { SPH_INTEGRATOR_PEC = 0, SPH_INTEGRATOR_EULER = 1, SPH_INTEGRATOR_VERLET = 2 };

/* host-side return codes */
enum {
  SPH_OK = 0,
  SPH_ERR_INVALID_ARGUMENT = 1,
  SPH_ERR_WORKSPACE_TOO_SMALL = 2,
  SPH_ERR_CUDA = 3,
  SPH_ERR_NOT_INITIALISED = 4,
  SPH_ERR_STATIC_LIMIT = 5 /* more particles than sph_compute_static's scratch holds */
};

/* device status bits (sticky, see sph_get_status) */
enum {
  /* a particle's flat cell id is >= n_cells of the reference grid: the
   * reference writes past heads[] there (src/Tools/NNLinkedList.py:129-141).
   * Such particles are left out of every neighbour list. */
  SPH_STATUS_CELL_OVERFLOW = 1u << 0,
  /* the traversal grid was coarsened to fit the workspace's cell capacity
   * (results stay exact, the search does more work) */
  SPH_STATUS_GRID_COARSENED = 1u << 1,
  /* a position, h or reduction input was not finite */
  SPH_STATUS_NONFINITE = 1u << 2,
  /* the reference grid has more than 2^30 cells per axis */
  SPH_STATUS_GRID_TOO_LARGE = 1u << 3,
  /* no fluid particle to take the time step from */
  SPH_STATUS_NO_FLUID = 1u << 4,
  /* TimeStep's dt fell below 1e-6 (the reference records it, src/Solver.py:219-224) */
  SPH_STATUS_SMALL_DT = 1u << 5,
  /* a bounded wait on asynchronous shared-memory copies ran out (the pair
   * kernels stage with per-thread cp.async copies, which each thread waits
   * for with cp.async.wait_all, and do not set it; the bit is kept so that
   * the values of the others stay fixed) */
  SPH_STATUS_STAGING_TIMEOUT = 1u << 6
};

/* WCSPH method constants, the attributes of src/Methods/WCSPH.py:33-79.
 * Fill them from the reference's formulas (co = 10 sqrt(2 g H),
 * B = co^2 rho0 / gamma, D = 5 g H) or set them directly, as the reference
 * allows (its jitclass attributes are mutable). */
typedef struct sph_wcsph {
  double rho0, gamma, co, B, Pb; /* Tait EOS (src/Equations/TaitEOS.py) */
  double alpha, beta;            /* artificial viscosity (src/Equations/Momentum.py) */
  double epsilon;                /* XSPH (src/Equations/XSPH.py) */
  double r0, D, p1, p2;          /* Lennard-Jones boundary (src/Equations/BoundaryForce.py) */
  double height;                 /* water column height H (TaitEOS_height) */
  int32_t use_xsph;              /* WCSPH.useXSPH */
  int32_t use_summation_density; /* WCSPH.useSummationDensity */
} sph_wcsph_t;

/* Solver / integrator / kernel / neighbour-finder settings */
typedef struct sph_config {
  int32_t kernel;       /* SPH_KERNEL_* (the Solver's kernel object) */
  int32_t precision;    /* SPH_PREC_* */
  int32_t integrator;   /* SPH_INTEGRATOR_* */
  int32_t pec_use_xsph; /* PEC(useXSPH=...) (src/Integrators/PEC.py:13) */
  int32_t pec_strict;   /* PEC(strict=...) */
  int32_t pad0;
  double nn_scale;      /* NNLinkedList(scale) -- the Solver uses 2.0 (src/Solver.py:109) */
  double h_fixed;       /* Solver(h=...): > 0 fixed h for fluid; <= 0: computeH(1.3, m, rho) */
  double cfl_c, cfl_f;  /* TimeStep.compute gamma_c, gamma_f (src/Solver.py:215 uses 0.25, 0.25) */
  double damping;       /* Solver damping factor passed to predict/correct */
  double dt_fixed;      /* Solver(timeStep=...): > 0 fixed dt, else TimeStep */
} sph_config_t;

/* The active particles as device structure-of-arrays: the fields of
 * particle_dtype (src/Common.py:26-57), 'deleted' excluded. */
typedef struct sph_particles {
  int64_t n;
  int8_t *label;
  double *m, *rho, *p, *c, *drho, *h, *x, *y, *vx, *vy, *ax, *ay, *xsphx, *xsphy;
  double *x0, *y0, *vx0, *vy0, *rho0;
} sph_particles_t;

/* A caller-allocated device workspace: ptr/bytes is device memory of at least
 * sph_workspace_size(n_cap, max_cells) bytes; n_cap bounds the particle count
 * of every call that uses it, max_cells the number of search cells.  The
 * workspace holds the cell table, the sort permutation, the sorted pair
 * records and the reduction and status words. */
typedef struct sph_workspace {
  void *ptr;
  size_t bytes;
  int64_t n_cap;
  int64_t max_cells;
} sph_workspace_t;

/* Library ABI version (SPH_ABI_VERSION of the build). */
int sph_abi_version(void);

/* Bytes of device workspace for up to n particles and max_cells search cells
 * (max_cells <= 0 picks the default, sph_default_max_cells(n)), including
 * the sorted state copy that sph_run steps on (19 doubles, a label and an
 * index per particle); a smaller workspace that holds everything else still
 * works, sph_run then steps on the caller's arrays. */
int sph_workspace_size(int64_t n, int64_t max_cells, size_t *bytes);
int64_t sph_default_max_cells(int64_t n);

/* Prepare a workspace (fills in ws->max_cells when it is <= 0): clears the
 * counters and the status word.  Synchronises the stream. */
int sph_workspace_init(sph_workspace_t *ws, sph_stream_t stream);

/* Read and clear the sticky device status word (SPH_STATUS_* bits).
 * Synchronises the stream. */
int sph_get_status(const sph_workspace_t *ws, uint32_t *status, sph_stream_t stream);

/* Human-readable name of a return code (SPH_OK, SPH_ERR_*). */
const char *sph_status_string(int code);

/* Human-readable name of a single device status bit (SPH_STATUS_*). */
const char *sph_status_bit_string(uint32_t bit);

/* Self-test of the bulk-copy primitives (a bulk asynchronous copy completing
 * on an mbarrier, and the bounded wait on it that gives up with a status
 * instead of hanging): src64 is 64 bytes of
 * device memory, 16-byte aligned; result (device, 2 x uint32) receives
 * {1 if the copy landed intact, 2 if a wait on bytes that never arrive gave
 * up after its bound}.  No host synchronisation. */
int sph_selftest_staging(const void *src64, uint32_t *result, sph_stream_t stream);

/* WCSPH.initialize + the fluid part of Solver.setup
 * (src/Methods/WCSPH.py:82-108, src/Solver.py:184-196): for fluid particles
 * set h (fixed or computeH), rho = TaitEOS_height(y), p = TaitEOS(rho) + Pb,
 * c = co. */
int sph_initialize(sph_particles_t *pa, const sph_wcsph_t *w, const sph_config_t *cfg, sph_stream_t stream);

/* WCSPH.compute_pressure and compute_speed_of_sound for every particle
 * (src/Methods/WCSPH.py:110-149, src/Equations/TaitEOS.py:6-31). */
int sph_eos(sph_particles_t *pa, const sph_wcsph_t *w, sph_stream_t stream);

/* Kernel.evaluate / Kernel.gradient as elementwise device maps over n values
 * (src/Kernels/CubicSpline.py:10-70, src/Kernels/Gaussian.py:16-59):
 * out[j] = W(r[j], h[j]), or the gradient component x[j] dW/dr / r for the
 * coordinate difference x[j]; sph_gauss_deriv is Gaussian.derivative
 * (dW/dq).  Arrays are device doubles. */
int sph_kernel_eval(int kernel, int64_t n, const double *r, const double *h, double *out, sph_stream_t stream);
int sph_kernel_grad(int kernel, int64_t n, const double *x, const double *r, const double *h, double *out,
                    sph_stream_t stream);
int sph_gauss_deriv(int64_t n, const double *r, const double *h, double *out, sph_stream_t stream);

/* NNLinkedList.update (src/Tools/NNLinkedList.py:37-39, 86-141): bins the
 * particles into the reference's cell grid (origin = min x, y; cell size =
 * scale * min h, or 1.0 below 1e-6) and builds the sorted cell table in the
 * workspace. */
int sph_nn_update(const sph_particles_t *pa, const sph_config_t *cfg, const sph_workspace_t *ws, sph_stream_t stream);

/* NNLinkedList.near(i) for every particle i (src/Tools/NNLinkedList.py:41-84)
 * on the table of the last sph_nn_update: counts[i] = number of neighbours
 * (device int64[n]).  Then, with offsets = exclusive prefix sum of counts
 * (device int64[n+1]), sph_nn_export writes the neighbour indices of i into
 * idx[offsets[i] .. offsets[i+1]).  The lists are those of the reference,
 * bit for bit and in its order: the 3x3 stencil cells with the x shift outer
 * and the y shift inner, descending index inside a cell (the head-insert
 * order of its linked lists, NNLinkedList.py:50-78, 129-141), including its
 * truncated stencil and its aliasing of x-overflow cells. */
int sph_nn_count(const sph_particles_t *pa, const sph_config_t *cfg, const sph_workspace_t *ws, int64_t *counts,
                 sph_stream_t stream);
int sph_nn_export(const sph_particles_t *pa, const sph_config_t *cfg, const sph_workspace_t *ws, const int64_t *offsets,
                  int64_t *idx, sph_stream_t stream);

/* NNLinkedList.nearPos (src/Tools/NNLinkedList.py:41-84) for np points
 * (px, py, ph device arrays) on the table of the last build in ws (as the
 * reference, distances use pa's current positions): the same count /
 * offsets / export protocol as sph_nn_count / sph_nn_export, each list in
 * the reference's order with its h_ij, q and r (device arrays, offsets[np]
 * entries). */
int sph_nn_probe_count(const sph_particles_t *pa, const sph_workspace_t *ws, int64_t np, const double *px,
                       const double *py, const double *ph, int64_t *counts, sph_stream_t stream);
int sph_nn_probe_export(const sph_particles_t *pa, const sph_workspace_t *ws, int64_t np, const double *px,
                        const double *py, const double *ph, const int64_t *offsets, int64_t *idx, double *hij,
                        double *q, double *r, sph_stream_t stream);

/* Density and pressure at np points, the interpolation the reference's
 * ice-coupling example builds from nearPos (examples/IceBreak.py:253-285):
 * over the nearPos set of (px, py, h_search), W = kernel(r, h_kernel), the
 * Shepard normalisation (src/Equations/Shepard.py) and summation density
 * (src/Equations/SummationDensity.py) give rho = sum_fluid m W /
 * sum_{fluid, rho >= 1e-3} W m / rho, and p = B ((rho / rho0)^gamma - 1).
 * Uses the table of the last build in ws. */
int sph_probe_density(const sph_particles_t *pa, const sph_wcsph_t *w, int kernel, const sph_workspace_t *ws,
                      int64_t np, const double *px, const double *py, const double *h_search, const double *h_kernel,
                      double *rho, double *p, sph_stream_t stream);

/* One particle's block of neighbours in the reference's computed_dtype layout
 * (src/Common.py:60-98) as device structure-of-arrays of n entries: label,
 * m, p, rho, h (the pair's averaged h), c, r, the kernel value w and
 * gradient dw_x, dw_y, and the differences x, y, vx, vy (particle minus
 * neighbour), as _assignProps fills it (src/Tools/SolverTools.py:74-104). */
typedef struct sph_block {
  int64_t n;
  const int8_t *label;
  const double *m, *p, *rho, *h, *c, *r, *w, *dw_x, *dw_y, *x, *y, *vx, *vy;
} sph_block_t;

/* The per-neighbour-block equations of one particle, the work of the
 * reference's plugin methods WCSPH.compute_density_change,
 * compute_acceleration and compute_velocity (src/Methods/WCSPH.py:151-203)
 * and of BoundaryForce (src/Equations/BoundaryForce.py:6-42), which _loop
 * calls per particle (src/Tools/SolverTools.py:143-173).  self4 (host) =
 * {p, rho, h, c} of the particle; out (device, 7 doubles) receives the sums
 * {Continuity, Momentum x, Momentum y (no gravity), BoundaryForce x, y,
 * XSPH x, y} (src/Equations/Continuity.py:4-16, Momentum.py:5-57,
 * XSPH.py:5-31), each in the block's order as the reference sums them.  The
 * methods' switches (summation density, XSPH, the -9.81 of gravity) are the
 * caller's.  Not a hot path: the step runs these equations fused in its
 * pair kernels. */
int sph_block_equations(const sph_block_t *blk, const double *self4, const sph_wcsph_t *w, double *out,
                        sph_stream_t stream);

/* Solver._compute (src/Solver.py:232-256) = NNLinkedList.update, the h reset
 * (fixed or computeH, src/Tools/SolverTools.py:106-118) and the derivative
 * loop _loop (src/Tools/SolverTools.py:120-175) as one fused pair kernel:
 * writes p, c (all particles), h (fluid) and, for fluid particles with at
 * least one neighbour, drho, ax, ay, xsphx, xsphy.  Also leaves in the
 * workspace the reductions the next sph_timestep would compute. */
int sph_compute(sph_particles_t *pa, const sph_wcsph_t *w, const sph_config_t *cfg, const sph_workspace_t *ws,
                sph_stream_t stream);

/* sph_compute without a caller workspace: the same evaluation, with the
 * scratch in a device array that the library owns.  It has no counterpart in
 * the reference; it is for callers that cannot allocate device memory
 * themselves (an application whose GPU memory belongs to another allocator or
 * a fixed budget, a foreign-function binding without a CUDA allocator).  The
 * caller still passes the particle arrays.
 *  - Limit: at most SPH_STATIC_MAX_PARTICLES particles (SPH_ERR_STATIC_LIMIT
 *    otherwise); the search grid is capped at SPH_STATIC_MAX_CELLS cells and
 *    is coarsened beyond that (results unchanged, search slower).
 *  - Every GPU that loads the library holds the SPH_STATIC_WS_BYTES array
 *    until the process exits.  The call itself allocates nothing.
 *  - The first call in a CUDA context looks up the array's device address
 *    there (once per context: the device's primary context, a caller's own
 *    context, and the new primary context after cudaDeviceReset each count as
 *    one); make that first call before any stream capture in the context.
 *  - All calls share the one array: calls whose work overlaps on the GPU (on
 *    different streams, or from different host threads without ordering) race
 *    on it.  Order them on one stream.
 *  - status: optional DEVICE pointer that receives the SPH_STATUS_* bits of
 *    this call (asynchronously, on the stream). */
#define SPH_STATIC_MAX_PARTICLES 32768
#define SPH_STATIC_MAX_CELLS 131072
#define SPH_STATIC_WS_BYTES 8388608
int sph_compute_static(sph_particles_t *pa, const sph_wcsph_t *w, const sph_config_t *cfg, uint32_t *status,
                       sph_stream_t stream);

/* TimeStep.compute over the fluid particles (src/Equations/TimeStep.py:7-91,
 * gamma_c = cfg->cfl_c, gamma_f = cfg->cfl_f): dt3[0..2] = {dt, dt_courant,
 * dt_force} (device doubles).  Sets SPH_STATUS_SMALL_DT when dt < 1e-6. */
int sph_timestep(const sph_particles_t *pa, const sph_wcsph_t *w, const sph_config_t *cfg, const sph_workspace_t *ws,
                 double *dt3, sph_stream_t stream);

/* Integrator.predict / correct on the fluid particles (src/Integrators/PEC.py:32-89,
 * src/Integrators/Euler.py:13-27), dt read from the device double *dt. */
int sph_predict(sph_particles_t *pa, const sph_config_t *cfg, const double *dt, sph_stream_t stream);
int sph_correct(sph_particles_t *pa, const sph_config_t *cfg, const double *dt, sph_stream_t stream);

/* NewmarkBeta.predict / correct (src/Integrators/NewmarkBeta.py:41-69), the
 * coupling integrator of Solver.run (src/Solver.py:381-382, 397-398), on the
 * particles labelled SPH_COUPLED, dt read from the device double *dt.
 * SPH_ERR_INVALID_ARGUMENT unless 2 beta >= gamma (NewmarkBeta.py:32). */
int sph_newmark_predict(sph_particles_t *pa, double beta, double gamma, const double *dt, sph_stream_t stream);
int sph_newmark_correct(sph_particles_t *pa, double beta, double gamma, const double *dt, sph_stream_t stream);

/* Scratch bytes of sph_newmark_acceleration for n nodes and matrices with
 * kl sub- and ku superdiagonals (0 <= kl, ku <= n - 1; n - 1: dense). */
int sph_newmark_work_size(int64_t n, int32_t kl, int32_t ku, size_t *bytes);

/* NewmarkBeta.acceleration (src/Integrators/NewmarkBeta.py:71-93):
 * a = (M + C gamma dt + K beta dt^2)^-1 (F - K r - C v).  M, K, C: device
 * n x (kl + ku + 1) row band storage (row i, column j at
 * [i (kl + ku + 1) + j - i + kl]); F, r, v, a: device n-vectors; work:
 * device scratch of work_bytes; info: device int32, set to 0, or to j + 1
 * when pivot j is exactly zero (the matrix is singular; a is not written). */
int sph_newmark_acceleration(int64_t n, int32_t kl, int32_t ku, const double *M, const double *K, const double *C,
                             double beta, double gamma, double dt, const double *F, const double *r, const double *v,
                             double *a, void *work, size_t work_bytes, int32_t *info, sph_stream_t stream);

/* nsteps bare time steps of Solver.run's loop body (src/Solver.py:366-410)
 * with settling and storage left out: dt (TimeStep or cfg->dt_fixed) ->
 * predict -> _compute -> correct, all on the device.  dt_hist, if not NULL,
 * receives 3 doubles per step {dt, dt_courant, dt_force} (device memory).
 * A run of 4 or more steps, in a workspace sized by sph_workspace_size,
 * steps on a copy of the state in the workspace, gathered once into the
 * sorted order of a first neighbour build and scattered back at the end;
 * the results are the same, bit for bit.  The workspace's neighbour table
 * then refers to that copy: call sph_nn_update before sph_nn_count,
 * sph_nn_export or the probes.  p, c and h are those of the last step, as
 * after nsteps single-step runs; with a fixed h and no summation density
 * the steps between the first and the last do not store them (no kernel of
 * the run reads them). */
int sph_run(sph_particles_t *pa, const sph_wcsph_t *w, const sph_config_t *cfg, const sph_workspace_t *ws, int64_t nsteps,
            double *dt_hist, sph_stream_t stream);

/* sph_run with a CUDA event recorded after every stage, for measurement:
 * the GPU time of each stage summed over the steps, in ms, into
 * stage_ms[SPH_NSTAGES] (host memory).  The events are recorded without
 * waiting on them and read after one synchronisation at the end, so a
 * stage's interval runs from the previous stage's last kernel to its own
 * last kernel, with no host round trip inside.  Synchronises once on return
 * and cannot be captured in a graph.  The stages are the parts of
 * Solver.run's step body (src/Solver.py:366-410); RECORDS is empty unless
 * summation density adds its pass (the records are written by the build). */
enum {
  SPH_STAGE_TIMESTEP = 0, /* initial TimeStep.compute */
  SPH_STAGE_PREDICT = 1,  /* the previous step's integrator.correct, this step's
                             integrator.predict and the bounds of nn.update, one pass */
  SPH_STAGE_BUILD = 2,    /* rest of nn.update: grid, keys, counting sort */
  SPH_STAGE_RECORDS = 3,  /* h reset + Tait EOS + sorted pair records */
  SPH_STAGE_PAIR = 4,     /* the fused pair interaction (+ next TimeStep) */
  SPH_STAGE_CORRECT = 5,  /* the last step's integrator.correct */
  SPH_NSTAGES = 6
};
int sph_run_profiled(sph_particles_t *pa, const sph_wcsph_t *w, const sph_config_t *cfg, const sph_workspace_t *ws,
                     int64_t nsteps, double *stage_ms, sph_stream_t stream);

/* ------------------------------------------------------------------------
 * Differentiation form.  The reference has no derivatives; these entry
 * points differentiate its step (fixed dt, src/Solver.py:370-372; PEC,
 * src/Integrators/PEC.py:32-89; fixed h; FP64 form; no XSPH, no summation
 * density) for losses built from a wall load: the x component of the
 * Lennard-Jones boundary force (src/Equations/BoundaryForce.py:6-42) that
 * the boundary particles at x >= wall_x exert on the fluid, with the sign of
 * the load on the wall: load = -sum_i m_i b_x,i.
 * ------------------------------------------------------------------------ */

/* sph_run (fixed dt) that also writes load_hist[s] = the wall load of step
 * s's evaluation (device doubles, nsteps of them), summed in a fixed order.
 * fr: device scratch, n doubles. */
int sph_run_wall_load(sph_particles_t *pa, const sph_wcsph_t *w, const sph_config_t *cfg, const sph_workspace_t *ws,
                      int64_t nsteps, double wall_x, double *fr, double *load_hist, sph_stream_t stream);

/* Adjoint of one step (cfg->precision: SPH_PREC_FP64, the reference's
 * arithmetic, or SPH_PREC_MIXED, the mixed form: the pair arithmetic of the
 * vector-Jacobian product in FP32 over the FP64 records and adjoint vectors;
 * the state update and the step-to-step accumulation stay FP64, and the
 * forward and its replay are FP64 either way).  On entry xb .. drhob hold
 * d loss / d S' for the
 * state after the step (fluid particles; caller order), on exit d loss / d S
 * for the state before it; S is pa's x, y, vx, vy, rho, ax, ay, drho (the
 * state before the step, as sph_run leaves it).  alphab[i] accumulates the
 * step's d loss / d alpha contribution of particle i (sum it for the
 * gradient).  omega: the weight of this step's wall load in the loss (dt for
 * a time integral).  The remaining pointers are device scratch of n doubles
 * each; half is a scratch particle set of n particles (all fields).
 * reuse_build != 0: ws already holds the neighbour build and FP64 records
 * of this step's evaluation (a copy of the workspace as sph_run_wall_load
 * left it after running this one step); the step then skips its own build
 * and does not touch half. */
typedef struct sph_adjoint {
  double *xb, *yb, *vxb, *vyb, *rhob, *axb, *ayb, *drhob;
  double *alphab;
  double *lax, *lay, *lad, *xhb, *yhb, *vxhb, *vyhb, *rhohb, *alb;
  int32_t reuse_build;
  int32_t pad0;
  double omega;
  double wall_x;
} sph_adjoint_t;
int sph_adjoint_step(const sph_particles_t *pa, sph_particles_t *half, const sph_wcsph_t *w, const sph_config_t *cfg,
                     const sph_workspace_t *ws, const sph_adjoint_t *adj, sph_stream_t stream);

/* ------------------------------------------------------------------------
 * Batched form.  No reference counterpart (the reference runs one tank per
 * Solver).  n_inst independent instances -- each a particle set the
 * reference's Solver would run on its own, with its own WCSPH constants,
 * fixed h and Courant dt -- live in one particle set, instance b in
 * [offsets[b], offsets[b+1]).  Each step is one launch per stage over all
 * instances (neighbour build, records, pair interaction, TimeStep, PEC), and
 * instance b's results are those of a single-instance run of it with
 * max_cells = sph_batch_instance_cells(...).  Mixed form, PEC, TimeStep dt,
 * no XSPH or summation density.
 * ------------------------------------------------------------------------ */

/* Workspace bytes for n_total particles in n_inst instances (max_cells <= 0:
 * a default of 8 cells per particle). */
int sph_batch_workspace_size(int64_t n_total, int64_t n_inst, int64_t max_cells, size_t *bytes);

/* Prepares ws (allocated with sph_batch_workspace_size and the same
 * max_cells) for the instances: offsets (host, n_inst + 1), w and h_fixed
 * (host, one per instance), cfg (shared settings).  tile_shift_max: the
 * largest tile shift of the own-grid cell numbering (0..4; -1: default).
 * Synchronises. */
int sph_batch_setup(const sph_workspace_t *ws, int64_t n_inst, const int64_t *offsets, const sph_wcsph_t *w,
                    const double *h_fixed, const sph_config_t *cfg, int32_t tile_shift_max, sph_stream_t stream);

/* The cell capacity instance b gets inside ws (what a single-instance run
 * of it must use to match the batched results bit for bit). */
int64_t sph_batch_instance_cells(const sph_workspace_t *ws, int64_t n_inst, const int64_t *offsets, int64_t b);

/* nsteps steps of every instance.  dt_hist (device, optional):
 * nsteps x n_inst x 3 doubles {dt, dt_courant, dt_force}.  tile_blocks:
 * resident blocks per SM of the pair tile kernel (<= 0: default).  No host
 * synchronisation, so a sequence of calls can be captured in a CUDA graph. */
int sph_batch_run(sph_particles_t *pa, const sph_config_t *cfg, const sph_workspace_t *ws, int64_t n_inst,
                  int64_t nsteps, double *dt_hist, int32_t tile_blocks, sph_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* SPH_GB300_H */

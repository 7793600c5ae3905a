"""CPU oracle for the WCSPH step -- TEST INFRASTRUCTURE ONLY.

A ctypes wrapper around ``sph_oracle.c``, a plain-C restatement of
Offshore-SPH's numba hot path (``src/Tools/NNLinkedList.py``,
``src/Tools/SolverTools.py``, ``src/Equations/*``, ``src/Kernels/{CubicSpline,
Gaussian}.py``, ``src/Integrators/{PEC,Euler}.py``, ``src/Solver.py`` step
body).  Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline leg use it, as the checker or as the timed CPU baseline; the product
package never imports it.

Parity of this restatement with the reference is pinned by the golden vectors
in ``tests/golden/`` (generated by running the unmodified reference source under
a pure-Python numba stand-in, ``tests/golden/make_golden.py``).
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libsph_oracle.so")
_SRC = os.path.join(_HERE, "sph_oracle.c")

OR_OK = 0
OR_ERR_CELL_OVERFLOW = 1

FIELDS = ["m", "rho", "p", "c", "drho", "h", "x", "y", "vx", "vy", "ax", "ay",
          "xsphx", "xsphy", "x0", "y0", "vx0", "vy0", "rho0"]


def build(force=False):
    """Compile sph_oracle.c into oracle/_build/libsph_oracle.so (gcc, OpenMP,
    no FMA contraction)."""
    os.makedirs(_BUILD, exist_ok=True)
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(_SRC)):
        return _LIB_PATH
    tmp = _LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
           "-o", tmp, _SRC, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        dp = C.POINTER(C.c_double)
        i64p = C.POINTER(C.c_int64)
        L.or_nn_new.restype = C.c_void_p
        L.or_nn_new.argtypes = [C.c_double]
        L.or_nn_free.argtypes = [C.c_void_p]
        L.or_nn_update.argtypes = [C.c_void_p, C.c_int64, dp, dp, dp]
        L.or_nn_grid.argtypes = [C.c_void_p, dp, i64p]
        L.or_nn_lists.argtypes = [C.c_void_p, i64p, i64p]
        L.or_nn_near.restype = C.c_int64
        L.or_nn_near.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double, dp, dp, dp,
                                 i64p, dp, dp, dp, C.c_int64]
        L.or_nn_all.argtypes = [C.c_void_p, C.c_int64, dp, dp, dp, C.c_void_p, C.c_int, i64p, C.c_void_p]
        L.or_nn_all_mt.argtypes = [C.c_void_p, C.c_int64, dp, dp, dp, C.c_void_p, C.c_int, i64p, C.c_void_p,
                                   C.c_int, C.c_int]
        L.or_loop_range.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64]
        L.or_loop.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.or_compute.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int]
        L.or_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
        L.or_timestep.argtypes = [C.c_int64, C.c_void_p, dp, dp, dp, dp, C.c_double, C.c_double, dp]
        L.or_pec_predict.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_int]
        L.or_pec_correct.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_int]
        L.or_euler_correct.argtypes = [C.c_void_p, C.c_void_p, C.c_double]
        L.or_verlet_predict.argtypes = [C.c_void_p, C.c_void_p, C.c_double]
        L.or_verlet_correct.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_int]
        L.or_eos.argtypes = [C.c_int64, C.c_void_p, dp, C.c_double, C.c_double, C.c_double, C.c_double, dp]
        L.or_tait_height.argtypes = [C.c_int64, dp, C.c_double, C.c_double, C.c_double, C.c_double, dp]
        L.or_kernel_eval.argtypes = [C.c_int, C.c_int64, dp, dp, dp]
        L.or_kernel_grad.argtypes = [C.c_int, C.c_int64, dp, dp, dp, dp]
        L.or_gauss_deriv.argtypes = [C.c_int64, dp, dp, dp]
        L.or_equations.argtypes = [C.c_int64, C.c_void_p] + [dp] * 12 + [dp, dp, C.c_double, dp]
        L.or_max_threads.restype = C.c_int
        _lib = L
    return _lib


def _dp(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i64p(a):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class WCSPHParams(C.Structure):
    """or_wcsph: the WCSPH constants (src/Methods/WCSPH.py:35-79)."""
    _fields_ = [(k, C.c_double) for k in
                ["gamma", "B", "rho0", "Pb", "co", "alpha", "beta", "epsilon", "r0", "D", "p1", "p2"]] + \
               [("use_xsph", C.c_int32), ("use_summation_density", C.c_int32),
                ("kernel", C.c_int32), ("sum_order", C.c_int32)]


class StepOpt(C.Structure):
    _fields_ = [("h_fixed", C.c_double), ("dt_fixed", C.c_double), ("gamma_c", C.c_double),
                ("gamma_f", C.c_double), ("damping", C.c_double), ("integrator", C.c_int32),
                ("pec_use_xsph", C.c_int32), ("pec_strict", C.c_int32), ("nthreads", C.c_int32)]


class _Particles(C.Structure):
    _fields_ = [("n", C.c_int64), ("label", C.c_void_p)] + [(k, C.c_void_p) for k in FIELDS]


def wcsph_params(height, r0, rho0, use_xsph=False, Pb=0.0, use_summation_density=False, kernel=0,
                 alpha=0.01, beta=0.0, sum_order=0):
    """The constants WCSPH.__init__ derives (WCSPH.py:35-79, TaitEOS.py:33-44).
    sum_order = 1 sums every particle's neighbours in reverse order: not a
    reference setting, but a control run that differs from the reference only
    by round-off, to size how round-off differences grow along a trajectory."""
    co = 10.0 * np.sqrt(2 * 9.81 * height)
    gamma = 7.0
    B = co * co * rho0 / gamma
    return WCSPHParams(gamma=gamma, B=B, rho0=rho0, Pb=Pb, co=co, alpha=alpha, beta=beta, epsilon=0.5,
                       r0=r0, D=5 * 9.81 * height, p1=4.0, p2=2.0, use_xsph=int(use_xsph),
                       use_summation_density=int(use_summation_density), kernel=int(kernel),
                       sum_order=int(sum_order))


class Particles:
    """SoA numpy arrays of the particle_dtype fields (src/Common.py:26-57)."""

    def __init__(self, n=None, arrays=None):
        if arrays is not None:
            n = len(arrays["x"])
        self.n = int(n)
        self.label = np.zeros(self.n, dtype=np.int8)
        for k in FIELDS:
            setattr(self, k, np.zeros(self.n, dtype=np.float64))
        if arrays is not None:
            for k, v in arrays.items():
                if k == "label":
                    self.label[:] = v
                elif k in FIELDS:
                    getattr(self, k)[:] = v

    def copy(self):
        return Particles(arrays=self.as_dict())

    def as_dict(self):
        d = {k: getattr(self, k).copy() for k in FIELDS}
        d["label"] = self.label.copy()
        return d

    def cstruct(self):
        s = _Particles(n=self.n, label=self.label.ctypes.data)
        for k in FIELDS:
            setattr(s, k, getattr(self, k).ctypes.data)
        return s


class NN:
    """NNLinkedList (src/Tools/NNLinkedList.py:21-208) restated in C."""

    def __init__(self, scale=2.0):
        self.h = lib().or_nn_new(scale)

    def __del__(self):
        try:
            if self.h:
                lib().or_nn_free(self.h)
        except Exception:
            pass

    def update(self, x, y, h):
        self._x, self._y, self._hh = _f64(x), _f64(y), _f64(h)
        return lib().or_nn_update(self.h, len(self._x), _dp(self._x), _dp(self._y), _dp(self._hh))

    def grid(self):
        d = np.zeros(5)
        i = np.zeros(3, dtype=np.int64)
        lib().or_nn_grid(self.h, _dp(d), _i64p(i))
        return dict(xmin=d[0], xmax=d[1], ymin=d[2], ymax=d[3], cell_size=d[4],
                    ncx=int(i[0]), ncy=int(i[1]), n_cells=int(i[2]))

    def lists(self):
        g = self.grid()
        heads = np.zeros(g["n_cells"], dtype=np.int64)
        nexts = np.zeros(len(self._x), dtype=np.int64)
        lib().or_nn_lists(self.h, _i64p(heads), _i64p(nexts))
        return heads, nexts

    def near(self, x, y, h):
        cap = len(self._x)
        idx = np.zeros(cap, dtype=np.int64)
        hij, q, r = np.zeros(cap), np.zeros(cap), np.zeros(cap)
        n = lib().or_nn_near(self.h, x, y, h, _dp(self._x), _dp(self._y), _dp(self._hh), _i64p(idx),
                             _dp(hij), _dp(q), _dp(r), cap)
        return hij[:n], q[:n], r[:n], idx[:n]

    def all(self, label=None, label_filter=-1, nthreads=1, sorted_lists=False):
        """CSR neighbour lists near(i) for all i (label_filter -1) or one label,
        each in the reference's traversal order (ascending index order with
        sorted_lists).  nthreads > 1 runs the queries on OpenMP threads."""
        if nthreads > 1 or sorted_lists:
            return self._all_mt(label, label_filter, nthreads, sorted_lists)
        n = len(self._x)
        lab = np.ascontiguousarray(label, dtype=np.int8) if label is not None else np.zeros(n, np.int8)
        off = np.zeros(n + 1, dtype=np.int64)
        lib().or_nn_all(self.h, n, _dp(self._x), _dp(self._y), _dp(self._hh), lab.ctypes.data,
                        label_filter, _i64p(off), None)
        idx = np.zeros(max(int(off[-1]), 1), dtype=np.int64)
        lib().or_nn_all(self.h, n, _dp(self._x), _dp(self._y), _dp(self._hh), lab.ctypes.data,
                        label_filter, _i64p(off), idx.ctypes.data)
        return off, idx[:int(off[-1])]

    def _all_mt(self, label, label_filter, nthreads, sorted_lists):
        n = len(self._x)
        lab = np.ascontiguousarray(label, dtype=np.int8) if label is not None else np.zeros(n, np.int8)
        off = np.zeros(n + 1, dtype=np.int64)
        args = (self.h, n, _dp(self._x), _dp(self._y), _dp(self._hh), lab.ctypes.data, label_filter, _i64p(off))
        if lib().or_nn_all_mt(*args, None, max(1, nthreads), int(sorted_lists)):
            raise RuntimeError("oracle neighbour export failed")
        idx = np.zeros(max(int(off[-1]), 1), dtype=np.int64)
        if lib().or_nn_all_mt(*args, idx.ctypes.data, max(1, nthreads), int(sorted_lists)):
            raise RuntimeError("oracle neighbour export failed")
        return off, idx[:int(off[-1])]


def kernel_eval(kernel, r, h):
    r, h = _f64(r), _f64(h)
    out = np.zeros_like(r)
    lib().or_kernel_eval(kernel, len(r), _dp(r), _dp(h), _dp(out))
    return out


def kernel_grad(kernel, x, r, h):
    x, r, h = _f64(x), _f64(r), _f64(h)
    out = np.zeros_like(r)
    lib().or_kernel_grad(kernel, len(r), _dp(x), _dp(r), _dp(h), _dp(out))
    return out


def gauss_deriv(r, h):
    r, h = _f64(r), _f64(h)
    out = np.zeros_like(r)
    lib().or_gauss_deriv(len(r), _dp(r), _dp(h), _dp(out))
    return out


def equations(comp, self5, par6, epsilon=0.5):
    """Continuity/Momentum/BoundaryForce/XSPH on one computed block.
    Returns (drho, ax, ay, bx, by, xsphx, xsphy) (gravity not included)."""
    J = len(comp["r"])
    lab = np.ascontiguousarray(comp["label"], dtype=np.int8)
    arrs = [_f64(comp[k]) for k in ["m", "p", "rho", "h", "r", "w", "dw_x", "dw_y", "x", "y", "vx", "vy"]]
    s5, p6 = _f64(self5), _f64(par6)
    out = np.zeros(7)
    lib().or_equations(J, lab.ctypes.data, *[_dp(a) for a in arrs], _dp(s5), _dp(p6), epsilon, _dp(out))
    return out


def eos(label, rho, params):
    rho = _f64(rho)
    lab = np.ascontiguousarray(label, dtype=np.int8)
    p = np.zeros_like(rho)
    lib().or_eos(len(rho), lab.ctypes.data, _dp(rho), params.gamma, params.B, params.rho0, params.Pb, _dp(p))
    return p


def tait_height(y, params, height):
    y = _f64(y)
    rho = np.zeros_like(y)
    lib().or_tait_height(len(y), _dp(y), params.rho0, height, params.B, params.gamma, _dp(rho))
    return rho


def timestep(P, gamma_c=0.25, gamma_f=0.25):
    out = np.zeros(3)
    lib().or_timestep(P.n, P.label.ctypes.data, _dp(P.h), _dp(P.c), _dp(P.ax), _dp(P.ay), gamma_c, gamma_f,
                      _dp(out))
    return out


def _mask(P, mask):
    if mask is None:
        return None, None
    m = np.ascontiguousarray(mask, dtype=np.uint8)
    return m, m.ctypes.data


def pec_predict(P, dt, damping=0.0, use_xsph=False, strict=True, mask=None):
    keep, mp = _mask(P, mask)
    s = P.cstruct()
    lib().or_pec_predict(C.byref(s), mp, dt, damping, int(use_xsph), int(strict))


def pec_correct(P, dt, damping=0.0, use_xsph=False, strict=True, mask=None):
    keep, mp = _mask(P, mask)
    s = P.cstruct()
    lib().or_pec_correct(C.byref(s), mp, dt, damping, int(use_xsph), int(strict))


def euler_correct(P, dt, mask=None):
    keep, mp = _mask(P, mask)
    s = P.cstruct()
    lib().or_euler_correct(C.byref(s), mp, dt)


def verlet_predict(P, dt, mask=None):
    keep, mp = _mask(P, mask)
    s = P.cstruct()
    lib().or_verlet_predict(C.byref(s), mp, dt)


def verlet_correct(P, dt, use_xsph=False, mask=None):
    keep, mp = _mask(P, mask)
    s = P.cstruct()
    lib().or_verlet_correct(C.byref(s), mp, dt, int(bool(use_xsph)))


def newmark_predict(P, dt, beta, gamma, mask=None):
    """NewmarkBeta.predict (src/Integrators/NewmarkBeta.py:41-54) on the
    particles in mask (all when None), elementwise in the reference's order."""
    m = np.ones(len(P.x), dtype=bool) if mask is None else np.asarray(mask)
    ax, ay = P.ax[m], P.ay[m]
    P.x[m] = P.x[m] + P.vx[m] * dt + ax * (0.5 - beta) * dt ** 2
    P.y[m] = P.y[m] + P.vy[m] * dt + ay * (0.5 - beta) * dt ** 2
    P.vx[m] = P.vx[m] + ax * (1 - gamma) * dt
    P.vy[m] = P.vy[m] + ay * (1 - gamma) * dt


def newmark_correct(P, dt, beta, gamma, mask=None):
    """NewmarkBeta.correct (src/Integrators/NewmarkBeta.py:56-69)."""
    m = np.ones(len(P.x), dtype=bool) if mask is None else np.asarray(mask)
    ax, ay = P.ax[m], P.ay[m]
    P.x[m] = P.x[m] + ax * beta * dt ** 2
    P.y[m] = P.y[m] + ay * beta * dt ** 2
    P.vx[m] = P.vx[m] + ax * gamma * dt
    P.vy[m] = P.vy[m] + ay * gamma * dt


def newmark_acceleration(M, K, Cm, beta, gamma, dt, F, r, v):
    """NewmarkBeta.acceleration (src/Integrators/NewmarkBeta.py:71-93):
    inv(M + C gamma dt + K beta dt^2) . (F - K r - C v)."""
    rhs = F - np.dot(K, r) - np.dot(Cm, v)
    lhs = M + Cm * gamma * dt + K * beta * dt ** 2
    return np.dot(np.linalg.inv(lhs), rhs)


def probe_density(nn, P, x, y, h_search, h_kernel, kernel, rho0, B, gamma):
    """The ice-coupling example's pressure interpolation at points
    (examples/IceBreak.py:253-285): nearPos (the C restatement), kernel values
    W(r, h_kernel), Shepard normalisation (src/Equations/Shepard.py:5-12),
    summation density (src/Equations/SummationDensity.py:5-13), Tait EOS.
    Returns (rho, p) arrays."""
    rho_out, p_out = [], []
    for xi, yi, hs, hk in zip(np.atleast_1d(x), np.atleast_1d(y), np.atleast_1d(h_search), np.atleast_1d(h_kernel)):
        hij, q, r, idx = nn.near(float(xi), float(yi), float(hs))
        w = kernel_eval(kernel, r, np.full(len(r), float(hk)))
        lab, m, rb = P.label[idx], P.m[idx], P.rho[idx]
        den = 0.0
        for k in range(len(w)):
            if rb[k] < 1e-3 or lab[k] != 0:
                continue
            den += w[k] * m[k] / rb[k]
        with np.errstate(divide="ignore", invalid="ignore"):  # as the reference: w / 0 on empty or boundary-only sets
            wt = w / den
        rho = 0.0
        for k in range(len(w)):
            if lab[k] != 0:
                continue
            rho += m[k] * wt[k]
        rho_out.append(rho)
        p_out.append(((rho / rho0) ** gamma - 1.0) * B)
    return np.array(rho_out), np.array(p_out)


def loop(params, nn, P, nthreads=1):
    s = P.cstruct()
    return lib().or_loop(C.byref(params), nn.h, C.byref(s), nthreads)


def loop_range(params, nn, P, i0, i1):
    """_loop's regular pass for the fluid particles in [i0, i1) on one thread
    (after the EOS pass over all particles), on the table of the last
    nn.update: a bounded sample of one evaluation, for timing."""
    s = P.cstruct()
    return lib().or_loop_range(C.byref(params), nn.h, C.byref(s), int(i0), int(i1))


def compute(params, nn, P, h_fixed, nthreads=1):
    """Solver._compute: nn.update + h + _loop (src/Solver.py:232-256)."""
    s = P.cstruct()
    nn._x, nn._y, nn._hh = P.x, P.y, P.h
    return lib().or_compute(C.byref(params), nn.h, C.byref(s), h_fixed, nthreads)


def run(params, nn, P, nsteps, h_fixed=0.0, dt_fixed=0.0, gamma_c=0.25, gamma_f=0.25, damping=0.0,
        integrator=0, pec_use_xsph=False, pec_strict=True, nthreads=1):
    """nsteps bare steps dt -> predict -> compute -> correct (src/Solver.py:366-410).
    Returns the (nsteps, 3) array of (dt, dt_courant, dt_force)."""
    s = P.cstruct()
    o = StepOpt(h_fixed=h_fixed, dt_fixed=dt_fixed, gamma_c=gamma_c, gamma_f=gamma_f, damping=damping,
                integrator=integrator, pec_use_xsph=int(pec_use_xsph), pec_strict=int(pec_strict),
                nthreads=nthreads)
    dts = np.zeros((max(nsteps, 1), 3))
    nn._x, nn._y, nn._hh = P.x, P.y, P.h
    st = lib().or_run(C.byref(params), nn.h, C.byref(s), C.byref(o), nsteps, _dp(dts))
    if st:
        raise RuntimeError("oracle run failed with status %d" % st)
    return dts[:nsteps]


def setup(P, params, height, h_fixed):
    """Solver.setup's state preparation (src/Solver.py:173-208): h for fluid,
    WCSPH.initialize (hydrostatic rho), p and c for fluid."""
    f = P.label == 0
    if h_fixed and h_fixed > 0:
        P.h[f] = h_fixed
    else:
        P.h[f] = np.where(P.rho[f] > 1e-12, 1.3 * np.power(P.m[f] / np.where(P.rho[f] > 1e-12, P.rho[f], 1.0), 0.5),
                          0.0)
    P.rho[f] = tait_height(P.y[f], params, height)
    P.p[f] = eos(P.label[f], P.rho[f], params)
    P.c[f] = params.co


def max_threads():
    return lib().or_max_threads()

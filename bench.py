#!/usr/bin/env python
"""WCSPH throughput benchmark (particle-steps/s) on one or more GB300s.

Workload (default ``dambreak1m``): a 1M-fluid 2D dam break -- the 1:2 column
of the 3200-particle case at 707 x 1414 particles, dx = 0.01, in a tank 4x its
width and 1.5x its height with 2 wall layers at dx/2 (28k boundary particles),
rho0 = 1000, H = 14.14 m, h = 1.3 dx, cubic spline, alpha = 0.01, Courant 0.3,
hydrostatic start -- advanced by full PEC time steps.  One step = TimeStep
(Courant/force dt) -> PEC predict -> neighbour build -> h reset + Tait EOS +
continuity + momentum + boundary force (the fused pair kernels) -> PEC
correct, all on the device.  Also: ``lattice1m`` / ``lattice1m_gauss`` (the
1000 x 1000 jittered lattice, cubic / Gaussian), ``dambreak2m`` (10 x 20 m
column, 2M fluid), ``dambreak3200``.

Metric: particle-steps/s = fluid particles x steps / device time of the
timed steps (whole job: summed over ranks; N > 1 runs independent replicas).

Lines printed: one JSON object (rank 0).  ``--impl reference`` times the CPU
reference implementation of the step (the C restatement in oracle/, OpenMP
over all host cores) on the same workload: ``--warmup`` untimed and
``--steps`` timed steps.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (REPO, os.path.join(REPO, "offshore-sph_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "WCSPH particle-steps/s"
UNIT = "particle-steps/s"
PAIR_BYTES = 81     # algorithmic bytes of the pair evaluation per particle (x,y,vx,vy,rho,m,h,label in; drho,ax,ay out)
STEP_BYTES = 385    # algorithmic bytes of one PEC step per particle (dt 32 + predict 144 + build 24 + pair 81 + correct 104)
# DRAM bytes (read + write) per particle of one pair launch: not measurable
# without a profiler, so taken from an ncu capture of the same kernel on the
# same workload (dram__bytes_read.sum + dram__bytes_write.sum over the
# particle count), with the capture's date
TRAFFIC_FROM_PROFILE = {("dambreak1m", "mixed"): (62.8, "2026-12-04, k_pair_tiles, one launch")}
# what bounds the pair kernel instead of HBM, read off the same captures
LIMITER_FROM_PROFILE = {"mixed": "instruction issue and the shared-memory pipe: 63.1% of active cycles issue, "
                                 "L1tex 76.0% of peak, DRAM 6.2% of peak (ncu, 2026-12-04)",
                        "fp64": "FP64 pipe: busy 86.5% of active cycles, DRAM 0.5% of peak (ncu, 2026-12-04)"}


def workload(name):
    from sph import scenarios as S
    if name == "dambreak1m":
        return dict(pa=S.cfg_dam_break_1m(), height=14.14, r0=0.01, h=0.013, kernel=0, gamma_c=0.3, setup=True,
                    desc="1M-fluid dam break: 7.07x14.14 m column at dx=0.01 (707x1414 fluid) in a 28.3x21.2 m "
                         "tank, 2 wall layers at dx/2, cubic, PEC, Courant 0.3")
    if name == "lattice1m":
        pa = S.jittered_lattice(1000, 1000, 0.01, seed=0)
        return dict(pa=pa, height=10.0, r0=0.01, h=0.013, kernel=0, gamma_c=0.25, setup=False,
                    desc="1000x1000 jittered lattice, dx=0.01, h=1.3dx, cubic, no boundaries, PEC step")
    if name == "lattice1m_gauss":
        pa = S.jittered_lattice(1000, 1000, 0.01, seed=0)
        return dict(pa=pa, height=10.0, r0=0.01, h=0.013, kernel=1, gamma_c=0.25, setup=False,
                    desc="1000x1000 jittered lattice, dx=0.01, h=1.3dx, Gaussian (q<=3), PEC step")
    if name == "dambreak2m":
        pa = S.cfg_dam_break_large()
        return dict(pa=pa, height=20.0, r0=0.01, h=0.013, kernel=0, gamma_c=0.3, setup=True,
                    desc="10x20 m column at dx=0.01 (2M fluid) in a 40x30 m tank, 2 wall layers at dx/2, "
                         "cubic, PEC, Courant 0.3")
    if name == "dambreak3200":
        pa = S.cfg_dam_break_small()
        return dict(pa=pa, height=2.0, r0=0.025, h=0.0325, kernel=0, gamma_c=0.3, setup=True,
                    desc="1x2 m column at dx=0.025 (3200 fluid) in a 4x3 m tank, cubic, PEC, Courant 0.3")
    raise SystemExit("unknown workload " + name)


def oracle_particles(wl, pa, height):
    import oracle
    par = oracle.wcsph_params(height, wl["r0"], 1000.0, kernel=wl["kernel"])
    d = {k: pa[k] for k in pa.dtype.names if k != "deleted"}
    P = oracle.Particles(arrays=d)
    if wl["setup"]:
        oracle.setup(P, par, height, wl["h"])
    else:
        P.h[P.label == 0] = wl["h"]
        P.p[:] = oracle.eos(P.label, P.rho, par)
        P.c[:] = par.co
    return P, par


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def prepare(wl, precision):
    import torch
    from sph import core, state
    pa = wl["pa"]
    dp = state.DeviceParticles.from_array(pa)
    wc = core.wcsph_struct(wl["height"], wl["r0"], 1000.0)
    cfg = core.config_struct(kernel=wl["kernel"], precision=precision, h_fixed=wl["h"], cfl_c=wl["gamma_c"],
                             cfl_f=0.25)
    if wl["setup"]:
        core.initialize(dp, wc, cfg)
    else:
        # Solver.setup without the hydrostatic initialise: h, p, c of fluid
        f = dp.label == 0
        dp.h[f] = wl["h"]
        core.eos(dp, wc)
    ws = state.DeviceWorkspace(dp.n)
    torch.cuda.synchronize()
    return dp, wc, cfg, ws


GRAPH_STEPS = 100  # steps per captured CUDA graph in the timed region


def graph_plan(k):
    """(steps per graph, replays, remainder steps) covering exactly k steps."""
    g = min(k, GRAPH_STEPS)
    return g, k // g, k % g


def make_graphs(core, dp, wc, cfg, ws, k):
    g, reps, rem = graph_plan(k)
    return core.StepGraph(dp, wc, cfg, ws, g), reps, (core.StepGraph(dp, wc, cfg, ws, rem) if rem else None)


def time_graph_steps(graphs):
    """Exactly the planned steps as replays of captured sph_run graphs."""
    import torch
    main, reps, tail = graphs
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record()
    for _ in range(reps):
        main.replay()
    if tail is not None:
        tail.replay()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / 1e3


def e2e_steps(core, dp, wc, cfg, ws, k, pa, result=None):
    """Steps through the C ABI with the particle state on the HOST: each step
    copies its inputs host -> device (pinned) and its results back, and the
    next step starts from the host's copy.  The host link carries about
    200 GB/s each way, so the transfers run on two copy streams, and two
    device copies of the state alternate between steps:
    - the fields that no step writes (m, h, c, label) go up for step s + 1
      while step s computes;
    - each result field goes up for step s + 1 as soon as its download of
      step s has finished, while the next field comes down.
    Returns (seconds, bytes in per step, bytes out per step); with a dict
    `result`, also the host copy of the last step's results in it."""
    import torch
    from sph import state
    fconst = ("m", "h", "c")
    fvar = ("x", "y", "vx", "vy", "rho", "drho", "ax", "ay")  # in the order they come down
    fout = fvar + ("p",)
    host = {f: torch.from_numpy(np.ascontiguousarray(dp.fields[f].cpu().numpy())).pin_memory()
            for f in fconst + fvar}
    host["p"] = torch.empty(dp.n, dtype=torch.float64).pin_memory()
    host_label = torch.from_numpy(dp.label.cpu().numpy()).pin_memory()
    h2d = sum(host[f].numel() * 8 for f in fconst + fvar) + host_label.numel()
    d2h = dp.n * 8 * len(fout)
    other = state.DeviceParticles(dp.n)
    other._buf.copy_(dp._buf)
    other.label.copy_(dp.label)
    bufs = (dp, other)
    comp = torch.cuda.current_stream()
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    ev_out = {f: None for f in fout}
    freed = [None, None]  # the last step on each device copy has finished
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record(comp)
    for step in range(k):
        d = bufs[step & 1]
        with torch.cuda.stream(s_in):
            if freed[step & 1] is not None:
                s_in.wait_event(freed[step & 1])  # step - 2 no longer reads this copy
            for f in fconst:
                d.fields[f].copy_(host[f], non_blocking=True)
            d.label.copy_(host_label, non_blocking=True)
            for f in fvar:
                if ev_out[f] is not None:
                    s_in.wait_event(ev_out[f])  # its host copy holds the previous step's result
                d.fields[f].copy_(host[f], non_blocking=True)
        comp.wait_stream(s_in)
        core.run(d, wc, cfg, ws, 1)
        done = torch.cuda.Event()
        done.record(comp)
        freed[step & 1] = done
        s_out.wait_event(done)
        with torch.cuda.stream(s_out):
            for f in fout:
                host[f].copy_(d.fields[f], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(s_out)
                ev_out[f] = ev
    comp.wait_stream(s_out)
    e.record(comp)
    torch.cuda.synchronize()
    del other
    if result is not None:
        result.update({f: host[f].numpy().copy() for f in fout})
    return s.elapsed_time(e) / 1e3, h2d, d2h


def arm_config(wl_name, wl):
    """The workload as both arms report it (identical dicts, so that the two
    lines name the same configuration)."""
    pa = wl["pa"]
    return {"workload": wl_name + ": " + wl["desc"], "n_particles": int(len(pa)),
            "n_fluid": int(np.sum(pa["label"] == 0)), "integrator": "PEC"}


def cpu_baseline(wl_name, wl, steps=3, budget_1t_s=8.0):
    """The oracle (C restatement of the reference's step) on the full
    workload: `steps` PEC steps on all host threads; then one thread, as the
    reference's numba loop runs (its prange has no parallel=True), on a
    bounded sample of one evaluation: _loop's pass over the first fluid
    particles (about budget_1t_s seconds of work), because a whole
    single-threaded step of the 1M workload takes minutes."""
    import oracle
    threads = oracle.max_threads()
    P, par = oracle_particles(wl, wl["pa"], wl["height"])
    nn = oracle.NN(2.0)
    nf = int(np.sum(P.label == 0))
    t0 = time.perf_counter()
    oracle.run(par, nn, P, steps, h_fixed=wl["h"], gamma_c=wl["gamma_c"], nthreads=threads)
    el = time.perf_counter() - t0
    # single thread: the table of the current state, then a timed probe and
    # a timed sample sized from it
    nn.update(P.x, P.y, P.h)
    fl = np.flatnonzero(P.label == 0)
    probe = min(len(fl), 512)
    t0 = time.perf_counter()
    oracle.loop_range(par, nn, P, int(fl[0]), int(fl[probe - 1]) + 1)
    per = max((time.perf_counter() - t0) / probe, 1e-9)
    cnt = int(min(len(fl), max(probe, budget_1t_s / per)))
    t0 = time.perf_counter()
    oracle.loop_range(par, nn, P, int(fl[0]), int(fl[cnt - 1]) + 1)
    el1 = time.perf_counter() - t0
    return {"value": nf * steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "the full workload (%d fluid), %d PEC steps, OpenMP over particles" % (nf, steps),
            "single_thread": {"value": cnt / el1, "unit": UNIT, "cores": 1,
                              "sample": "the pair loop (_loop) of one evaluation over %d of the %d fluid "
                                        "particles, one thread (neighbour build and integrator, O(N) "
                                        "and a small share of a step, not included)" % (cnt, nf)}}


REFERENCE_BUDGET_S = 150.0  # timed CPU steps of the reference arm: about this many seconds at most


def run_reference(args, wl_name):
    """--impl reference: the CPU reference implementation of the step (the C
    restatement of the reference's algorithm in oracle/, all host threads)
    on the same workload and configuration as the GPU arm.  One untimed step
    (a CPU needs no more warm-up) measures a step's cost; then full steps
    are timed, `steps` of them or as many as fit in REFERENCE_BUDGET_S,
    whichever is fewer (a full step of the 1M-particle workload takes
    seconds on the host cores, so the GPU arm's step counts would take
    hours)."""
    import oracle
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    oracle.build()
    wl = workload(wl_name)
    threads = oracle.max_threads()
    P, par = oracle_particles(wl, wl["pa"], wl["height"])
    nn = oracle.NN(2.0)
    nf = int(np.sum(P.label == 0))
    t0 = time.perf_counter()
    oracle.run(par, nn, P, 1, h_fixed=wl["h"], gamma_c=wl["gamma_c"], nthreads=threads)
    t_step = time.perf_counter() - t0
    n_t = int(max(1, min(args.steps, REFERENCE_BUDGET_S // max(t_step, 1e-9))))
    t0 = time.perf_counter()
    oracle.run(par, nn, P, n_t, h_fixed=wl["h"], gamma_c=wl["gamma_c"], nthreads=threads)
    el = time.perf_counter() - t0
    v = nf * n_t / el
    smp = "the full workload (%d fluid), %d timed PEC steps after 1 untimed, OpenMP over particles" % (nf, n_t)
    if n_t < args.steps:
        smp += " (%d of the %d requested: the timed steps are bounded to about %d s)" % (
            n_t, args.steps, int(REFERENCE_BUDGET_S))
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "steps_timed": n_t, "warmup": args.warmup, "ms_per_step": el / n_t * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": arm_config(wl_name, wl),
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": smp},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def solver_run_bench(wl, precision="mixed", lengths=(20, 120)):
    """The drop-in Solver.run (the reference's driver loop: TimeStep with its
    0.25 / 0.25 numbers, settling ended by customSettle at the first check,
    no export properties, no incremental write-out) on the workload, timed
    around run() with the host clock for two run lengths; the steady
    throughput is the difference of fluid particle-steps over the difference
    of times, so set-up, the two settling steps and the settling transfer
    cancel."""
    import torch
    import sph
    kernels = {0: sph.CubicSpline, 1: sph.Gaussian, 2: sph.Wendland}
    pa = wl["pa"]
    nf = int(np.sum(pa["label"] == 0))
    co = 10.0 * np.sqrt(2 * 9.81 * wl["height"])
    dt_c = 0.25 * wl["h"] / co
    runs = []
    for n in lengths:
        s = sph.Solver(sph.WCSPH(wl["height"], wl["r0"], 1000.0, False, 0.0), sph.PEC(False, True),
                       kernels[wl["kernel"]](), duration=n * dt_c, h=wl["h"], exportProperties=[],
                       incrementalWriteout=False, customSettle=lambda pA, sv: True, precision=precision)
        s.addParticles(pa.copy())
        s.setup()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.run()
        el = time.perf_counter() - t0
        runs.append((s.t_step, el))
        del s
        torch.cuda.empty_cache()
    (k1, t1), (k2, t2) = runs
    return {"value": nf * (k2 - k1) / (t2 - t1), "unit": UNIT, "precision": precision,
            "steps": [k1, k2], "seconds": [t1, t2], "ms_per_step_steady": (t2 - t1) / (k2 - k1) * 1e3,
            "how": "sph.Solver.run (no per-step exports: each settled chunk of up to 256 steps is one device "
                   "run with one host synchronisation), host clock around run(), steady rate from two run lengths"}


def replica_value(el, nfluid, steps, world, device):
    """Whole-job throughput of N independent replicas: the slowest rank's
    elapsed time (max over ranks) and the fluid particle-steps of all ranks
    over it."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([el], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    el = float(t.item())
    return el, world * nfluid * steps / el


def adjoint_case(nsteps=200, adjoint_precision="fp64"):
    """The differentiation form's case: a 1.0 x 2.0 m column at dx = 0.01
    (20k fluid) against the right wall of the 4 x 3 m tank, 200 PEC steps,
    checkpoints every 20; loss = time integral of the load on the right wall.
    Fixed dt = 5e-5 s: at 1e-4 s (Courant number 0.48 with co = 62.6 m/s and
    h = 0.013) this configuration diverges after about 40 steps, on the GPU
    and in the CPU restatement alike; the reference's own TimeStep would take
    5.2e-5 s here."""
    from sph import adjoint, scenarios
    pa = scenarios.cfg_adjoint()
    return adjoint.WallLoadCase(pa, height=2.0, r0=0.01, h=0.013, dt=5e-5, nsteps=nsteps, wall_x=4.0,
                                checkpoint=20 if nsteps >= 100 else 10, adjoint_precision=adjoint_precision)


def _adjoint_timed(case, pos, vel, reps):
    """Median forward (loss only), forward with checkpoints and backward
    times (ms, CUDA events) and the last gradients."""
    import torch
    from sph import adjoint
    a = torch.tensor(0.01, dtype=torch.float64, device="cuda", requires_grad=True)
    p = pos.clone().requires_grad_(True)
    v = vel.clone().requires_grad_(True)
    torch.autograd.grad(adjoint.WallLoadLoss.apply(a, p, v, case), (a, p, v))  # warm-up
    case.loss(0.01, pos, vel)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    fwd, fwd_ckpt, bwd = [], [], []
    for _ in range(reps):
        torch.cuda.synchronize()
        ev[0].record()
        case.loss(0.01, pos, vel)
        ev[1].record()
        loss = adjoint.WallLoadLoss.apply(a, p, v, case)
        ev[2].record()
        ga, gp, gv = torch.autograd.grad(loss, (a, p, v))
        ev[3].record()
        torch.cuda.synchronize()
        fwd.append(ev[0].elapsed_time(ev[1]))
        fwd_ckpt.append(ev[1].elapsed_time(ev[2]))
        bwd.append(ev[2].elapsed_time(ev[3]))
    return (float(np.median(fwd)), float(np.median(fwd_ckpt)), float(np.median(bwd)), loss.item(), ga, gp, gv)


def adjoint_cost(reps=3):
    """The differentiation form, FP64 and mixed adjoint: forward pass (loss
    only) and backward pass (replay + adjoint), CUDA-event timed; gradient
    checks against central differences (eps = 1e-6, FP64 forward) along
    alpha and one random direction each for the initial velocities (over the
    configured 200 steps) and positions (over 50 steps: over 200 the loss is
    kinked in the positions, where pairs cross the Lennard-Jones cutoff, and
    the differences do not converge in eps); the mixed adjoint's gradients
    against the FP64 adjoint's."""
    import torch
    from sph import adjoint
    case = adjoint_case()
    case_m = adjoint_case(adjoint_precision="mixed")
    # a small seeded initial velocity field, N(0, 0.01 m/s) per component:
    # at rest every pair sits on the kink of the artificial-viscosity switch
    # (v_ij . x_ij = 0), where the loss has only one-sided derivatives
    torch.manual_seed(3)
    pos = case.positions()
    vel = case.velocities() + 0.01 * torch.randn_like(pos)
    f, fc, b, loss, ga, gp, gv = _adjoint_timed(case, pos, vel, reps)
    fm, fcm, bm, loss_m, gam, gpm, gvm = _adjoint_timed(case_m, pos, vel, reps)
    torch.manual_seed(2)
    dpos = torch.randn_like(pos)
    dpos /= torch.linalg.norm(dpos)
    dvel = torch.randn_like(vel)
    dvel /= torch.linalg.norm(dvel)
    fd = {"alpha": adjoint.central_difference(case, 0.01, pos, vel, d_alpha=1.0),
          "v0_direction": adjoint.central_difference(case, 0.01, pos, vel, d_vel=dvel)}
    grads = {"fp64": {"alpha": ga.item(), "v0_direction": (gv * dvel).sum().item()},
             "mixed": {"alpha": gam.item(), "v0_direction": (gvm * dvel).sum().item()}}
    short = adjoint_case(nsteps=50)
    short_m = adjoint_case(nsteps=50, adjoint_precision="mixed")
    _, _, gp50, gv50 = adjoint.gradients(short, 0.01, pos, vel)
    _, _, gp50m, gv50m = adjoint.gradients(short_m, 0.01, pos, vel)
    fd["x0_direction_50_steps"] = adjoint.central_difference(short, 0.01, pos, vel, d_pos=dpos)
    fd["v0_direction_50_steps"] = adjoint.central_difference(short, 0.01, pos, vel, eps=1e-5, d_vel=dvel)
    grads["fp64"]["x0_direction_50_steps"] = (gp50 * dpos).sum().item()
    grads["fp64"]["v0_direction_50_steps"] = (gv50 * dvel).sum().item()
    grads["mixed"]["x0_direction_50_steps"] = (gp50m * dpos).sum().item()
    grads["mixed"]["v0_direction_50_steps"] = (gv50m * dvel).sum().item()
    # over 200 steps along positions, as a figure only (no convergence in eps)
    x0_200 = {"adjoint": (gp * dpos).sum().item(),
              "central_difference": adjoint.central_difference(case, 0.01, pos, vel, d_pos=dpos)}

    def nrel(a, b):
        return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()

    return {"case": "20k-fluid dam break against the right wall, v0 ~ N(0, 0.01 m/s), 200 PEC steps, dt=5e-5, "
                    "FP64 forward, checkpoints every 20",
            "n_fluid": case.nf, "loss": loss, "forward_ms": f, "forward_with_checkpoints_ms": fc,
            "backward_ms": b, "backward_over_forward": b / f, "forward_plus_backward_over_forward": (fc + b) / f,
            "fd_rel_err": {k: abs(grads["fp64"][k] - d) / abs(d) for k, d in fd.items()},
            "grad_vs_fd": {k: [grads["fp64"][k], d] for k, d in fd.items()},
            "x0_direction_200_steps": x0_200,
            "mixed": {"what": "FP32 pair arithmetic in the adjoint pair product, FP64 forward and replay",
                      "backward_ms": bm, "backward_over_forward": bm / f,
                      "forward_plus_backward_over_forward": (fcm + bm) / f,
                      "fd_rel_err": {k: abs(grads["mixed"][k] - d) / abs(d) for k, d in fd.items()},
                      "vs_fp64_adjoint": {"alpha": abs(gam.item() - ga.item()) / abs(ga.item()),
                                          "positions": nrel(gpm, gp), "velocities": nrel(gvm, gv),
                                          "positions_50_steps": nrel(gp50m, gp50),
                                          "velocities_50_steps": nrel(gv50m, gv50)}}}


def batch_bench(count=256, steps=50, warmup=5):
    """The batched form: 256 seeded dam breaks (column width U(0.5, 2.0) m,
    height U(1.0, 3.0) m, dx U(0.02, 0.05) m, tank 4x by 1.5x), mixed form,
    every instance with its own Courant dt.  Autotunes, captures `steps`
    steps in a CUDA graph and times its replays with CUDA events."""
    import torch
    from sph import batch, scenarios
    cases = scenarios.ensemble(count=count, seed=1)
    E = batch.Ensemble(cases)
    nf = E.fluid_count()
    E.run(warmup)
    E.check()
    t0 = time.perf_counter()
    tune = E.autotune(steps=5, warmup=2)
    tune_s = time.perf_counter() - t0
    g = E.capture(steps)
    g.replay()  # warm replay
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3
    ev0.record()
    for _ in range(reps):
        g.replay()
    ev1.record()
    torch.cuda.synchronize()
    el = ev0.elapsed_time(ev1) / 1e3
    E.check()
    # the same steps launched eagerly, for the graph's effect
    ev0.record()
    E.run(steps)
    ev1.record()
    torch.cuda.synchronize()
    el_eager = ev0.elapsed_time(ev1) / 1e3
    sizes = [int(np.sum(pa["label"] == 0)) for pa, _ in cases]
    best = min(tune, key=tune.get)
    return {"case": "%d dam breaks, width U(0.5,2.0) m, height U(1.0,3.0) m, dx U(0.02,0.05) m, seed 1, "
                    "mixed form, PEC, Courant 0.3 per instance" % count,
            "instances": count, "n_particles": E.n, "n_fluid": nf, "fluid_per_instance": [min(sizes), max(sizes)],
            "value": nf * steps * reps / el, "unit": UNIT, "ms_per_step": el / (steps * reps) * 1e3,
            "eager_ms_per_step": el_eager / steps * 1e3, "graph_steps": steps,
            "autotune": {"chosen": {"tile_shift": best[0], "tile_blocks_per_sm": best[1]},
                         "ms_per_step": {"%d/%d" % k: v for k, v in sorted(tune.items())}, "seconds": tune_s}}


def accuracy(names):
    """Mixed form against the GPU's own FP64 path (the oracle for the mixed
    form) from identical states: the per-step derivative error of one
    evaluation (drho, ax, ay: norm-wise relative error over fluid) and the
    trajectory error (x, y, vx, vy, rho) after 1, 10 and 100 PEC steps.  One
    JSON line per workload."""
    import torch
    from sph import build as sph_build
    sph_build.build()
    from sph import core

    def rel(a, b):
        a = a.double()
        b = b.double()
        n = torch.linalg.norm(b).item()
        d = torch.linalg.norm(a - b).item()
        return d / n if n > 0 else d

    for name in names:
        wl = workload(name)
        f = torch.from_numpy(wl["pa"]["label"] == 0).cuda()
        out = {"workload": name + ": " + wl["desc"], "n_fluid": int(f.sum().item())}
        st = {}
        for prec in ("fp64", "mixed"):
            dp, wc, cfg, ws = prepare(wl, prec)
            core.compute(dp, wc, cfg, ws)
            ws.check()
            st[prec] = (dp, wc, cfg, ws)
        d64, dmx = st["fp64"][0], st["mixed"][0]
        out["derivative"] = {k: rel(dmx.fields[k][f], d64.fields[k][f]) for k in ("drho", "ax", "ay")}
        traj = {}
        done = 0
        for s in (1, 10, 100):
            for prec in ("fp64", "mixed"):
                dp, wc, cfg, ws = st[prec]
                core.run(dp, wc, cfg, ws, s - done)
                ws.check()
            done = s
            traj[str(s)] = {k: rel(dmx.fields[k][f], d64.fields[k][f]) for k in ("x", "y", "vx", "vy", "rho")}
        out["trajectory"] = traj
        print(json.dumps(out), flush=True)
        del st, d64, dmx
        torch.cuda.empty_cache()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dambreak1m")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-extras", action="store_true", help="skip the FP64 / e2e / CPU / profile passes")
    ap.add_argument("--accuracy", default=None,
                    help="comma-separated workloads: mixed vs FP64 derivative and trajectory errors, then exit")
    ap.add_argument("--batch", action="store_true",
                    help="batched form only: 256-instance ensemble in a CUDA graph, then exit")
    ap.add_argument("--adjoint", action="store_true",
                    help="differentiation form only: adjoint/forward cost and finite-difference checks, then exit")
    args = ap.parse_args()
    if args.accuracy:
        accuracy(args.accuracy.split(","))
        return
    if args.adjoint:
        from sph import build as sph_build
        sph_build.build()
        print(json.dumps(adjoint_cost()))
        return
    if args.batch:
        from sph import build as sph_build
        sph_build.build()
        print(json.dumps(batch_bench()))
        return
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args, args.workload)
        return

    import torch
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from sph import build as sph_build
    sph_build.build()
    from sph import core

    wl = workload(args.workload)
    nfluid = int(np.sum(wl["pa"]["label"] == 0))
    dp, wc, cfg, ws = prepare(wl, args.precision)
    core.run(dp, wc, cfg, ws, args.warmup)
    ws.check()

    def barrier():
        if world > 1:
            dist.barrier()

    # the timed steps run as replays of CUDA graphs of sph_run (captured here,
    # outside the timed region; capturing runs one step per graph)
    graphs = make_graphs(core, dp, wc, cfg, ws, args.steps)
    ws.check()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier()
    el = time_graph_steps(graphs)
    barrier()
    clk = clocks.stop()
    ws.check()
    el, value = replica_value(el, nfluid, args.steps, world, "cuda")
    # per step: k_bounds (corrector + predictor + bounds + grid), k_keys,
    # k_scan_cells, k_scatter_rank, k_cellsort (+ records), then
    # k_pair_tiles + k_pair_list (mixed) or k_pair (FP64); per sph_run call
    # also the initial TimeStep and the last corrector
    launches_per_step = 7 if args.precision == "mixed" else 6
    gsteps, reps, rem = graph_plan(args.steps)
    launches = launches_per_step * args.steps + 2 * (reps + (1 if rem else 0))
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 pair / f64 state" if args.precision == "mixed" else "f64",
           "data": "synthetic",
           "config": arm_config(args.workload, wl),
           "precision": args.precision,
           "l2": "inputs larger than L2 (state + records ~%.0f MB per step)"
                 % ((dp.n * (19 * 8 + 1) + ws.buf.numel()) / 1e6),
           "parallelism": "replicas" if world > 1 else "single GPU",
           "clocks": clk, "gpu_launches": launches,
           "timing": "CUDA events around %d replays of a %d-step CUDA graph of sph_run%s"
                     % (reps, gsteps, " and one of %d steps" % rem if rem else "")}
    del graphs
    if not args.no_extras and rank == 0:
        hbm, peak_kind = peaks()
        kprof = min(args.steps, 50)
        stages = core.run_profiled(dp, wc, cfg, ws, kprof)
        pair_s = stages["pair"] / 1e3 / kprof
        step_s = sum(stages.values()) / 1e3 / kprof
        ach = dp.n * PAIR_BYTES / pair_s / 1e9
        out["stages_ms_per_step"] = {k: v / kprof for k, v in stages.items()}
        traffic = TRAFFIC_FROM_PROFILE.get((args.workload, args.precision))
        out["roofline"] = {"bound": "hbm",
                           "kernel": "k_pair_tiles + k_pair_list" if args.precision == "mixed" else "k_pair (FP64)",
                           "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                           "peak_kind": peak_kind, "traffic": traffic[0] * dp.n if traffic else None,
                           "traffic_source": ("from_profile: ncu dram__bytes_read.sum + dram__bytes_write.sum, "
                                              + traffic[1]) if traffic else None,
                           "algorithmic_bytes_per_launch": dp.n * PAIR_BYTES,
                           "step_achieved_gbs": dp.n * STEP_BYTES / step_s / 1e9,
                           "limiter_from_profile": LIMITER_FROM_PROFILE.get(args.precision)}
        # the GPU's own FP64 path on the same workload, timed the same way
        # (replays of a captured CUDA graph of sph_run)
        if args.precision == "mixed":
            dp64, wc64, cfg64, ws64 = prepare(wl, "fp64")
            core.run(dp64, wc64, cfg64, ws64, 3)
            k64 = max(20, min(args.steps, 100))
            g64 = make_graphs(core, dp64, wc64, cfg64, ws64, k64)
            ws64.check()
            el64 = time_graph_steps(g64)
            ws64.check()
            v64 = nfluid * k64 / el64
            out["fp64"] = {"value": v64, "steps": k64, "ms_per_step": el64 / k64 * 1e3,
                           "timing": "CUDA events around a graph replay of %d steps of sph_run" % k64,
                           "mixed_over_fp64": value / world / v64}
            del g64, dp64, ws64
        # end to end through host buffers
        ke = max(3, min(args.steps, 100))
        el_e, h2d, d2h = e2e_steps(core, dp, wc, cfg, ws, ke, wl["pa"])
        out["e2e"] = {"value": nfluid * ke / el_e, "unit": UNIT,
                      "how": "sph_run one step per call on the state held in pinned host memory; 11 fields and "
                             "the labels up, 9 fields down every step, on two copy streams into two "
                             "alternating device copies of the state",
                      "h2d_bytes_per_step": h2d,
                      "d2h_bytes_per_step": d2h, "steps": ke}
        del dp, ws
        torch.cuda.empty_cache()
        out["solver_run"] = solver_run_bench(wl, args.precision)
        out["cpu_baseline"] = cpu_baseline(args.workload, wl)
        torch.cuda.empty_cache()
        out["adjoint"] = adjoint_cost()
        torch.cuda.empty_cache()
        out["batched"] = batch_bench()
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

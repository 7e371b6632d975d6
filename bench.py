#!/usr/bin/env python
"""Benchmark of the Lagrangian Voronoi time step on GB300.

Default workload: the double shear layer, periodic unit square, 2048 x 2048
= 4,194,304 seeds on a jittered lattice (SplitMix64 seed 12345,
U(-0.1h, 0.1h)), u = tanh(80(y - 1/4)) for y <= 1/2 else tanh(80(3/4 - y)),
v = 0.05 sin(2 pi x), Re = 10,000 (mu = 1e-4), ideal gas (gamma = 1.4,
P0 = 100/gamma), dt = 0.1 dr / 2, FP64 state and geometry.  One step is the
reference's step! (examples/doubleshear.jl: move!, ideal_eos!,
find_pressure! with 10 fixed-point sweeps, pressure_step!, find_D!,
viscous_step!, find_dv!, relaxation_step!) with both remeshes.  The
pressure sweeps are solved by the learned-preconditioned mixed-precision
solver (FP32 inner CG inside FP64 iterative refinement) to an FP64 residual
||b - A x|| <= 1e-8 ||b||; every timed sweep is checked to have converged.
--config selects another of the five flows (gresho 50^2, taylor_green 256^2,
rayleigh_taylor 512x1024, cavity 1024^2, double_shear 2048^2), --solver the
pressure solver.

Metric: particle-steps/s (particles x steps / device time of the steps).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--config NAME] [--solver jacobi_pcg|mixed_ir|learned_pcg]

--impl reference times the CPU restatement of the reference's algorithm
(the oracle, with the reference's solver settings: MINRES atol = rtol =
1e-6, itmax = 1000) on all host cores for the same workload.  With --gpus N
> 1 (torchrun) every rank runs an independent replica of the workload.
"""
import argparse
import atexit
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC = "particle-steps/s at 1 GB300; pressure solve ms & CG iters, learned vs plain PCG @1e-8"
UNIT = "particle-steps/s"
L2_BYTES = 129 << 20
L2_FLUSH_BYTES = 512 << 20
# bytes of device state per particle (x, v, dv, momentum, D, GP, e, P, rho,
# c2, mass, energy, quality, mu, phase), the mesh and the operator excluded
STATE_BYTES_PER_PARTICLE = 196

# (default lattice nx, ny) of each flow: the sizes of the five workloads
CONFIG_SIZES = {"gresho": (50, 50), "taylor_green": (256, 256), "rayleigh_taylor": (512, 1024),
                "cavity": (1024, 1024), "double_shear": (2048, 2048)}


# the step counts the five workloads are specified with
CONFIG_STEPS = {"gresho": 100, "taylor_green": 200, "rayleigh_taylor": 300, "cavity": 500, "double_shear": 500}


class Workload:
    def __init__(self, name, nx=None):
        import workloads as W
        dnx, dny = CONFIG_SIZES[name]
        nx = int(nx) if nx else dnx
        ny = nx * dny // dnx
        self.name = name
        self.flow = W.rayleigh_taylor(nx, ny) if name == "rayleigh_taylor" else W.FLOWS[name](nx)
        if name == "taylor_green":
            # the 256 x 256 workload has dt = 5e-4; other sizes keep its CFL number
            self.flow.dt = 5e-4 * 256.0 / nx
        self.nx, self.ny = nx, ny
        self.n = nx * ny
        self.label = f"{name}_{nx}x{ny}"

    def describe(self):
        f = self.flow
        d = {"workload": self.label, "particles": self.n, "dt": f.dt, "periodic": bool(f.periodic)}
        if f.eos == "stiffened":
            d["eos"] = f"stiffened gamma={f.gamma} P0={f.P0:.6g}"
        elif f.eos == "ideal":
            d["eos"] = f"ideal gamma={f.gamma}"
        else:
            d["eos"] = "incompressible (c2 = Inf)"
        d["mu"] = getattr(f, "mu", None) if self.name != "rayleigh_taylor" else f"rho/{f.Re}"
        d["artificial_viscosity"] = bool(f.artificial_viscosity)
        if f.walls is not None:
            d["walls"] = {str(k): v for k, v in f.walls.items()} or "no-slip"
        return d


def load_package():
    import __graft_entry__ as ge
    ge.build()
    return ge._package()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, v):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region.
    The sampler is started, and its first sample awaited, before the region
    begins, so that its start-up does not overlap the timed work."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.marks = []
        self._first = threading.Event()

    def _reader(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line))
            self._first.set()

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return self
        threading.Thread(target=self._reader, daemon=True).start()
        atexit.register(self.stop)  # never leave the sampler running
        self._first.wait(5.0)
        return self

    def mark(self):
        self.marks.append(time.perf_counter())

    def stop(self):
        if self.proc is not None and self.proc.poll() is None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0=None, t1=None):
        rows = []
        for ts, line in self.lines:
            if t0 is not None and not (t0 <= ts <= t1 + 0.25):
                continue
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for _, _, r in rows for k in range(4) if r[k].lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------ our arm

# the fields that carry a state from one step to the next (the mesh follows
# from x by remesh)
STATE_FIELDS = ["x", "v", "e", "P", "rho", "c2", "dv", "mass", "momentum", "energy", "phase", "quality", "D", "mu"]


def setup_grid(lv, wl):
    import harness as H
    from lvgpu import populate as pop
    import workloads as W
    fl = wl.flow
    x = H.seeds(pop, fl)
    g = lv.VoronoiGrid(lv.Rectangle(fl.xlims, fl.ylims), fl.dr, xperiodic=fl.periodic, yperiodic=fl.periodic)
    g.push(x)
    lv.remesh(g)
    for k, v in W.initial_fields(fl, g["x"], g["area"]).items():
        g[k] = v
    return g


def gpu_step(lv, g, solver, fl, snapshot=False, stats=False):
    """The reference's step! of the flow (tests/workloads.py:step_sequence),
    through the package's public API; returns the per-sweep solver stats
    when stats=True (which synchronises)."""
    import workloads as W
    dt, seq = W.step_sequence(fl)
    st = None
    for op, kw in seq:
        if op == "move":
            lv.move(g, dt)
        elif op == "gravity_step":
            lv.gravity_step(g, kw["g"], dt)
        elif op == "stiffened_eos":
            lv.stiffened_eos(g, kw["gamma"], kw["P0"])
        elif op == "ideal_eos":
            lv.ideal_eos(g, kw["gamma"])
        elif op == "find_pressure":
            # the examples call find_pressure!(solver, dt) with zero_vbc
            st = lv.find_pressure(solver, dt, 10, stats=stats)
            if snapshot:
                assert lv._lib.load().lv_learn_add_system(g._ctx) == 0
        elif op == "pressure_step":
            lv.pressure_step(g, dt)
        elif op == "find_D":
            lv.find_D(g)
        elif op == "viscous_step":
            lv.viscous_step(g, dt, kw["artificial_viscosity"])
        elif op == "bdary_friction":
            lv.bdary_friction(g, kw["walls"], dt)
        elif op == "find_dv":
            lv.find_dv(g, dt)
        elif op == "multiphase_projection":
            lv.multiphase_projection(lv.MultiphaseSolver(g))
        elif op == "relaxation_step":
            lv.relaxation_step(g, dt)
        else:
            raise ValueError(op)
    return st


def unconverged(L, g):
    n = C.c_int64()
    assert L.lv_solver_unconverged(g._ctx, C.byref(n)) == 0
    return n.value


def solver_comparison(lv, L, g, fl, steps, train_info):
    """Pressure solve of the same workload with each solver: device ms of the
    solve kernels (+ operator/RHS/factor kernels) and CG iterations per step."""
    fam = lv._lib.KERNEL_FAMILIES
    out = {}
    for method in ("jacobi_pcg", "mixed_ir", "learned_pcg", "minres"):
        # minres: the reference's own solve (tol 1e-6 absolute + relative, itmax 1000)
        solver = lv.PressureSolver(g, method=method, tol=None if method == "minres" else 1e-8)
        gpu_step(lv, g, solver, fl)  # settle
        g.synchronize()
        L.lv_kernel_timing(g._ctx, 1)
        for f in fam.values():
            L.lv_kernel_time(g._ctx, f, None, None, 1)
        s0, i0 = C.c_int64(), C.c_int64()
        L.lv_solver_counters(g._ctx, C.byref(s0), C.byref(i0))
        u0 = unconverged(L, g)
        fallbacks = 0
        per_sweep = []
        for _ in range(steps):
            st = gpu_step(lv, g, solver, fl, stats=True)
            fallbacks += sum(1 for rec in st if method == "learned_pcg" and rec[3] != 2)
            per_sweep.append([rec[0] for rec in st])
        s1, i1 = C.c_int64(), C.c_int64()
        L.lv_solver_counters(g._ctx, C.byref(s1), C.byref(i1))
        ms = {}
        for name, f in fam.items():
            nl, t = C.c_int64(), C.c_double()
            L.lv_kernel_time(g._ctx, f, C.byref(nl), C.byref(t), 1)
            ms[name] = t.value
        L.lv_kernel_timing(g._ctx, 0)
        out[method] = {"solve_ms_per_step": (ms["pcg"] + ms["rhs"] + ms["learn"]) / steps,
                       "factor_ms_per_step": ms["learn"] / steps,
                       "pcg_kernel_ms_per_step": ms["pcg"] / steps,
                       "cg_iters_per_step": (i1.value - i0.value) / steps,
                       "cg_iters_per_sweep_last_step": per_sweep[-1],
                       "us_per_iteration": 1e3 * ms["pcg"] / max(i1.value - i0.value, 1),
                       "unconverged_sweeps": unconverged(L, g) - u0}
        if method == "learned_pcg":
            out[method]["fallbacks_to_jacobi"] = fallbacks
    out["learned_pcg"]["training"] = train_info
    j, lrn = out["jacobi_pcg"], out["learned_pcg"]
    # solve: the solver kernels and the learned factor; find_pressure: also the
    # right-hand side passes every method shares
    lin = lambda r: r["pcg_kernel_ms_per_step"] + r["factor_ms_per_step"]
    out["learned_vs_plain"] = {"iteration_ratio": j["cg_iters_per_step"] / max(lrn["cg_iters_per_step"], 1e-9),
                               "solve_time_ratio": lin(j) / max(lin(lrn), 1e-9),
                               "find_pressure_time_ratio": j["solve_ms_per_step"] / max(lrn["solve_ms_per_step"], 1e-9)}
    return out


def train_learned(L, g, args):
    t_tr = time.perf_counter()
    train_steps = args.train_steps if (args.solver == "learned_pcg" or not args.no_compare) else 0
    losses = np.zeros(max(train_steps, 1), np.float32)
    assert L.lv_learn_init(g._ctx, 1234) == 0
    assert L.lv_learn_set_pattern(g._ctx, args.learn_hops) == 0
    if train_steps:
        assert L.lv_learn_train(g._ctx, train_steps, args.train_lr, args.train_probes, 99,
                                losses.ctypes.data_as(C.POINTER(C.c_float))) == 0
    return {"systems": int(L.lv_learn_num_systems(g._ctx)), "adam_steps": train_steps,
            "objective": "fsai-kaporin" if args.train_probes == 0 else f"hutchinson x{args.train_probes}",
            "pattern": "lower triangle" if args.learn_hops == 1 else "lower triangle + two-hop",
            "lr": args.train_lr, "seconds": time.perf_counter() - t_tr, "loss_first": float(losses[0]),
            "loss_last": float(losses[-10:].mean())}


def full_run(args, wl):
    """The whole run of a workload (its specified step count, or --full-steps)
    through the public API: warm-up steps with the Jacobi mixed solver, which
    also give the learned preconditioner its training systems, then the
    remaining steps with --solver.  Reports the wall time per step, the
    solves that missed the tolerance, the CG iterations, and the totals of
    mass, momentum, energy and kinetic energy every 50 steps (with their
    drift over the run).  Not a bench line: a check that the run completes."""
    lv = load_package()
    L = lv._lib.load()
    fl = wl.flow
    g = setup_grid(lv, wl)
    total = args.full_steps or CONFIG_STEPS[wl.name]
    learned = args.solver == "learned_pcg"
    tol = None if args.solver == "minres" else 1e-8
    solver = lv.PressureSolver(g, method="mixed_ir" if learned else args.solver, tol=tol)

    def totals(step):
        m, v, e, P, area = g["mass"], g["v"], g["e"], g["P"], g["area"]
        return {"step": step, "mass": float(m.sum()), "momentum": [float((m * v[:, 0]).sum()), float((m * v[:, 1]).sum())],
                "energy": float((m * e).sum()), "kinetic": float(0.5 * (m * (v * v).sum(axis=1)).sum()),
                "v_max": float(np.abs(v).max()), "P_range": [float(P.min()), float(P.max())],
                "area_min_rel": float(area.min() / area.mean()),
                "finite": bool(np.isfinite(v).all() and np.isfinite(e).all() and np.isfinite(g["x"]).all())}

    rec = [totals(0)]
    warm = min(max(args.warmup, 3), total)
    t_run = 0.0
    t0 = time.perf_counter()
    for _ in range(warm):
        gpu_step(lv, g, solver, fl, snapshot=learned)
    g.synchronize()
    t_run += time.perf_counter() - t0
    train = train_learned(L, g, args) if learned else None
    solver = lv.PressureSolver(g, method=args.solver, tol=tol)
    u0 = unconverged(L, g)
    s0, i0 = C.c_int64(), C.c_int64()
    L.lv_solver_counters(g._ctx, C.byref(s0), C.byref(i0))
    step = warm
    failure = None
    while step < total and failure is None:
        seg = min(50 - step % 50, total - step)
        t0 = time.perf_counter()
        try:
            for _ in range(seg):
                gpu_step(lv, g, solver, fl)
            g.synchronize()
        except lv.LvError as err:  # the run stops: report where
            failure = {"error": str(err), "segment": [step, step + seg]}
            break
        t_run += time.perf_counter() - t0
        step += seg
        rec.append(totals(step))
    s1, i1 = C.c_int64(), C.c_int64()
    L.lv_solver_counters(g._ctx, C.byref(s1), C.byref(i1))
    rel = lambda a, b: (b - a) / abs(a) if a else b - a
    first, last = rec[0], rec[-1]
    return {"mode": "full_run", "workload": wl.label, "particles": wl.n, "steps": step, "failure": failure,
            "solver": args.solver,
            "wall_ms_per_step": 1e3 * t_run / total, "unconverged_sweeps": unconverged(L, g) - u0,
            "solves": s1.value - s0.value, "cg_iters_per_step": (i1.value - i0.value) / max(total - warm, 1),
            "all_finite": all(r["finite"] for r in rec), "training": train,
            "drift": {"mass": rel(first["mass"], last["mass"]), "energy": rel(first["energy"], last["energy"]),
                      "momentum_abs": [last["momentum"][0] - first["momentum"][0],
                                       last["momentum"][1] - first["momentum"][1]],
                      "kinetic": rel(first["kinetic"], last["kinetic"])},
            "totals": rec}


def run_ours(args, world, rank, local, wl):
    import torch
    torch.cuda.set_device(local)
    lv = load_package()
    L = lv._lib.load()
    fl = wl.flow
    N = wl.n
    g = setup_grid(lv, wl)
    # warm-up with the Jacobi mixed solver: its iteration count is the
    # learned solver's fallback reference
    solver = lv.PressureSolver(g, method="mixed_ir" if args.solver == "learned_pcg" else args.solver,
                               tol=None if args.solver == "minres" else 1e-8)
    stream = torch.cuda.ExternalStream(L.lv_stream(g._ctx), device=local)
    # between timed steps an L2 flush when the state fits in L2
    flush_l2 = N * STATE_BYTES_PER_PARTICLE < L2_BYTES
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}") if flush_l2 else None
    if flush is not None:
        # the first fill loads torch's kernel (~0.25 s of host time): once here, outside the timed steps
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
    # warm-up steps also snapshot the pressure operators the learned
    # preconditioner is trained on (the solver's own systems)
    for _ in range(args.warmup):
        gpu_step(lv, g, solver, fl, snapshot=True)
    g.synchronize()
    train_info = train_learned(L, g, args)

    solver = lv.PressureSolver(g, method=args.solver, tol=None if args.solver == "minres" else 1e-8)
    # the state the passes start from: each pass restores it, forgets the
    # sweep-guess history and runs one untimed step with the timed solver, so
    # the timed, the instrumented and the end-to-end passes run the same steps
    state = g.get_many(STATE_FIELDS)

    def restore():
        g.set_many(dict(zip(STATE_FIELDS, state)))
        lv.remesh(g)
        assert L.lv_solver_forget(g._ctx) == 0
        gpu_step(lv, g, solver, fl)
        g.synchronize()

    # events around the L2 flush (outside the step events), to report its time
    ev_f = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]

    def between_steps(ev0, k=None):
        with torch.cuda.stream(stream):
            if flush is not None:
                if k is not None:
                    ev_f[k][0].record(stream)
                flush.zero_()
                if k is not None:
                    ev_f[k][1].record(stream)
            ev0.record(stream)

    restore()

    # ---- timed region: K steps, device time from events on the library's stream
    # (an L2 flush between steps outside the events when the state fits in L2);
    # no per-family instrumentation inside it
    fam = lv._lib.KERNEL_FAMILIES
    s0, i0 = C.c_int64(), C.c_int64()
    L.lv_solver_counters(g._ctx, C.byref(s0), C.byref(i0))
    u0 = unconverged(L, g)
    launches0 = g.launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clk = ClockSampler(local).start()
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        between_steps(ev[k][0], k)
        gpu_step(lv, g, solver, fl)
        with torch.cuda.stream(stream):
            ev[k][1].record(stream)
    g.synchronize()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    wall = t1 - t0
    timed_span = (t0, t1)
    barrier(world)
    launches = g.launch_count() - launches0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    flush_ms = float(sum(a.elapsed_time(b) for a, b in ev_f)) / args.steps if flush is not None else 0.0
    dev_ms = float(sum(step_ms))
    s1, i1 = C.c_int64(), C.c_int64()
    L.lv_solver_counters(g._ctx, C.byref(s1), C.byref(i1))
    solves, iters = s1.value - s0.value, i1.value - i0.value
    n_unconverged = unconverged(L, g) - u0
    if n_unconverged:
        raise RuntimeError(f"{n_unconverged} of {solves} timed pressure sweeps did not reach the 1e-8 residual")
    max_ms = allmax(world, dev_ms)
    # ---- the same number of steps again with every kernel family bracketed by
    # CUDA events (lv_kernel_timing): the per-family device times and the
    # roofline of the dominant kernel come from this pass
    restore()
    L.lv_kernel_timing(g._ctx, 1)
    for f in fam.values():
        L.lv_kernel_time(g._ctx, f, None, None, 1)
    L.lv_solver_counters(g._ctx, C.byref(s0), C.byref(i0))
    ev_i = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k in range(args.steps):
        between_steps(ev_i[k][0])
        gpu_step(lv, g, solver, fl)
        with torch.cuda.stream(stream):
            ev_i[k][1].record(stream)
    g.synchronize()
    torch.cuda.synchronize()
    instr_ms = float(sum(a.elapsed_time(b) for a, b in ev_i))
    L.lv_solver_counters(g._ctx, C.byref(s1), C.byref(i1))
    iters_i = i1.value - i0.value  # CG iterations of the instrumented pass
    kt = {}
    for name, f in fam.items():
        nl, ms = C.c_int64(), C.c_double()
        L.lv_kernel_time(g._ctx, f, C.byref(nl), C.byref(ms), 1)
        kt[name] = (nl.value, ms.value)
    L.lv_kernel_timing(g._ctx, 0)

    # ---- end to end through the public API: per step, host (pinned) -> device
    # upload of the evolving state, the step, device -> host read of the result
    # (from the same starting state as the timed steps)
    restore()
    # two sets of pinned buffers: the outputs of one step are the inputs of the next
    in_names = ("v", "e", "P", "mass")
    out_names = ["x", "v", "e", "P", "mass"]
    bufs = [{k: torch.empty(g.get(k).shape, dtype=torch.float64, pin_memory=True).numpy() for k in out_names}
            for _ in range(2)]
    for k in out_names:
        bufs[1][k][...] = g.get(k)
    h2d = sum(bufs[0][k].nbytes for k in in_names)
    d2h = sum(bufs[0][k].nbytes for k in out_names)
    e2e_steps = max(1, args.steps)
    u0 = unconverged(L, g)
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        src, dst = bufs[(k + 1) % 2], bufs[k % 2]
        g.set_many({n_: src[n_] for n_ in in_names})  # one call, one synchronisation for the uploads
        gpu_step(lv, g, solver, fl)
        g.get_many(out_names, out=[dst[n_] for n_ in out_names])
    g.synchronize()
    e2e_t1 = time.perf_counter()
    e2e_s = allmax(world, e2e_t1 - t0)
    # the sampler ran on through the instrumented and end-to-end passes
    clk.stop()
    e2e_span = (t0, e2e_t1)
    e2e_unconverged = unconverged(L, g) - u0
    if e2e_unconverged:
        raise RuntimeError(f"{e2e_unconverged} end-to-end pressure sweeps did not reach the 1e-8 residual")

    comparison = solver_comparison(lv, L, g, fl, 3, train_info) if not args.no_compare else None
    if rank != 0:
        return None
    value = world * N * args.steps / (max_ms / 1e3)
    e2e_value = world * N * e2e_steps / e2e_s
    ms_per_step = max_ms / args.steps
    clocks = clk.summary(*timed_span)
    e2e_clocks = clk.summary(*e2e_span)

    # ---- roofline of the dominant kernel family
    # interior faces (= off-diagonal nonzeros of the pressure operator)
    nfc = C.c_int64()
    rc = L.lv_get_faces(g._ctx, C.byref(nfc), None, None, None, None, None, None)
    F = nfc.value if rc == 0 and nfc.value > 0 else 6 * N
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    # per CG iteration, the bytes a streaming implementation moves: FP64
    # Jacobi-PCG 12 B per nonzero (value + column) + 60 B per row (vectors);
    # FP32 inner CG 8 B per nonzero + 28 B per row, and the learned M^-1:
    # about 10 more nonzeros per row (explicit, the staged solver) or, in the
    # factored form of the streaming solver (systems beyond 152 x 1024 rows),
    # two passes over ~3 entries of G per row with their vectors (92 B per
    # row).  The register-resident kernels keep the matrix on chip, so these
    # are upper bounds of their DRAM traffic.
    if args.solver == "jacobi_pcg":
        per_it = 12 * (F + N) + 60 * N
    else:
        m_bytes = (92 * N if N > 152 * 1024 else 80 * N) if args.solver == "learned_pcg" else 0
        per_it = 8 * (F + N) + 28 * N + m_bytes
    pcg_bytes = iters * per_it
    clip_unit = 16 * N + 28 * F + 28 * N  # per remesh: read x; write nbr, lrr, mid; area, centroid, nface
    fams = {"pcg": iters_i * per_it, "clip": kt["clip"][0] * clip_unit}  # bytes of the instrumented pass
    # compulsory bytes of the whole step (per kernel family, the per-unit
    # counts above): re-bin 32N and clip 16N + 28F + 28N per remesh; CSR
    # assembly 28F + 68N + 12 nnz per find_pressure; RHS 28F + 80N per sweep;
    # the CG iterations; ten other face passes of 28F + 40N
    remeshes = kt["clip"][0]
    step_bytes = (remeshes * (32 * N + clip_unit)
                  + args.steps * (28 * F + 68 * N + 12 * (F + N))
                  + solves * (28 * F + 80 * N)
                  + pcg_bytes
                  + args.steps * 10 * (28 * F + 40 * N))
    step_gbs = step_bytes / (dev_ms / 1e3) / 1e9
    dom = max(("pcg", "clip"), key=lambda k: kt[k][1])
    dom_ms = kt[dom][1]
    dom_launches = max(kt[dom][0], 1)
    achieved = (fams[dom] / dom_launches) / ((dom_ms / dom_launches) / 1e3) / 1e9 if dom_ms > 0 else 0.0
    if dom == "pcg":
        if args.solver == "minres":
            kname = "k_minres"
        elif args.solver == "jacobi_pcg":
            kname = "k_pcg_reg<2>" if N <= 2 * 128 * 2 * 152 else "k_pcg"
        else:
            staged = 1 if args.solver == "learned_pcg" else 0
            kname = (f"k_fcg<1,{staged}>" if N <= 152 * 512 else
                     (f"k_fcg<2,{staged}>" if N <= 152 * 1024 else f"k_big<{'true' if staged else 'false'}>"))
    else:
        kname = "k_clip"
    roofline = {"kernel": kname, "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak,
                "traffic": read_traffic(wl.label, dom, kname,
                                        {"per_polygon": N, "per_iteration": iters_i / max(kt["pcg"][0], 1)}),
                "peak_source": peak_src, "units_per_launch": N if dom == "clip" else None,
                "algorithmic_bytes_per_launch": fams[dom] / dom_launches,
                "launch_ms": dom_ms / dom_launches, "note": ROOFLINE_NOTE.get(kname, "")}
    if dom == "clip":
        # the bound that applies: FP64 operations per polygon over the measured
        # FP64 rate of this part (a microbenchmark: 0.60 T FP64 thread
        # operations per second)
        roofline["fp64"] = {"ops_per_polygon": CLIP_FP64_OPS, "peak_ops_per_s": FP64_OPS_PEAK,
                            "frac": CLIP_FP64_OPS * N / (dom_ms / dom_launches / 1e3) / FP64_OPS_PEAK}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 (fp32 inner CG)" if args.solver != "jacobi_pcg" else "f64",
        "data": "synthetic (seeded jittered lattice, analytic initial field)",
        "config": dict(wl.describe(), **{
            "solver": SOLVER_DESC[args.solver] + ("" if args.solver == "minres" else
                                                  ", tol 1e-8 (FP64 residual)") + ", 10 sweeps/step",
            "parallelism": f"replicas x{world}",
            "l2": ("512 MiB buffer written between timed steps (the state fits in L2)" if flush_l2 else
                   f"no flush: the state ({N * STATE_BYTES_PER_PARTICLE / 1e9:.2f} GB) is larger than L2")}),
        "pressure": {"solve_ms_per_step": (kt["pcg"][1] + kt["rhs"][1] + kt["learn"][1]) / args.steps,
                     "pcg_ms_per_step": kt["pcg"][1] / args.steps, "cg_iters_per_step": iters / args.steps,
                     "solves": solves, "unconverged_sweeps": n_unconverged,
                     "e2e_unconverged_sweeps": e2e_unconverged, "solvers": comparison},
        "kernel_ms_per_step": {k: v[1] / args.steps for k, v in kt.items()},
        "instrumented_pass": {"ms_per_step": instr_ms / args.steps, "cg_iters_per_step": iters_i / args.steps},
        "full_step_roofline": {"bytes_per_step": step_bytes / args.steps, "achieved": step_gbs, "peak": hbm_peak,
                               "unit": "GB/s", "frac": step_gbs / hbm_peak},
        "roofline": roofline,
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "clocks": e2e_clocks},
        "gpu_launches": launches,
        "wall_s_timed": wall,
        "host_gap_ms_per_step": (wall * 1e3 - dev_ms) / args.steps,
        "l2_flush_ms_per_step": flush_ms,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, wl)
    return line


# FP64 thread operations per polygon of k_clip (ncu: dadd + dmul + dfma thread
# instructions per polygon of one remesh of the 1024x1024 double shear) and
# this part's FP64 rate
CLIP_FP64_OPS = 1074
FP64_OPS_PEAK = 0.60e12

# what bounds each dominant kernel instead of HBM (from the ncu summaries in profiles/)
ROOFLINE_NOTE = {
    "k_clip": "FP64-pipe and FP64-latency bound (profiles/k_clip_*.md); its compulsory traffic is 212 B per"
              " polygon, so its HBM fraction is small by construction: see roofline.fp64",
    "k_fcg<1,1>": "synchronisation-latency bound: a grid-wide reduction and a neighbour exchange per CG iteration"
                  " (profiles/k_fcg_taylor_green_256.md)",
    "k_fcg<1,0>": "synchronisation-latency bound (profiles/k_fcg_taylor_green_256.md)",
}

SOLVER_DESC = {
    "jacobi_pcg": "jacobi_pcg fp64",
    "mixed_ir": "mixed_ir: fp32 jacobi CG inside fp64 refinement",
    "learned_pcg": "learned_pcg: fp32 CG preconditioned by the trained factor inside fp64 refinement",
    "minres": "minres fp64 (the reference's solve: atol = rtol = 1e-6, itmax 1000)",
}


def read_traffic(workload, family, kernel, units):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum)
    of the kernel on this workload, from the committed ncu summary table
    profiles/traffic.txt (columns: family workload bytes kernel note...),
    whose bytes are per launch or, when the note starts with per_polygon or
    per_iteration, per unit: units[that unit] scales them to a launch."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    for ln in open(path):
        f = ln.split()
        if len(f) >= 4 and not ln.startswith("#") and f[0] == family and f[1] == workload and f[3] == kernel:
            unit = f[4].rstrip(";") if len(f) > 4 else ""
            if unit in units:
                return float(f[2]) * units[unit]
            return float(f[2])
    return None


# ------------------------------------------------------------ reference arm

def oracle_grid(wl):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import lvref
    import harness as H
    import workloads as W
    from importlib import util
    fl = wl.flow
    spec = util.spec_from_file_location("pop_b", os.path.join(ROOT, "lagrangianvoronoi.jl_gb300", "populate.py"))
    pop = util.module_from_spec(spec)
    spec.loader.exec_module(pop)
    lvref.build()
    threads = lvref.set_threads(os.cpu_count() or 1)
    x = H.seeds(pop, fl)
    og = lvref.OracleGrid(fl.xlims, fl.ylims, fl.dr, len(x), xperiodic=fl.periodic, yperiodic=fl.periodic,
                          max_edges=20)
    og.set("x", x)
    assert og.remesh() == 0
    for k, v in W.initial_fields(fl, x, og.edges()["area"]).items():
        og.set(k, v)
    return og, threads


def oracle_step(og, wl):
    """The same step! on the oracle, with the reference's solver settings."""
    import harness as H
    import workloads as W
    fl = wl.flow
    dt, seq = W.step_sequence(fl)
    for op, kw in seq:
        if op == "find_pressure":
            og.find_pressure(dt, 10, None, method="minres", tol=1e-6, itmax=1000)
        else:
            H.apply(None, fl, og, op, kw, False)


def cpu_baseline(args, wl):
    """The oracle on the host cores: one warm-up step and one timed step for
    workloads above 1M particles, else two timed steps."""
    og, threads = oracle_grid(wl)
    big = wl.n > 1_000_000
    if not big:
        oracle_step(og, wl)  # warm-up
    sample_steps = 1 if big else 2
    t0 = time.perf_counter()
    for _ in range(sample_steps):
        oracle_step(og, wl)
    dt = time.perf_counter() - t0
    return {"value": wl.n * sample_steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{sample_steps} full step(s) of {wl.label}" + ("" if big else " after 1 warm-up step") +
                      f", oracle restatement with the reference's solver (MINRES atol=rtol=1e-6, itmax=1000), "
                      f"OpenMP {threads} threads"}


REF_BUDGET_S = 150.0


def run_reference(args, world, rank, wl):
    if rank != 0:
        return None
    og, threads = oracle_grid(wl)
    # warm-up, then as many of the K steps as fit the time budget (at least one)
    warm = max(0, min(args.warmup, 1))
    t_w = None
    for _ in range(warm):
        t0 = time.perf_counter()
        oracle_step(og, wl)
        t_w = time.perf_counter() - t0
    steps = args.steps
    if t_w is not None:
        steps = max(1, min(args.steps, int(REF_BUDGET_S / max(t_w, 1e-9))))
    t0 = time.perf_counter()
    for _ in range(steps):
        oracle_step(og, wl)
    dt = time.perf_counter() - t0
    value = wl.n * steps / dt
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3 / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered lattice, analytic initial field)",
        "config": dict(wl.describe(), **{
            "solver": "minres fp64 atol=rtol=1e-6 itmax=1000, 10 sweeps/step (reference settings)",
            "parallelism": "host threads"}),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{steps} of the {args.steps} requested full steps after {warm} warm-up "
                                   f"step(s) (as many as fit {REF_BUDGET_S:.0f} s); the reference is Julia and no "
                                   "Julia runtime exists on this machine, so its algorithm runs as the C++ "
                                   "restatement (oracle/)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="double_shear", choices=sorted(CONFIG_SIZES),
                    help="flow of the workload (default: the double shear layer, 2048 x 2048)")
    ap.add_argument("--nx", type=int, default=0, help="lattice columns (0: the workload's size; others for profiling)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-compare", action="store_true", help="skip the per-solver comparison")
    ap.add_argument("--solver", default="learned_pcg", choices=["jacobi_pcg", "mixed_ir", "learned_pcg", "minres"],
                    help="pressure solver of the timed steps")
    ap.add_argument("--train-steps", type=int, default=400, help="Adam steps of the learned preconditioner")
    ap.add_argument("--train-probes", type=int, default=0, help="0: FSAI/Kaporin objective; K: Hutchinson, K probes")
    ap.add_argument("--train-lr", type=float, default=5e-3)
    ap.add_argument("--learn-hops", type=int, default=1, choices=[1, 2],
                    help="pattern of the learned factor: 1 the operator's lower triangle, 2 with two-hop neighbours")
    ap.add_argument("--full-run", action="store_true",
                    help="run the workload for its specified step count and report completion and drift (no bench line)")
    ap.add_argument("--full-steps", type=int, default=0, help="steps of --full-run (0: the workload's own)")
    args = ap.parse_args()
    wl = Workload(args.config, args.nx or None)
    if args.full_run:
        print(json.dumps(full_run(args, wl)), flush=True)
        return
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    world, rank, local = dist_setup()
    if args.impl == "reference":
        line = run_reference(args, world, rank, wl)
    else:
        line = run_ours(args, world, rank, local, wl)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

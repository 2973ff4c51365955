#!/usr/bin/env python
"""Benchmark of the GB300 WCSPH right-hand side: particle-steps/s of the 3D dam break.

Workload (N=1 line): the 3D WCSPH dam break in its plain Float64 GPU drop-in form -- fluid block
1.0 x 0.5 x 1.0 m at dx = 0.008 in a 3.2 x 1.0 x 1.4 m tank with 3 wall layers, h = 1.75 dx,
WendlandC2, Cole EOS (gamma 7, c = 20 sqrt(9.81)), Monaghan alpha 0.02, Molteni-Colagrossi delta
0.1, Adami walls, gravity -9.81, CarpenterKennedy2N54 at dt = 5e-5.  One step = one CK2N54 step
(5 RHS evaluations + the fused 2N update).  particle-steps/s = (n_fluid + n_wall) * steps / s.

Timed window: the dam break in motion.  Before the window (untimed) the precision form advances
the hydrostatic start by --flow-time seconds of physical time (default 0.2 s = 4000 steps; the
collapsing column then moves at up to ~2 m/s, so the neighbour search is rebuilt every few
steps); the FP64 drop-in takes that state, runs --warmup steps and then the --steps timed steps.
The line carries the number of neighbour-search rebuilds inside the window, the same window
from the hydrostatic start (`at_rest`, where no rebuild happens) and with a rebuild at every stage
(`rebuild_every_stage`, skin 0: the reference's update_nhs! schedule).

The `forms` object adds the precision form (FP32 pair arithmetic) and the FP64 drop-in on the
finer dx = 0.0064 geometry over the same kind of window (flowing start, same --steps), with the
FP32-vs-FP64 field errors after the timed steps.

Synthetic data: the inputs are the reference's own dam-break setup (RectangularTank with
hydrostatic density), generated here; no dataset is involved.  The state (> 300 MB) is larger
than the 129 MB L2, so no L2 flush is needed between steps.

--impl reference: the FP64 CPU restatement of the reference (oracle/, OpenMP on all host cores)
on the same workload; each timed step is one full CK2N54 step of the full state (the oracle
rebuilds its cell list at every stage, so its cost per step does not depend on the start state).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s (3D WCSPH) FP32 vs FP64 at stated error; % of HBM roofline"
UNIT = "particle-steps/s"

# Algorithmic byte model: compulsory unique bytes per RHS stage in 3D, every array touched once
# per pass (neighbour re-reads assumed on chip).  FP64 per fluid particle: NHS 32 (x read, key and
# permutation written) + Adami-side read of x, rho 32 + pair 64 (x, v, rho, m) + fused 2N update
# 224 (7 scalars, state and register read and written); per wall particle: Adami 40 + pair-side
# read 48.  FP32 form: 32 + 20 + 36 + 160 per fluid, 56 per wall.
BYTES_STAGE = {"float64": (352, 88), "float32": (248, 56)}   # (per fluid, per wall)
BYTES_PAIR = {"float64": (288, 48), "float32": (196, 24)}    # pair kernel + fused update share

CFG1 = dict(name="3D WCSPH dam break FP64 drop-in, dx=0.008 (fluid 1.0x0.5x1.0 m, tank "
                 "3.2x1.0x1.4 m, 3 layers), CarpenterKennedy2N54 dt=5e-5",
            dx=0.008, fluid=(1.0, 0.5, 1.0), tank=(3.2, 1.0, 1.4), layers=3, dt=5e-5)
CFG2 = dict(name="3D WCSPH dam break dx=0.0064 (same geometry)", dx=0.0064,
            fluid=(1.0, 0.5, 1.0), tank=(3.2, 1.0, 1.4), layers=3, dt=5e-5)


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_profile_value(key: str, kernel: str):
    """`key[kernel]: value` line of the committed ncu summaries (profiles/*.md): (value, file)."""
    for f in sorted((ROOT / "profiles").glob("*.md")):
        for line in f.read_text().splitlines():
            if line.startswith(f"{key}[{kernel}]:"):
                try:
                    return float(line.split(":", 1)[1].split()[0]), f"profiles/{f.name}"
                except ValueError:
                    return None, f"profiles/{f.name}"
    return None, None


def load_traffic(kernel: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary: (value, file)."""
    return load_profile_value("traffic_bytes_per_launch", kernel)


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}",
                                      f"--query-gpu={self.Q}", "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if len(s) > 5 + k and s[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def replica_value(dist, ms_local, particles, steps, device="cpu"):
    """Whole-job particle-steps/s of independent replicas: every rank advanced `particles`
    particles for `steps` steps; the job time is the slowest rank's (max over ranks)."""
    import torch

    world = dist.get_world_size() if dist is not None else 1
    ms = float(ms_local)
    if dist is not None:
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return particles * steps * world / (ms / 1e3), ms


def make_case(pkg, cfg, precision, device):
    tank, eos = pkg.dam_break(3, cfg["dx"], cfg["fluid"], cfg["tank"], n_layers=cfg["layers"])
    semi = pkg.dam_break_semidiscretization(tank, eos, 1.75 * cfg["dx"], precision=precision,
                                            device=device)
    return semi, tank


def run_form(pkg, torch, semi, ode, steps, warmup, dt, precision, with_timing=True):
    """Device-resident timing of `steps` CK2N54 steps (one fused library call)."""
    v, u = ode.v0.clone(), ode.u0.clone()
    lib = semi._lib
    semi._set_stream()
    if warmup:
        semi._call("tp_integrate_ck2n54", v.data_ptr(), u.data_ptr(), ctypes.c_double(0.0),
                   ctypes.c_double(dt), ctypes.c_int64(warmup))
    semi.sync()
    lib.tp_enable_timing(semi._handle, 1 if with_timing else 0)
    l0 = lib.tp_kernel_launches(semi._handle)
    stream = torch.cuda.current_stream(semi.device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    semi._call("tp_integrate_ck2n54", v.data_ptr(), u.data_ptr(), ctypes.c_double(0.0),
               ctypes.c_double(dt), ctypes.c_int64(steps))
    e1.record(stream)
    torch.cuda.synchronize()
    semi.sync()
    ms = e0.elapsed_time(e1)
    launches = lib.tp_kernel_launches(semi._handle) - l0
    ph = (ctypes.c_double * 3)()
    lib.tp_phase_times(semi._handle, ph, 3)
    lib.tp_enable_timing(semi._handle, 0)
    return v, u, ms, launches, list(ph)


def roofline_for(precision, nf, nw, stages, pair_ms, hbm, peak_kind, kernel):
    bf, bw = BYTES_PAIR[precision]
    bytes_launch = nf * bf + nw * bw
    avg_s = pair_ms / 1e3 / stages
    achieved = bytes_launch / avg_s / 1e9
    traffic, tsrc = load_traffic(kernel)
    fp64, fsrc = load_profile_value("fp64_pipe_active_pct", kernel)
    issue, isrc = load_profile_value("issue_active_pct", kernel)
    l1, lsrc = load_profile_value("l1tex_throughput_pct", kernel)
    return {"bound": "hbm", "kernel": kernel, "achieved": round(achieved, 2),
            "peak": hbm, "unit": "GB/s", "frac": round(achieved / hbm, 4),
            "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "bytes_per_launch": bytes_launch, "avg_launch_ms": round(pair_ms / stages, 4),
            "traffic": traffic,
            # what bounds the kernel instead; these four are NOT measured in this run: they are
            # copied from the committed ncu summary of the same kernel and workload
            "from_profiles": {"traffic": tsrc, "fp64_pipe_active_pct": fp64,
                              "issue_active_pct": issue, "l1tex_throughput_pct": l1,
                              "source": fsrc or isrc or lsrc or tsrc}}


def flow_state(pkg, torch, cfg, device, flow_steps):
    """Untimed prefix: the precision form advances the hydrostatic dam break `flow_steps`
    CarpenterKennedy2N54 steps; returns the state (device tensors, caller order) and seconds."""
    semi, _ = make_case(pkg, cfg, "float32", device)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    v, u = ode.v0.clone(), ode.u0.clone()
    semi._set_stream()
    t0 = time.perf_counter()
    if flow_steps:
        semi._call("tp_integrate_ck2n54", v.data_ptr(), u.data_ptr(), ctypes.c_double(0.0),
                   ctypes.c_double(cfg["dt"]), ctypes.c_int64(flow_steps))
    semi.sync()
    el = time.perf_counter() - t0
    semi.close()
    del ode
    return v, u, el


def rebuilds(semi):
    c = ctypes.c_int64()
    semi._call("tp_rebuild_count", ctypes.byref(c))
    return int(c.value)


def timed_window(torch, semi, v, u, steps, warmup, dt, clk=None, dist=None, label="window"):
    """`warmup` untimed steps, then `steps` timed CK2N54 steps of (v, u) in one fused call
    (CUDA events on the launching stream, synchronised on both sides); phase times from the
    library's event pool; rebuilds of the neighbour search inside the timed steps.  The timed
    call runs inside the NVTX range `label` (ncu --nvtx --nvtx-include selects its launches)."""
    lib = semi._lib
    semi._set_stream()
    if warmup:
        semi._call("tp_integrate_ck2n54", v.data_ptr(), u.data_ptr(), ctypes.c_double(0.0),
                   ctypes.c_double(dt), ctypes.c_int64(warmup))
    semi.sync()
    r0 = rebuilds(semi)
    lib.tp_enable_timing(semi._handle, 1)
    l0 = lib.tp_kernel_launches(semi._handle)
    stream = torch.cuda.current_stream(semi.device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    import contextlib

    with (clk if clk is not None else contextlib.nullcontext()):
        torch.cuda.nvtx.range_push(label)
        e0.record(stream)
        semi._call("tp_integrate_ck2n54", v.data_ptr(), u.data_ptr(), ctypes.c_double(0.0),
                   ctypes.c_double(dt), ctypes.c_int64(steps))
        e1.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
    semi.sync()
    if dist:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    launches = lib.tp_kernel_launches(semi._handle) - l0
    ph = (ctypes.c_double * 3)()
    lib.tp_phase_times(semi._handle, ph, 3)
    lib.tp_enable_timing(semi._handle, 0)
    return {"ms": ms, "launches": int(launches), "phases": list(ph),
            "rebuilds": rebuilds(semi) - r0}


def phases_per_step(ph, steps):
    return {"update nhs": ph[0] / steps, "compute boundary pressure": ph[1] / steps,
            "system interaction": ph[2] / steps}


def workload_config(cfg, nf, nw):
    """The `config` object of both arms (the same keys and values)."""
    return {"workload": cfg["name"], "n_fluid": nf, "n_wall": nw, "particles": nf + nw,
            "dx": cfg["dx"], "dt": cfg["dt"],
            "l2": "inputs larger than L2 (state + records > 300 MB), no flush"}


def e2e_run(pkg, torch, semi, v0, u0, steps, dt):
    """Through the public C ABI with HOST buffers: every step copies the state host->device from
    pinned memory, advances one CK2N54 step and reads the result back to pinned memory."""
    v_h = v0.cpu().pin_memory()
    u_h = u0.cpu().pin_memory()
    v_d, u_d = torch.empty_like(v0), torch.empty_like(u0)
    stream = torch.cuda.current_stream(semi.device)
    semi._set_stream()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        v_d.copy_(v_h, non_blocking=True)
        u_d.copy_(u_h, non_blocking=True)
        semi._call("tp_integrate_ck2n54", v_d.data_ptr(), u_d.data_ptr(), ctypes.c_double(0.0),
                   ctypes.c_double(dt), ctypes.c_int64(1))
        v_h.copy_(v_d, non_blocking=True)
        u_h.copy_(u_d, non_blocking=True)
    stream.synchronize()
    el = time.perf_counter() - t0
    semi.sync()
    nbytes = (v_h.numel() + u_h.numel()) * 8
    return el, nbytes


def cpu_baseline(semi, tank, cfg, v, u, state):
    """Bounded CPU sample: full CK2N54 steps of the same state (host arrays v (N, 4), u (N, 3))
    with the FP64 oracle on all host cores."""
    import __graft_entry__ as g

    orc = g.load_oracle()
    orc.build()
    model = orc.Model(semi.config, tank.boundary.coordinates, tank.boundary.mass,
                      tank.fluid.mass)
    v, u = v.copy(), u.copy()
    t0 = time.perf_counter()
    steps = 0
    while steps < 8 and (steps == 0 or time.perf_counter() - t0 < 10.0):
        v, u, _ = model.integrate(v, u, cfg["dt"], 1)
        steps += 1
    el = time.perf_counter() - t0
    n = tank.fluid.n_particles + tank.boundary.n_particles
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": n * steps / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{steps} CarpenterKennedy2N54 steps (5 RHS each) of the full workload "
                      f"({n} particles, {state}) with the FP64 C++ oracle, OpenMP, {el:.1f} s"}


def run_ensemble(pkg, torch, args, n_instances=512, seed=0, steps_per_replay=5):
    """Batching form: 512 seeded 2D dam breaks (FP32), three spacing groups in one CUDA graph of
    `steps_per_replay` CK2N54 steps; autotuned launch shape and skin; both graph layouts (the
    groups as parallel branches, one persistent pair launch per stage) timed, the faster kept.
    Aggregate particle-steps/s over all instances, plus the agreement of one instance per group
    with the same instance run alone."""
    e = pkg.ensemble
    t0 = time.perf_counter()
    specs = e.ensemble_specs(n_instances, seed)
    groups = e.build_ensemble(specs)
    setup_s = time.perf_counter() - t0
    tuned = e.autotune(groups, trial_steps=6)
    reps = max(1, min(args.steps, 4))

    def time_graph(eg):
        eg.reset()
        eg.replay()  # warm-up replay
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        launch = torch.cuda.current_stream()  # the batch graph launches on the current stream
        ev0.record(launch)
        for _ in range(reps):
            eg.replay()
        ev1.record(launch)
        torch.cuda.synchronize()
        eg.check()
        return ev0.elapsed_time(ev1)

    # both graph layouts of the same groups and tuning: the groups as parallel branches, and
    # one persistent pair launch per stage for all groups (possible when every group runs the
    # list pass); the faster one is the form's number
    layouts = {}
    eg = e.EnsembleGraph(groups, steps_per_replay)
    layouts["branches"] = time_graph(eg)
    if all(g.tuned["pair_mode"] == "lists" for g in groups):
        eg.close()
        eg = e.EnsembleGraph(groups, steps_per_replay, persistent=True)
        layouts["persistent"] = time_graph(eg)
        if layouts["persistent"] > layouts["branches"]:
            eg.close()
            eg = e.EnsembleGraph(groups, steps_per_replay)
    best = "persistent" if eg.persistent else "branches"
    ms = layouts[best]
    steps = reps * steps_per_replay
    n = eg.n_particles
    # agreement with the single-instance path after one replay from the initial state
    eg.reset()
    eg.replay()
    torch.cuda.synchronize()
    agree = {}
    for g in groups:
        one = e.single_instance(specs[g.instances[0]])
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            e.prepare(one, s)
            one.semi._call("tp_set_skin", ctypes.c_double(g.tuned["skin"]))
            e.prepare(one, s)
            e._integrate(one, steps_per_replay)
        s.synchronize()
        (xa, va, ra), (xb, vb, rb) = e.instance_state(g, 0), e.instance_state(one, 0)

        def rl2(a, b):
            return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

        agree[str(g.dx)] = {"rel_l2_x": rl2(xa, xb), "rel_l2_v": rl2(va, vb),
                            "rel_l2_rho": rl2(ra, rb), "after_steps": steps_per_replay}
        one.semi.close()
    out = {"workload": f"{n_instances} seeded 2D dam breaks (width U[0.5,2], height U[0.25,1], "
                       f"dx in {{0.005,0.01,0.02}}, 5.366x4.0 tank, 3 layers), FP32 form, "
                       f"dt = 5e-3 dx",
           "value": n * steps / (ms / 1e3), "unit": UNIT, "particles": n,
           "n_fluid": eg.n_fluid, "steps": steps, "ms_per_step": ms / steps,
           "graph": (f"{len(groups)} groups x {steps_per_replay} steps per replay, "
                     + ("one persistent pair launch per stage for all groups"
                        if best == "persistent" else "the groups as concurrent branches")),
           "ms_per_step_by_layout": {k: v / steps for k, v in layouts.items()},
           "autotuned": {str(k): v for k, v in tuned.items()},
           "per_instance_agreement": agree, "host_setup_s": round(setup_s, 2)}
    for g in groups:
        g.semi.close()
    return out


def run_adjoint(pkg, torch, dx=0.01, n_steps=500, every=25, fd_h=1e-4, seed=7):
    """Differentiation form: 2D dam break at dx = 0.01 (20 000 fluid), v0 ~ N(0, 0.1^2) m/s,
    FP32 forward + adjoint over 500 CK2N54 steps with checkpoints every 25; objective = mean
    final height of the initial top layer.  Gradients w.r.t. alpha, delta, |g| and v0 (seeded
    direction) against central differences (h = 1e-4) through the fused FP64 integrator, and
    the cost of the backward pass per step relative to one forward step."""
    dt = 5e-3 * dx
    tank, eos = pkg.dam_break(2, dx, (2.0, 1.0), (5.366, 4.0), n_layers=3)
    n = tank.fluid.n_particles
    rng = np.random.default_rng(seed)
    v0 = np.zeros((n, 3))
    v0[:, :2] = rng.normal(0.0, 0.1, (n, 2))
    v0[:, 2] = tank.fluid.density
    u0 = tank.fluid.coordinates.copy()
    w = np.random.default_rng(11).normal(size=(n, 2))
    idx = pkg.adjoint.top_layer_indices(tank)
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device="cuda")

    def semi_of(precision, **kw):
        p = dict(alpha=0.02, delta=0.1, gravity=9.81)
        p.update(kw)
        s = pkg.dam_break_semidiscretization(tank, eos, 1.75 * dx, precision=precision, **p)
        pkg.semidiscretize(s, (0.0, 1.0))
        return s

    semi = semi_of("float32")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    stream = torch.cuda.current_stream()
    pkg.adjoint.Trajectory(semi, dev(v0), dev(u0), dt=dt, n_steps=every, checkpoint_every=every)
    torch.cuda.synchronize()
    ev[0].record(stream)
    traj = pkg.adjoint.Trajectory(semi, dev(v0), dev(u0), dt=dt, n_steps=n_steps,
                                  checkpoint_every=every)
    ev[1].record(stream)
    loss, ubar = pkg.adjoint.surface_height_loss(traj.u, idx, 2)
    vbar = torch.zeros_like(traj.v)
    torch.cuda.synchronize()
    ev[2].record(stream)
    vb, ub, pbar = traj.pullback(vbar, ubar)
    ev[3].record(stream)
    torch.cuda.synchronize()
    fwd_ms, bwd_ms = ev[0].elapsed_time(ev[1]), ev[2].elapsed_time(ev[3])
    # the fused FP32 integrator step (product forward) for the cost ratio
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    vi, ui = dev(v0), dev(u0)
    semi._set_stream()
    semi._call("tp_integrate_ck2n54", vi.data_ptr(), ui.data_ptr(), ctypes.c_double(0.0),
               ctypes.c_double(dt), ctypes.c_int64(10))
    torch.cuda.synchronize()
    ev[0].record(stream)
    semi._call("tp_integrate_ck2n54", vi.data_ptr(), ui.data_ptr(), ctypes.c_double(0.0),
               ctypes.c_double(dt), ctypes.c_int64(100))
    ev[1].record(stream)
    torch.cuda.synchronize()
    integ_ms = ev[0].elapsed_time(ev[1]) / 100
    del ode
    grad = dict(pbar, v0=float((vb.view(-1, 3)[:, :2].cpu().numpy() * w).sum()))
    semi.close()

    def fd_loss(v, **kw):
        s = semi_of("float64", **kw)
        vv, uu = dev(v), dev(u0)
        s._set_stream()
        s._call("tp_integrate_ck2n54", vv.data_ptr(), uu.data_ptr(), ctypes.c_double(0.0),
                ctypes.c_double(dt), ctypes.c_int64(n_steps))
        s.sync()
        val = float(uu.view(-1, 2)[torch.as_tensor(idx, device="cuda"), 1].mean())
        s.close()
        return val

    base = dict(alpha=0.02, delta=0.1, gravity=9.81)
    fd = {}
    for name in ("alpha", "delta", "gravity"):
        fd[name] = (fd_loss(v0, **{name: base[name] + fd_h})
                    - fd_loss(v0, **{name: base[name] - fd_h})) / (2 * fd_h)
    vp, vm = v0.copy(), v0.copy()
    vp[:, :2] += fd_h * w
    vm[:, :2] -= fd_h * w
    fd["v0"] = (fd_loss(vp) - fd_loss(vm)) / (2 * fd_h)
    fwd_step = fwd_ms / n_steps
    bwd_step = bwd_ms / n_steps
    return {"workload": f"2D dam break dx={dx} ({n} fluid, {tank.boundary.n_particles} wall), "
                        f"v0 ~ N(0, 0.1^2), {n_steps} steps dt={dt:g}, checkpoints every "
                        f"{every}; loss = mean final height of the initial top layer "
                        f"({len(idx)} particles)",
            "loss": float(loss), "gradient": grad, "central_fd_fp64": fd, "fd_h": fd_h,
            "rel_err": {k: abs(grad[k] - fd[k]) / max(abs(fd[k]), 1e-300) for k in fd},
            "forward_ms_per_step": fwd_step, "backward_ms_per_step": bwd_step,
            "fused_fp32_integrator_ms_per_step": integ_ms,
            "backward_over_forward_step": bwd_step / fwd_step,
            "backward_over_fused_step": bwd_step / integ_ms}


def run_profile_adjoint(args, dx=0.01, every=25, seed=7):
    """Profiling mode of the differentiation form: the FP32 adjoint of the 2D dam break at
    dx = 0.01 (20 000 fluid) over --steps steps (checkpoints every 25), forward then backward,
    without the finite-difference checks; one summary line.  Used under ncu for the launch list
    of the backward pass."""
    import torch

    import __graft_entry__ as g

    pkg = g.load_package()
    pkg.load_library()
    dt = 5e-3 * dx
    tank, eos = pkg.dam_break(2, dx, (2.0, 1.0), (5.366, 4.0), n_layers=3)
    n = tank.fluid.n_particles
    rng = np.random.default_rng(seed)
    v0 = np.zeros((n, 3))
    v0[:, :2] = rng.normal(0.0, 0.1, (n, 2))
    v0[:, 2] = tank.fluid.density
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device="cuda")
    semi = pkg.dam_break_semidiscretization(tank, eos, 1.75 * dx, precision="float32")
    pkg.semidiscretize(semi, (0.0, 1.0))
    idx = pkg.adjoint.top_layer_indices(tank)
    k = min(every, args.steps)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    stream = torch.cuda.current_stream()
    ev[0].record(stream)
    traj = pkg.adjoint.Trajectory(semi, dev(v0), dev(tank.fluid.coordinates), dt=dt,
                                  n_steps=args.steps, checkpoint_every=k)
    ev[1].record(stream)
    loss, ubar = pkg.adjoint.surface_height_loss(traj.u, idx, 2)
    torch.cuda.synchronize()
    ev[2].record(stream)
    traj.pullback(torch.zeros_like(traj.v), ubar)
    ev[3].record(stream)
    torch.cuda.synchronize()
    print(json.dumps({"profile_adjoint": n, "steps": args.steps, "checkpoint_every": k,
                      "forward_ms_per_step": ev[0].elapsed_time(ev[1]) / args.steps,
                      "backward_ms_per_step": ev[2].elapsed_time(ev[3]) / args.steps}),
          flush=True)
    semi.close()
    return 0


def run_precision_study(pkg, torch, checkpoints=(100, 500, 1000), jitters=(0.0, 0.05),
                        seed=2024):
    """Precision form against the FP64 drop-in on the dx = 0.0064 geometry: relative L2 errors of
    rho, v and x after 100 / 500 / 1000 CK2N54 steps, on the lattice start and on a jittered
    start (fluid positions perturbed by uniform +-0.05 dx noise from a seeded generator, the
    same perturbed input for both forms).  The FP64 drop-in stands in for the FP64 oracle at
    this size (it matches the oracle to 1e-9 relative in the parity tests)."""
    cfg = CFG2
    out = {"workload": cfg["name"], "checkpoints": list(checkpoints), "cases": []}
    for jit in jitters:
        tank, eos = pkg.dam_break(3, cfg["dx"], cfg["fluid"], cfg["tank"], n_layers=3)
        if jit:
            rng = np.random.default_rng(seed)
            tank.fluid.coordinates += rng.uniform(-jit * cfg["dx"], jit * cfg["dx"],
                                                  tank.fluid.coordinates.shape)
        states = {}
        semis = {}
        for prec in ("float64", "float32"):
            semi = pkg.dam_break_semidiscretization(tank, eos, 1.75 * cfg["dx"], precision=prec)
            ode = pkg.semidiscretize(semi, (0.0, 1.0))
            semis[prec] = semi
            states[prec] = (ode.v0.clone(), ode.u0.clone())
        rows = []
        done = 0
        t_form = {"float64": 0.0, "float32": 0.0}
        for cp in checkpoints:
            for prec, semi in semis.items():
                v, u = states[prec]
                semi._set_stream()
                t0 = time.perf_counter()
                semi._call("tp_integrate_ck2n54", v.data_ptr(), u.data_ptr(), ctypes.c_double(0.0),
                           ctypes.c_double(cfg["dt"]), ctypes.c_int64(cp - done))
                semi.sync()
                t_form[prec] += time.perf_counter() - t0
            v64 = states["float64"][0].view(-1, 4).cpu().numpy()
            v32 = states["float32"][0].view(-1, 4).cpu().numpy()
            u64 = states["float64"][1].view(-1, 3).cpu().numpy()
            u32 = states["float32"][1].view(-1, 3).cpu().numpy()

            def rl2(a, b):
                return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

            rows.append({"step": cp, "rel_l2_rho": rl2(v32[:, 3], v64[:, 3]),
                         "rel_l2_v": rl2(v32[:, :3], v64[:, :3]), "rel_l2_x": rl2(u32, u64)})
            done = cp
        for semi in semis.values():
            semi.close()
        out["cases"].append({"jitter_dx": jit, "seed": seed if jit else None,
                             "n_fluid": tank.fluid.n_particles,
                             "n_wall": tank.boundary.n_particles, "errors": rows,
                             "seconds": {k: round(v, 2) for k, v in t_form.items()}})
    return out


def run_reference(args):
    """--impl reference: the oracle (C++ FP64 restatement of the reference) on host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import __graft_entry__ as g

    pkg = g.load_package()
    orc = g.load_oracle()
    orc.build()
    tank, eos = pkg.dam_break(3, CFG1["dx"], CFG1["fluid"], CFG1["tank"], n_layers=3)
    semi = pkg.dam_break_semidiscretization(tank, eos, 1.75 * CFG1["dx"])
    model = orc.Model(semi.config, tank.boundary.coordinates, tank.boundary.mass,
                      tank.fluid.mass)
    v = np.zeros((tank.fluid.n_particles, 4))
    v[:, 3] = tank.fluid.density
    u = tank.fluid.coordinates.copy()
    n = tank.fluid.n_particles + tank.boundary.n_particles
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    warm = min(args.warmup, 1)
    steps = max(1, min(args.steps, 2))
    for _ in range(warm):
        v, u, _ = model.integrate(v, u, CFG1["dt"], 1)
    t0 = time.perf_counter()
    for _ in range(steps):
        v, u, st = model.integrate(v, u, CFG1["dt"], 1)
    el = time.perf_counter() - t0
    val = n * steps / el
    line = {"metric": METRIC, "value": val, "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": steps, "warmup": warm,
            "ms_per_step": el / steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(CFG1, tank.fluid.n_particles, tank.boundary.n_particles),
            "parallelism": f"host threads ({cores})",
            "start_state": "hydrostatic start (the oracle rebuilds its cell list at every "
                           "stage, so the cost of a step does not depend on the state)",
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{steps} full CarpenterKennedy2N54 steps of the "
                                       f"workload (Julia is absent: the C++ FP64 oracle stands "
                                       f"in for the reference's threaded CPU path)"},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_profile_form(args):
    import torch

    import __graft_entry__ as g

    prec, wl = args.profile_form.split(":")
    cfg = {"cfg1": CFG1, "cfg2": CFG2}[wl]
    pkg = g.load_package()
    pkg.load_library()
    flow_steps = int(round(args.profile_flow_time / cfg["dt"]))
    if flow_steps:
        v_f, u_f, _ = flow_state(pkg, torch, cfg, 0, flow_steps)
    semi, tank = make_case(pkg, cfg, prec, 0)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    if args.pair_mode is not None:
        semi._call("tp_set_pair_mode", args.pair_mode)
    if flow_steps:
        win = timed_window(torch, semi, v_f, u_f, args.steps, args.warmup, cfg["dt"])
        ms, launches, ph, reb = win["ms"], win["launches"], win["phases"], win["rebuilds"]
    else:
        v, u, ms, launches, ph = run_form(pkg, torch, semi, ode, args.steps, args.warmup,
                                          cfg["dt"], prec)
        reb = None
    n = semi.n_fluid + semi.n_wall
    print(json.dumps({"profile_form": args.profile_form, "pair_mode": args.pair_mode,
                      "flow_time": args.profile_flow_time, "n_fluid": semi.n_fluid,
                      "n_wall": semi.n_wall, "steps": args.steps, "ms_per_step": ms / args.steps,
                      "value": n * args.steps / (ms / 1e3), "launches": launches,
                      "rebuilds": reb, "phase_ms": ph}), flush=True)
    semi.close()
    return 0


def run_profile_ensemble(args, n_instances=512, seed=0, steps_per_replay=5):
    """Profiling mode of the batching form: the 512-instance ensemble with the library's default
    launch shape and skin (no autotuning trials), one warm-up replay of the CUDA graph and then
    `--steps` replays; one summary line.  Used under ncu for the launch list of the graph."""
    import torch

    import __graft_entry__ as g

    pkg = g.load_package()
    pkg.load_library()
    e = pkg.ensemble
    groups = e.build_ensemble(e.ensemble_specs(n_instances, seed))
    eg = e.EnsembleGraph(groups, steps_per_replay,
                         persistent=args.batch_layout == "persistent")
    eg.reset()
    eg.replay()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launch = torch.cuda.current_stream()
    ev0.record(launch)
    for _ in range(max(1, args.steps)):
        eg.replay()
    ev1.record(launch)
    torch.cuda.synchronize()
    eg.check()
    steps = max(1, args.steps) * steps_per_replay
    ms = ev0.elapsed_time(ev1)
    print(json.dumps({"profile_ensemble": n_instances, "layout": args.batch_layout,
                      "particles": eg.n_particles,
                      "groups": [{"dx": gr.dx, "particles": gr.n_particles} for gr in groups],
                      "steps": steps, "ms_per_step": ms / steps,
                      "value": eg.n_particles * steps / (ms / 1e3)}), flush=True)
    for gr in groups:
        gr.semi.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--flow-time", type=float, default=0.2,
                    help="physical time (s) the precision form advances the dam break before "
                         "the timed window (untimed); 0 = hydrostatic start")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-forms", action="store_true", help="skip the dx=0.0064 form comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-ensemble", action="store_true",
                    help="skip the 512-instance 2D ensemble (batching form)")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the differentiated 2D dam break (differentiation form)")
    ap.add_argument("--profile-form", default=None, metavar="PRECISION:WORKLOAD",
                    help="profiling mode (e.g. float32:cfg2): only warm-up + timed steps of that "
                         "form, one summary line; used under ncu")
    ap.add_argument("--profile-flow-time", type=float, default=0.0,
                    help="--profile-form: start from the dam break advanced this many seconds "
                         "by the precision form (untimed; default 0 = hydrostatic start)")
    ap.add_argument("--profile-adjoint", action="store_true",
                    help="profiling mode of the differentiation form: FP32 adjoint of the 2D dam "
                         "break (dx = 0.01) over --steps steps, forward and backward only")
    ap.add_argument("--profile-ensemble", action="store_true",
                    help="profiling mode of the batching form: default launch shape, one warm-up "
                         "replay and --steps replays of the ensemble graph; used under ncu")
    ap.add_argument("--batch-layout", default="branches", choices=["branches", "persistent"],
                    help="graph layout of --profile-ensemble: the groups as parallel branches, "
                         "or one persistent pair launch per stage for all groups")
    ap.add_argument("--pair-mode", type=int, default=None, choices=[0, 1, 2],
                    help="pair pass of --profile-form: 0 gather (lists), 1 symmetric (FP64), "
                         "2 tiled (FP32)")
    ap.add_argument("--precision-study", action="store_true",
                    help="FP32 form vs FP64 drop-in errors after 100/500/1000 steps (dx=0.0064, "
                         "lattice and jittered starts); prints one JSON line")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.precision_study:
        import torch

        import __graft_entry__ as g

        pkg = g.load_package()
        pkg.load_library()
        print(json.dumps(run_precision_study(pkg, torch)), flush=True)
        return 0
    if args.profile_form:
        return run_profile_form(args)
    if args.profile_ensemble:
        return run_profile_ensemble(args)
    if args.profile_adjoint:
        return run_profile_adjoint(args)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import __graft_entry__ as g

    pkg = g.load_package()
    if rank == 0:
        pkg.build()
    if dist:
        dist.barrier()
    pkg.load_library()
    hbm, peak_kind = load_peaks()

    dt = CFG1["dt"]
    flow_steps = int(round(args.flow_time / dt))
    # untimed prefix: the dam break in motion (precision form, then handed to the FP64 drop-in)
    v_flow, u_flow, flow_s = flow_state(pkg, torch, CFG1, local, flow_steps)

    semi, tank = make_case(pkg, CFG1, "float64", local)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    nf, nw = semi.n_fluid, semi.n_wall
    ntot = nf + nw

    # timed window on the flowing state (barrier + synchronize on both sides, max over ranks)
    v, u = v_flow.clone(), u_flow.clone()
    clk = ClockSampler(local)
    win = timed_window(torch, semi, v, u, args.steps, args.warmup, dt, clk=clk, dist=dist)
    ms = win["ms"]
    ph = win["phases"]
    value, ms_max = replica_value(dist, ms, ntot, args.steps, semi.device)
    stages = 5 * args.steps
    bf, bw = BYTES_STAGE["float64"]
    step_bytes = 5 * (nf * bf + nw * bw)

    # the same window from the hydrostatic start (no particle moves far enough for a rebuild)
    v0, u0 = ode.v0.clone(), ode.u0.clone()
    rest = timed_window(torch, semi, v0, u0, args.steps, args.warmup, dt, label="at_rest")
    del v0, u0

    # end to end through the C ABI with host buffers, from the flowing state
    e2e_steps = max(1, min(args.steps, 10))
    el, nbytes = e2e_run(pkg, torch, semi, v_flow, u_flow, e2e_steps, dt)
    e2e_val = ntot * e2e_steps * world / el

    # the reference's schedule: cell list and neighbour lists rebuilt at every stage (skin 0)
    semi._call("tp_set_skin", ctypes.c_double(0.0))
    v, u = v_flow.clone(), u_flow.clone()
    every = timed_window(torch, semi, v, u, args.steps, args.warmup, dt,
                         label="rebuild_every_stage")

    out = None
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": workload_config(CFG1, nf, nw),
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "window": {"start_state": f"dam break in motion: hydrostatic start advanced "
                                      f"{flow_steps} steps (t = {args.flow_time:g} s) by the "
                                      f"precision form, untimed ({flow_s:.1f} s), then "
                                      f"{args.warmup} FP64 warm-up steps",
                       "rebuilds_in_window": win["rebuilds"],
                       "rebuilds_per_step": win["rebuilds"] / args.steps},
            "roofline": roofline_for("float64", nf, nw, stages, ph[2], hbm, peak_kind,
                                     "k_pair64"),
            "step_roofline": {"bytes_per_step": step_bytes,
                              "achieved_gbs": round(step_bytes / (ms_max / args.steps / 1e3)
                                                    / 1e9, 2),
                              "frac": round(step_bytes / (ms_max / args.steps / 1e3) / 1e9
                                            / hbm, 4)},
            "phase_ms_per_step": phases_per_step(ph, args.steps),
            "at_rest": {"value": ntot * args.steps / (rest["ms"] / 1e3),
                        "ms_per_step": rest["ms"] / args.steps,
                        "rebuilds_in_window": rest["rebuilds"],
                        "phase_ms_per_step": phases_per_step(rest["phases"], args.steps)},
            "rebuild_every_stage": {"value": ntot * args.steps / (every["ms"] / 1e3),
                                    "ms_per_step": every["ms"] / args.steps,
                                    "rebuilds_in_window": every["rebuilds"],
                                    "phase_ms_per_step": phases_per_step(every["phases"],
                                                                         args.steps)},
            "e2e": {"value": e2e_val, "unit": UNIT, "steps": e2e_steps,
                    "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes},
            "gpu_launches": win["launches"],
            "clocks": clk.summary(),
        }
    semi.close()
    del ode

    # precision forms on the finer geometry over the same kind of window (rank 0 only)
    if rank == 0 and not args.no_forms:
        k = args.steps
        forms = {}
        res = {}
        vf2, uf2, flow2_s = flow_state(pkg, torch, CFG2, local, flow_steps)
        for prec in ("float64", "float32"):
            s2, t2 = make_case(pkg, CFG2, prec, local)
            o2 = pkg.semidiscretize(s2, (0.0, 1.0))
            v2, u2 = vf2.clone(), uf2.clone()
            w2 = timed_window(torch, s2, v2, u2, k, args.warmup, CFG2["dt"], label=f"form_{prec}")
            n2 = s2.n_fluid + s2.n_wall
            forms[prec] = {
                "value": n2 * k / (w2["ms"] / 1e3), "ms_per_step": w2["ms"] / k, "steps": k,
                "warmup": args.warmup, "n_fluid": s2.n_fluid, "n_wall": s2.n_wall,
                "rebuilds_in_window": w2["rebuilds"],
                "phase_ms_per_step": phases_per_step(w2["phases"], k),
                "roofline": roofline_for(prec, s2.n_fluid, s2.n_wall, 5 * k, w2["phases"][2],
                                         hbm, peak_kind,
                                         "k_pair64" if prec == "float64" else "k_pair32"),
                "step_hbm_frac": round(5 * (s2.n_fluid * BYTES_STAGE[prec][0] + s2.n_wall
                                            * BYTES_STAGE[prec][1]) / (w2["ms"] / k / 1e3)
                                       / 1e9 / hbm, 4),
            }
            res[prec] = (v2.view(-1, 4).cpu().numpy(), u2.view(-1, 3).cpu().numpy())
            s2.close()
            del o2
        del vf2, uf2
        (v64, u64), (v32, u32) = res["float64"], res["float32"]

        def rl2(a, b):
            return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

        forms["fp32_vs_fp64"] = {
            "speedup": forms["float32"]["value"] / forms["float64"]["value"],
            "after_steps": k + args.warmup,
            "start_state": f"the same flowing state (t = {args.flow_time:g} s) for both forms",
            "rel_l2_rho": rl2(v32[:, 3], v64[:, 3]),
            "rel_l2_v": rl2(v32[:, :3], v64[:, :3]),
            "rel_l2_x": rl2(u32, u64)}
        forms["workload"] = CFG2["name"]
        out["forms"] = forms

    if rank == 0 and not args.no_ensemble:
        out.setdefault("forms", {})["batching"] = run_ensemble(pkg, torch, args)
    if rank == 0 and not args.no_adjoint:
        out.setdefault("forms", {})["differentiation"] = run_adjoint(pkg, torch)

    if rank == 0 and not args.no_cpu:
        semi_c, tank_c = make_case(pkg, CFG1, "float64", local)
        out["cpu_baseline"] = cpu_baseline(
            semi_c, tank_c, CFG1, v_flow.view(-1, 4).cpu().numpy(),
            u_flow.view(-1, 3).cpu().numpy(), f"the flowing state at t = {args.flow_time:g} s")
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Benchmark of the BVE RK4 direct-sum path on GB300.

Workload (default, the metric's configuration): barotropic vorticity on the
unit sphere, icosahedral level 7 (327,680 leaf faces = sources, 163,842
vertices = passive targets), Gaussian vortex 4 pi exp(-(1 - x.x0)/0.25^2)
centred at lat 0.05 pi, lon 0, plus 2 Omega z, Omega = 2 pi, smoothing
eps = 0.01, RK4 with dt = 0.005.  A step is one RK4 step: four direct-sum
evaluations over (vertices + leaf faces) x leaf faces.  Inputs are synthetic
(the mesh and the vorticity are generated, no dataset is read).

Interactions are counted as in the metric: (Nv + Nf) * Nf per evaluation, Nf =
leaf faces.  `value` uses the FP32-compensated path with inputs resident in
HBM; the FP64 path (reference arithmetic) is reported beside it, as are the
relative errors of the FP32 path against FP64 on the same state, and the
learned form (octree far field + tcgen05 MLP correction, network trained in
the run) with its error against the same FP64 evaluation.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import math
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

METRIC = "BVE RK4 Ginteractions/s: plain FP64 vs FP32-comp/learned at equal L∞ error"
UNIT = "Ginteractions/s"
LEVEL = 7
EPS = 0.01
DT = 0.005
OMEGA = 2 * math.pi
FLOPS_PER_PAIR = 24  # credited flops of the sphere u pair (eps form)
L2_FLUSH_BYTES = 512 << 20


def workload_config(level: int, nv: int, nf: int) -> dict:
    return {
        "workload": f"BVE sphere icosahedral level {level} RK4, Gaussian vortex + 2*Omega*z, "
                    f"eps={EPS}, dt={DT}",
        "level": level, "vertices": nv, "leaf_faces": nf, "eps": EPS, "dt": DT,
        "interactions_per_step": 4 * (nv + nf) * nf,
        "l2": "flushed between timed steps (512 MiB write)",
        "parallelism": "replicas (one independent problem per GPU)",
    }


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for name, v in zip(names, s[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


# ---------------------------------------------------------------------------
# workload setup
# ---------------------------------------------------------------------------
def make_state(level: int):
    from lpm_gb300 import core

    vx, fx, fa, fm = core.build_mesh(core.MESH_ICOS_TRI, level, 1.0)
    params = (4 * math.pi, 4.0, 0.0, 0.05 * math.pi, 0.0, OMEGA)
    vz = core.eval_ic(core.IC_GAUSSIAN_SPHERE, params, vx)
    fz = core.eval_ic(core.IC_GAUSSIAN_SPHERE, params, fx)
    return vx, fx, fa, fm, vz, fz


class DeviceState:
    def __init__(self, host, device):
        import torch

        vx, fx, fa, fm, vz, fz = host
        d = torch.device("cuda", device)
        self.vx = torch.from_numpy(vx).to(d)
        self.fx = torch.from_numpy(fx).to(d)
        self.fa = torch.from_numpy(fa).to(d)
        self.fm = torch.from_numpy(fm).to(d)
        self.vz = torch.from_numpy(vz).to(d)
        self.fz = torch.from_numpy(fz).to(d)
        self.vu = torch.zeros_like(self.vx)
        self.fu = torch.zeros_like(self.fx)

    def clone(self):
        c = DeviceState.__new__(DeviceState)
        for k, v in self.__dict__.items():
            setattr(c, k, v.clone())
        return c

    def velocity(self, ctx, precision):
        """Velocities of the current state (eps sphere kernel, faces skip i == j)."""
        from lpm_gb300 import functors as F

        ctx.set_precision(precision)
        F.ic2d_passive_sums(ctx, self.vu, None, self.vx, self.fx, self.fz, self.fa, self.fm, EPS)
        F.ic2d_active_sums(ctx, self.fu, None, self.fx, self.fz, self.fa, self.fm, EPS,
                           self_rule=1)


def make_stepper(ctx, st, precision, flags):
    import ctypes as C

    from lpm_gb300 import core

    h = C.c_void_p()
    core.check(core.lib().lpm_bve_rk4_create(ctx.handle, C.byref(h), st.vx.shape[0],
                                             st.fx.shape[0], DT, OMEGA, EPS, precision, flags))
    return h


def advance(h, st):
    from lpm_gb300 import core
    from lpm_gb300.core import ptr, view

    core.check(core.lib().lpm_bve_rk4_advance_timestep(
        h, view(st.vx), ptr(st.vz), view(st.vu), view(st.fx), ptr(st.fz), view(st.fu),
        ptr(st.fa), ptr(st.fm)))


def fp32_peak(device) -> tuple[float, float, int]:
    """Computed FP32 FMA peak (TFLOP/s) 2*128*SMs*sm_max_mhz, with sm_max_mhz and SMs."""
    import torch

    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
        if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    nsm = torch.cuda.get_device_properties(device).multi_processor_count
    return 2 * 128 * nsm * sm_max * 1e6 / 1e12, sm_max, nsm


def rel_errors(got, ref, mask=None):
    import torch

    g = got if got.dim() == 2 else got.reshape(-1, 1)
    r = ref if ref.dim() == 2 else ref.reshape(-1, 1)
    if mask is not None:
        keep = mask == 0
        g, r = g[keep], r[keep]
    em = torch.linalg.norm(g - r, dim=1)
    xm = torch.linalg.norm(r, dim=1)
    return {"linf": float(em.max() / xm.max()), "l2": float(torch.sqrt((em ** 2).sum() / (xm ** 2).sum()))}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args, rank, world, device):
    import torch
    import torch.distributed as dist

    from lpm_gb300 import build as B
    from lpm_gb300 import core

    B.build()
    torch.cuda.set_device(device)
    ctx = core.Context(device)
    stream = torch.cuda.current_stream(device)
    ctx.set_stream(stream)
    if args.fp32_shape is not None:  # else the stepper times the shapes once
        ctx.set_kernel_shape(args.fp32_shape)

    host = make_state(args.level)
    vx, fx, fa, fm, vz, fz = host
    nv, nleaf = vx.shape[0], int((fm == 0).sum())
    ipe = (nv + nleaf) * nleaf  # interactions per evaluation
    base = DeviceState(host, device)
    base.velocity(ctx, core.FP32C)
    torch.cuda.synchronize(device)

    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)

    def barrier():
        if world > 1:
            dist.barrier()

    # ---- headline: FP32C stepper, graph-replayed, inputs resident ----------
    # FP64 position update with reprojection onto the sphere; divided parent
    # slots (which nothing reads) are neither evaluated nor moved.
    st = base.clone()
    flags = core.STEP_SKIP_MASKED_TARGETS | core.STEP_REPROJECT
    h = make_stepper(ctx, st, core.FP32C, flags)
    for _ in range(args.warmup):
        advance(h, st)
    torch.cuda.synchronize(device)
    barrier()
    sampler = ClockSampler(device) if rank == 0 else None
    if sampler:
        sampler.start()
    launches0 = ctx.kernel_launches
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    torch.cuda.synchronize(device)
    barrier()
    for k in range(args.steps):
        flush.fill_(float(k))  # evict L2 between timed steps (untimed)
        ev[k][0].record(stream)
        advance(h, st)
        ev[k][1].record(stream)
    torch.cuda.synchronize(device)
    barrier()
    clocks = sampler.stop() if sampler else None
    launches = ctx.kernel_launches - launches0
    ms = sum(a.elapsed_time(b) for a, b in ev)
    if world > 1:
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = world * 4 * ipe * args.steps / (ms * 1e-3) / 1e9
    core.lib().lpm_bve_rk4_destroy(h)

    result = {}
    if args.only_headline:
        if rank == 0:
            result = {"metric": METRIC, "value": round(value, 3), "unit": UNIT,
                      "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": round(ms_per_step, 4), "gpu_launches": launches,
                      "config": workload_config(args.level, nv, nleaf),
                      "note": "headline leg only (profiling run)"}
        return result
    if rank == 0:
        # ---- kernel timing for the roofline (events around each N-body) ----
        st2 = base.clone()
        h2 = make_stepper(ctx, st2, core.FP32C, flags | core.STEP_TIME_NBODY)
        advance(h2, st2)  # warm
        import ctypes as C
        msn, nn = C.c_double(), C.c_int64()
        core.check(core.lib().lpm_bve_rk4_nbody_time(h2, C.byref(msn), C.byref(nn)))
        for _ in range(2):
            flush.fill_(1.0)
            advance(h2, st2)
        core.check(core.lib().lpm_bve_rk4_nbody_time(h2, C.byref(msn), C.byref(nn)))
        shp = [C.c_int() for _ in range(3)]
        core.check(core.lib().lpm_bve_rk4_kernel_shape(h2, *[C.byref(v) for v in shp]))
        kernel_shape = "%d threads x %d targets, %d CTAs per SM (autotuned)" % tuple(
            v.value for v in shp)
        core.lib().lpm_bve_rk4_destroy(h2)
        nbody_ms = msn.value / max(nn.value, 1)
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
            if (ROOT / "MEASURED_PEAKS.json").exists() else {}
        sm_max = float(peaks.get("sm_max_mhz", 2070.0))
        nsm = torch.cuda.get_device_properties(device).multi_processor_count
        peak_fp32 = 2 * 128 * nsm * sm_max * 1e6 / 1e12
        achieved = ipe * FLOPS_PER_PAIR / (nbody_ms * 1e-3) / 1e12
        traffic = None
        tf = ROOT / "profiles" / "roofline_traffic.json"
        if tf.exists():
            try:
                traffic = json.loads(tf.read_text()).get("nbody_f32_sphere_u_bytes_per_launch")
            except Exception:
                traffic = None
        fma32 = ctx.fma_peak_tflops(core.FP32C)
        fma64 = ctx.fma_peak_tflops(core.FP64)

        # ---- accuracy 1: one evaluation on the initial (unit-sphere) state,
        # FP32C vs the reference's FP64 arithmetic; also the FP64 throughput ----
        s64 = base.clone()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s64.velocity(ctx, core.FP64)
        e1.record(stream)
        torch.cuda.synchronize(device)
        ms64_eval = e0.elapsed_time(e1)
        e_v = rel_errors(base.vu, s64.vu)
        e_f = rel_errors(base.fu, s64.fu, base.fm)

        # ---- the learned far field on the same state (the metric's third
        # form): network trained here (untimed), then timed velocity
        # evaluations of the initial state, error vs the FP64 evaluation ----
        learned = run_learned_eval(args, ctx, stream, base, s64, ipe, device) \
            if not args.no_learned else None
        c5 = run_c5_leg(args, ctx, stream, device, run_learned_eval.weights) \
            if learned is not None and not args.no_c5 else None
        other = run_other_legs(args, device) if not args.no_other else None

        # ---- accuracy 2: one RK4 step, FP32C vs the same algorithm in FP64
        # (chord form, LPM_FP64_CHORD), same flags; also its throughput ----
        sa, sb = base.clone(), base.clone()
        ha = make_stepper(ctx, sa, core.FP32C, flags | core.STEP_NO_GRAPH)
        hb = make_stepper(ctx, sb, core.FP64_CHORD, flags | core.STEP_NO_GRAPH)
        advance(ha, sa)
        torch.cuda.synchronize(device)
        e0.record(stream)
        advance(hb, sb)
        e1.record(stream)
        torch.cuda.synchronize(device)
        ms64c = e0.elapsed_time(e1)
        core.lib().lpm_bve_rk4_destroy(ha)
        core.lib().lpm_bve_rk4_destroy(hb)
        step_err = {"velocity_vertices": rel_errors(sa.vu, sb.vu),
                    "velocity_leaf_faces": rel_errors(sa.fu, sb.fu, base.fm),
                    "position_leaf_faces": rel_errors(sa.fx, sb.fx, base.fm),
                    "vorticity_leaf_faces": rel_errors(sa.fz, sb.fz, base.fm)}

        # ---- e2e: host buffers through the C ABI, copies inside the timing ----
        hostbufs = {k: getattr(base, k).cpu().pin_memory() for k in ("vx", "vz", "vu", "fx", "fz", "fu")}
        se = base.clone()
        he = make_stepper(ctx, se, core.FP32C, flags)
        h2d = d2h = 0
        for name in hostbufs:
            h2d += hostbufs[name].numel() * 8
        d2h = h2d
        advance(he, se)
        torch.cuda.synchronize(device)
        e2e_ms = 0.0
        for k in range(args.steps):
            flush.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for name, hb in hostbufs.items():
                getattr(se, name).copy_(hb, non_blocking=True)
            advance(he, se)
            for name, hb in hostbufs.items():
                hb.copy_(getattr(se, name), non_blocking=True)
            b.record(stream)
            torch.cuda.synchronize(device)
            e2e_ms += a.elapsed_time(b)
        core.lib().lpm_bve_rk4_destroy(he)
        e2e_value = 4 * ipe * args.steps / (e2e_ms * 1e-3) / 1e9

        cpu = cpu_baseline(host, args, e2e_value, ipe / (ms64_eval * 1e-3) / 1e9) \
            if not args.no_cpu else None

        result = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (generated icosahedral mesh + Gaussian vortex; no dataset)",
            "config": workload_config(args.level, nv, nleaf),
            "clocks": clocks,
            "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "roofline": {"bound": "fp32", "achieved": round(achieved, 3),
                         "peak": round(peak_fp32, 3), "unit": "TFLOP/s",
                         "frac": round(achieved / peak_fp32, 4), "traffic": traffic,
                         "peak_kind": f"computed FP32 FMA peak 2*128*{nsm} SMs*{sm_max:.0f} MHz "
                                      "(sm_max_mhz of MEASURED_PEAKS.json)",
                         "kernel": "nbody_chord<float,3,u> (sphere velocity, FP32 pairs, "
                                   "compensated)",
                         "kernel_shape": kernel_shape,
                         "kernel_ms": round(nbody_ms, 4),
                         "flops_per_pair_credited": FLOPS_PER_PAIR,
                         "measured_fma_tflops": {"fp32": round(fma32, 2), "fp64": round(fma64, 3)},
                         "frac_of_measured_fp32_fma": round(achieved / fma32, 4)},
            "fp64": {"value": round(ipe / (ms64_eval * 1e-3) / 1e9, 4), "unit": UNIT,
                     "ms_per_evaluation": round(ms64_eval, 2),
                     "frac_of_measured_fp64_fma": round(
                         ipe / (ms64_eval * 1e-3) * FLOPS_PER_PAIR / 1e12 / fma64, 4),
                     "note": "one velocity evaluation (vertices + leaf faces) of the initial "
                             "state in the reference's FP64 kernel (LPM_FP64: cross product "
                             "out of the sum, Newton-Raphson quotients; 1e-12 parity), "
                             f"{FLOPS_PER_PAIR} credited flops per pair"},
            "fp64_chord": {"value": round(4 * ipe / (ms64c * 1e-3) / 1e9, 4), "unit": UNIT,
                           "ms_per_step": round(ms64c, 2),
                           "note": "one RK4 step of the FP32C algorithm carried out in FP64"},
            "errors_fp32c_vs_fp64": {
                "one_evaluation_vs_reference_fp64": {"velocity_vertices": e_v,
                                                     "velocity_leaf_faces": e_f},
                "one_rk4_step_vs_fp64_chord": step_err},
            "learned": learned,
            "c5_level8_far_field": c5,
            "other_configurations": other,
            "cpu_baseline": cpu,
        }
    return result


def run_learned_eval(args, ctx, stream, base, s64, ipe, device):
    """Octree far field with the learned correction (theta = 0.5, leaves <= 64,
    order-4 expansion, tcgen05 BF16 MLP for rho >= --ff-rho-min) on the
    headline workload: RK4 steps of the same state with the far field as the
    stepper's velocity evaluator (tree topology built once, cell records and
    lists rebuilt on the device every evaluation), timed like the headline
    (--warmup, --steps, L2 flushed), and one velocity evaluation of every
    vertex and leaf face of the initial state compared with the
    reference-arithmetic FP64 evaluation."""
    import torch

    from lpm_gb300 import core
    from lpm_gb300.farfield import FarField

    theta = 0.4 if args.ff_theta is None else args.ff_theta
    # the network is trained on (cell, target) pairs with h/D in [rho_min,
    # 0.5], the range of every setting used here and in the level-8 leg
    trainer = FarField(theta=0.5, leaf_max=64, rho_min=args.ff_rho_min, ctx=ctx)
    t0 = time.perf_counter()
    if args.ff_weights:
        saved = np.load(args.ff_weights)
        weights = (saved["w"], saved["norm"])
    else:
        trainer.train(nsamples=args.ff_samples, epochs=args.ff_epochs, batch=16384, lr=2e-3,
                      seed=20261203, level_min=5, level_max=8, eps=EPS)
        weights = trainer.get_weights()
    torch.cuda.synchronize(device)
    train_s = time.perf_counter() - t0
    trainer.close()
    ff = FarField(theta=theta, leaf_max=64, rho_min=args.ff_rho_min, ctx=ctx)
    ff.set_weights(*weights)
    ff.set_network(True)
    leaf = base.fm == 0
    xall = torch.cat([base.vx, base.fx[leaf]]).contiguous()
    u64 = torch.cat([s64.vu, s64.fu[leaf]])
    uall = torch.zeros_like(xall)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)
    errs = {}
    for tag, net in (("expansion_only", False), ("learned", True)):
        ff.set_network(net)
        ff.velocity(uall, xall, base.fx, base.fz, base.fa, base.fm, EPS)
        torch.cuda.synchronize(device)
        nv = base.vx.shape[0]
        errs[tag] = {"velocity_vertices": rel_errors(uall[:nv], u64[:nv]),
                     "velocity_leaf_faces": rel_errors(uall[nv:], u64[nv:])}
    stats = ff.stats()
    flags = core.STEP_SKIP_MASKED_TARGETS | core.STEP_REPROJECT

    def timed_steps(net):
        ff.set_network(net)
        st = base.clone()
        h = make_stepper(ctx, st, core.FP64_CHORD, flags)
        core.check(core.lib().lpm_bve_rk4_set_farfield(h, ff.handle, 0))
        for _ in range(args.warmup):
            advance(h, st)
        torch.cuda.synchronize(device)
        ms = 0.0
        for k in range(args.steps):
            flush.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            advance(h, st)
            b.record(stream)
            torch.cuda.synchronize(device)
            ms += a.elapsed_time(b)
        core.lib().lpm_bve_rk4_destroy(h)
        return ms / args.steps

    ms_x = timed_steps(False)
    ms = timed_steps(True)
    run_learned_eval.weights = weights
    return {"value": round(4 * ipe / (ms * 1e-3) / 1e9, 3), "unit": UNIT,
            "ms_per_step": round(ms, 3), "theta": theta, "rho_min": args.ff_rho_min,
            "train_s": round(train_s, 2),
            "errors_one_evaluation_vs_reference_fp64": errs,
            "expansion_only": {"value": round(4 * ipe / (ms_x * 1e-3) / 1e9, 3),
                               "ms_per_step": round(ms_x, 3),
                               "note": "the same steps without the network (order-4 "
                                       "expansion on every accepted cell)"},
            "network_rows_per_evaluation": stats.get("network_rows"),
            "note": "direct-equivalent interactions per RK4 step with the octree far field "
                    "and the learned correction as the velocity evaluator (FP64 stage "
                    "updates); the network is trained in this run on seeded random vortex "
                    "fields of icosahedral levels 5-8"}


def run_other_legs(args, device):
    """Short runs of configurations C3 (planar dipoles, quad level 9) and C4
    (256-problem ensemble) inside the default run: the same measurement as
    --config c3 / c4 with 2 timed steps after 1 warm-up step."""
    import copy

    a = copy.copy(args)
    a.steps, a.warmup = 2, 1
    out = {}
    for name, fn in (("c3_plane", run_plane), ("c4_ensemble", run_ensemble)):
        r = fn(a, device)
        keep = ("metric", "value", "unit", "ms_per_step", "steps", "warmup", "config",
                "roofline", "clocks", "gpu_launches", "errors_fp32c_vs_fp64_16384_vertex_targets")
        out[name] = {k: r[k] for k in keep if k in r}
    return out


C5_SETTINGS = (  # (form, theta, rho_min): the configuration's setting first
    ("learned", 0.5, 0.25), ("learned", 0.5, 0.30), ("learned", 0.5, 0.35),
    ("learned", 0.45, 0.25), ("learned", 0.4, 0.30), ("learned", 0.35, 0.30),
    ("expansion_only", 0.5, None), ("expansion_only", 0.4, None), ("expansion_only", 0.35, None),
    ("expansion_only", 0.3, None))
NET_MODE = {"expansion_only": 0, "learned": 1}


def run_c5_leg(args, ctx, stream, device, weights):
    """Configuration C5 inside the default run: icosahedral level 8
    (1,310,720 leaf faces, 655,362 vertices), Rossby-Haurwitz R = 4,
    eps = 0.01, RK4 dt = 0.005, the octree far field (leaves <= 64, order-4
    expansion, exact FP32C near field) with the network trained earlier in
    this run (its inputs are scale-free: trained on levels 5-8).  For each
    setting of C5_SETTINGS: one evaluation of every target, its error against
    the GPU FP64 direct sum (reference arithmetic) on 16,384 seeded targets
    and against the FP32C direct sum on every target (the larger of the two
    decides "<= 1e-4"), and the mean of --c5-steps timed RK4 steps after one
    warm-up step.  The FP64 time per evaluation is the sample's scaled to all
    targets."""
    import torch

    from lpm_gb300 import core
    from lpm_gb300 import functors as F
    from lpm_gb300.farfield import FarField

    L = 8
    vx, fx, fa, fm = core.build_mesh(core.MESH_ICOS_TRI, L, 1.0)
    w = OMEGA / 12.5
    vz = core.eval_ic(core.IC_RH54, (w, -w), vx)
    fz = core.eval_ic(core.IC_RH54, (w, -w), fx)
    nv, nleaf = vx.shape[0], int((fm == 0).sum())
    ipe = (nv + nleaf) * nleaf
    st0 = DeviceState((vx, fx, fa, fm, vz, fz), device)
    xall = torch.cat([st0.vx, st0.fx[st0.fm == 0]])
    rng = np.random.default_rng(20261203)
    idx = torch.from_numpy(np.sort(rng.choice(xall.shape[0], 16384, replace=False))).to(device)
    xs = xall[idx].contiguous()
    ctx.set_precision(core.FP64)
    u64 = torch.zeros_like(xs)
    F.ic2d_passive_sums(ctx, u64, None, xs, st0.fx, st0.fz, st0.fa, st0.fm, EPS)  # warm
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    F.ic2d_passive_sums(ctx, u64, None, xs, st0.fx, st0.fz, st0.fa, st0.fm, EPS)
    b.record(stream)
    torch.cuda.synchronize(device)
    fp64_ms = a.elapsed_time(b) * xall.shape[0] / xs.shape[0]
    fp64 = ipe / (fp64_ms * 1e-3) / 1e9
    # every target: the FP32C direct sum (1.5e-7 from FP64, checked on the
    # sample) as the reference, since the sample's maximum misses the peaks
    ctx.set_precision(core.FP32C)
    uall32 = torch.zeros_like(xall)
    F.ic2d_passive_sums(ctx, uall32, None, xall, st0.fx, st0.fz, st0.fa, st0.fm, EPS)
    torch.cuda.synchronize(device)
    fp32c_vs_fp64 = rel_errors(uall32[idx], u64)
    flags = core.STEP_SKIP_MASKED_TARGETS | core.STEP_REPROJECT
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)
    st = st0.clone()
    st.velocity(ctx, core.FP64_CHORD)  # entry velocities of the RK4 runs
    rows = []
    for form, theta, rho in C5_SETTINGS:
        ff = FarField(theta=theta, leaf_max=64, rho_min=rho if rho else 0.25, ctx=ctx)
        ff.set_weights(*weights)
        ff.set_network(NET_MODE[form])
        uall = torch.zeros_like(xall)
        ff.velocity(uall, xall, st0.fx, st0.fz, st0.fa, st0.fm, EPS)
        torch.cuda.synchronize(device)
        err = rel_errors(uall[idx], u64)
        err_all = rel_errors(uall, uall32)
        run = st.clone()
        h = make_stepper(ctx, run, core.FP64_CHORD, flags)
        core.check(core.lib().lpm_bve_rk4_set_farfield(h, ff.handle, 0))
        advance(h, run)  # warm: builds the tree
        torch.cuda.synchronize(device)
        ms = 0.0
        for k in range(args.c5_steps):
            flush.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            advance(h, run)
            b.record(stream)
            torch.cuda.synchronize(device)
            ms += a.elapsed_time(b)
        core.lib().lpm_bve_rk4_destroy(h)
        ms /= args.c5_steps
        rows.append({"form": form, "theta": theta, "rho_min": rho,
                     "value": round(4 * ipe / (ms * 1e-3) / 1e9, 1), "ms_per_step": round(ms, 2),
                     "error_vs_fp64": err, "error_all_targets_vs_fp32c_direct": err_all,
                     "network_rows": ff.stats().get("network_rows")
                     if form != "expansion_only" else 0})
        ff.close()
    spec = rows[0]

    def worst(r):
        return max(r["error_vs_fp64"]["linf"], r["error_all_targets_vs_fp32c_direct"]["linf"])

    ok = [r for r in rows if worst(r) <= 1e-4]
    best = {f: max((r for r in ok if r["form"] == f), key=lambda r: r["value"], default=None)
            for f in NET_MODE}
    return {"workload": "BVE sphere icosahedral level 8 RK4, Rossby-Haurwitz R=4, eps=0.01, "
                        "dt=0.005, octree far field (leaves <= 64, order-4 expansion)",
            "value": spec["value"], "unit": UNIT, "theta": spec["theta"],
            "rho_min": spec["rho_min"], "error_vs_fp64": spec["error_vs_fp64"],
            "error_all_targets_vs_fp32c_direct": spec["error_all_targets_vs_fp32c_direct"],
            "fp32c_direct_vs_fp64_on_sample": fp32c_vs_fp64,
            "fp64_direct": {"value": round(fp64, 3), "unit": UNIT,
                            "ms_per_evaluation": round(fp64_ms, 1),
                            "note": "GPU FP64 direct sum (reference kernel), 16,384 seeded "
                                    "targets timed and scaled to all targets"},
            "speedup_vs_fp64_direct": round(spec["value"] / fp64, 1),
            "settings": rows,
            "best_at_1e-4": {f: (None if r is None else
                                 {"theta": r["theta"], "rho_min": r["rho_min"],
                                  "value": r["value"], "linf": worst(r)})
                             for f, r in best.items()},
            # the learned correction moves the frontier only if its fastest
            # setting at <= 1e-4 beats the expansion's fastest there
            "learned_faster_than_expansion_at_1e-4": (
                None if best["learned"] is None or best["expansion_only"] is None
                else best["learned"]["value"] > best["expansion_only"]["value"]),
            "steps_timed_per_setting": args.c5_steps,
            "interactions_per_step": 4 * ipe}


def make_state_oracle(level: int):
    """The workload's inputs built by the oracle alone: the reference's mesh
    (tree_init restated from its seed file) and Gaussian vortex.  The
    reference arm uses these, so it loads no code of the library; they equal
    make_state's bit for bit (tests/test_mesh_seeds.py)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import lpm_oracle as O

    vx, fx, fa, fm = O.mesh(O.MESH_ICOS_TRI, level, 1.0)
    params = (4 * math.pi, 4.0, 0.0, 0.05 * math.pi, 0.0, OMEGA)
    vz = O.ic_eval(O.IC_GAUSSIAN_SPHERE, params, vx)
    fz = O.ic_eval(O.IC_GAUSSIAN_SPHERE, params, fx)
    return vx, fx, fa, fm, vz, fz


CPU_TARGETS_NOTE = ("the reference's Kokkos-OpenMP build cannot be compiled (Kokkos, "
                    "KokkosKernels, MPI, spdlog, Catch2 absent); this is the FP64 CPU "
                    "restatement of its functors in oracle/, built -O3 with native code "
                    "generation for this host (like Kokkos_ARCH_NATIVE), contraction off")


def cpu_sample(host, n_sample):
    vx = host[0]
    rng = np.random.default_rng(20261203)
    return np.sort(rng.choice(vx.shape[0], min(n_sample, vx.shape[0]), replace=False))


def cpu_time_eval(host, idx, want_psi, reps, warmup):
    """Seconds per FP64 passive-sum evaluation of the targets idx against all
    face slots (Incompressible2DPassiveSums, sphere kernel with eps), on every
    host thread; median of reps runs after warmup runs."""
    import lpm_oracle

    vx, fx, fa, fm, vz, fz = host
    lpm_oracle.use_native(True)
    lpm_oracle.set_threads(os.cpu_count() or 1)
    for _ in range(warmup):
        lpm_oracle.ic2d_passive_sums(vx, fx, fz, fa, fm, EPS, tgt_idx=idx, want_psi=want_psi)
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        lpm_oracle.ic2d_passive_sums(vx, fx, fz, fa, fm, EPS, tgt_idx=idx, want_psi=want_psi)
        ts.append(time.perf_counter() - t0)
    lpm_oracle.use_native(False)
    return statistics.median(ts), ts


def cpu_baseline(host, args, gpu_fp32c_e2e=None, gpu_fp64=None):
    """FP64 oracle (CPU restatement of the reference functors) on a bounded
    target sample: --cpu-targets seeded vertex targets against all face slots,
    velocity only (the GPU arm's per-pair work), median of 5 after 1 warm-up;
    the reference kernel's velocity + stream function (one log per pair) once
    beside it."""
    sys.path.insert(0, str(ROOT / "oracle"))
    nleaf = int((host[3] == 0).sum())
    idx = cpu_sample(host, args.cpu_targets)
    t_u, ts = cpu_time_eval(host, idx, False, 5, 1)
    t_up, _ = cpu_time_eval(host, idx, True, 1, 0)
    pairs = idx.size * nleaf
    value = pairs / t_u / 1e9
    out = {"value": round(value, 4), "unit": UNIT, "cores": os.cpu_count() or 1,
           "kind": "port",
           "sample": f"{idx.size} seeded vertex targets x {nleaf} leaf sources, one FP64 "
                     f"velocity evaluation (eps kernel, velocity only as timed on the GPU), "
                     f"median of 5 after 1 warm-up: {t_u:.2f} s "
                     f"(runs {', '.join(f'{t:.2f}' for t in ts)})",
           "with_stream_function": {"value": round(pairs / t_up / 1e9, 4), "unit": UNIT,
                                    "note": "the reference's passive-sum kernel as written "
                                            "(velocity and stream function, one log per pair)"},
           "note": CPU_TARGETS_NOTE}
    if gpu_fp32c_e2e is not None:
        out["gpu_fp32c_e2e_over_cpu_fp64"] = round(gpu_fp32c_e2e / value, 1)
    if gpu_fp64 is not None:
        out["gpu_fp64_over_cpu_fp64"] = round(gpu_fp64 / value, 2)
    return out


# ---------------------------------------------------------------------------
# reference arm: the reference's CPU algorithm (FP64 port; the Kokkos build is
# not buildable here), on this workload, all host threads; inputs and code
# from oracle/ only
# ---------------------------------------------------------------------------
def run_reference(args):
    sys.path.insert(0, str(ROOT / "oracle"))
    import lpm_oracle

    host = make_state_oracle(args.level)
    vx, fx, fa, fm, vz, fz = host
    nv, nleaf = vx.shape[0], int((fm == 0).sum())
    threads = os.cpu_count() or 1
    idx = cpu_sample(host, args.cpu_targets)
    lpm_oracle.use_native(True)
    lpm_oracle.set_threads(threads)
    for _ in range(max(args.warmup, 0)):
        lpm_oracle.ic2d_passive_sums(vx, fx, fz, fa, fm, EPS, tgt_idx=idx, want_psi=False)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        lpm_oracle.ic2d_passive_sums(vx, fx, fz, fa, fm, EPS, tgt_idx=idx, want_psi=False)
        ts.append(time.perf_counter() - t0)
    dt = sum(ts)
    t0 = time.perf_counter()
    lpm_oracle.ic2d_passive_sums(vx, fx, fz, fa, fm, EPS, tgt_idx=idx, want_psi=True)
    t_up = time.perf_counter() - t0
    lpm_oracle.use_native(False)
    pairs = idx.size * nleaf
    value = args.steps * pairs / dt / 1e9
    sample = (f"each step: one FP64 velocity evaluation (eps kernel, velocity only: the "
              f"GPU arm's per-pair work) of {idx.size} seeded vertex targets x {nleaf} leaf "
              f"sources, a bounded sample of the RK4 step; median step "
              f"{statistics.median(ts):.2f} s")
    loaded = []
    try:
        with open("/proc/self/maps") as f:
            loaded = sorted({ln.split()[-1] for ln in f if ln.rstrip().endswith(".so")
                             and str(ROOT) in ln})
    except OSError:
        pass
    return {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(dt / args.steps * 1e3, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": "synthetic (the reference's icosahedral mesh from its seed file, "
                    "Gaussian vortex; built by oracle/)",
            "config": workload_config(args.level, nv, nleaf),
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": threads,
                             "kind": "port", "sample": sample,
                             "with_stream_function": {
                                 "value": round(pairs / t_up / 1e9, 4), "unit": UNIT,
                                 "note": "the reference's passive-sum kernel as written "
                                         "(velocity and stream function, one log per pair)"}},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "libraries_loaded_from_repo": loaded,
            "note": CPU_TARGETS_NOTE}


def run_ensemble(args, device):
    """Configuration C4: 256 independent BVE problems, icosahedral levels 3-6
    drawn uniformly from a seed, 1-4 Gaussian vortices each (centres uniform
    on the sphere, amplitudes U[pi, 4 pi], widths U[0.1, 0.4]), eps = 0.01,
    RK4 dt = 0.005, FP32C; one N-body launch per evaluation, RK4 steps
    replayed from a captured graph, chunk length, kernel shape and launch form
    autotuned (or fixed by --ens-plan)."""
    import torch

    from lpm_gb300 import build as B
    from lpm_gb300 import core
    from lpm_gb300.ensemble import BVEEnsemble, random_vortex_params

    B.build()
    torch.cuda.set_device(device)
    ctx = core.Context(device)
    stream = torch.cuda.current_stream(device)
    ctx.set_stream(stream)
    rng = np.random.default_rng(20261203)
    levels = rng.integers(3, 7, size=args.problems)
    params = [random_vortex_params(rng) for _ in levels]
    flags = core.STEP_SKIP_MASKED_TARGETS | core.STEP_REPROJECT
    ens = BVEEnsemble(levels, params, DT, eps=EPS, precision=core.FP32C, flags=flags, ctx=ctx)
    if args.ens_plan:  # a fixed plan: chunk length, shape index, persistent (0/1)
        chunk, shape, persistent = (int(v) for v in args.ens_plan.split(","))
        ens.set_kernel(shape, bool(persistent))
        ens.set_chunk_len(chunk)
    t0 = time.perf_counter()
    ens.velocity()  # autotunes chunk length, kernel shape and launch form
    torch.cuda.synchronize(device)
    tune_s = time.perf_counter() - t0
    ipe = ens.interactions_per_evaluation()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)
    for _ in range(args.warmup):
        ens.advance_timestep()
    torch.cuda.synchronize(device)
    sampler = ClockSampler(device)
    sampler.start()
    l0 = ctx.kernel_launches
    ms = 0.0
    for k in range(args.steps):
        flush.fill_(float(k))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ens.advance_timestep()
        b.record(stream)
        torch.cuda.synchronize(device)
        ms += a.elapsed_time(b)
    clocks = sampler.stop()
    launches = ctx.kernel_launches - l0
    info = ens.info()
    peak, sm_max, nsm = fp32_peak(device)
    ach = 4 * ipe * args.steps * FLOPS_PER_PAIR / (ms * 1e-3) / 1e12
    return {"metric": METRIC, "value": round(4 * ipe * args.steps / (ms * 1e-3) / 1e9, 3),
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded meshes and vortex fields)",
            "config": {"workload": f"ensemble of {args.problems} BVE sphere problems, icosahedral "
                                   "levels 3-6, 1-4 Gaussian vortices each, eps=0.01, dt=0.005",
                       "levels_histogram": {int(l): int((levels == l).sum()) for l in range(3, 7)},
                       "interactions_per_step": 4 * ipe, "chunk_len": info["chunk_len"],
                       "kernel_shape": "%d threads x %d targets, %s" % (
                           ens.shape()[:2] + ("persistent" if ens.shape()[2]
                                              else "one CTA per work item",)),
                       "work_items_per_evaluation": info["items"], "autotune_s": round(tune_s, 2)},
            "roofline": {"bound": "fp32", "achieved": round(ach, 2), "peak": round(peak, 2),
                         "unit": "TFLOP/s", "frac": round(ach / peak, 4), "traffic": None,
                         "kernel": "ensemble N-body (%s), whole RK4 step timed" % (
                             "persistent" if ens.shape()[2] else "one CTA per work item"),
                         "flops_per_pair_credited": FLOPS_PER_PAIR,
                         "peak_kind": f"computed FP32 FMA peak 2*128*{nsm} SMs*{sm_max:.0f} MHz"},
            "clocks": clocks, "gpu_launches": launches}


def run_c1(args, device):
    """Configuration C1: plain FP64 BVE, icosahedral level 4 (5,120 leaf
    faces, 2,562 vertices), Rossby-Haurwitz R=4 with omega = K = Omega/12.5,
    eps = 0, 10 RK4 steps of dt = 0.01, the reference's arithmetic and
    quirks (all face slots evaluated, facevort4, no reprojection).  Parity:
    the whole run against the FP64 oracle; CPU baseline: the oracle's run."""
    import torch

    sys.path.insert(0, str(ROOT / "oracle"))
    import lpm_oracle
    from lpm_gb300 import build as B
    from lpm_gb300 import core
    from lpm_gb300.bve import BVERK4, BVESphere, rossby_haurwitz_params

    B.build()
    torch.cuda.set_device(device)
    ctx = core.Context(device, precision=core.FP64)
    stream = torch.cuda.current_stream(device)
    ctx.set_stream(stream)
    sph = BVESphere(4, ctx=ctx)
    sph.init_vorticity(core.IC_RH54, rossby_haurwitz_params())
    sph.init_velocity()
    torch.cuda.synchronize(device)
    ref = lpm_oracle.BVEState(sph.vert_x.cpu().numpy(), sph.rel_vort_verts.cpu().numpy(),
                              sph.velocity_verts.cpu().numpy(), sph.face_x.cpu().numpy(),
                              sph.rel_vort_faces.cpu().numpy(), sph.velocity_faces.cpu().numpy(),
                              sph.host_face_area, sph.host_face_mask)
    nv, nleaf = sph.n_vertices_host(), sph.n_leaves()
    ipe = (nv + nleaf) * nleaf
    st = BVERK4(0.01, sph, precision=core.FP64)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = ctx.kernel_launches
    a.record(stream)
    for _ in range(10):
        st.advance_timestep(sph)
    b.record(stream)
    torch.cuda.synchronize(device)
    ms = a.elapsed_time(b)
    launches = ctx.kernel_launches - l0
    threads = os.cpu_count() or 1
    lpm_oracle.set_threads(threads)
    t0 = time.perf_counter()
    for _ in range(10):
        ref.step(0.01, OMEGA)
    cpu_s = time.perf_counter() - t0
    leaf = sph.host_face_mask == 0

    def rel(g, r):
        g, r = np.asarray(g), np.asarray(r)
        return float(np.abs(g - r).max() / np.abs(r).max())

    parity = {"vertex_positions": rel(sph.vert_x.cpu(), ref.vx),
              "leaf_positions": rel(sph.face_x.cpu().numpy()[leaf], ref.fx[leaf]),
              "vertex_velocity": rel(sph.velocity_verts.cpu(), ref.vvel),
              "leaf_velocity": rel(sph.velocity_faces.cpu().numpy()[leaf], ref.fvel[leaf]),
              "leaf_vorticity": rel(sph.rel_vort_faces.cpu().numpy()[leaf], ref.fzeta[leaf])}
    return {"metric": METRIC, "value": round(40 * ipe / (ms * 1e-3) / 1e9, 4), "unit": UNIT,
            "n_gpus": 1, "steps": 10, "warmup": 0, "ms_per_step": round(ms / 10, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (generated mesh + Rossby-Haurwitz wave)",
            "config": {"workload": "BVE sphere icosahedral level 4 RK4, RH R=4, eps=0, dt=0.01, "
                                   "10 steps, reference arithmetic (FP64)", "vertices": nv,
                       "leaf_faces": nleaf, "interactions_per_step": 4 * ipe},
            "parity_vs_oracle_after_10_steps": parity,
            "cpu_baseline": {"value": round(40 * ipe / cpu_s / 1e9, 4), "unit": UNIT,
                             "cores": threads, "kind": "port",
                             "sample": "the whole 10-step run (all face slots as targets)"},
            "gpu_launches": launches}


def c3_roofline(device, pairs_per_s: float) -> dict:
    """Planar RK2 step: the stage evaluation computes the velocity only (13
    credited flops per pair, one special-function result: the reciprocal),
    the final evaluation velocity and stream function (16 flops; the
    logarithm from the MUFU, the reciprocal from the MUFU for 5 sources in 8
    and from Newton's method on the FMA pipe for the other 3: soft_rcp_sources
    in lpm_gb300/csrc/nbody.cuh); the stage's stream function would be
    overwritten.  Per pair of the step: 14.5 credited flops against the FP32
    FMA peak.  The XU pipe bounds the step: it delivers 16 MUFU results per
    clock per SM (each reciprocal or log2 holds it two cycles: ncu shows the
    final kernel's XU pipe 94.5 % busy at 47.9 % of its instruction peak when
    every reciprocal is a MUFU one), so 16 pairs per clock per SM in the stage
    and 16 / 1.625 in the final evaluation, 2 / (1/16 + 1.625/16) = 12.2 for
    the step."""
    peak, sm_max, nsm = fp32_peak(device)
    ach = pairs_per_s * 14.5 / 1e12
    mufu_final = 2 - 3 / 8
    xu_pairs = 2 / (1 / 16 + mufu_final / 16) * nsm * sm_max * 1e6
    return {"bound": "fp32", "achieved": round(ach, 2), "peak": round(peak, 2), "unit": "TFLOP/s",
            "frac": round(ach / peak, 4), "traffic": None,
            "kernel": "nbody_chord<float,2,u> + nbody_chord<float,2,u,psi>, whole RK2 step timed",
            "flops_per_pair_credited": 14.5,
            "xu_bound_pairs_per_s": xu_pairs, "frac_of_xu_bound": round(pairs_per_s / xu_pairs, 4),
            "peak_kind": f"computed FP32 FMA peak 2*128*{nsm} SMs*{sm_max:.0f} MHz"}


def run_fp64(args, device):
    """The metric's plain-FP64 leg on its own: one velocity evaluation of
    every vertex and face slot (Incompressible2DPassiveSums +
    Incompressible2DActiveSums with the BVE face rule, eps = 0.01) of the C2
    workload at --level, LPM_FP64 (the reference kernel, cross product taken
    out of the sum) and, once, LPM_FP64_EXACT (every pair term in the
    reference's operation order) beside it.  value = interactions/s of
    LPM_FP64, mean of --steps evaluations after --warmup; roofline: 24
    credited flops per pair against the measured FP64 FMA peak."""
    import torch

    from lpm_gb300 import build as B
    from lpm_gb300 import core

    B.build()
    torch.cuda.set_device(device)
    ctx = core.Context(device)
    stream = torch.cuda.current_stream(device)
    ctx.set_stream(stream)
    vx, fx, fa, fm, vz, fz = make_state(args.level)
    nv, nleaf = vx.shape[0], int((fm == 0).sum())
    ipe = (nv + nleaf) * nleaf
    st = DeviceState((vx, fx, fa, fm, vz, fz), device)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)

    def timed(precision, n, warm):
        for _ in range(warm):
            st.velocity(ctx, precision)
        torch.cuda.synchronize(device)
        ms = 0.0
        for k in range(n):
            flush.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            st.velocity(ctx, precision)
            b.record(stream)
            torch.cuda.synchronize(device)
            ms += a.elapsed_time(b)
        return ms / max(n, 1)

    sampler = ClockSampler(device)
    sampler.start()
    l0 = ctx.kernel_launches
    ms = timed(core.FP64, args.steps, args.warmup)
    clocks = sampler.stop()
    launches = ctx.kernel_launches - l0
    u64 = (st.vu.clone(), st.fu.clone())
    ms_exact = timed(core.FP64_EXACT, 1, 0)
    err = {"velocity_vertices": rel_errors(u64[0], st.vu),
           "velocity_leaf_faces": rel_errors(u64[1], st.fu, st.fm)}
    fma64 = ctx.fma_peak_tflops(core.FP64)
    value = ipe / (ms * 1e-3) / 1e9
    ach = value * FLOPS_PER_PAIR / 1e3
    return {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (generated icosahedral mesh + Gaussian vortex; no dataset)",
            "config": dict(workload_config(args.level, nv, nleaf),
                           step="one velocity evaluation of every target (FP64)"),
            "roofline": {"bound": "fp64", "achieved": round(ach, 4), "peak": round(fma64, 4),
                         "unit": "TFLOP/s", "frac": round(ach / fma64, 4), "traffic": None,
                         "kernel": "nbody_f64h (reference kernel, cross product hoisted)",
                         "flops_per_pair_credited": FLOPS_PER_PAIR,
                         "peak_kind": "measured FP64 FMA microbenchmark (lpm_measure_fma_peak)"},
            "fp64_exact": {"value": round(ipe / (ms_exact * 1e-3) / 1e9, 3),
                           "ms_per_evaluation": round(ms_exact, 2),
                           "difference_from_fp64": err},
            "clocks": clocks, "gpu_launches": launches}


def run_plane(args, device):
    """Configuration C3: planar incompressible flow, colliding Lamb dipoles of
    radius 1 and strength +-2 centred at (-+2, 0), uniform quad mesh of
    [-4, 4]^2 at level 9 (1024 x 1024 leaf cells), eps = 0.02, RK2 dt = 0.01;
    velocity and stream function of every step (FP32C; the stage evaluation
    computes the velocity only, its stream function being overwritten by the
    final evaluation as in the reference).  Accuracy: FP32C vs the reference
    FP64 arithmetic on 16,384 seeded vertex targets."""
    import torch

    from lpm_gb300 import build as B
    from lpm_gb300 import core
    from lpm_gb300 import functors as F
    from lpm_gb300.ic2d import Incompressible2D, Incompressible2DRK2, colliding_dipoles_params

    B.build()
    torch.cuda.set_device(device)
    ctx = core.Context(device)
    stream = torch.cuda.current_stream(device)
    ctx.set_stream(stream)
    if args.fp32_shape is not None:  # else the stepper times the six shapes once
        ctx.set_kernel_shape(args.fp32_shape)
    ic = Incompressible2D(core.MESH_QUAD_RECT, args.plane_level, radius=4.0, eps=0.02, ctx=ctx)
    ic.init_vorticity(core.IC_DIPOLE_PAIR, colliding_dipoles_params())
    ctx.set_precision(core.FP32C)
    ic.init_direct_sums()
    nv, nleaf = ic.n_vertices_host(), int((ic.host_face_mask == 0).sum())
    ipe = (nv + nleaf) * nleaf
    # accuracy on a target subsample, initial state
    idx = torch.from_numpy(np.sort(np.random.default_rng(20261203).choice(nv, 16384, replace=False))).to(ic.vert_x.device)
    xs = ic.vert_x[idx].contiguous()
    outs = {}
    for prec in (core.FP32C, core.FP64):
        ctx.set_precision(prec)
        u = torch.zeros(xs.shape[0], 2, dtype=torch.float64, device=xs.device)
        p = torch.zeros(xs.shape[0], dtype=torch.float64, device=xs.device)
        F.ic2d_passive_sums(ctx, u, p, xs, ic.face_x, ic.rel_vort_active, ic.face_area,
                            ic.face_mask, ic.eps)
        outs[prec] = (u, p)
    torch.cuda.synchronize(device)
    err = {"velocity": rel_errors(outs[core.FP32C][0], outs[core.FP64][0]),
           "stream_fn": rel_errors(outs[core.FP32C][1], outs[core.FP64][1])}
    solver = Incompressible2DRK2(0.01, ic, precision=core.FP32C,
                                 flags=core.STEP_SKIP_MASKED_TARGETS)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)
    for _ in range(args.warmup):
        ic.advance_timestep(solver)
    torch.cuda.synchronize(device)
    sampler = ClockSampler(device)
    sampler.start()
    l0 = ctx.kernel_launches
    ms = 0.0
    for k in range(args.steps):
        flush.fill_(float(k))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ic.advance_timestep(solver)
        b.record(stream)
        torch.cuda.synchronize(device)
        ms += a.elapsed_time(b)
    clocks = sampler.stop()
    inv = (ic.total_vorticity(), ic.total_enstrophy(), ic.total_kinetic_energy())
    return {"metric": "incompressible2d RK2 Ginteractions/s (planar, velocity + stream function)",
            "value": round(2 * ipe * args.steps / (ms * 1e-3) / 1e9, 3), "unit": UNIT,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (generated quad mesh + Lamb dipoles)",
            "config": {"workload": f"planar colliding dipoles, quad level {args.plane_level} on "
                                   "[-4,4]^2, eps=0.02, RK2 dt=0.01", "vertices": nv,
                       "leaf_faces": nleaf, "interactions_per_step": 2 * ipe},
            "roofline": c3_roofline(device, 2 * ipe * args.steps / (ms * 1e-3)),
            "errors_fp32c_vs_fp64_16384_vertex_targets": err,
            "invariants_after": {"circulation": inv[0], "enstrophy": inv[1],
                                 "kinetic_energy": inv[2]},
            "clocks": clocks, "gpu_launches": ctx.kernel_launches - l0}

# credited FP64 flops of the spherical SWE pair as evaluated (FMA = 2, the
# reciprocal = 1): x.y 5, D 2, 1/D 1, scalings 6, c 9, w 6, v 3, velocity 12,
# [y]x and P sums 8, rank-2 gradient update 6 + 36
SWE_FLOPS_PER_PAIR = 94
# FP32C form (chord moments): d from hi/lo parts 6, |d|^2 + c0 6, 1/q 1,
# scalings 6, first moments 12 + 12, second moments 24, scalar sums 4
SWE32_FLOPS_PER_PAIR = 71


def swe_plane_measure(ctx, stream, flush, args, lpm_oracle):
    """Planar SWE sums with PSE (PlanarSWEVertexSums + PlanarSWEFaceSums): quad
    mesh of [-4, 4]^2 at level --swe-plane-level, a dipole-like vorticity, a
    smooth divergence and surface, eps = 0.02, pse_eps = h^0.55.  `value` is
    the FP32C form (--steps timed vertex + face evaluations); the FP64 form is
    timed once and checked against the oracle on 2,048 vertex targets, and
    FP32C against FP64 on every vertex."""
    import torch

    from lpm_gb300 import core
    from lpm_gb300 import functors as F

    level = args.swe_plane_level
    vx, fx, fa, fm = core.build_mesh(core.MESH_QUAD_RECT, level, 4.0)
    zeta = 2 * np.exp(-np.sum((fx - [1.0, 0.0]) ** 2, 1)) - 2 * np.exp(-np.sum((fx + [1.0, 0.0]) ** 2, 1))
    sigma = 0.3 * np.cos(fx[:, 0]) * np.exp(-np.sum(fx ** 2, 1) / 8)
    fs = 1 + 0.1 * np.exp(-np.sum(fx ** 2, 1))
    vs = 1 + 0.1 * np.exp(-np.sum(vx ** 2, 1))
    eps, pse_eps = 0.02, float(np.sqrt(fa[fm == 0].mean())) ** 0.55
    dev = torch.device("cuda", torch.cuda.current_device())
    T = {k: torch.tensor(v, device=dev) for k, v in
         dict(vx=vx, fx=fx, fa=fa, fm=fm, z=zeta, s=sigma, fs=fs, vs=vs).items()}
    ctx.set_precision(core.FP64)

    def step():
        gv = F.swe_plane_vertex_sums(ctx, T["vx"], T["vs"], T["fx"], T["z"], T["s"], T["fa"],
                                     T["fm"], T["fs"], eps, pse_eps)
        F.swe_plane_face_sums(ctx, T["fx"], T["z"], T["s"], T["fa"], T["fm"], T["fs"], eps,
                              pse_eps)
        return gv

    def timed(n):
        ms, out = 0.0, None
        for k in range(n):
            flush.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            out = step()
            b.record(stream)
            torch.cuda.synchronize()
            ms += a.elapsed_time(b)
        return ms / n, out

    step()
    torch.cuda.synchronize()
    ms, gv = timed(1)
    ctx.set_precision(core.FP32C)
    step()
    ms32, gv32 = timed(max(1, args.steps))
    ctx.set_precision(core.FP64)
    nv, ntot, nleaf = vx.shape[0], fx.shape[0], int((fm == 0).sum())
    idx = np.sort(np.random.default_rng(20261203).choice(nv, min(2048, nv), replace=False))
    ref = lpm_oracle.swe_plane_sums(vx[idx], vs[idx], fx, zeta, sigma, fa, fm, fs, eps, pse_eps)
    err, err32 = {}, {}
    for k, col in (("u", slice(0, 2)), ("du1dx1", 2), ("du1dx2", 3), ("laps", 6), ("psi", 7),
                   ("phi", 8)):
        g = gv[k].cpu().numpy()[idx]
        r = ref[:, col]
        err[k] = float(np.max(np.abs(g - r)) / np.max(np.abs(r)))
        g32, g64 = gv32[k].cpu().numpy(), gv[k].cpu().numpy()
        err32[k] = float(np.max(np.abs(g32 - g64)) / np.max(np.abs(g64)))
    pairs = (nv + ntot) * nleaf
    return {"value": round(pairs / (ms32 * 1e-3) / 1e9, 3), "unit": UNIT, "dtype": "f32",
            "ms_per_step": round(ms32, 3),
            "fp64": {"value": round(pairs / (ms * 1e-3) / 1e9, 4), "ms_per_step": round(ms, 2)},
            "workload": f"planar SWE vertex + face sums with PSE, quad level {level} on "
                        f"[-4,4]^2, eps={eps}, pse_eps={pse_eps:.4f}",
            "interactions_per_step": pairs,
            "errors_fp32c_vs_fp64_all_vertex_targets": err32,
            "errors_fp64_vs_oracle_2048_vertex_targets": err}


def run_swe(args, device):
    """Spherical shallow-water direct sums (SphereVertexSums + SphereFaceSums,
    src/lpm_swe_kernels.hpp:723-940): icosahedral level --swe-level, every
    vertex and every face slot a target (as the functors launch), leaf faces
    the sources, vorticity 2 Omega z + a Rossby-Haurwitz-like wave, divergence
    a smooth seeded field, eps = 0.01.  A step is one vertex + one face
    evaluation (velocity and the double dot product).  `value` is the
    FP32-compensated form (context precision FP32C); the FP64 form (the
    reference's arithmetic) is timed on one step beside it.  Accuracy:
    FP32C against the FP64 path on every leaf target; FP64 against the CPU
    oracle on 2,048 seeded vertex targets."""
    import torch

    from lpm_gb300 import build as B
    from lpm_gb300 import core
    from lpm_gb300 import functors as F

    B.build()
    torch.cuda.set_device(device)
    ctx = core.Context(device)
    stream = torch.cuda.current_stream(device)
    ctx.set_stream(stream)
    level, eps = args.swe_level, 0.01
    vx, fx, fa, fm = core.build_mesh(core.MESH_ICOS_TRI, level, 1.0)
    zeta = 2 * OMEGA * fx[:, 2] + 0.5 * fx[:, 2] * (1 - fx[:, 2] ** 2) ** 2 * np.cos(
        4 * np.arctan2(fx[:, 1], fx[:, 0]))
    sigma = 0.2 * np.sin(3 * fx[:, 0]) * fx[:, 1] + 0.05 * np.random.default_rng(7).standard_normal(fx.shape[0])
    d = torch.device("cuda", device)
    T = {k: torch.tensor(v, device=d) for k, v in
         dict(vx=vx, fx=fx, fa=fa, fm=fm, z=zeta, s=sigma).items()}
    nv, ntot, nleaf = vx.shape[0], fx.shape[0], int((fm == 0).sum())
    pairs = (nv + ntot) * nleaf
    outs = {p: (F.swe_sphere_vertex_sums(ctx, T["vx"], T["fx"], T["z"], T["s"], T["fa"], T["fm"],
                                         eps),
                F.swe_sphere_face_sums(ctx, T["fx"], T["z"], T["s"], T["fa"], T["fm"], eps))
            for p in (core.FP64, core.FP32C)}

    def step(prec):
        ctx.set_precision(prec)
        ov, of = outs[prec]
        F.swe_sphere_vertex_sums(ctx, T["vx"], T["fx"], T["z"], T["s"], T["fa"], T["fm"], eps,
                                 out=ov)
        F.swe_sphere_face_sums(ctx, T["fx"], T["z"], T["s"], T["fa"], T["fm"], eps, out=of)

    def timed(prec, n, flush_buf):
        ms = 0.0
        for k in range(n):
            flush_buf.fill_(float(k))
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step(prec)
            b.record(stream)
            torch.cuda.synchronize(device)
            ms += a.elapsed_time(b)
        return ms

    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)
    step(core.FP64)
    torch.cuda.synchronize(device)
    ms64 = timed(core.FP64, 1, flush)
    for _ in range(args.warmup):
        step(core.FP32C)
    torch.cuda.synchronize(device)
    fma64 = ctx.fma_peak_tflops(core.FP64)
    peak32, sm_max, nsm = fp32_peak(device)
    sampler = ClockSampler(device)
    sampler.start()
    l0 = ctx.kernel_launches
    ms = timed(core.FP32C, args.steps, flush)
    clocks = sampler.stop()
    launches = ctx.kernel_launches - l0
    pairs_per_s = pairs * args.steps / (ms * 1e-3)
    # end to end (FP32C): host inputs in, velocity + ddot out, every step
    host = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in
            dict(vx=vx, fx=fx, fa=fa, fm=fm, z=zeta, s=sigma).items()}
    h_out = [torch.empty(nv, 3, dtype=torch.float64).pin_memory(),
             torch.empty(nv, dtype=torch.float64).pin_memory(),
             torch.empty(ntot, 3, dtype=torch.float64).pin_memory(),
             torch.empty(ntot, dtype=torch.float64).pin_memory()]
    bi = sum(t.numel() * t.element_size() for t in host.values())
    bo = sum(t.numel() * t.element_size() for t in h_out)
    ov32, of32 = outs[core.FP32C]
    ms_e2e = 0.0
    n_e2e = max(1, args.steps // 2)
    for k in range(n_e2e):
        flush.fill_(float(k))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for key, t in host.items():
            T[key].copy_(t, non_blocking=True)
        step(core.FP32C)
        for dst, src in zip(h_out, (ov32["u"], ov32["ddot"], of32["u"], of32["ddot"])):
            dst.copy_(src, non_blocking=True)
        b.record(stream)
        torch.cuda.synchronize(device)
        ms_e2e += a.elapsed_time(b)
    e2e = pairs * n_e2e / (ms_e2e * 1e-3) / 1e9
    # FP32C against FP64 on every leaf target (vertices and leaf faces)
    ov64, of64 = outs[core.FP64]
    leaf = T["fm"] == 0
    err32 = {"velocity_vertices": rel_errors(ov32["u"], ov64["u"]),
             "velocity_leaf_faces": rel_errors(of32["u"][leaf], of64["u"][leaf]),
             "ddot_vertices": rel_errors(ov32["ddot"], ov64["ddot"]),
             "ddot_leaf_faces": rel_errors(of32["ddot"][leaf], of64["ddot"][leaf])}
    # FP64 against the CPU oracle, and the CPU baseline on the same sample
    sys.path.insert(0, str(ROOT / "oracle"))
    import lpm_oracle

    threads = os.cpu_count() or 1
    lpm_oracle.set_threads(threads)
    idx = np.sort(np.random.default_rng(20261203).choice(nv, min(2048, nv), replace=False))
    t0 = time.perf_counter()
    ref = lpm_oracle.swe_sphere_sums(vx[idx], fx, zeta, sigma, fa, fm, eps)
    cpu_s = time.perf_counter() - t0
    got_u = ov64["u"].cpu().numpy()[idx]
    got_d = ov64["ddot"].cpu().numpy()[idx]
    ref_d = lpm_oracle.double_dot(ref[:, 3:])
    err64 = {"velocity_linf": float(np.abs(got_u - ref[:, :3]).max() / np.abs(ref[:, :3]).max()),
             "ddot_linf": float(np.abs(got_d - ref_d).max() / np.abs(ref_d).max())}
    plane = swe_plane_measure(ctx, stream, flush, args, lpm_oracle)
    ach = pairs_per_s * SWE32_FLOPS_PER_PAIR / 1e12
    ach64 = pairs / (ms64 * 1e-3) * SWE_FLOPS_PER_PAIR / 1e12
    return {"metric": "spherical SWE direct sums Ginteractions/s (velocity + double dot)",
            "value": round(pairs_per_s / 1e9, 3), "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (generated icosahedral mesh, analytic + seeded fields)",
            "config": {"workload": f"spherical SWE vertex + face sums, icosahedral level {level}, "
                                   f"eps={eps}", "vertices": nv, "face_slots": ntot,
                       "leaf_faces": nleaf, "interactions_per_step": pairs,
                       "l2": "flushed between timed steps (512 MiB write)"},
            "e2e": {"value": round(e2e, 3), "unit": UNIT, "h2d_bytes_per_step": bi,
                    "d2h_bytes_per_step": bo},
            "roofline": {"bound": "fp32", "achieved": round(ach, 3), "peak": round(peak32, 2),
                         "unit": "TFLOP/s", "frac": round(ach / peak32, 4), "traffic": None,
                         "kernel": "k_swe_sphere32 (whole step timed)",
                         "flops_per_pair_credited": SWE32_FLOPS_PER_PAIR,
                         "peak_kind": f"computed FP32 FMA peak 2*128*{nsm} SMs*{sm_max:.0f} MHz"},
            "fp64": {"value": round(pairs / (ms64 * 1e-3) / 1e9, 4), "unit": UNIT,
                     "ms_per_step": round(ms64, 2),
                     "roofline": {"bound": "fp64", "achieved": round(ach64, 4),
                                  "peak": round(fma64, 4), "unit": "TFLOP/s",
                                  "frac": round(ach64 / fma64, 4),
                                  "flops_per_pair_credited": SWE_FLOPS_PER_PAIR,
                                  "peak_kind": "measured FP64 FMA peak (lpm_measure_fma_peak)"}},
            "errors_fp32c_vs_fp64_all_leaf_targets": err32,
            "plane": plane,
            "errors_fp64_vs_oracle_2048_vertex_targets": err64,
            "cpu_baseline": {"value": round(idx.size * nleaf / cpu_s / 1e9, 5), "unit": UNIT,
                             "cores": threads, "kind": "port",
                             "sample": f"{idx.size} vertex targets x {nleaf} leaf faces, FP64"},
            "clocks": clocks, "gpu_launches": launches}


def run_c5(args, device):
    """Configuration C5: BVE sphere at icosahedral level 8 (1,310,720 leaf
    faces, 655,362 vertices), Rossby-Haurwitz R=4 (omega = K = Omega/12.5),
    eps = 0.01, RK4 dt = 0.005, evaluated by the octree far field (leaves <= 64
    points, opening angle 0.5, order-4 expansion, exact FP32-compensated near
    field) with the learned correction: a BF16 MLP (moments to order 4 in the
    target's cell frame, 3 x 128 SiLU) trained on the GPU by the tcgen05
    kernels on 2^24 cell-target samples from seeded random vortex fields.
    value = direct-equivalent interactions ((Nv + Nf) Nf per evaluation) per
    second.  References for the error: the GPU FP64 direct sum (reference
    arithmetic) on a seeded 16,384-target subsample for one evaluation, and
    the FP32C direct-sum trajectory (1.6e-7 from FP64 after a step, C2) for
    the steps; the FP64 time per evaluation is the subsample's time scaled
    linearly to all targets."""
    import torch

    from lpm_gb300 import build as B
    from lpm_gb300 import core
    from lpm_gb300 import functors as F
    from lpm_gb300.farfield import FarField

    B.build()
    torch.cuda.set_device(device)
    ctx = core.Context(device)
    stream = torch.cuda.current_stream(device)
    ctx.set_stream(stream)
    L = args.c5_level
    t0 = time.perf_counter()
    vx, fx, fa, fm = core.build_mesh(core.MESH_ICOS_TRI, L, 1.0)
    mesh_host_s = time.perf_counter() - t0
    core.build_mesh_device(ctx, core.MESH_ICOS_TRI, L)  # warm
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    core.build_mesh_device(ctx, core.MESH_ICOS_TRI, L)
    torch.cuda.synchronize(device)
    mesh_dev_s = time.perf_counter() - t0
    w = OMEGA / 12.5
    vz = core.eval_ic(core.IC_RH54, (w, -w), vx)
    fz = core.eval_ic(core.IC_RH54, (w, -w), fx)
    nv, nleaf = vx.shape[0], int((fm == 0).sum())
    ipe = (nv + nleaf) * nleaf
    st0 = DeviceState((vx, fx, fa, fm, vz, fz), device)
    # ---- network: trained here on the GPU (not in the timed region) ----------
    theta = 0.5 if args.ff_theta is None else args.ff_theta
    ff = FarField(theta=theta, leaf_max=64, rho_min=args.ff_rho_min, ctx=ctx)
    t0 = time.perf_counter()
    if args.ff_weights:
        saved = np.load(args.ff_weights)
        ff.set_weights(saved["w"], saved["norm"])
        ff.set_network(True)
        loss = [float(x) for x in saved["loss"]] if "loss" in saved else []
    else:
        loss = ff.train(nsamples=args.ff_samples, epochs=args.ff_epochs, batch=16384, lr=2e-3,
                        seed=20261203, level_min=5, level_max=8, eps=EPS)
    torch.cuda.synchronize(device)
    train_s = time.perf_counter() - t0
    if args.ff_save:
        wv, nv_ = ff.get_weights()
        np.savez(args.ff_save, w=wv, norm=nv_, loss=np.array(loss))
    # ---- one evaluation: learned / expansion only vs the GPU FP64 direct sum --
    xall = torch.cat([st0.vx, st0.fx[st0.fm == 0]])
    rng = np.random.default_rng(20261203)
    idx = torch.from_numpy(np.sort(rng.choice(xall.shape[0], 16384, replace=False))).to(xall.device)
    xs = xall[idx].contiguous()
    ctx.set_precision(core.FP64)
    u64 = torch.zeros_like(xs)
    F.ic2d_passive_sums(ctx, u64, None, xs, st0.fx, st0.fz, st0.fa, st0.fm, EPS)  # warm
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    F.ic2d_passive_sums(ctx, u64, None, xs, st0.fx, st0.fz, st0.fa, st0.fm, EPS)
    b.record(stream)
    torch.cuda.synchronize(device)
    fp64_eval_s = a.elapsed_time(b) * 1e-3 * xall.shape[0] / xs.shape[0]
    ctx.set_precision(core.FP32C)  # every target: the FP32C direct sum as the reference
    uall32 = torch.zeros_like(xall)
    F.ic2d_passive_sums(ctx, uall32, None, xall, st0.fx, st0.fz, st0.fa, st0.fm, EPS)
    uall = torch.zeros_like(xall)
    errs, errs_all = {}, {}
    for tag, net in (("expansion_only", False), ("learned", True)):
        ff.set_network(net)
        ff.velocity(uall, xall, st0.fx, st0.fz, st0.fa, st0.fm, EPS)
        torch.cuda.synchronize(device)
        errs[tag] = rel_errors(uall[idx], u64)
        errs_all[tag] = rel_errors(uall, uall32)
    errs_all["fp32c_direct_vs_fp64_on_the_16384_targets"] = rel_errors(uall32[idx], u64)
    stats = ff.stats()
    ff.set_network(True)
    # ---- RK4 steps on the learned far field --------------------------------
    flags = core.STEP_SKIP_MASKED_TARGETS | core.STEP_REPROJECT
    st = st0.clone()
    st.velocity(ctx, core.FP64_CHORD)
    h = make_stepper(ctx, st, core.FP64_CHORD, flags)
    core.check(core.lib().lpm_bve_rk4_set_farfield(h, ff.handle, 0))
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=device)
    for _ in range(args.warmup):
        advance(h, st)
    torch.cuda.synchronize(device)
    sampler = ClockSampler(device)
    sampler.start()
    l0 = ctx.kernel_launches
    ms = 0.0
    for k in range(args.steps):
        flush.fill_(float(k))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        advance(h, st)
        b.record(stream)
        torch.cuda.synchronize(device)
        ms += a.elapsed_time(b)
    clocks = sampler.stop()
    launches = ctx.kernel_launches - l0
    # ---- e2e: the state in host buffers, copied in and out inside the timing
    # (the device state is restored afterwards for the trajectory comparison)
    names = ("vx", "vz", "vu", "fx", "fz", "fu")
    keep = {k: getattr(st, k).clone() for k in names}
    hostbufs = {k: getattr(st, k).cpu().pin_memory() for k in names}
    h2d = sum(t.numel() * t.element_size() for t in hostbufs.values())
    ms_e2e = 0.0
    n_e2e = max(1, args.steps // 2)
    for k in range(n_e2e):
        flush.fill_(float(k))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for name, hb in hostbufs.items():
            getattr(st, name).copy_(hb, non_blocking=True)
        advance(h, st)
        for name, hb in hostbufs.items():
            hb.copy_(getattr(st, name), non_blocking=True)
        b.record(stream)
        torch.cuda.synchronize(device)
        ms_e2e += a.elapsed_time(b)
    e2e = {"value": round(4 * ipe * n_e2e / (ms_e2e * 1e-3) / 1e9, 3), "unit": UNIT,
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d}
    for k in names:
        getattr(st, k).copy_(keep[k])
    torch.cuda.synchronize(device)
    core.lib().lpm_bve_rk4_destroy(h)
    # ---- the same steps with the FP32C direct sum (trajectory reference) --------
    ref = st0.clone()
    ref.velocity(ctx, core.FP32C)
    hr = make_stepper(ctx, ref, core.FP32C, flags)
    for _ in range(args.warmup + args.steps):
        advance(hr, ref)
    torch.cuda.synchronize(device)
    core.lib().lpm_bve_rk4_destroy(hr)
    traj = {"position_leaf_faces": rel_errors(st.fx, ref.fx, st.fm),
            "vorticity_leaf_faces": rel_errors(st.fz, ref.fz, st.fm),
            "velocity_leaf_faces": rel_errors(st.fu, ref.fu, st.fm),
            "velocity_vertices": rel_errors(st.vu, ref.vu)}
    # ---- kernel split of one step (events around the tree and network parts)
    hs = make_stepper(ctx, st, core.FP64_CHORD, flags | core.STEP_TIME_NBODY)
    core.check(core.lib().lpm_bve_rk4_set_farfield(hs, ff.handle, 0))
    ff.timing(True)
    advance(hs, st)
    tree_ms, net_ms, nev = ff.timing(False)
    core.lib().lpm_bve_rk4_destroy(hs)
    rows = stats["network_rows"]
    flops_row = 2 * (48 * 128 + 2 * 128 * 128 + 128 * 16)  # one (target, cell) row, 4 layers
    peaks = {}
    pp = ROOT / "MEASURED_PEAKS.json"
    if pp.exists():
        peaks = json.loads(pp.read_text())
    peak = peaks.get("bf16_tflops")
    net_tf = rows * flops_row / (net_ms / nev * 1e-3) / 1e12 if nev and net_ms > 0 else None
    step_s = ms / args.steps * 1e-3
    return {"metric": METRIC,
            "value": round(4 * ipe / step_s / 1e9, 3), "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+bf16", "data": "synthetic (generated mesh + Rossby-Haurwitz wave; "
                                          "network trained on seeded random vortex fields)",
            "config": {"workload": f"BVE sphere icosahedral level {L} RK4, RH R=4, eps={EPS}, "
                                   f"dt={DT}, octree far field theta={theta} leaf<=64 + learned "
                                   f"correction for rho >= {args.ff_rho_min}", "vertices": nv, "leaf_faces": nleaf,
                       "direct_equivalent_interactions_per_step": 4 * ipe,
                       "l2": "flushed between timed steps (512 MiB write)",
                       "training": ({"loaded": str(args.ff_weights)} if args.ff_weights else
                                    {"samples": args.ff_samples, "epochs": args.ff_epochs,
                                     "batch": 16384, "seconds": round(train_s, 2),
                                     "loss_per_epoch": [round(float(x), 6) for x in loss]})},
            "mesh_build_seconds": {"host": round(mesh_host_s, 3), "device": round(mesh_dev_s, 4)},
            "e2e": e2e,
            "speedup_vs_gpu_fp64_direct": round(fp64_eval_s / (step_s / 4), 1),
            "fp64_direct": {"seconds_per_evaluation": round(fp64_eval_s, 3),
                            "value": round(ipe / fp64_eval_s / 1e9, 3),
                            "note": "reference arithmetic on 16,384 seeded targets, scaled "
                                    "linearly to all targets"},
            "errors_one_evaluation_vs_fp64_direct_16384_targets": errs,
            "errors_one_evaluation_all_targets_vs_fp32c_direct": errs_all,
            "errors_after_steps_vs_fp32c_direct": traj,
            "far_field": {**stats, "tree_ms_per_evaluation": round(tree_ms / max(nev, 1), 3),
                          "network_ms_per_evaluation": round(net_ms / max(nev, 1), 3)},
            "roofline": {"bound": "tensor", "kernel": "k_ff_mlp (tcgen05 BF16 MLP, 4 layers)",
                         "achieved": round(net_tf, 2) if net_tf else None,
                         "peak": peak, "unit": "TFLOP/s",
                         "frac": round(net_tf / peak, 4) if (net_tf and peak) else None,
                         "traffic": None,
                         "flops_per_row": flops_row, "rows_per_evaluation": rows,
                         "tiles_of_128_rows": -(-rows // 128),
                         "peak_kind": "bf16_tflops of MEASURED_PEAKS.json (burst)"},
            "clocks": clocks, "gpu_launches": launches}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--level", type=int, default=LEVEL)
    ap.add_argument("--config", choices=["c1", "c2", "c3", "c4", "c5", "swe", "fp64"],
                    default="c2",
                    help="c2: the metric's workload (default); c1: FP64 level 4; "
                         "c3: planar dipoles; c4: 256-problem ensemble; "
                         "c5: level 8 on the learned octree far field; "
                         "swe: spherical shallow-water sums (FP64)")
    ap.add_argument("--swe-level", type=int, default=6)
    ap.add_argument("--swe-plane-level", type=int, default=7)
    ap.add_argument("--ff-samples", type=int, default=1 << 24)
    ap.add_argument("--ff-epochs", type=int, default=16)
    ap.add_argument("--ff-theta", type=float, default=None,
                    help="far field opening angle (cells accepted when h <= theta (D - r)); "
                         "default 0.5 for c5 (its specification), 0.4 for the learned "
                         "block of c2")
    ap.add_argument("--ff-rho-min", type=float, default=0.25,
                    help="c5: learned correction for cells with h/(D - r_block) >= this")
    ap.add_argument("--ff-save", default=None, help="c5: save the trained network (.npz)")
    ap.add_argument("--ff-weights", default=None,
                    help="c5: load a saved network instead of training")
    ap.add_argument("--plane-level", type=int, default=9)
    ap.add_argument("--fp32-shape", type=int, default=None, choices=range(6),
                    help="c2/c3: fixed FP32 kernel shape instead of the per-size autotuner")
    ap.add_argument("--problems", type=int, default=256)
    ap.add_argument("--ens-plan", default=None,
                    help="c4: fixed plan 'chunk_len,shape,persistent' instead of the autotuner")
    ap.add_argument("--cpu-targets", type=int, default=16384)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-learned", action="store_true",
                    help="c2: skip the learned far-field evaluation")
    ap.add_argument("--no-other", action="store_true",
                    help="c2: skip the short C3 and C4 legs")
    ap.add_argument("--no-c5", action="store_true",
                    help="c2: skip the level-8 far-field leg (configuration C5)")
    ap.add_argument("--c5-level", type=int, default=8,
                    help="c5: icosahedral level (the configuration's is 8)")
    ap.add_argument("--c5-steps", type=int, default=3,
                    help="c2: timed RK4 steps per far-field setting of the level-8 leg")
    ap.add_argument("--only-headline", action="store_true",
                    help="time the FP32C steps only (for profiler runs)")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return

    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    if args.config == "c4":
        res = run_ensemble(args, local) if rank == 0 else {}
    elif args.config == "c3":
        res = run_plane(args, local) if rank == 0 else {}
    elif args.config == "c1":
        res = run_c1(args, local) if rank == 0 else {}
    elif args.config == "c5":
        res = run_c5(args, local) if rank == 0 else {}
    elif args.config == "swe":
        res = run_swe(args, local) if rank == 0 else {}
    elif args.config == "fp64":
        res = run_fp64(args, local) if rank == 0 else {}
    else:
        res = run_ours(args, rank, world, local)
    if rank == 0:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

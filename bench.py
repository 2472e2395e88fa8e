"""Benchmark of the GB300 WCSPH step (one JSON line on stdout).

Workload: ``obstacle_1m`` — 1,048,576 FP32 particles (128 x 128 x 64 jittered lattice, spacing
0.0075 m, h = 0.015 m) in a 2 x 1 x 1 m box with a sphere obstacle (r = 0.2 m, 128^3 volume map),
dt = 1e-4. A step is one WCSPH substep of every particle (key, sort, cells + reorder, boundary +
density, pressure + viscosity + integration).

* ``value``  particle-steps/s with the state resident in HBM, device-timed with CUDA events per
  step on the launching stream; L2 is flushed (256 MiB write) between timed steps.
* ``e2e``    the same metric through the public C ABI with host buffers: per step the state is
  uploaded from pinned memory, one substep runs, and positions, velocities and densities are
  read back, in one vfs_model_step_host call (one wait); wall-clock over the K steps.
* ``roofline`` the dominant kernel's algorithmic bytes per launch / its mean event-timed duration
  against the measured HBM copy bandwidth.
* ``cpu_baseline`` the oracle (the project's restatement of the reference's shader math) on the
  host's cores, on a bounded sample of the same workload.
* ``full_run`` the configured 1000-substep run timed end to end from the initial state (the run
  blows up near substep 250 with the configured parameters, in the oracle as on the GPU; its
  per-segment times show what that does to the cost).

``--impl reference`` times the reference's own step code on every host thread: its Slang compute
shaders compiled as C++ for the host and driven in the order of its host code (oracle/_ref), or,
where that build is absent, the oracle. The reference's Vulkan pipeline itself has no runnable
form here (no Vulkan stack or software renderer exists).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from dataclasses import replace
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s @1M (plain vs batched vs fwd+adjoint, 1e-5 rel), % HBM roofline"
UNIT = "particle-steps/s"
# Algorithmic HBM bytes per particle-step and per pass (compulsory traffic between the passes'
# global dependencies, float3 fields): key 16, sort 12, cell starts 8, reorder 52,
# density + boundary 28, force + integrate 64.
B_STEP = 180
STRESS_NBR_SLOTS = 1536
B_PHASE = {"keys": 16, "sort": 12, "cells_reorder": 60, "density": 28, "force": 64}
FLUSH_BYTES = 256 << 20


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class _Nvml:
    """Read-only NVML queries through ctypes (the driver's libnvidia-ml): SM clock, its maximum
    and the active clock-event reasons of one device. None when the library is unavailable."""

    # nvmlClocksEventReason* bits (nvml.h).
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, index: int):
        import ctypes as C

        lib = C.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.C, self.lib = C, lib
        self.h = C.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(index), C.byref(self.h)) != 0:
            raise OSError("no NVML device")
        mx = C.c_uint()
        lib.nvmlDeviceGetMaxClockInfo(self.h, C.c_int(1), C.byref(mx))  # NVML_CLOCK_SM
        self.max_mhz = float(mx.value)
        self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")

    def sample(self):
        C = self.C
        clk, bits = C.c_uint(), C.c_ulonglong()
        self.lib.nvmlDeviceGetClockInfo(self.h, C.c_int(1), C.byref(clk))
        self.reasons_fn(self.h, C.byref(bits))
        return float(clk.value), int(bits.value)


class ClockSampler:
    """SM clock and clock-event reasons during a timed region: NVML polled every ~2 ms from a
    thread (the timed regions last milliseconds), else nvidia-smi at its 200 ms period."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.nvml = None
        self.samples = []
        self.out = ""

    def _poll(self):
        while not self._stop.is_set():
            try:
                self.samples.append(self.nvml.sample())
            except Exception:
                return
            self._stop.wait(0.002)

    def __enter__(self):
        try:
            self.nvml = _Nvml(self.index)
        except Exception:
            self.nvml = None
        if self.nvml is not None:
            import threading

            self._stop = threading.Event()
            self.samples.append(self.nvml.sample())
            self._thread = threading.Thread(target=self._poll, daemon=True)
            self._thread.start()
            return self
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.nvml is not None:
            self._stop.set()
            self._thread.join(timeout=5)
            self.samples.append(self.nvml.sample())
            return
        if self.proc:
            self.proc.terminate()
            try:
                self.out = self.proc.communicate(timeout=5)[0]
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""

    def summary(self):
        if self.nvml is not None:
            reasons = set()
            for _, bits in self.samples:
                for bit, name in _Nvml.REASONS.items():
                    if bits & bit:
                        reasons.add(name)
            sm = [c for c, _ in self.samples]
            return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": self.nvml.max_mhz,
                    "reasons": sorted(reasons), "samples": len(sm), "source": "nvml"}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm), "source": "nvidia-smi"}


def issue_roofline(inst_pp, phase_ms, n, device, clocks):
    """The neighbour passes against the instruction-issue roofline: warp instructions per launch
    (per particle from one ncu capture of this workload, smsp__inst_executed.sum, times N) over the
    pass's event-timed duration, against one warp instruction per cycle on each of an SM's four
    schedulers at the SM clock sampled during the timed region."""
    import torch

    sms = torch.cuda.get_device_properties(device).multi_processor_count
    mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz")
    if not inst_pp or not mhz:
        return None
    peak = sms * 4 * mhz * 1e6
    out = {"unit": "G warp-instructions/s", "peak": peak / 1e9, "sms": sms, "sm_mhz": mhz,
           "source": "profiles/ncu_traffic.json warp_instructions_per_particle"}
    for k in ("density", "force"):
        if k in inst_pp and k in phase_ms:
            inst = inst_pp[k] * n
            achieved = inst / (phase_ms[k] * 1e-3)
            out[k] = {"warp_instructions_per_launch": inst, "achieved": achieved / 1e9,
                      "frac": achieved / peak}
    return out


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x: float, world: int, device=None) -> float:
    """The largest x over all ranks (the job's time is its slowest replica's); x itself at N=1."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: int, steps: int, total_ms: float, world: int,
                       device=None) -> tuple[float, float]:
    """Whole-job throughput of `world` independent replicas, each processing units_per_rank units
    per step for `steps` steps: all ranks' units over the slowest rank's time. Returns (value,
    max total ms)."""
    ms = max_over_ranks(total_ms, world, device)
    return world * units_per_rank * steps / (ms / 1e3), ms


def oracle_for_workload(w, model=None):
    """CPU oracle of the workload; boundary grids from the GPU model or built on the CPU."""
    from oracle import binding as ob

    o = ob.OracleModel(ob.params_from(w.sim, w.sph, w.wcsph), w.n)
    if model is not None:
        for i in range(model.n_boundary_objects):
            o.add_object(model.get_boundary_object(i))
    else:
        for a in w.objects:
            bs, bp, sdf, vm = ob.volume_map(a.shape, a.params, w.sim.smooth_radius, a.resolution,
                                            np.float32(8.0 * w.sim.smooth_radius))
            T = np.eye(4, dtype=np.float32)
            T[:3, 3] = -np.asarray(a.position, np.float32)
            o.add_object(type("Obj", (), dict(
                transform=T.T.ravel(), rotation=np.eye(4, dtype=np.float32).ravel(),
                box_size=bs, box_pos=bp, resolution=tuple(a.resolution), sdf=sdf,
                volume_map=vm)))
    o.set_state(w.pos, w.vel)
    return o


def time_cpu(w, model=None, budget_s=12.0, max_steps=200, threads=None):
    from oracle import binding as ob

    o = oracle_for_workload(w, model)  # boundary grids built with every host thread
    if threads:
        ob.set_threads(threads)
    o.substeps(1)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps:
        o.substeps(1)
        steps += 1
        if time.perf_counter() - t0 >= budget_s and steps >= 2:
            break
    dt = time.perf_counter() - t0
    return {"value": w.n * steps / dt, "unit": UNIT, "cores": ob.get_threads(), "kind": "port",
            "sample": f"{w.name}: {steps} substeps of {w.n} particles after 1 warm-up substep "
                      f"({dt:.1f} s wall)"}


def workload_config(name: str, n: int, h: float, dt: float, boundary: str) -> dict:
    """The `config` both arms print for the timed workload (identical dicts: the arms run the
    same scene from the same seeded initial state and time the same substeps)."""
    return {"workload": name, "particles": int(n), "h": float(h), "dt": float(dt),
            "boundary": boundary, "substeps_timed": "the --steps substeps after --warmup, from "
                                                    "the seeded initial state",
            "l2": "GPU arm: flushed between timed steps (256 MiB write)"}


def _mapped_libraries() -> list:
    """Shared objects of this repository mapped into this process (from /proc/self/maps)."""
    out = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                p = line.split()[-1] if line.strip() else ""
                if p.endswith(".so") and str(ROOT) in p:
                    out.add(os.path.relpath(p, ROOT))
    except OSError:
        pass
    return sorted(out)


def run_reference(args):
    """The reference arm, on every host thread, on the same workload as the GPU arm: --warmup
    untimed substeps, then exactly --steps timed substeps (wall clock). It runs the reference's
    own step code (its Slang compute shaders compiled as C++ for the host, oracle/_ref, driven in
    the order of its host code) when that build exists, else the project's CPU restatement of it
    (the oracle, pinned bit for bit to that build). It never imports the product package."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import binding as ob
    from oracle import ref_binding as rb
    from oracle.workloads import Obstacle1M

    w = Obstacle1M()
    w.objects()  # the sphere's grids, built by the oracle's generator on every host thread
    threads = os.cpu_count() or 1
    if rb.available():
        r = rb.RefShaderModel(w.params(), w.n)
        for info in w.objects():
            r.add_object(info)
        r.set_state(w.pos, w.vel)
        rb.set_threads(threads)
        step, kind, cores = r.step, "reference", rb.get_threads()
        what = ("the reference's step shaders compiled as C++ for the host (oracle/_ref), OpenMP "
                "over each dispatch's ids; the counting sort's atomic passes in index order")
    else:
        o = w.oracle()
        ob.set_threads(threads)
        step, kind, cores = o.substeps, "port", ob.get_threads()
        what = ("the project's CPU restatement of the reference's shader math (oracle), OpenMP "
                "on all host threads")
    step(args.warmup)
    t0 = time.perf_counter()
    step(args.steps)
    dt = time.perf_counter() - t0
    value = w.n * args.steps / dt
    libs = _mapped_libraries()
    if any("vkfluidsim_gb300" in p for p in libs):
        raise RuntimeError(f"the reference arm mapped the product library: {libs}")
    cpu = {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
           "sample": f"{w.name}: {args.steps} substeps of {w.n} particles after {args.warmup} "
                     f"warm-up substeps ({dt:.1f} s wall)"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded jittered lattice (no dataset exists for this path)",
            "impl": "reference",
            "config": workload_config(w.name, w.n, w.h, w.dt, "sphere r=0.2, 128^3 volume map"),
            "cpu_baseline": cpu,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "libraries_mapped": libs,
            "note": "the reference's own pipeline is Vulkan/Slang, which cannot run on this box "
                    "(no Vulkan stack or software renderer); timed here: " + what}
    print(json.dumps(line), flush=True)


def time_batched(args, stream, torch):
    """Batched scenes (256 independent dam breaks, 4.58M particles): one batched substep against a
    loop of one plain model per scene on the same stream; both device-timed with CUDA events."""
    from vkfluidsim_gb300 import workloads as W

    scenes = W.batched_scenes(n_scenes=args.batch_scenes)
    total = sum(w.n for w in scenes)
    b = W.build_batch(scenes)
    b.set_stream(stream.cuda_stream)
    tuned = b.autotune(repeats=2) if args.autotune else b.get_tune_config()
    for _ in range(args.warmup):
        b.substeps(1)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.substeps(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    t_batch = e0.elapsed_time(e1) / args.steps
    b.synchronize()
    prof = b.profile_substeps(3)
    del b
    models = [W.build_model(w) for w in scenes]
    for m in models:
        m.set_stream(stream.cuda_stream)
        for _ in range(args.warmup):
            m.substeps(1)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        for m in models:
            m.substeps(1)
    e1.record(stream)
    torch.cuda.synchronize()
    t_loop = e0.elapsed_time(e1) / args.steps
    for m in models:
        m.synchronize()
    del models
    return {"scenes": len(scenes), "particles": total,
            "value": total / (t_batch * 1e-3), "ms_per_step": t_batch,
            "loop_value": total / (t_loop * 1e-3), "loop_ms_per_step": t_loop,
            "speedup_vs_loop": t_loop / t_batch, "phase_ms": prof, "launch_shapes": tuned,
            "config": "N_s log-uniform [2048, 65536], nu_s log-uniform [1e-3, 5e-2], "
                      "k_s uniform [20, 100], own 64^3 container map per scene, dt 2e-4; "
                      "working set > L2"}


def time_adjoint(args, stream, torch):
    """Differentiable rollout (65,536-particle dam break, 300 substeps, checkpoint every
    25). The target is the rollout with viscosity 0.02, stiffness 60 and a smooth initial velocity
    (8 Fourier modes, 0.5 m/s); the optimised run starts from viscosity 0.01, stiffness 50, zero
    velocity; loss = MSE of final positions by id. Times the plain forward rollout against forward
    + checkpointed adjoint (wall clock around synchronised C-ABI calls on the model's stream), each
    after one untimed pass that captures its CUDA graphs."""
    import vkfluidsim_gb300 as vfs
    from vkfluidsim_gb300 import workloads as W
    from vkfluidsim_gb300.adjoint import Rollout

    base = W.dam_break_64k()
    steps, every = base.steps, 25
    tw = replace(base, vel=vfs.generate_fourier_velocity(base.pos, 8, 0.5, 4),
                 wcsph=replace(base.wcsph, viscosity_strenght=0.02, stiffness=60.0))
    tm = W.build_model(tw)
    tm.set_stream(stream.cuda_stream)
    tm.substeps(steps)
    ts = tm.copy_data_buffers()
    target = np.empty_like(ts["positions"])
    target[tm.get_ids()] = ts["positions"]
    del tm
    m = W.build_model(base)
    m.set_stream(stream.cuda_stream)
    m.substeps(3)  # warm-up (graph capture)
    m.set_particle_state(base.pos, base.vel)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    m.substeps(steps)
    m.synchronize()
    t_fwd = time.perf_counter() - t0
    ro = Rollout(m, steps, every)
    for timed in (False, True):  # the first pass captures the segment graph
        m.set_particle_state(base.pos, base.vel)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ro.forward()
        xf = ro.final_positions_by_id()
        g = ro.backward(2.0 * (xf - target) / xf.size)
        t_all = time.perf_counter() - t0
    return {"particles": base.n, "steps": steps, "checkpoint_every": every,
            "forward_ms_per_step": 1e3 * t_fwd / steps,
            "fwd_adjoint_ms_per_step": 1e3 * t_all / steps,
            "cost_vs_forward": t_all / t_fwd,
            "value": base.n * steps / t_all,
            "loss": float(np.mean((xf - target) ** 2)),
            "grads": {"dnu": g["dnu"], "dk": g["dk"], "dv0_max": float(np.abs(g["dv0"]).max())}}


def time_stress(args, stream, torch):
    """Stress workload (4,194,304 uniform particles in a 4 x 2 x 2 box plus a 419,430-particle
    Gaussian blob, sigma 0.1, h = 0.02, 128^3 container volume map): one substep from the same
    initial state, repeated (state re-uploaded untimed before each repeat). Reports the sort's
    pair throughput (N x 16 B per pass-equivalent: read + write of key and value) and the
    density/force fractions of the HBM roofline."""
    from vkfluidsim_gb300 import workloads as W

    w = W.stress_4m()
    m = W.build_model(w)
    m.set_stream(stream.cuda_stream)
    m.set_neighbor_capacity(STRESS_NBR_SLOTS)  # the blob's ~900 neighbours fit the lists
    # Launch shapes for this state (the autotuner restores the state before every candidate).
    tuned = m.autotune(repeats=3, use_cache=False) if args.autotune else m.get_tune_config()
    reps = max(3, min(args.steps, 10))
    for _ in range(args.warmup):
        m.set_particle_state(w.pos, w.vel)
        m.substeps(1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ms = []
    for _ in range(reps):
        m.set_particle_state(w.pos, w.vel)
        torch.cuda.synchronize()
        e0.record(stream)
        m.substeps(1)
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    phase = {}
    for _ in range(3):
        m.set_particle_state(w.pos, w.vel)
        for k, v in m.profile_substeps(1).items():
            phase.setdefault(k, []).append(v)
    phase = {k: float(np.median(v)) for k, v in phase.items()}
    hbm, _ = peaks()
    n = w.n
    digits, items, passes = m.get_sort_config()
    frac = {k: B_PHASE[k] * n / (phase[k] * 1e-3) / 1e9 / hbm for k in ("density", "force") if k in phase}
    del m
    return {"workload": w.name, "particles": n, "repeats": reps, "neighbor_slots": STRESS_NBR_SLOTS,
            "launch_shapes": tuned,
            "ms_per_step": float(np.median(ms)), "value": n / (float(np.median(ms)) * 1e-3),
            "phase_ms": phase,
            "sort": {"digit_bits": digits, "passes": passes,
                     "pair_gbs": 16 * n / (phase["sort"] * 1e-3) / 1e9},
            "roofline_frac": frac}


def time_next_rows(args, stream, torch, model, rank):
    """Setup and output paths beside the step: GPU volume-map generation (analytic sphere at 128^3
    and 64^3, a 320-triangle mesh at 64^3) against the oracle's OpenMP CPU generator at 64^3,
    headless rendering of the 1M scene at 1920 x 1080, and one state snapshot (bin + JSON)."""
    import tempfile

    import vkfluidsim_gb300 as vfs
    from vkfluidsim_gb300 import workloads as W

    out = {}
    probe = W.build_model(W.dam_break(dims=(4, 4, 4), map_res=0))
    probe.set_stream(stream.cuda_stream)

    def gpu_ms(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        probe.synchronize()
        return 1e3 * (time.perf_counter() - t0)

    h = float(probe.get_parameters()[0].smooth_radius)
    for res in (128, 64):
        obj = vfs.AnalyticObject(vfs.SHAPE_SPHERE, (0.25,), resolution=(res,) * 3)
        out[f"sphere_map_{res}_gpu_ms"] = gpu_ms(lambda: probe.add_analytic_object(obj))
    # A 320-triangle icosphere (radius 0.25).
    g = (1 + 5 ** 0.5) / 2
    v = [(-1, g, 0), (1, g, 0), (-1, -g, 0), (1, -g, 0), (0, -1, g), (0, 1, g), (0, -1, -g),
         (0, 1, -g), (g, 0, -1), (g, 0, 1), (-g, 0, -1), (-g, 0, 1)]
    v = [np.array(q, np.float64) / np.linalg.norm(q) for q in v]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
         (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(2):
        mid, nf = {}, []
        for a, b, c in f:
            ks = []
            for x, y in ((a, b), (b, c), (c, a)):
                k = (min(x, y), max(x, y))
                if k not in mid:
                    q = v[x] + v[y]
                    v.append(q / np.linalg.norm(q))
                    mid[k] = len(v) - 1
                ks.append(mid[k])
            nf += [(a, ks[0], ks[2]), (b, ks[1], ks[0]), (c, ks[2], ks[1]), tuple(ks)]
        f = nf
    mesh = vfs.MeshObject(vertices=np.array(v) * 0.25, triangles=np.array(f), resolution=(64,) * 3)
    out["mesh_map_64_gpu_ms"] = gpu_ms(lambda: probe.add_mesh_object(mesh))
    out["mesh_triangles"] = len(f)
    if rank == 0 and not args.no_cpu:
        from oracle import binding as ob

        t0 = time.perf_counter()
        ob.volume_map(0, (0.25,), h, (64, 64, 64), np.float32(8 * h))
        out["sphere_map_64_cpu_oracle_ms"] = 1e3 * (time.perf_counter() - t0)
        out["cpu_threads"] = ob.get_threads()
    del probe
    eye, center = (1.0, -1.6, 1.2), (1.0, 0.5, 0.25)
    mv, pj = vfs.look_at(eye, center), vfs.perspective(0.8, 1920 / 1080, 0.05, 20.0)
    model.render_particles(mv, pj, 1920, 1080, quad_side=0.01)  # warm-up
    t0 = time.perf_counter()
    model.render_particles(mv, pj, 1920, 1080, quad_side=0.01)
    out["render_1920x1080_ms"] = 1e3 * (time.perf_counter() - t0)
    # The density field of the scene on 256 x 128 x 128 nodes over its 2 x 1 x 1 m box and its
    # raymarch (raymarch.slang, 0.01 m steps) at 1920 x 1080, both into device buffers.
    import ctypes as C

    from vkfluidsim_gb300._abi import check

    lo, hi = np.zeros(3, np.float32), np.array([2.0, 1.0, 1.0], np.float32)
    res = np.array([256, 128, 128], np.int32)
    grid = torch.empty((128, 128, 256), dtype=torch.float32, device="cuda")
    img = torch.zeros((1080, 1920, 4), dtype=torch.float32, device="cuda")
    tp = lambda t_: C.cast(C.c_void_p(t_.data_ptr()), C.POINTER(C.c_float))  # noqa: E731
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    ip = res.ctypes.data_as(C.POINTER(C.c_int32))
    lib = model._lib
    for k in range(2):  # the first call warms up
        t0 = time.perf_counter()
        check(lib.vfs_model_density_grid(model._h, fp(lo), fp(hi), ip, tp(grid)))
        out["density_grid_256x128x128_ms"] = 1e3 * (time.perf_counter() - t0)
    grid /= 1000.0
    torch.cuda.synchronize()
    center, half = (lo + hi) / 2, (hi - lo) / 2
    for k in range(2):
        t0 = time.perf_counter()
        check(lib.vfs_render_density_raymarch(tp(grid), ip, fp(center), fp(half), fp(mv), fp(pj),
                                              1920, 1080, 0.01, 1000, 5.0, 2.0, tp(img)))
        out["raymarch_1920x1080_ms"] = 1e3 * (time.perf_counter() - t0)
    with tempfile.TemporaryDirectory() as d:
        t0 = time.perf_counter()
        model.export_state(f"{d}/snap")
        out["snapshot_ms"] = 1e3 * (time.perf_counter() - t0)
    out["particles"] = model.n_particles
    return out


def time_full_run(args, stream, torch):
    """The configured obstacle_1m run end to end: 1000 graphed substeps from the initial state,
    timed with CUDA events around the whole run (no L2 flush: one continuous simulation). The
    configured run does not stay physical (the column starts below rest density, free-falls and
    is blown apart by the impact near substep 250, in the CPU oracle as on the GPU), so the peak
    speed is reported beside the time."""
    from vkfluidsim_gb300 import workloads as W

    w = W.obstacle_1m()
    m = W.build_model(w)
    m.set_stream(stream.cuda_stream)
    tuned = m.autotune(repeats=3) if args.autotune else m.get_tune_config()
    m.set_particle_state(w.pos, w.vel)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    marks = {}
    e0.record(stream)
    done = 0
    for chunk in (250, 250, 500):
        m.substeps(chunk)
        done += chunk
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(stream)
        marks[done] = ev
    e1.record(stream)
    torch.cuda.synchronize()
    total = e0.elapsed_time(e1)
    v = np.linalg.norm(m.copy_data_buffers()["velocities"], axis=1)
    seg, prev = {}, e0
    for k, ev in marks.items():
        seg[f"to_{k}"] = prev.elapsed_time(ev) / (250 if k <= 500 else 500)
        prev = ev
    return {"workload": w.name, "particles": w.n, "substeps": done, "ms_total": total,
            "ms_per_substep": total / done, "value": w.n * done / (total * 1e-3),
            "ms_per_substep_by_segment": seg, "final_max_speed_m_s": float(v.max()),
            "skin_builds": m.skin_builds(), "launch_shapes": tuned}


def time_small(args, stream, torch):
    """The 32,768-particle dam break (32^3 lattice at 0.02, h = 0.04, 64^3 box-wall volume map,
    dt = 2e-4): device-timed graphed substeps, and the oracle on one host core for comparison."""
    from vkfluidsim_gb300 import workloads as W

    w = W.dam_break_32k()
    m = W.build_model(w)
    m.set_stream(stream.cuda_stream)
    for _ in range(args.warmup):
        m.substeps(1)
    steps = max(args.steps, 50)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    m.substeps(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    out = {"workload": w.name, "particles": w.n, "steps": steps, "ms_per_step": ms,
           "value": w.n / (ms * 1e-3)}
    del m
    return out


def run_gpu(args):
    import torch

    from vkfluidsim_gb300 import workloads as W

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    w = W.obstacle_1m(seed=1 + rank)
    m = W.build_model(w)
    m.set_stream(stream.cuda_stream)
    n = w.n
    tuned = m.autotune(repeats=3) if args.autotune else m.get_tune_config()
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    # Warm-up (graph capture happens in the first substep).
    for _ in range(args.warmup):
        m.substeps(1)
    barrier()

    # ---- value: device-timed substeps, L2 flushed between steps.
    builds0 = m.skin_builds()  # candidate-list builds so far (read outside the timed region)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        t_wall0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()
            starts[k].record(stream)
            m.substeps(1)
            ends[k].record(stream)
        barrier()
        t_wall = time.perf_counter() - t_wall0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    builds_timed = m.skin_builds() - builds0
    value, total_ms = replica_throughput(n, args.steps, sum(step_ms), world, device="cuda")
    ms_per_step = total_ms / args.steps

    # ---- per-kernel timing (same stream, CUDA events between the passes).
    prof = m.profile_substeps(max(3, min(args.steps, 10)))
    skin_build_ms = None
    if m.skin > 0:
        # set_skin drops every list, so the next substep rebuilds them: the median of three such
        # build substeps' density phases.
        builds = []
        for _ in range(3):
            m.set_skin(m.skin)
            builds.append(m.profile_substeps(1)["density"])
        skin_build_ms = float(statistics.median(builds))
    digits, items, passes = m.get_sort_config()
    kernel_phases = {k: v for k, v in prof.items() if k in B_PHASE}
    dom = max(kernel_phases, key=kernel_phases.get)
    hbm, peak_kind = peaks()
    achieved = B_PHASE[dom] * n / (kernel_phases[dom] * 1e-3) / 1e9
    traffic = None
    inst_pp = {}
    tfile = ROOT / "profiles" / "ncu_traffic.json"
    if tfile.exists():
        t = json.loads(tfile.read_text())
        per = t.get("bytes_per_particle", {}).get(dom)
        if per is not None:
            traffic = per * n
        inst_pp = t.get("warp_instructions_per_particle", {})

    # ---- e2e through the C ABI with pinned host buffers.
    s0 = m.copy_data_buffers()
    hp = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    hv = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    hd = torch.empty((n,), dtype=torch.float32, pin_memory=True)
    hp.numpy()[:] = s0["positions"]
    hv.numpy()[:] = s0["velocities"]
    lib = m._lib
    import ctypes as C

    fp = lambda t_: C.cast(C.c_void_p(t_.data_ptr()), C.POINTER(C.c_float))  # noqa: E731
    from vkfluidsim_gb300._abi import check

    # Each step: the state uploaded from the pinned buffers, one substep, positions, velocities
    # and densities read back into them, one wait (vfs_model_step_host: the upload kernel reads
    # the buffers before the substep's passes run; the density and force passes write the
    # outputs). The call's pointer arguments are made once, as a frame loop would.
    args_e2e = (m._h, fp(hp), fp(hv), 1, fp(hp), fp(hv), fp(hd))

    def e2e_step():
        check(lib.vfs_model_step_host(*args_e2e))

    for _ in range(max(3, args.warmup)):  # the same untimed warm-up as the device-timed leg
        e2e_step()
    e2e_builds0 = m.skin_builds()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    barrier()
    e2e_value, _ = replica_throughput(n, args.steps, 1e3 * (time.perf_counter() - t0), world,
                                      device="cuda")
    e2e = {"value": e2e_value, "unit": UNIT,
           "h2d_bytes_per_step": 24 * n, "d2h_bytes_per_step": 28 * n,
           "skin_builds": m.skin_builds() - e2e_builds0}

    batched = None
    if args.batch_scenes > 0:
        batched = time_batched(args, stream, torch)
    adjoint = time_adjoint(args, stream, torch) if args.adjoint else None
    stress = time_stress(args, stream, torch) if args.stress else None
    next_rows = time_next_rows(args, stream, torch, m, rank) if args.next_rows else None

    small = time_small(args, stream, torch) if args.small else None
    full_run = time_full_run(args, stream, torch) if args.full_run else None

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import binding as ob

        all_threads = ob.get_threads()
        cpu = time_cpu(w, m, budget_s=args.cpu_budget)
        one = time_cpu(w, m, budget_s=max(2.0, args.cpu_budget / 3), max_steps=3, threads=1)
        cpu["single_core"] = {k: one[k] for k in ("value", "cores", "sample")}
        if small:
            s1 = time_cpu(W.dam_break_32k(), None, budget_s=max(2.0, args.cpu_budget / 3), threads=1)
            small["cpu_single_core"] = {k: s1[k] for k in ("value", "cores", "sample")}
        ob.set_threads(all_threads)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded jittered lattice (no dataset exists for this path)",
            "config": workload_config(w.name, n, w.sim.smooth_radius, w.sph.fixed_dt,
                                      "sphere r=0.2, 128^3 volume map"),
            "impl_config": {"sort": {"digit_bits": digits, "tile_items": items, "passes": passes},
                            "launch_shapes": tuned, "autotuned": bool(args.autotune),
                            "cuda_graph": True, "parallelism": f"replicas x{world}"},
            "e2e": e2e,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm,
                         "unit": "GB/s", "frac": achieved / hbm, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": B_PHASE[dom] * n, "traffic": traffic,
                         # the DRAM bytes the pass really moves per launch (one ncu capture)
                         # over its live event time: what the memory system sustains for it
                         "traffic_gbs": traffic / (kernel_phases[dom] * 1e-3) / 1e9 if traffic else None,
                         "traffic_frac": traffic / (kernel_phases[dom] * 1e-3) / 1e9 / hbm if traffic else None},
            "issue_roofline": issue_roofline(inst_pp, kernel_phases, n, local, clk.summary()),
            "step_roofline": {"bytes_per_particle_step": B_STEP,
                              "achieved_gbs": B_STEP * n / (ms_per_step * 1e-3) / 1e9,
                              "frac": B_STEP * n / (ms_per_step * 1e-3) / 1e9 / hbm},
            "phase_ms": prof,
            # the key pass's two kernels (flags, compaction; the 1M scene is below the 4M
            # particles where a tile scan joins them), `passes` onesweep passes, merge,
            # cells+reorder, density (with skin lists:
            # the list pass, the one-warp-per-particle walk of the queued particles and the
            # per-thread walk, which returns at once unless the scene is stale), force.
            "gpu_launches": (6 + passes + (2 if m.skin > 0 else 0)) * args.steps,
            "skin": {"fraction": m.skin, "builds_in_timed_region": builds_timed,
                     "build_substep_density_ms": skin_build_ms},
            "clocks": clk.summary(),
            "wall_s_timed_region": t_wall,
        }
        if batched:
            line["batched"] = batched
        if adjoint:
            line["fwd_adjoint"] = adjoint
        if stress:
            line["stress"] = stress
        if next_rows:
            line["next_rows"] = next_rows
        if small:
            line["small"] = small
        if full_run:
            line["full_run"] = full_run
        if cpu:
            line["cpu_baseline"] = cpu
        # The figures the other legs exist for, last on the line (short keys).
        summ = {"plain_ms": ms_per_step, "plain_value": value, "e2e_value": e2e_value,
                "dominant_frac": achieved / hbm, "step_frac": B_STEP * n / (ms_per_step * 1e-3) / 1e9 / hbm,
                "skin_builds_timed": builds_timed}
        if full_run:
            summ["amortised_ms_1000"] = full_run["ms_per_substep"]
            summ["amortised_ms_first_250"] = full_run["ms_per_substep_by_segment"].get("to_250")
            summ["full_run_builds"] = full_run.get("skin_builds")
        if batched:
            summ["batched_value"] = batched["value"]
            summ["batched_ms"] = batched["ms_per_step"]
            summ["batched_loop_ms"] = batched["loop_ms_per_step"]
            summ["batched_speedup"] = batched["speedup_vs_loop"]
        if adjoint:
            summ["fwd_adjoint_cost"] = adjoint["cost_vs_forward"]
            summ["fwd_ms"] = adjoint["forward_ms_per_step"]
        if stress:
            summ["stress_ms"] = stress["ms_per_step"]
        if cpu:
            summ["cpu_value"] = cpu["value"]
        line["summary"] = summ
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def run_profile(args):
    """A short run for profilers (no timing line): `--profile step` runs --steps substeps of
    --workload with one launch per pass (no CUDA graph) after one warm-up substep and prints the
    per-pass event times; `--profile adjoint` runs a checkpointed forward + adjoint rollout of the
    65,536-particle dam break over --steps substeps."""
    from vkfluidsim_gb300 import workloads as W

    if args.profile == "step":
        w = W.WORKLOADS[args.workload]()
        m = W.build_model(w)
        m.use_graph(False)
        m.substeps(1)
        prof = m.profile_substeps(max(1, args.steps - 1))
        m.synchronize()
        print(json.dumps({"workload": w.name, "particles": w.n, "phase_ms": prof,
                          "sort": m.get_sort_config()}))
        return
    import vkfluidsim_gb300 as vfs
    from vkfluidsim_gb300.adjoint import Rollout

    w = W.dam_break_64k()
    w.vel = vfs.generate_fourier_velocity(w.pos, 8, 0.5, 4)
    m = W.build_model(w)
    ro = Rollout(m, args.steps, 25)
    t0 = time.perf_counter()
    ro.forward()
    xf = ro.final_positions_by_id()
    g = ro.backward(2.0 * (xf - w.pos) / xf.size)
    print(json.dumps({"particles": w.n, "steps": args.steps, "seconds": time.perf_counter() - t0,
                      "dnu": g["dnu"], "dk": g["dk"], "dv0_max": float(np.abs(g["dv0"]).max())}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--batch-scenes", type=int, default=256)
    ap.add_argument("--adjoint", type=int, default=1)
    ap.add_argument("--stress", type=int, default=1)
    ap.add_argument("--autotune", type=int, default=1)
    ap.add_argument("--next-rows", type=int, default=1)
    ap.add_argument("--small", type=int, default=1)
    ap.add_argument("--full-run", type=int, default=1)
    ap.add_argument("--profile", choices=["step", "adjoint"], default=None,
                    help="a short untimed run for profilers instead of the benchmark")
    ap.add_argument("--workload", default="obstacle_1m", help="workload of --profile step")
    args = ap.parse_args()
    if args.profile:
        run_profile(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

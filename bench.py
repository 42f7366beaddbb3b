"""Benchmark: forward + adjoint DiffDFSPH steps per second at 1M fluid particles.

Workload (default): the 1,000,000-particle dam break with a dropped sphere
(100 x 100 x 100 lattice, r = 0.005 m, 2.4 x 1.2 x 1.2 m box, dt = 0.5 ms), FP32 fluid
and FP64 rigid arithmetic. One step = one DiffDFSPH time step with the per-sweep pair
Jacobians accumulated and the chain step matrix recorded; the timed region also runs
the reverse (adjoint) sweep over the recorded steps once.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0). Under torchrun (N > 1) every rank runs an independent
replica on its own GPU (no data exchange; "replicas only") and value is the sum.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "fwd+adjoint steps/s at 1M particles; warm-start vs plain solve at 0.01% rho err"
UNIT = "steps/s"

# Algorithmic DRAM bytes per particle of each kernel class (FP32 fields, compulsory
# traffic, neighbour gathers assumed cache-resident): the per-unit figures of the
# measurement model.
ALGO_BYTES = {
    "sort": 92, "lists_density_factor": 32, "density_pass": 32, "velocity_pass": 52,
    "xsph_advect": 40, "integrate": 36, "bf_lists": 16, "pairs": 32, "rigid": 32,
}


# DRAM bytes per particle and launch (dram__bytes_read.sum + dram__bytes_write.sum) from an
# ncu capture of the same passes on the 262,144-particle copy of the dam break (L2 flushed
# by ncu before each launch), scaled by the launch's particle count; a capture of one
# launch of each at 1M particles measured 179 and 183 B per particle.
MEASURED_TRAFFIC = {"density_pass": 178.3, "velocity_pass": 179.5}
# The passes' binding resource as ncu measured it on one launch of each at 1M particles:
# L1 data-pipe wavefronts (l1tex__data_pipe_lsu_wavefronts) as a fraction of their peak.
MEASURED_L1_WAVEFRONT_FRAC = {"density_pass": 0.777, "velocity_pass": 0.696}


def load_sm_max_mhz():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f).get("sm_max_mhz", 2070.0))
    return 2070.0


def load_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """SM clock and clock-event (throttle) reasons sampled during the timed region: NVML
    read through ctypes every 2 ms (a background thread), or nvidia-smi every 200 ms
    where NVML cannot be loaded. Read-only: no clock or setting is changed."""
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None
        self.thread = None
        self.samples = []
        self.max_mhz = None

    def _nvml(self):
        import ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit")
        dev = ctypes.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.gpu), ctypes.byref(dev)) != 0:
            raise RuntimeError("nvml handle")
        reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
        mx = ctypes.c_uint()
        if lib.nvmlDeviceGetMaxClockInfo(dev, ctypes.c_int(1), ctypes.byref(mx)) == 0:
            self.max_mhz = float(mx.value)
        return lib, dev, reasons_fn

    def start(self):
        import threading
        try:
            import ctypes
            lib, dev, reasons_fn = self._nvml()
            self.stop_flag = threading.Event()

            def run():
                clk, rs = ctypes.c_uint(), ctypes.c_ulonglong()
                while not self.stop_flag.is_set():
                    if lib.nvmlDeviceGetClockInfo(dev, ctypes.c_int(1), ctypes.byref(clk)) == 0 and \
                            reasons_fn(dev, ctypes.byref(rs)) == 0:
                        self.samples.append((float(clk.value), int(rs.value)))
                    time.sleep(0.002)
            self.thread = threading.Thread(target=run, daemon=True)
            self.thread.start()
            return
        except Exception:
            self.thread = None
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.thread is not None:
            self.stop_flag.set()
            self.thread.join(timeout=2)
            if self.samples:
                reasons = set()
                for _, r in self.samples:
                    for bit, nm in self.REASONS.items():
                        if r & bit:
                            reasons.add(nm)
                out = {"sm_mhz": statistics.median(c for c, _ in self.samples), "sm_max_mhz": self.max_mhz,
                       "reasons": sorted(reasons), "samples": len(self.samples), "source": "nvml, 2 ms"}
            return out
        if self.proc is None:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    smax.append(float(p[2]))
                except ValueError:
                    continue
                for nm, val in zip(names, p[5:9]):
                    if val.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                   "samples": len(sm), "source": "nvidia-smi, 200 ms"}
        return out


def make_scene(args, enable_gradient=1, seed=0):
    from difffr_gb300 import scene as scn
    if args.config == 1:
        sc = scn.dam_break_sphere(seed=seed, enable_gradient=enable_gradient)
    elif args.config == 5:
        sc = scn.dam_break_sphere(n=(64, 64, 64), seed=seed, enable_gradient=enable_gradient)
    elif args.config == 0:
        sc = scn.config0(seed=seed, enable_gradient=enable_gradient)  # FP64 fluid, as configured
    elif args.config == 2:
        sc = scn.pool_ellipsoid(seed=seed, enable_gradient=enable_gradient)
    else:
        sc = scn.billiards_on_water(seed=seed, enable_gradient=enable_gradient)
    return sc


def scene_dtype(sc):
    """The arithmetic type of the fluid path ("f64" for an FP64 scene; the bodies are FP64 always)."""
    from difffr_gb300 import _abi
    return "f64" if sc.params.fluid_precision == _abi.DFSPH_FP64 else "f32"


def oracle_mode(sc):
    """The oracle build matching the scene's split: FP64 throughout, or FP32 fluid / FP64 rigid."""
    import oracle
    return oracle.MODE_F64 if scene_dtype(sc) == "f64" else oracle.MODE_MIXED


def split_name(sc):
    return "FP64 fluid / FP64 rigid" if scene_dtype(sc) == "f64" else "FP32 fluid / FP64 rigid"


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def config_dict(args, sc):
    """The workload description both arms print (same keys, same values)."""
    # the neighbour passes' working set: the particle records and the int32 neighbour lists
    # (about 35 entries per particle), against the 129 MB L2
    wide = 2 if scene_dtype(sc) == "f64" else 1
    ws_mb = sc.n_fluid * (32 * wide + 16 * wide + 35 * 4) / 1e6
    l2 = ("inputs larger than L2" if ws_mb > 129.0 else
          f"working set about {ws_mb:.0f} MB, inside the 129 MB L2 (not flushed between steps)")
    phase = " (collapse phase)" if args.config == 1 else ""
    return {"workload": args.config_name, "n_fluid": sc.n_fluid, "n_boundary": sc.n_boundary,
            "dt": sc.params.time_step, "gradient_mode": "incomplete",
            "window": f"steps {args.start_step + args.warmup}-{args.start_step + args.warmup + args.steps - 1} "
                      f"of the trajectory{phase}, after {args.warmup} warm-up steps from step "
                      f"{args.start_step}",
            "l2": l2, "parallelism": f"replicas{args.gpus}" if args.gpus > 1 else "single GPU"}


def oracle_steps(o, steps):
    """Times `steps` oracle steps; returns (steps/s, seconds, pressure sweeps per step)."""
    t0 = time.perf_counter()
    st = o.step(steps)
    dt = time.perf_counter() - t0
    return steps / dt, dt, st["total_pressure_iterations"] / steps


def cpu_baseline(args, sim, steps, threads):
    """The CPU oracle (C++/OpenMP restatement of the reference step) on this host's cores,
    continuing from the GPU context's current state (fluid fields, warm-start stiffness,
    bodies, time), so that it times the same phase of the trajectory."""
    import oracle
    oracle.build()
    sc = make_scene(args, enable_gradient=1)
    o = oracle.Oracle(sc, mode=oracle_mode(sc), threads=threads)
    o.load_state(sim)
    o.step(1)
    return oracle_steps(o, steps)


def run_reference(args):
    """The reference arm: the oracle port on all host cores, run from step 0 through the same
    pre-roll as the GPU arm (untimed), then `warmup` untimed and `steps` timed steps."""
    world, rank, local, pg = dist_setup()
    if rank != 0:
        return 0
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    sc = make_scene(args, enable_gradient=1)
    o = oracle.Oracle(sc, mode=oracle_mode(sc), threads=threads)
    if args.start_step > 0:
        o.step(args.start_step)
    o.step(args.warmup)
    steps = args.steps
    val, dt, ip = oracle_steps(o, steps)
    sample = (f"{steps} timed steps (steps {args.start_step + args.warmup}-{args.start_step + args.warmup + steps - 1}, "
              f"{ip:.2f} pressure sweeps per step) of the full {args.config_name} workload after an untimed "
              f"pre-roll from step 0; oracle port, {split_name(sc)}, gradient on, {threads} OpenMP threads "
              f"on {cpu_model()}")
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * dt / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": scene_dtype(sc), "data": "synthetic (seeded lattice + sampled boundaries)",
        "config": config_dict(args, sc),
        "pressure_iterations_per_step": ip,
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                         "cpu_model": cpu_model()},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def nvtx(name=None):
    """Pushes (name given) or pops an NVTX range; a profiler's launch list can then select the
    timed window (``ncu --nvtx --nvtx-include "timed_window/"``). Does nothing without NVTX."""
    try:
        import torch
        if name is None:
            torch.cuda.nvtx.range_pop()
        else:
            torch.cuda.nvtx.range_push(name)
    except Exception:
        pass


def timed_fwd_adjoint(sim, steps, dL):
    """K forward steps with the pair Jacobians recorded, then the reverse sweep once; CUDA
    events on the context's stream. Returns (ms, step stats)."""
    sim.synchronize()
    sim.record_event(0)
    st = sim.step(steps)
    sim.backward(dL)
    sim.record_event(1)
    return sim.event_elapsed_ms(0, 1), st


def run_ours(args):
    world, rank, local, pg = dist_setup()
    import numpy as np
    from difffr_gb300 import _abi
    from difffr_gb300.sim import DiffDFSPH

    lib = _abi.load_library()
    _abi.check(lib, lib.dfsph_set_device(local))
    peak, peak_kind = load_peaks()
    sc = make_scene(args, enable_gradient=1, seed=rank)
    sim = DiffDFSPH(sc)
    nb = sim.n_bodies
    dL = np.zeros((nb, 13))
    dL[:, 0:3] = 1.0

    # ---- early phase (steps W..W+K-1 from rest: both solves at their minimum sweep counts)
    for _ in range(args.warmup):
        sim.step(1)
    sim.reset_gradient()
    early_ms, early_st = timed_fwd_adjoint(sim, args.steps, dL)
    early_ms = allmax(pg, early_ms)

    # ---- untimed pre-roll to the start of the headline window, kept as a device checkpoint
    t_now, sc_now = sim.time()
    if args.start_step > sc_now:
        sim.step(args.start_step - sc_now)
    slot = sim.checkpoint_save()

    # ---- headline: forward + adjoint over the window (collapse phase)
    for _ in range(args.warmup):
        sim.step(1)
    slot_w = sim.checkpoint_save()  # the window's first state, for the end-to-end leg
    sim.reset_gradient()
    barrier(pg)
    clocks = ClockSampler(local)
    clocks.start()
    l0 = sim.launch_count()
    sim.synchronize()
    barrier(pg)
    nvtx("timed_window")
    ms, st = timed_fwd_adjoint(sim, args.steps, dL)
    nvtx()
    launches = sim.launch_count() - l0
    clk = clocks.stop()
    ms_max = allmax(pg, ms)
    value = world * args.steps / (ms_max / 1000.0)
    iters_p = st["total_pressure_iterations"] / args.steps
    iters_v = st["total_divergence_iterations"] / args.steps

    # ---- per-kernel device times over the next K steps of the same phase (profiling on)
    sim.profile_enable(True)
    sim.step(args.steps)
    prof = sim.profile()
    sim.profile_enable(False)
    from difffr_gb300._abi import KERNEL_CLASSES
    dom = max(KERNEL_CLASSES, key=lambda k: prof[k]["ms"])
    d = prof[dom]
    avg_launch_s = d["ms"] / max(d["launches"], 1) / 1000.0
    units_per_launch = d["units"] / max(d["launches"], 1)
    # FP64 fluid fields are twice the bytes; the measured traffic is of the FP32 passes
    wide = 2 if scene_dtype(sc) == "f64" else 1
    algo_bytes = wide * ALGO_BYTES.get(dom, 32) * units_per_launch
    achieved = algo_bytes / avg_launch_s / 1e9
    traffic = MEASURED_TRAFFIC[dom] * units_per_launch if dom in MEASURED_TRAFFIC and wide == 1 else None
    # the L1 side of the same kernel: each neighbour visit gathers one 32-byte record (the
    # density and XSPH passes; 16 bytes in the velocity pass) and reads a 4-byte list entry
    from difffr_gb300 import _abi as abi_mod
    nbar = sim.neighbor_total(abi_mod.NB_FLUID_FLUID) / max(sim.n_fluid, 1)
    rec = {"density_pass": 32, "xsph_advect": 32, "velocity_pass": 16}.get(dom)
    rec = rec * wide if rec is not None else None
    l1 = None
    if rec is not None:
        import torch
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        l1_peak = 128.0 * sms * load_sm_max_mhz() * 1e6 / 1e9  # GB/s: 128 B per clock per SM
        l1_achieved = nbar * (rec + 4) * units_per_launch / avg_launch_s / 1e9
        l1 = {"fluid_neighbours_per_particle": nbar, "bytes_per_particle": nbar * (rec + 4),
              "achieved": l1_achieved, "peak": l1_peak, "unit": "GB/s", "frac": l1_achieved / l1_peak,
              "peak_basis": "128 B per clock per SM at the maximum SM clock",
              # the used record bytes fill fewer wavefronts than a scattered gather costs
              "ncu_wavefront_frac": MEASURED_L1_WAVEFRONT_FRAC.get(dom) if wide == 1 else None}

    # ---- forward-only steps/s over the same window (no pair Jacobians, no tape)
    sim.checkpoint_restore(slot)
    sim.set_gradient_enabled(False)
    for _ in range(args.warmup):
        sim.step(1)
    sim.synchronize()
    sim.record_event(0)
    sim.step(args.steps)
    sim.record_event(1)
    fwd_ms = sim.event_elapsed_ms(0, 1)
    sim.set_gradient_enabled(True)

    # ---- end to end through the public API with host buffers: one optimisation-loop
    # trajectory over the headline's window. The fluid state comes from the device
    # checkpoint of the window's first state (the trajectory's saved starting state, as the
    # reference's scripts load theirs), the bodies' states are uploaded from host memory,
    # K single-step calls each followed by a read-back of every body's state, then the
    # adjoint with its host input and output.
    n = sim.n_fluid
    sim.checkpoint_restore(slot_w)
    host_bodies = [sim.rigid_state(b) for b in range(nb)]
    sim.synchronize()
    t0 = time.perf_counter()
    sim.checkpoint_restore(slot_w)
    sim.reset_gradient()
    for b in range(nb):
        sim.set_rigid_state(b, *host_bodies[b])
    for _ in range(args.steps):
        sim.step(1)
        for b in range(nb):
            sim.rigid_state(b)
    sim.backward(dL)
    sim.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_s = allmax(pg, e2e_s)
    body_state_bytes = 1656  # one device BodyState record per body per transfer
    h2d = (nb * body_state_bytes + nb * 13 * 8) / args.steps     # the bodies' states, adjoint input
    d2h = nb * body_state_bytes + (nb * 6 * 8) / args.steps       # per-step read-back, gradient
    e2e_value = world * args.steps / e2e_s

    # ---- the CPU oracle over the same window, from the same device state
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sim.checkpoint_restore(slot_w)
        threads = os.cpu_count() or 1
        cpu_steps = args.cpu_steps
        cval, cdt, cip = cpu_baseline(args, sim, cpu_steps, threads)
        t_start, sc_start = sim.time()
        cpu = {"value": cval, "unit": UNIT, "cores": threads, "kind": "port", "cpu_model": cpu_model(),
               "sample": f"{cpu_steps} steps (after 1 warm-up step) from the GPU context's state at step "
                         f"{sc_start} of the full {args.config_name} workload ({cip:.2f} pressure sweeps per "
                         f"step), oracle port with {split_name(sc)}, gradient on, {threads} OpenMP threads"}
    sim.checkpoint_free(slot)
    sim.checkpoint_free(slot_w)

    # ---- the whole trajectory of the configuration (steps 0..T-1 in one call, gradient
    # recorded, then the adjoint), the average over all its phases
    traj = None
    if rank == 0 and args.config == 1 and args.trajectory_steps > 0:
        sim.reset()
        sim.reset_gradient()
        sim.synchronize()
        sim.record_event(0)
        st_t = sim.step(args.trajectory_steps)
        sim.backward(dL)
        sim.record_event(1)
        t_ms = sim.event_elapsed_ms(0, 1)
        traj = {"steps": args.trajectory_steps, "value": args.trajectory_steps / (t_ms / 1000.0), "unit": UNIT,
                "ms_per_step": t_ms / args.trajectory_steps,
                "pressure_iterations_per_step": st_t["total_pressure_iterations"] / args.trajectory_steps,
                "divergence_iterations_per_step": st_t["total_divergence_iterations"] / args.trajectory_steps,
                "window": f"steps 0-{args.trajectory_steps - 1} from rest, forward with gradient recording, then the adjoint"}

    # ---- learned warm start vs the reference warm start (collapse phase of a held-out seed)
    ws = None
    if rank == 0 and args.config == 1 and args.ws_steps > 0:
        sim.close()
        sim = None
        ws = warm_start_ab(args)

    # ---- the rigid contact solver and the gradient manager at the same size
    contact = None
    if rank == 0 and args.config == 1 and args.contact_steps > 0:
        if sim is not None:
            sim.close()
            sim = None
        contact = contact_leg(args)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": scene_dtype(sc),
            "data": "synthetic (seeded lattice + sampled boundaries)",
            "config": config_dict(args, sc),
            "fwd_only_steps_per_s": world * args.steps / (fwd_ms / 1000.0),
            "pressure_iterations_per_step": iters_p, "divergence_iterations_per_step": iters_v,
            "early_phase": {"value": world * args.steps / (early_ms / 1000.0), "unit": UNIT,
                            "ms_per_step": early_ms / args.steps,
                            "window": f"steps {args.warmup}-{args.warmup + args.steps - 1} from rest",
                            "pressure_iterations_per_step": early_st["total_pressure_iterations"] / args.steps,
                            "divergence_iterations_per_step": early_st["total_divergence_iterations"] / args.steps},
            "gpu_launches": launches,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "algo_bytes_per_particle": wide * ALGO_BYTES.get(dom, 32),
                         "avg_launch_us": avg_launch_s * 1e6},
            "l1_gather": l1,
            "kernel_ms_per_step": {k: v["ms"] / args.steps for k, v in prof.items()},
            "clocks": clk,
            "cpu_baseline": cpu,
            "trajectory": traj,
            "warm_start": ws,
            "contact": contact,
        }
        print(json.dumps(line), flush=True)
    if sim is not None:
        sim.close()
    return 0


def roofline_of(sim, prof, peak, peak_kind):
    """The dominant kernel class's achieved algorithmic bandwidth against the measured peak."""
    from difffr_gb300._abi import KERNEL_CLASSES
    dom = max(KERNEL_CLASSES, key=lambda k: prof[k]["ms"])
    d = prof[dom]
    avg_launch_s = d["ms"] / max(d["launches"], 1) / 1000.0
    units = d["units"] / max(d["launches"], 1)
    achieved = ALGO_BYTES.get(dom, 32) * units / avg_launch_s / 1e9
    traffic = MEASURED_TRAFFIC[dom] * units if dom in MEASURED_TRAFFIC else None
    return {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "peak_kind": peak_kind, "algo_bytes_per_particle": ALGO_BYTES.get(dom, 32),
            "avg_launch_us": avg_launch_s * 1e6}


def run_basin(args):
    """The full pipeline at 4M particles (200 x 100 x 200 lattice at r = 0.0025 m in a
    1.2 x 0.8 x 1.2 m box, two R 0.03 m spheres colliding on the water, a static box): the
    learned warm start is trained on the scene's own plain-solver samples (steps 40-59 of
    seed 0), then K forward + adjoint steps with it (the leg's value: the gradient with
    respect to the 12 initial velocities), K forward-only steps with it, and K forward +
    adjoint steps with the reference warm start, all after W warm-up steps, CUDA events on
    the context's stream; the dominant kernel's roofline from a profiled repeat."""
    import numpy as np
    from difffr_gb300 import _abi
    from difffr_gb300 import scene as scn
    from difffr_gb300.sim import DiffDFSPH
    from difffr_gb300.warmstart import WarmStartModel, collect_samples, train
    lib = _abi.load_library()
    _abi.check(lib, lib.dfsph_set_device(0))
    peak, peak_kind = load_peaks()
    t0 = time.perf_counter()
    sc0 = scn.billiards_on_water(seed=0, enable_gradient=0)
    sim = DiffDFSPH(sc0)
    sim.step(40)
    x, y = collect_samples(sim, 20)
    sim.close()
    model = WarmStartModel(seed=0)
    losses = train(model, x, y, epochs=2, batch=65536, lr=2e-3, lr_final=1e-4, seed=0)
    training = {"samples": int(x.shape[0]), "epochs": 2, "final_loss": float(losses[-1]) if losses else None,
                "wall_s": time.perf_counter() - t0}
    del x, y

    def leg(model_on, gradient):
        s = DiffDFSPH(scn.billiards_on_water(seed=0, enable_gradient=1 if gradient else 0))
        s.set_warmstart_model(model if model_on else None)
        nb = s.n_bodies
        dL = np.zeros((nb, 13))
        dL[:, 0:3] = 1.0
        for _ in range(args.warmup):
            s.step(1)
        s.reset_gradient()
        s.synchronize()
        s.record_event(0)
        st = s.step(args.steps)
        if gradient:
            g = s.backward(dL)
        s.record_event(1)
        ms = s.event_elapsed_ms(0, 1)
        out = {"steps_per_s": args.steps / (ms / 1000.0), "ms_per_step": ms / args.steps,
               "pressure_iterations_per_step": st["total_pressure_iterations"] / args.steps}
        if gradient:
            out["gradient_finite"] = bool(np.all(np.isfinite(g)))
            s.profile_enable(True)
            s.step(args.steps)
            prof = s.profile()
            s.profile_enable(False)
            out["roofline"] = roofline_of(s, prof, peak, peak_kind)
            out["kernel_ms_per_step"] = {k: v["ms"] / args.steps for k, v in prof.items()}
        s.set_warmstart_model(None)
        s.close()
        return out

    clocks = ClockSampler(0)
    clocks.start()
    learned = leg(True, True)
    clk = clocks.stop()
    fwd = leg(True, False)
    plain = leg(False, True)
    model.close()
    line = {
        "metric": METRIC, "value": learned["steps_per_s"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": learned["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded lattice + sampled boundaries)",
        "config": {"workload": args.config_name, "n_fluid": sc0.n_fluid, "n_boundary": sc0.n_boundary,
                   "dt": sc0.params.time_step, "gradient": "12 initial velocity variables (2 spheres x (v, omega))",
                   "warm_start": "learned, trained on this scene's steps 40-59 (seed 0)",
                   "l2": "inputs larger than L2", "parallelism": "single GPU"},
        "pressure_iterations_per_step": learned["pressure_iterations_per_step"],
        "gradient_finite": learned["gradient_finite"],
        "fwd_only_steps_per_s": fwd["steps_per_s"],
        "plain_warm_start": {"fwd_adjoint_steps_per_s": plain["steps_per_s"],
                             "pressure_iterations_per_step": plain["pressure_iterations_per_step"]},
        "roofline": learned["roofline"], "kernel_ms_per_step": learned["kernel_ms_per_step"],
        "warm_start_training": training, "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    return 0


def contact_leg(args):
    """Forward + adjoint steps/s of the 1M dam break with two spheres in contact (the rigid
    contact solver and the gradient manager on), and the rigid-stream time that includes the
    contact samples, the sequential impulses and the manager's chain."""
    import numpy as np
    from difffr_gb300 import scene as scn
    from difffr_gb300.sim import DiffDFSPH
    sc = scn.dam_break_two_spheres()
    s = DiffDFSPH(sc)
    for _ in range(max(args.warmup, 3)):
        s.step(1)
    s.profile_enable(True)
    k = args.contact_steps
    s.record_event(0)
    s.step(k)
    s.record_event(1)
    ms = s.event_elapsed_ms(0, 1)
    prof = s.profile()
    nc, na = s.contact_count()
    g = s.manager_grad(2, 1)
    s.close()
    return {"workload": f"{sc.name} (two R 0.05 spheres 0.01 m apart, 0.5 m/s towards each other)",
            "value": k / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms / k,
            # wall time of the rigid stream's kernels, most of it overlapping the fluid stream
            "rigid_stream_busy_ms_per_step": prof["rigid"]["ms"] / k,
            "contact_samples_last_step": nc, "force_samples_last_step": na,
            "cross_gradient_finite": bool(np.all(np.isfinite(g))), "steps": k}


def warm_start_ab(args):
    """Pressure solve from the reference warm start vs from the learned one, both to the
    0.01 % density tolerance, on seed 1 from the state after `ws_start` plain steps (the
    collapse phase, where the solve needs more than its minimum sweeps). The model is the
    committed one trained on seed 0 (difffr_gb300/train_warmstart.py), or trained here."""
    from difffr_gb300 import train_warmstart as tw
    from difffr_gb300.warmstart import WarmStartModel
    t0 = time.perf_counter()
    if os.path.exists(tw.DEFAULT_MODEL) and not args.train_warm_start:
        model = WarmStartModel(seed=0)
        model.load(tw.DEFAULT_MODEL)
        source = "committed weights " + os.path.basename(tw.DEFAULT_MODEL)
    else:
        model, info = tw.train_model(start=args.ws_start)
        source = f"trained here on seed 0 ({info['samples']} samples, {info['train_s']:.2f} s)"
    r = tw.evaluate(model, 1, args.ws_start, args.ws_steps)
    model.close()
    r.update({"workload": f"dam_break_sphere_1M seed 1, steps {args.ws_start}-{args.ws_start + args.ws_steps - 1}",
              "model": source, "tolerance": "0.01 % average density error (both runs)",
              "wall_s": time.perf_counter() - t0})
    return r


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--cpu-steps", type=int, default=10)
    # the headline window: from step 400 of the dam break the pressure solve needs 7-12 sweeps
    # per step (2 before step 275); the early phase is reported beside it
    ap.add_argument("--start-step", type=int, default=400)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ws-start", type=int, default=300)
    ap.add_argument("--ws-steps", type=int, default=200)
    ap.add_argument("--train-warm-start", action="store_true")
    ap.add_argument("--contact-steps", type=int, default=20)
    ap.add_argument("--trajectory-steps", type=int, default=500)
    args = ap.parse_args()
    args.config_name = {0: "tank_sphere_8k (20^3 lattice, r 0.025, FP64)",
                        1: "dam_break_sphere_1M (100^3 lattice, r 0.005, 2.4x1.2x1.2 box, R 0.05 sphere)",
                        2: "pool_ellipsoid_250k (125x16x125, r 0.004)",
                        4: "billiards_on_water_4M (200x100x200, r 0.0025, 2 spheres)",
                        5: "dam_break_sphere_262k (64^3 lattice, r 0.005; reduced copy for profiling)"}[args.config]
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.config == 4:
        return run_basin(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

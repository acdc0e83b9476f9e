"""Throughput of the GB300 force engine on its headline workload.

Workload (one step = one production MD step of nve_md.c:359-418): the 3-site
water recipe scaled to 32,000 molecules (96,000 sites, L = 98.65 A, density
0.1 sites/A^3), SPME 96^3 order 4, kappa 0.32, rc 10 A with the LJ switched
from 8 A, Verlet list 12 A rebuilt every 10 steps, NVE velocity Verlet with
dt = 0.5 fs, mixed precision (FP32 pair/PME math, 64-bit fixed-point force
sums, FP64 integration).  Synthetic seeded input (no dataset is involved).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  ``value`` is atom-steps/s with all state resident on
the GPU (steps timed with CUDA events on the engine's stream); ``e2e`` is the
same metric through the C ABI with host buffers: every step uploads the
state integrate_vverlet reads (atom, atnopbc, vv, ff from pinned host
arrays) and reads back what it writes (those, uu and the energies),
in one fe_integrate_vverlet_host call per step, then kinet, as the
reference's host loop (nve_md.c) calls them.
Under torchrun each rank runs its own replica (the single-box path does not
shard: replicas only) and the slowest rank's time is used.
``--impl reference`` times the reference's CPU implementation of the path
(the pinned CPU restatement, built with the reference makefile's flags) on a
bounded sample of the same workload, on rank 0 only: W + K real MD steps of
the CPU path (at most 5 + 40), each step timed as it runs.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_MOL = 32000
SEED = 2025
R_SWITCH = 8.0  # LJ switched from 8 A to rc = 10 A in every leg
METRIC = "atom-steps/s"
PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}
PROFILE = os.path.join(ROOT, "profiles", "k_mx_pair_water96k.md")
WORKLOAD = ("water 3-site, 96,000 sites (32,000 molecules), L=98.65 A, SPME 96^3 order 4, "
            "kappa 0.32, rc 10 A, LJ switch 8-10 A (CHARMM), list 12 A every 10 steps, "
            "NVE velocity Verlet dt 0.5 fs")
CONFIG = {"workload": WORKLOAD, "cache": "inputs larger than L2 (pair list > 129 MB per step)"}
EN_TERMS = ("bond", "bend", "nbond", "nbonds", "coulomb", "rewald", "rewalds", "kewald",
            "sewald", "iewald", "tewald")


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return PEAKS_FALLBACK, "fallback"


def profile_traffic():
    """dram read+write bytes per launch of the pair kernel from the committed
    ncu summary (None if absent)."""
    if not os.path.exists(PROFILE):
        return None
    with open(PROFILE) as f:
        for line in f:
            m = re.match(r"\s*traffic_bytes_per_launch:\s*([0-9.eE+]+)", line)
            if m:
                return float(m.group(1))
    return None


class NvmlSampler:
    """SM clock and clock-event reasons read through NVML (libnvidia-ml, read
    only) every millisecond from a thread, so that timed regions shorter than
    nvidia-smi's sampling period still get samples."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, device: int):
        import ctypes as C
        import threading
        self.C = C
        self.samples = []
        self.stop_ev = threading.Event()
        self.thread = None
        self.ok = False
        try:
            lib = C.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return
            h = C.c_void_p()
            if lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(device), C.byref(h)) != 0:
                return
            self.lib, self.h = lib, h
            mx = C.c_uint()
            self.max_mhz = (float(mx.value) if lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx)) == 0
                            else None)
            self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
            self.ok = True
        except (OSError, AttributeError):
            self.ok = False

    def _run(self):
        C = self.C
        clk = C.c_uint()
        rs = C.c_ulonglong()
        while not self.stop_ev.is_set():
            if self.lib.nvmlDeviceGetClockInfo(self.h, 1, C.byref(clk)) == 0:
                r = rs.value if self.reasons_fn(self.h, C.byref(rs)) == 0 else 0
                self.samples.append((float(clk.value), int(r)))
            time.sleep(0.001)

    def start(self):
        if self.ok:
            import threading
            self.thread = threading.Thread(target=self._run, daemon=True)
            self.thread.start()

    def stop(self):
        if not self.ok or self.thread is None:
            return None
        self.stop_ev.set()
        self.thread.join()
        if not self.samples:
            return None
        reasons = set()
        for _, r in self.samples:
            for bit, nm in self.REASONS.items():
                if r & bit:
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(c for c, _ in self.samples), "sm_max_mhz": self.max_mhz,
                "samples": len(self.samples), "reasons": sorted(reasons), "source": "nvml 1 ms"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return world, rank, local


def allreduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_sample(sysm, nsteps_cap: int = 3):
    """Times the CPU restatement of the path (reference makefile flags) on a
    bounded sample: one O(N^2) list build and a few force+integration steps;
    the per-step cost charges the list build once per nlist_freq steps as the
    workload does."""
    from oracle import oracle as orc
    o = orc.Oracle(sysm, fast=True)
    t0 = time.perf_counter()
    o.nblist(sysm.pos)
    t_list = time.perf_counter() - t0
    ns = nsteps_cap
    t0 = time.perf_counter()
    o.run_md(ns - 1)  # list + forces, then ns-1 steps: ns force evaluations
    t_md = time.perf_counter() - t0
    t_step = (t_md - t_list) / ns
    per_step = t_step + t_list / sysm.nlist_freq
    return {
        "value": sysm.n / per_step, "unit": METRIC, "cores": 1, "kind": "port",
        "sample": (f"{sysm.n} sites: 1 O(N^2) list build ({t_list:.2f} s) + {ns} force/VV "
                   f"evaluations ({t_step:.2f} s each); list charged every {sysm.nlist_freq} "
                   "steps; single thread, reference makefile flags"),
        "seconds": t_list + t_md,
    }


def run_reference(args, world, rank):
    """The CPU path of the reference on the same workload: W warm-up and K
    timed MD steps (list every 10 steps, as the workload) of the CPU
    restatement built with the reference makefile's flags, one thread (the
    reference is single-threaded).  At most 5 + 40 steps are run; the line
    says how many were timed.  The box is placed with numpy only: no
    compiled code of the engine is loaded."""
    if rank != 0:
        return
    from oracle import oracle as orc
    from thecodecombo_7_gb300 import systems
    sysm = systems.water_box(N_MOL, density=0.1, seed=SEED, r_switch=R_SWITCH, helper=False)
    W = min(args.warmup, 5)
    K = min(args.steps, 40)
    o = orc.Oracle(sysm, fast=True)
    md = o.run_md(W + K, timed=True)
    ts = md["tstamp"]
    sec = float(ts[W + K] - ts[W])
    value = sysm.n * K / sec
    sample = (f"{K} timed MD steps after {W} warm-up steps ({sec:.1f} s; list rebuilt "
              f"(O(N^2)) at every 10th step as in the workload), 96,000 sites, single thread, "
              "CPU restatement built with the reference makefile's flags")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC,
        "n_gpus": args.gpus, "steps": K, "warmup": W,
        "ms_per_step": 1000.0 * sec / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(CONFIG, parallelism=f"replicas x{world}"),
        "precision": "fp64 CPU (reference arithmetic)",
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": 1, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    if K != args.steps or W != args.warmup:
        line["steps_requested"] = args.steps
        line["warmup_requested"] = args.warmup
    print(json.dumps(line))


def nve_drift(rec, sysm, dt=None):
    """Linear drift of the total energy (kinetic + bond + bend + shifted
    non-bonded) over an NVE run, in kT per ns per degree of freedom
    (kJ/mol, kT = RG T / 1000), with the fit's standard error and the rms
    fluctuation about the line (kJ/mol)."""
    dt = sysm.dt if dt is None else dt
    tot = rec[:, 0] + rec[:, 1] + rec[:, 2] + rec[:, 4]  # kinet + bond + bend + nbonds
    if rec.shape[1] > 12:  # + urey + tors + impr (calcvalue.c:45-53)
        tot = tot + rec[:, 12] + rec[:, 13] + rec[:, 14]
    t_ps = np.arange(len(tot)) * dt
    kT = 1.380662e-23 * 6.022045e23 * sysm.T * 1e-3
    nfree = 3 * sysm.n - 3
    if len(tot) < 3:
        return {"kT_per_ns_per_dof": 0.0, "steps": int(len(tot))}
    A = np.vstack([t_ps, np.ones_like(t_ps)]).T
    coef, res, _, _ = np.linalg.lstsq(A, tot, rcond=None)
    resid = tot - A @ coef
    # standard error of the slope from the means of 0.25 ps blocks (the
    # fluctuations are correlated over many steps; block means much less)
    nb = max(int(t_ps[-1] // 0.25), 3)
    blk = [b for b in np.array_split(np.arange(len(tot)), nb) if len(b)]
    tm = np.array([t_ps[b].mean() for b in blk])
    em = np.array([tot[b].mean() for b in blk])
    cb = np.polyfit(tm, em, 1)
    rb = em - np.polyval(cb, tm)
    se = float(np.sqrt((rb ** 2).sum() / max(len(tm) - 2, 1) / ((tm - tm.mean()) ** 2).sum()))
    scale = 1000.0 / (kT * nfree)
    return {"kT_per_ns_per_dof": float(coef[0]) * scale,
            "stderr_kT_per_ns_per_dof": se * scale,
            "fluct_rms_kJ_mol": float(np.sqrt(np.mean(resid ** 2))),
            "steps": int(len(tot)), "span_ps": float(t_ps[-1]), "dt_fs": dt * 1e3}


def drift_study(local, n_mol, equil_steps, nve_steps, fp64=True, seed=SEED + 9):
    """NVE energy drift on an equilibrated box: Nose-Hoover (M=3) at 300 K for
    equil_steps from the random start (mixed precision), then from that state
    NVE for nve_steps at dt = 0.5 fs and 2 * nve_steps at dt/2, in mixed
    precision and (fp64=True) in the FP64 drop-in.  Drift from the
    integrator scales as dt^2; drift from the force field's cutoffs does not."""
    from thecodecombo_7_gb300 import engine, systems
    s = systems.water_box(n_mol, density=0.1, seed=seed, r_switch=R_SWITCH)
    nfree = 3 * s.n - 3
    RG = 8.31441e-3  # kJ/mol/K
    chunk = 500
    out = {"sites": s.n,
           "equilibration": f"{equil_steps} steps (mixed): NVE in chunks of {chunk} with the "
                            "velocities rescaled to 300 K after each (the reference's isokin), "
                            f"then {equil_steps // 4} Nose-Hoover steps at 300 K"}
    with engine.Box(s, precision=engine.FE_PREC_MIXED, device=local) as b:
        b.nblist()
        b.forces()
        b.kinet()
        step = 1
        for _ in range(max(equil_steps // chunk, 1)):
            b.run_md(chunk, first_step=step, record=False)
            step += chunk
            kin, _ = b.kinet()
            v, u = b.get_velocities()
            f = np.sqrt(s.T / (2.0 * kin / (nfree * RG)))
            b.set_velocities(v * f, u * f)
        rec = b.run_md(equil_steps // 4, first_step=step, use_nhc=True, record=True)
        out["T_end_K"] = float(2.0 * rec[-1, 0] / (nfree * RG))
        pos, nop = b.get_positions(), b.get_positions_nopbc()
        vel, _ = b.get_velocities()
    precs = [("mixed", engine.FE_PREC_MIXED)] + ([("fp64", engine.FE_PREC_FP64)] if fp64 else [])
    for name, prec in precs:
        for div in (1, 2):
            sd = s.copy()
            sd.dt = s.dt / div
            with engine.Box(sd, precision=prec, device=local) as b:
                b.set_positions(pos)
                b.set_positions_nopbc_array(nop)
                b.set_velocities(vel)
                b.nblist()
                b.forces()
                b.kinet()
                rec = b.run_md(nve_steps * div, first_step=1, record=True)
            out[f"{name}_dt{'' if div == 1 else '/2'}"] = nve_drift(rec, sd, sd.dt)
    return out


def config0_sample(local):
    """The plain FP64 drop-in on the 4,095-site box (1,365 molecules, L 34.47 A,
    SPME 32^3, LJ switch 8-10 A, list every 10 steps, dt 0.5 fs): 1,000 NVE
    steps timed with CUDA events; CPU: 10 real steps of the CPU restatement
    (reference makefile flags, one thread) on the same box."""
    import torch

    from oracle import oracle as orc
    from thecodecombo_7_gb300 import engine, systems
    s = systems.water_box(1365, density=0.1, seed=SEED + 1, r_switch=R_SWITCH)
    stream = torch.cuda.Stream(device=local)
    with engine.Box(s, precision=engine.FE_PREC_FP64, device=local) as b:
        b.set_stream(stream.cuda_stream)
        b.nblist()
        b.forces()
        b.kinet()
        b.run_md(10, first_step=1, record=False)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run_md(1000, first_step=11, record=False)
        e1.record(stream)
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / 1000.0
    md = orc.Oracle(s, fast=True).run_md(10, timed=True)
    cpu_sec = float(md["tstamp"][10] - md["tstamp"][0])
    return {"value": s.n * 1000 / sec, "unit": METRIC, "sites": s.n, "steps": 1000,
            "ns_per_day": 1000 / sec * 0.0005e-3 * 86400.0, "ms_per_step": 1000.0 * sec / 1000,
            "cpu_port_1_thread": s.n * 10 / cpu_sec,
            "workload": "4,095 sites (1,365 molecules), L 34.47 A, SPME 32^3 order 4, rc 10 A, "
                        "LJ switch 8-10 A, list 12 A every 10 steps, NVE dt 0.5 fs, FP64 drop-in"}


def batched_sample(local, steps):
    """32 NHC replicas of the 3-site recipe, 2,000-12,000 molecules each
    (seeded), own L at 0.1 sites/A^3 and grid ~1 point/A, T linear 300-400 K,
    exchange every 500 steps, all boxes in one graph per step; timed with
    CUDA events on the batch stream."""
    import torch

    from thecodecombo_7_gb300 import engine, systems
    R = 32
    rng = np.random.default_rng(SEED + 4)
    nmol = rng.integers(2000, 12001, R)
    temps = np.linspace(300.0, 400.0, R)
    ss = [systems.water_box(int(m), density=0.1, seed=SEED + 100 + k, T=float(temps[k]),
                            r_switch=R_SWITCH)
          for k, m in enumerate(nmol)]
    boxes = [engine.Box(s, precision=engine.FE_PREC_MIXED, device=local) for s in ss]
    try:
        shapes = []
        for b in boxes:
            b.nblist()
            b.forces()
            shapes.append(b.autotune()[:3])  # per-box launch shape (uneven sizes)
        batch = engine.Batch(boxes, seed=SEED)
        # box by box (one graph branch per box) first, then the fused step
        # (one launch per kernel for all boxes), continuing the same run
        batch.set_fused(False)
        batch.run(240, nlist_freq=10, swap_freq=500, first_step=1, use_nhc=True)
        st = torch.cuda.ExternalStream(batch.stream(), device=local)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        batch.run(100, nlist_freq=10, swap_freq=500, first_step=241, use_nhc=True)
        e1.record(st)
        torch.cuda.synchronize()
        ms_unfused = e0.elapsed_time(e1) / 100
        lv_unfused = batch.step_launches()
        batch.set_fused(True)
        # warm up to step 480 so that the timed steps include the exchange at step 500
        batch.run(140, nlist_freq=10, swap_freq=500, first_step=341, use_nhc=True)
        first = 481
        e0.record(st)
        batch.run(steps, nlist_freq=10, swap_freq=500, first_step=first, use_nhc=True)
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        n_atoms = int(sum(s.n for s in ss))
        state = batch.state()
        lv = batch.step_launches()
        n_list = sum(1 for i in range(first, first + steps) if i % 10 == 0)
        n_ex = sum(1 for i in range(first, first + steps) if i % 500 == 0)
        batch.close()
    finally:
        for b in boxes:
            b.close()
    return {"value": n_atoms * steps / (ms / 1000.0), "unit": METRIC, "replicas": R,
            "sites": n_atoms, "steps": steps, "ms_per_step": ms / steps,
            "workload": "32 NHC (M=3) replicas, 2,000-12,000 molecules each, own L at 0.1 "
                        "sites/A^3, grid ~1 point/A, LJ switch 8-10 A, T 300-400 K, exchange "
                        "every 500 steps",
            "exchange_attempts": int(state["attempts"]),
            "exchanges_in_timed_steps": n_ex, "list_steps": n_list,
            "graph_launches_per_step": {"plain": lv[0], "list": lv[1], "list_exchange": lv[3]},
            "stepping": "fused: each kernel launched once for all 32 boxes (box ranges of "
                        "blocks), batched FFTs per grid shape, list rebuilds of all boxes in six launches",
            "box_by_box": {"value": n_atoms / (ms_unfused * 1e-3), "ms_per_step": ms_unfused,
                           "graph_launches_per_step": {"plain": lv_unfused[0],
                                                       "list": lv_unfused[1]},
                           "steps": 100},
            "pair_launch_shapes": sorted(set(tuple(x) for x in shapes))}


def go_sample(local):
    """64 Go-model replicas (60-400 beads, seeded compact native structures),
    Langevin NVT at temperatures geometric 280-450 K, exchange every 1,000
    steps: one persistent launch per segment.  Timed: 5 segments (5,000
    steps) with CUDA events on the batch stream; CPU port: one replica of
    the same kind for a few steps on one thread."""
    import torch

    from oracle import oracle as orc
    from thecodecombo_7_gb300 import engine, systems
    g = systems.go_chains(64, seed=SEED)
    b = engine.GoBatch(g, device=local, seed=SEED)
    try:
        b.run(1000, swap_freq=1000)
        st = torch.cuda.ExternalStream(b.stream(), device=local)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        b.run(5000, swap_freq=1000)
        e1.record(st)
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / 1000.0
        s = b.state()
        lay = b.layout()
    finally:
        b.close()
    nb = int(g.nbeads.sum())
    r = int(np.argmax(g.nbeads))
    t0 = time.perf_counter()
    orc.go_baoab(g, r, 20, seed=SEED)
    cpu = int(g.nbeads[r]) * 20 / (time.perf_counter() - t0)
    return {"value": nb * 5000 / sec, "unit": "bead-steps/s", "replicas": 64, "beads": nb,
            "steps": 5000, "us_per_step": 1e6 * sec / 5000,
            "exchange_attempts": int(s["attempted"].sum()),
            "exchanges_accepted": int(s["accepted"].sum()),
            "ctas": lay["ncta"], "resident_ctas": lay["slots"],
            "chains_by_ctas": {str(k): int((lay["parts"] == k).sum()) for k in (1, 2, 3, 4)},
            "workload": "64 Go-model C-alpha chains (60-400 beads), bonds 3.8 A k=100 "
                        "kcal/mol/A^2, natives 12-10 eps=1 kcal/mol, non-native (4 A/r)^12, "
                        "BAOAB Langevin dt 10 fs gamma 1/ps, T 280-450 K geometric, exchange "
                        "every 1,000 steps",
            "cpu_port_bead_steps_per_s_1_thread": cpu}


def mc_sample(local):
    """Monte Carlo on the 4,095-site box: exact-dE chains against delayed
    acceptance with the surrogate trained on 2x10^5 exact moves of the same
    method; accepted moves/s for one chain (2x10^5 timed moves per mode) and
    for 152 chains (one per SM, 10^6 timed moves in total)."""
    import torch

    from thecodecombo_7_gb300 import engine, systems
    s = systems.water_box(1365, density=0.1, seed=SEED + 3, r_switch=R_SWITCH)
    box = engine.Box(s, precision=engine.FE_PREC_FP64, device=local)
    stream = torch.cuda.Stream(device=local)
    box.set_stream(stream.cuda_stream)
    net = engine.Mlp(device=local, seed=SEED)
    out = {"workload": "4,095 sites (1,365 rigid 3-site molecules, L 34.47 A), translation "
                       "<= 0.3 A / rotation <= 15 deg, Ewald kappa 0.32, |n|^2 <= 49 "
                       "(783 k-vectors), rc 10 A, LJ switch 8-10 A, 300 K"}
    try:
        # training set: 2x10^5 exact moves (152 chains x 1,316)
        box.mc_chains_setup(nchains=152, kmax=7, T=300.0, seed=SEED)
        box.mc_chains_collect(1316)
        box.mc_chains_run(1316)
        t0 = time.perf_counter()
        hist = box.mc_chains_train_surrogate(net, epochs=20, batch=512, lr=2e-3, seed=SEED)
        t_train = time.perf_counter() - t0
        box.mc_chains_setup(nchains=16, kmax=7, T=300.0, seed=SEED + 1)
        box.mc_chains_collect(512)
        box.mc_chains_run(512)
        held = box.mc_chains_samples()
        B = (len(held) // 64) * 64
        _, _, g = net.grad(held[:B, :128], held[:B, 128])
        y = held[:B, 128].astype(np.float64)
        res = (g[B:] - g[:B]).astype(np.float64) - y
        out["surrogate"] = {"train_samples": 152 * 1316, "epochs": 20, "train_s": t_train,
                            "loss_first_last": [float(hist[0]), float(hist[-1])],
                            "heldout_dEk_rms": float(np.sqrt(np.mean(y * y))),
                            "heldout_residual_rms": float(np.sqrt(np.mean(res * res)))}
        for mode, name in ((0, "exact"), (1, "delayed_acceptance")):
            for nch, moves in ((1, 200000), (152, 6600)):
                box.mc_chains_setup(nchains=nch, kmax=7, T=300.0, seed=SEED + 7)
                if mode:
                    box.mc_chains_set_surrogate(net)
                    box.mc_chains_set_mode(1)
                box.mc_chains_run(2000)
                st0 = [box.mc_chains_stats(c) for c in range(nch)]
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                box.mc_chains_run(moves)
                e1.record(stream)
                torch.cuda.synchronize()
                sec = e0.elapsed_time(e1) / 1000.0
                st1 = [box.mc_chains_stats(c) for c in range(nch)]
                acc = sum(b["accepted"] - a["accepted"] for a, b in zip(st0, st1))
                s1 = sum(b["stage1"] - a["stage1"] for a, b in zip(st0, st1))
                tot = nch * moves
                out[f"{name}_{nch}_chain{'s' if nch > 1 else ''}"] = {
                    "accepted_moves_per_s": acc / sec, "moves_per_s": tot / sec,
                    "acceptance": acc / tot, "stage1_acceptance": s1 / tot,
                    "moves_per_chain": moves, "chains": nch, "us_per_move": 1e6 * sec / moves}
        out["da_over_exact_accepted_per_s"] = (
            out["delayed_acceptance_1_chain"]["accepted_moves_per_s"] /
            out["exact_1_chain"]["accepted_moves_per_s"])
        # against the reference's exact evaluation: the reciprocal change
        # recomputed from every site before and after each move (modes 2, 3)
        for mode, name in ((2, "exact_full_recompute"), (3, "delayed_acceptance_full_recompute")):
            box.mc_chains_setup(nchains=1, kmax=7, T=300.0, seed=SEED + 7)
            if mode == 3:
                box.mc_chains_set_surrogate(net)
            box.mc_chains_set_mode(mode)
            box.mc_chains_run(50)
            a0 = box.mc_chains_stats(0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            moves = 1500
            e0.record(stream)
            box.mc_chains_run(moves)
            e1.record(stream)
            torch.cuda.synchronize()
            sec = e0.elapsed_time(e1) / 1000.0
            a1 = box.mc_chains_stats(0)
            acc = a1["accepted"] - a0["accepted"]
            out[f"{name}_1_chain"] = {"accepted_moves_per_s": acc / sec, "moves_per_s": moves / sec,
                                      "acceptance": acc / moves,
                                      "stage1_acceptance": (a1["stage1"] - a0["stage1"]) / moves,
                                      "us_per_move": 1e6 * sec / moves, "moves_per_chain": moves}
        out["da_over_exact_full_recompute_accepted_per_s"] = (
            out["delayed_acceptance_full_recompute_1_chain"]["accepted_moves_per_s"] /
            out["exact_full_recompute_1_chain"]["accepted_moves_per_s"])
        # the reference's exact dE recomputes the whole structure factor twice
        # per move (ewald_mc.c:109-156 via forces_mc); its CPU restatement,
        # one thread, reference makefile flags, on 40 translation moves
        from oracle import oracle as orc
        o = orc.Oracle(s, fast=True)
        rng = np.random.default_rng(SEED)
        t0 = time.perf_counter()
        for _ in range(40):
            m = int(rng.integers(0, 1365))
            pn = s.pos.copy()
            pn[3 * m:3 * m + 3] += (rng.uniform(size=3) - 0.5) * 0.6
            o.mc_delta_energy(s.pos, pn, 3 * m, 3 * m + 3, kmax=7, max_k_square=49)
        out["cpu_port_full_recompute_moves_per_s_1_thread"] = 40 / (time.perf_counter() - t0)
    finally:
        net.close()
        box.close()
    return out


def energy_errors(en_mixed, en_fp64):
    """Per-term relative error of the mixed-precision energies against the
    FP64 drop-in on the same coordinates (equal to the FP64 oracle to 1e-12
    in the parity tests); terms that vanish (bond, bend at a rigid start) get
    their absolute error instead."""
    out = {}
    for k in EN_TERMS:
        a, b = en_fp64[k], en_mixed[k]
        out[k] = (b - a) / abs(a) if abs(a) > 1e-6 else {"abs": b - a}
    return out


def run_ours(args, world, rank, local):
    import torch

    from thecodecombo_7_gb300 import build as fe_build
    from thecodecombo_7_gb300 import engine, systems

    if not os.path.exists(engine.LIB_PATH):
        fe_build.build()
    torch.cuda.set_device(local)
    sysm = systems.water_box(N_MOL, density=0.1, seed=SEED + rank, r_switch=R_SWITCH)
    n = sysm.n
    stream = torch.cuda.Stream(device=local)
    box = engine.Box(sysm, precision=engine.FE_PREC_MIXED, device=local)
    box.set_stream(stream.cuda_stream)
    box.nblist()
    en_mixed0 = box.forces()
    box.kinet()
    f_mixed0 = box.get_forces()
    tune = box.autotune()  # launch shape of the pair kernel for this box (untimed)
    W = max(args.warmup, 3)
    K = args.steps
    box.run_md(W, first_step=1)
    first = W + 1
    nl = sysm.nlist_freq
    clocks = ClockSampler(local)
    nvml = NvmlSampler(local)
    clocks.start()
    nvml.start()
    barrier(world)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    _, _, prunes0 = box.inner_list_stats()
    ev0.record(stream)
    box.run_md(K, nlist_freq=nl, first_step=first, record=False)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    clk_nvml = nvml.stop()
    if clk_nvml and (clk.get("samples") or 0) < 3:
        clk = dict(clk_nvml, nvidia_smi_samples=clk.get("samples"))
    ms = ev0.elapsed_time(ev1)
    ms_max = allreduce_max(ms, world)
    value = world * n * K / (ms_max / 1000.0)
    n_list_steps = sum(1 for i in range(first, first + K) if i % nl == 0)
    lp, ll = box.step_launches(False)
    launches = lp * (K - n_list_steps) + ll * n_list_steps
    # dominant kernel: the pair loop over the inner list (its steady state
    # between prunes), timed live on the same stream
    _, _, prunes1 = box.inner_list_stats()
    pair_us = box.time_kernel(engine.FE_KERNEL_PAIR, reps=20)
    outer_entries, _ = box.list_stats()
    entries, max_row, _ = box.inner_list_stats()
    alg_bytes = 4.0 * entries + n * (16.0 + 4.0 + 4.0 + 24.0)
    peaks, peak_kind = load_peaks()
    achieved = alg_bytes / (pair_us * 1e-6) / 1e9
    peak = float(peaks["hbm_gbs"])
    traffic = profile_traffic()
    pipe = {"fp32_tflops": engine.pipe_peak(0, local), "fp64_tflops": engine.pipe_peak(1, local),
            "mufu_tera_ops": engine.pipe_peak(2, local),
            "how": "fe_pipe_peak: FMA / ex2.approx chains, 8 per thread, 8 blocks of 256 per "
                   "SM, best of 3 (CUDA events)"}
    # plain FP64 drop-in on the same workload (the 10x denominator), a few steps
    fp64 = None
    force_err = None
    en_err = None
    counts = None
    b64 = None
    if rank == 0:
        b64 = engine.Box(sysm, precision=engine.FE_PREC_FP64, device=local)
        b64.set_stream(stream.cuda_stream)
        b64.nblist()
        en64 = b64.forces()
        f64 = b64.get_forces()
        counts = b64.pair_counts()
        d = f_mixed0 - f64
        force_err = {"rms_rel": float(np.sqrt((d ** 2).sum() / (f64 ** 2).sum())),
                     "max_abs": float(np.abs(d).max())}
        en_err = energy_errors(en_mixed0, en64)
        b64.kinet()
        b64.run_md(3, first_step=1)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        k64 = 20
        e0.record(stream)
        b64.run_md(k64, first_step=4)
        e1.record(stream)
        torch.cuda.synchronize()
        fp64 = n * k64 / (e0.elapsed_time(e1) / 1000.0)
    # end to end through the C ABI with host buffers (pinned)
    ke = min(K, 30)
    pos_h = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    nop_h = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    vv_h = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    uu_h = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    ff_h = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    pos_h[:] = box.get_positions()
    nop_h[:] = box.get_positions_nopbc()
    v, u = box.get_velocities()
    vv_h[:] = v
    uu_h[:] = u
    lib = box.lib
    import ctypes as C

    def ptr(a):
        return a.ctypes.data_as(C.c_void_p)

    ff_h[:] = box.get_forces()
    en = np.empty(engine.FE_EN_COUNT)
    io = engine.FeMdIo(pos_h.ctypes.data, 24, 0, nop_h.ctypes.data, 24, 0, vv_h.ctypes.data,
                       uu_h.ctypes.data, ff_h.ctypes.data)
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(first + K, first + K + ke):
        # nve_md.c's loop: the list when due, integrate_vverlet with the host
        # state it reads (atom, atnopbc, vv, ff: uploaded before the step)
        # and writes (those and uu: read back after it), kinet
        if i % nl == 0:
            box._check(lib.fe_nblist(box.h))
        box._check(lib.fe_integrate_vverlet_host(box.h, C.c_double(1.0), C.byref(io), ptr(en)))
        box._check(lib.fe_kinet(box.h, None, None))
    torch.cuda.synchronize()
    t_e2e = allreduce_max(time.perf_counter() - t0, world)
    e2e = world * n * ke / t_e2e
    h2d = 4 * 24 * n
    d2h = 5 * 24 * n + 8 * engine.FE_EN_COUNT
    # accuracy along one continuous trajectory: mixed-precision forces against
    # the FP64 engine on the same coordinates at steps 0, 1,000 and 10,000
    accuracy = None
    if b64 is not None:
        def fp64_error():
            b64.set_positions(box.get_positions())
            b64.nblist()
            e64 = b64.forces()
            f64 = b64.get_forces()
            em = box.forces()
            d = box.get_forces() - f64
            return {"rms_rel": float(np.sqrt((d ** 2).sum() / (f64 ** 2).sum())),
                    "max_abs": float(np.abs(d).max())}, energy_errors(em, e64)
        done = W + K + ke
        if done < 1000:
            box.run_md(1000 - done, nlist_freq=nl, first_step=done + 1, record=False)
        err1k, en1k = fp64_error()
        box.run_md(9000, nlist_freq=nl, first_step=1001, record=False)
        err10k, en10k = fp64_error()
        accuracy = {"force_error_vs_fp64": {"step_0": force_err, "step_1000": err1k,
                                            "step_10000": err10k, "unit_max_abs": "kJ/mol/A"},
                    "energy_rel_error_vs_fp64": {"step_0": en_err, "step_1000": en1k,
                                                 "step_10000": en10k}}
        b64.close()
    box.close()
    if rank != 0:
        return
    cpu = None
    if world == 1:
        try:
            c = cpu_sample(sysm)
            cpu = {k: c[k] for k in ("value", "unit", "cores", "kind", "sample")}
        except Exception as exc:  # the GPU line must still print
            cpu = {"value": None, "unit": METRIC, "cores": 1, "kind": "port",
                   "sample": f"failed: {exc}"}
    steps_per_s = K / (ms_max / 1000.0)
    extras = {}
    for name, fn in (("batched_replicas", lambda: batched_sample(local, min(max(K, 100), 500))),
                     ("mc", lambda: mc_sample(local)), ("go_replicas", lambda: go_sample(local)),
                     ("config0_fp64", lambda: config0_sample(local)),
                     ("nve_drift_4095", lambda: drift_study(local, 1365, 20000, 10000)),
                     ("nve_drift_96000", lambda: drift_study(local, N_MOL, 8000, 10000,
                                                             fp64=False))):
        try:
            extras[name] = fn()
        except Exception as exc:  # the headline line must still print
            extras[name] = {"failed": str(exc)}
    # the pair loop's algorithmic FLOPs per step (half-list units, counted
    # from the reference loop): 11 per list entry, +30 per pair inside rc,
    # +17 per LJ pair, +12 per excluded pair inside rc
    L_pairs, P_rc, P_lj, P_x = counts if counts else (0, 0, 0, 0)
    flops = 11.0 * L_pairs + 30.0 * P_rc + 17.0 * P_lj + 12.0 * P_x
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": (value / world) / fp64 if fp64 else None,
        "vs_baseline_basis": "mixed-precision engine / plain FP64 drop-in on the same box and "
                             "the same GPU, this run (the metric's denominator)",
        "dtype": "fp32", "data": "synthetic",
        "config": dict(CONFIG, parallelism=f"replicas x{world}"),
        "precision": "mixed (FP32 pair/PME math, int64 fixed-point force sums, FP64 "
                     "integration and energy sums)",
        "ns_per_day": steps_per_s * 0.0005e-3 * 86400.0,
        "roofline": {"kernel": "k_mx_pair", "bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_kind, "algorithmic_bytes": alg_bytes,
                     "us_per_launch": pair_us, "list_entries": entries, "max_row": max_row,
                     "fp32_pipe": {"algorithmic_gflop_per_launch": flops * 1e-9,
                                   "achieved_tflops": flops / (pair_us * 1e-6) * 1e-12,
                                   "peak_tflops": pipe["fp32_tflops"],
                                   "frac": flops / (pair_us * 1e-6) * 1e-12 / pipe["fp32_tflops"],
                                   "half_list_counts": {"entries": L_pairs, "pairs_in_rc": P_rc,
                                                        "lj_pairs_in_rc": P_lj,
                                                        "excluded_in_rc": P_x}},
                     "list": f"inner list (rc + 0.8 A, {entries} entries) between prunes; "
                             f"outer list (rlist, {outer_entries} entries) read by the "
                             f"{prunes1 - prunes0} pruning launches of the {K} timed steps",
                     "launch_shape": {"warps_per_block": tune[0], "registers": tune[1],
                                      "blocks": tune[2],
                                      "chosen_by": "autotune (events, this box)"}},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e, "unit": METRIC, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": ke},
        "gpu_launches": launches,
        "clocks": clk,
        "pipe_peaks": pipe,
    }
    line.update(extras)
    # last, so that a truncated tail of the line still carries them
    line["accuracy"] = accuracy
    line["fp64_drop_in"] = {"value": fp64, "unit": METRIC,
                            "ratio": (value / world) / fp64 if fp64 else None}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2500)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--drift-study", type=int, default=0, metavar="NVE_STEPS",
                    help="only the NVE drift study of the 4,095-site box, NVE_STEPS steps at "
                         "dt (twice as many at dt/2), FP64 and mixed; prints one JSON line")
    args = ap.parse_args()
    if args.drift_study:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps({"nve_drift_4095": drift_study(0, 1365, 40000, args.drift_study)}))
        return
    world, rank, local = dist_setup() if args.impl == "ours" else (
        int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

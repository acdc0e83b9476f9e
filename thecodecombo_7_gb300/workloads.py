"""A single box of the water workload stepped on the GPU, for timing and for
profiling one kernel at a time (a small driver: it builds only the box it
is asked for).

    python -m thecodecombo_7_gb300.workloads [--molecules 32000] [--precision mixed]
        [--steps 30] [--warmup 10] [--switch 8.0]
    python -m thecodecombo_7_gb300.workloads --batch [--replicas 32] [--unfused]
    python -m thecodecombo_7_gb300.workloads --go [--replicas 64] [--steps 1000]

With --profile-range the timed steps alone are bracketed by
cudaProfilerStart/Stop, so `ncu --profile-from-start off` lists the launches
of the production steps without the set-up, autotuning and warm-up.

Builds the seeded 3-site water box (0.1 sites/A^3, SPME grid ~1 point/A),
picks the pair kernel's launch shape, runs the warm-up steps, then the timed
steps of the production loop (list every 10 steps) with CUDA events, and
prints one JSON line: ms per step and the mean device time of the pair,
spreading and list kernels re-launched on the final state.
"""
from __future__ import annotations

import argparse
import json

from . import engine, systems


def batch_main(a):
    """The uneven replica batch: 32 NHC boxes of 2,000-12,000 molecules (the
    bench's batch leg), stepped together; prints one JSON line."""
    import numpy as np
    import torch
    rng = np.random.default_rng(a.seed + 4)
    nmol = rng.integers(2000, 12001, a.replicas)
    temps = np.linspace(300.0, 400.0, a.replicas)
    ss = [systems.water_box(int(m), density=0.1, seed=a.seed + 100 + k, T=float(temps[k]),
                            r_switch=a.switch) for k, m in enumerate(nmol)]
    boxes = [engine.Box(s, precision=engine.FE_PREC_MIXED) for s in ss]
    out = {"replicas": a.replicas, "sites": int(sum(s.n for s in ss))}
    try:
        for b in boxes:
            b.nblist()
            b.forces()
        batch = engine.Batch(boxes, seed=a.seed)
        batch.set_fused(not a.unfused)
        batch.run(a.warmup, nlist_freq=10, swap_freq=500, first_step=1, use_nhc=True)
        st = torch.cuda.ExternalStream(batch.stream())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        if a.profile_range:
            torch.cuda.profiler.start()
        e0.record(st)
        batch.run(a.steps, nlist_freq=10, swap_freq=500, first_step=a.warmup + 1, use_nhc=True)
        e1.record(st)
        if a.profile_range:
            torch.cuda.profiler.stop()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        out.update(ms_per_step=ms / a.steps, atom_steps_per_s=out["sites"] * a.steps / (ms * 1e-3),
                   launches=batch.step_launches(), fused=not a.unfused)
        batch.close()
    finally:
        for b in boxes:
            b.close()
    print(json.dumps(out))


def go_main(a):
    """Go-model replica exchange: 64 chains of 60-400 beads (the bench's Go
    leg), one persistent launch per exchange segment of --steps steps; times
    --warmup segments untimed and then 5 segments; prints one JSON line."""
    import torch
    g = systems.go_chains(a.replicas, seed=a.seed)
    b = engine.GoBatch(g, seed=a.seed)
    try:
        b.run(a.warmup * a.steps, swap_freq=a.steps)
        st = torch.cuda.ExternalStream(b.stream())
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        if a.profile_range:
            torch.cuda.profiler.start()
        e0.record(st)
        b.run(5 * a.steps, swap_freq=a.steps)
        e1.record(st)
        if a.profile_range:
            torch.cuda.profiler.stop()
        torch.cuda.synchronize()
        us = 1e3 * e0.elapsed_time(e1) / (5 * a.steps)
        lay = b.layout()
    finally:
        b.close()
    nb = int(g.nbeads.sum())
    print(json.dumps({"replicas": a.replicas, "beads": nb, "us_per_step": us,
                      "bead_steps_per_s": nb / (us * 1e-6), "ctas": lay["ncta"],
                      "resident_ctas": lay["slots"],
                      "chains_by_ctas": {str(k): int((lay["parts"] == k).sum())
                                         for k in (1, 2, 3, 4)}}))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--molecules", type=int, default=32000)
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--switch", type=float, default=8.0)
    ap.add_argument("--seed", type=int, default=2025)
    ap.add_argument("--batch", action="store_true",
                    help="the 32-replica uneven batch instead of one box")
    ap.add_argument("--go", action="store_true",
                    help="the Go-model replica exchange instead of water")
    ap.add_argument("--replicas", type=int, default=None,
                    help="batch: 32 boxes; go: 64 chains")
    ap.add_argument("--unfused", action="store_true", help="batch: box by box")
    ap.add_argument("--profile-range", action="store_true",
                    help="bracket the timed steps with cudaProfilerStart/Stop")
    a = ap.parse_args(argv)
    if a.go:
        a.replicas = a.replicas or 64
        return go_main(a)
    if a.batch:
        a.replicas = a.replicas or 32
        return batch_main(a)
    import torch
    s = systems.water_box(a.molecules, density=0.1, seed=a.seed, r_switch=a.switch)
    prec = engine.FE_PREC_MIXED if a.precision == "mixed" else engine.FE_PREC_FP64
    stream = torch.cuda.Stream()
    out = {"sites": s.n, "precision": a.precision, "grid": list(s.grid)}
    with engine.Box(s, precision=prec) as b:
        b.set_stream(stream.cuda_stream)
        b.nblist()
        b.forces()
        b.kinet()
        if prec == engine.FE_PREC_MIXED:
            out["launch_shape"] = b.autotune()
        b.run_md(a.warmup, first_step=1, record=False)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        if a.profile_range:
            torch.cuda.profiler.start()
        e0.record(stream)
        b.run_md(a.steps, first_step=a.warmup + 1, record=False)
        e1.record(stream)
        if a.profile_range:
            torch.cuda.profiler.stop()
        torch.cuda.synchronize()
        out["ms_per_step"] = e0.elapsed_time(e1) / a.steps
        out["atom_steps_per_s"] = s.n * a.steps / (e0.elapsed_time(e1) * 1e-3)
        for name, k in (("pair", engine.FE_KERNEL_PAIR), ("spread", engine.FE_KERNEL_SPREAD),
                        ("list", engine.FE_KERNEL_LIST)):
            out[f"{name}_us"] = b.time_kernel(k, reps=10)
        out["list_entries"], out["max_row"] = b.list_stats()
        if prec == engine.FE_PREC_MIXED:
            out["inner_entries"] = b.inner_list_stats()[0]
    print(json.dumps(out))


if __name__ == "__main__":
    main()

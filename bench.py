"""Benchmark of the push: FP64 particle-turns/s on the thick LHC-like ring.

Workload: the synthetic thick ring (8 arcs x 23 FODO cells, 6993 elements,
drift-kick-drift-expanded magnets with 8 kicks and order-10 multipole
errors) with 10^6 Gaussian protons at 7 TeV (xtrack_gb300.workloads). A step
is one turn of the whole ring for the whole beam, so particle-turns/s =
particles x steps / time. The particle arrays (19 x 8 B x 10^6 = 152 MB) are
larger than the 129 MB L2, so no flush is needed between steps.

value   device-timed: CUDA events on the launching stream around the K steps.
e2e     the same steps through the C-ABI with pinned host buffers: each step
        copies the particle arrays host->device, tracks one turn and copies
        them back, all inside the timed region.
roofline  FP64 pipe: counted FLOPs (canonical minimal formulation, FMA = 2)
        per particle-turn x particle-turns / kernel time, against the FP64
        DFMA peak measured in the same run (the driver's peak file has no
        FP64 figure).
cpu_baseline  the CPU oracle (a C port of the reference's OpenMP track_line)
        on all host cores, on a bounded sample of the same workload.

--impl reference  times that CPU implementation alone and prints its line.
Multi-GPU (torchrun, N > 1): each rank tracks its own 10^6 particles
(weak scaling, no data-path collective); timing is the max over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

METRIC = "FP64 particle-turns/s on thick ring (1 GB300)"
UNIT = "particle-turns/s"


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.gpu}",
                                      f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([v.strip() for v in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        smax = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for n, v in zip(names, s[3:7]):
                if v.strip().lower() in ("active", "1"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(float(s[2]) for s in self.samples
                                   if s[2].replace(".", "").isdigit()) if self.samples else None,
                "samples": len(self.samples), "reasons": sorted(reasons)}


def cpu_baseline(line, n_target_seconds=12.0):
    """The oracle's port of the reference OpenMP track_line on all host
    cores, on a sample of the workload sized to ~n_target_seconds."""
    import pyoracle
    from xtrack_gb300 import workloads
    pyoracle.ensure_built(with_ref=False)
    recs = line._element_records()
    L = line.get_length()
    p0c = float(line.particle_ref.p0c[0])
    cores = pyoracle.max_threads()
    # calibrate on a small sample
    n_cal = 4 * cores
    cal = pyoracle.host_arrays(workloads.gaussian_beam(n_cal, p0c, seed=5, device="cpu").to_numpy())
    t0 = time.perf_counter()
    pyoracle.track(recs, cal, num_turns=1, line_length=L, mode=pyoracle.MODE_OPENMP)
    dt = time.perf_counter() - t0
    rate = n_cal / dt
    n = int(max(cores, min(200000, rate * n_target_seconds)))
    beam = pyoracle.host_arrays(workloads.gaussian_beam(n, p0c, seed=6, device="cpu").to_numpy())
    t0 = time.perf_counter()
    pyoracle.track(recs, beam, num_turns=1, line_length=L, mode=pyoracle.MODE_OPENMP)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{n} particles x 1 turn of the {len(recs)}-element thick ring "
                      f"({dt:.1f} s, OpenMP, element-outer chunks as the reference CPU path)"}


def run_reference(args):
    rank, world, _ = _dist()
    if rank != 0:
        return
    from xtrack_gb300 import workloads
    line = workloads.thick_ring()
    vals = []
    base = None
    for i in range(args.warmup + args.steps):
        b = cpu_baseline(line, n_target_seconds=max(2.0, 30.0 / max(1, args.steps + args.warmup)))
        if i >= args.warmup:
            vals.append(b["value"])
            base = b
    v = float(np.median(vals))
    base["value"] = v
    out = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "thick ring 6993 elements, 1e6 protons 7 TeV (CPU sample)",
                      "particles": base["sample"]},
           "cpu_baseline": base,
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_gpu(args):
    import ctypes

    import torch
    from xtrack_gb300 import _abi, workloads

    rank, world, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    line = workloads.thick_ring()
    p0c = float(line.particle_ref.p0c[0])
    n = args.particles
    beam = workloads.gaussian_beam(n, p0c, seed=100 + rank, device=dev)
    tracker = line.build_tracker(device=dev, arith=args.arith)
    lib = _abi.load_library()
    n_el = len(line.element_names)
    flops_pt = tracker.flops_per_particle()

    peak = ctypes.c_double()
    _abi.check(lib.xtg_measure_fp64_peak(ctypes.byref(peak)))
    fp64_peak = peak.value

    stream = torch.cuda.current_stream(dev)

    def step():
        tracker._track(beam, num_turns=1)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    n_alive0 = int((beam.state > 0).sum().item())
    launches0 = lib.xtg_launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1)
    launches = lib.xtg_launch_count() - launches0
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    n_alive1 = int((beam.state > 0).sum().item())
    particle_turns = float(n) * args.steps * world
    value = particle_turns / (ms * 1e-3)
    ms_per_step = ms / args.steps
    kernel_s = ms * 1e-3 / args.steps
    achieved = flops_pt * n / kernel_s

    # e2e through the C-ABI with pinned host buffers
    fields = _abi.PARTICLE_DOUBLE_FIELDS + _abi.PARTICLE_INT_FIELDS
    host = {f: getattr(beam, f).cpu().pin_memory() for f in fields}
    devbuf = {f: torch.empty_like(getattr(beam, f)) for f in fields}
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    pstruct = _abi.particles_struct_from_ptrs(n, beam.q0, beam.mass0, beam.t_sim,
                                              {f: devbuf[f].data_ptr() for f in fields})

    def e2e_step():
        for f in fields:
            devbuf[f].copy_(host[f], non_blocking=True)
        tracker._launch(pstruct, 1, 0, n_el, True, 0, None, 0, stream.cuda_stream)
        for f in fields:
            host[f].copy_(devbuf[f], non_blocking=True)

    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    torch.cuda.synchronize(dev)
    e2e_steps = max(1, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize(dev)
    e2e_s = time.perf_counter() - t0
    e2e_value = float(n) * e2e_steps * world / e2e_s

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "arith": args.arith,
           "config": {"workload": "thick LHC-like ring, 8x23 FODO cells, 6993 elements, "
                                  "1e6 protons 7 TeV, 1 turn per step",
                      "particles_per_gpu": n, "elements": n_el, "turns_per_step": 1,
                      "l2": "inputs larger than L2 (152 MB of particle arrays), no flush",
                      "alive_before": n_alive0, "alive_after": n_alive1},
           "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                   "d2h_bytes_per_step": h2d},
           "gpu_launches": int(launches),
           "roofline": {"bound": "fp64", "achieved": achieved / 1e12, "peak": fp64_peak / 1e12,
                        "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                        "peak_source": "in-run DFMA probe (FP64 pipe, FMA = 2)",
                        "flops_per_particle_turn": flops_pt, "traffic": _traffic()},
           "clocks": clk.summary()}
    if not args.no_alt:
        # the other arithmetic mode on the same beam, same step count
        alt = "exact" if args.arith == "fast" else "fast"
        t_alt = line.build_tracker(device=dev, arith=alt)
        for _ in range(args.warmup):
            t_alt._track(beam, num_turns=1)
        torch.cuda.synchronize(dev)
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        for _ in range(args.steps):
            t_alt._track(beam, num_turns=1)
        a1.record(stream)
        torch.cuda.synchronize(dev)
        ms_alt = a0.elapsed_time(a1)
        v_alt = float(n) * args.steps * world / (ms_alt * 1e-3)
        out[alt] = {"value": v_alt, "unit": UNIT, "ms_per_step": ms_alt / args.steps,
                    "roofline_frac": flops_pt * n / (ms_alt * 1e-3 / args.steps) / fp64_peak}
        line.tracker = tracker
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(line)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def _traffic():
    """DRAM bytes per launch of the track kernel from the committed ncu
    summary, when present."""
    p = os.path.join(ROOT, "profiles", "track_kernel_traffic.json")
    if os.path.exists(p):
        try:
            return json.load(open(p)).get("dram_bytes_per_launch")
        except Exception:
            return None
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--arith", default="fast", choices=["exact", "fast"])
    ap.add_argument("--no-alt", action="store_true",
                    help="skip the timing of the other arithmetic mode")
    ap.add_argument("--particles", type=int, default=1_000_000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

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
           "config": {"workload": "thick LHC-like ring, 8x23 FODO cells, 6993 elements, "
                                  f"{args.particles:.3g} protons 7 TeV, 1 turn per step",
                      "particles_per_gpu": args.particles, "elements": 6993,
                      "turns_per_step": 1,
                      "sample": "each step times a bounded sample of the beam on the host "
                                "cores: " + base["sample"]},
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
    tuning = tracker.set_tuning(**_tuning_args(args))
    lib = _abi.load_library()
    n_el = len(line.element_names)
    flops_pt = tracker.flops_per_particle()

    peak = ctypes.c_double()
    _abi.check(lib.xtg_measure_fp64_peak(ctypes.byref(peak)))
    fp64_peak = peak.value
    # multiply+add chains with the products on the integer pipes
    er = ctypes.c_double()
    _abi.check(lib.xtg_measure_emul_rate(ctypes.byref(er)))
    emul_rate = er.value

    stream = torch.cuda.current_stream(dev)
    monitor = None
    if args.monitor_first:
        # turn-by-turn monitor of the first particles, 6 coordinates, over
        # the timed steps (the monitor-stress configuration)
        from xtrack_gb300.monitors import ParticlesMonitor
        t0_turn = args.warmup
        monitor = ParticlesMonitor(start_at_turn=t0_turn, stop_at_turn=t0_turn + args.steps,
                                   num_particles=min(args.monitor_first, n),
                                   fields=("x", "px", "y", "py", "zeta", "delta"), device=dev)

    def step():
        tracker._track(beam, num_turns=1, turn_by_turn_monitor=monitor)

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
    # particle-turns survived: particles alive after the last timed step
    # times the steps (a lower bound: particles lost inside the timed
    # region are not counted for the turns they did survive)
    n_alive1 = int((beam.state > 0).sum().item())
    alive_all = float(n_alive1)
    if world > 1:
        t = torch.tensor([alive_all], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t)
        alive_all = float(t.item())
    particle_turns = alive_all * args.steps
    value = particle_turns / (ms * 1e-3)
    ms_per_step = ms / args.steps
    kernel_s = ms * 1e-3 / args.steps
    achieved = flops_pt * n_alive1 / kernel_s

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
    e2e_value = alive_all * e2e_steps / e2e_s

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "arith": args.arith,
           "config": {"workload": "thick LHC-like ring, 8x23 FODO cells, 6993 elements, "
                                  f"{n:.3g} protons 7 TeV, 1 turn per step",
                      "particles_per_gpu": n, "elements": n_el, "turns_per_step": 1,
                      "l2": f"inputs larger than L2 ({n * 152 / 1e6:.0f} MB of particle "
                            "arrays), no flush" if n * 152 > 129e6 else
                            "inputs smaller than L2 (not a headline configuration)",
                      "alive_before": n_alive0, "alive_after": n_alive1,
                      "tuning": tuning,
                      "monitor": (None if monitor is None else
                                  {"particles": monitor.part_id_end, "fields": 6,
                                   "bytes_per_step": monitor.part_id_end * 48})},
           "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                   "d2h_bytes_per_step": h2d},
           "gpu_launches": int(launches),
           "roofline": {"bound": "fp64", "achieved": achieved / 1e12, "peak": fp64_peak / 1e12,
                        "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                        "peak_source": "in-run DFMA probe (FP64 pipe, FMA = 2)",
                        "flops_per_particle_turn": flops_pt, "traffic": _traffic(args.arith),
                        "note": "the push runs its stand-alone FP64 products on the integer "
                                "pipes (bit-identical), next to the FP64 pipe; the peak is the "
                                "FP64 pipe's alone",
                        "emul_probe_ops_per_s": emul_rate},
           "clocks": clk.summary()}
    if not args.no_alt:
        # the other arithmetic mode on the same beam, same step count
        alt = "exact" if args.arith == "fast" else "fast"
        t_alt = line.build_tracker(device=dev, arith=alt)
        t_alt.set_tuning(**_tuning_args(args))
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
        v_alt = alive_all * args.steps / (ms_alt * 1e-3)
        out[alt] = {"value": v_alt, "unit": UNIT, "ms_per_step": ms_alt / args.steps,
                    "roofline_frac": flops_pt * n_alive1 / (ms_alt * 1e-3 / args.steps) / fp64_peak}
        line.tracker = tracker
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(line)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def _tuning_args(args):
    kw = {}
    for k in ("block_size", "compact_every", "chunk_bytes", "use_graph"):
        v = getattr(args, k)
        if v is not None:
            kw[k] = v
    return kw


def run_da_screen(args):
    """DA-scan time, screened vs plain, on seeds of the thick ring. The
    seeds are scanned on a polar grid (11 angles x 2 momentum offsets x
    amplitudes up to --da-rmax sigma) with all seeds in one persistent
    launch. A survival MLP is trained with the library's kernels on the
    training seeds' outcomes (features: coordinates, the seed's tunes,
    closed-orbit extremes, the ray's linear aperture and, by default, the
    seed's 32 multipole-error features). The test seeds are then scanned
    plainly (every particle tracked) and screened six ways: (1) the
    network's uncertain band alone (one pass); (2) sentinels every
    --da-stride amplitudes plus that band, then each ray's bracket (two
    passes); (3) the same two passes without the network; (4) three passes
    without the network (coarse sentinels every --da-coarse amplitudes, a
    fine window below the first coarse loss, brackets); (5) two passes with
    the fine window placed by the network around its predicted boundary;
    (6) the same two passes without the network (coarse sentinels, brackets
    of one coarse step). value = plain time / time of (1), the
    configuration's one-pass screening. The DA error per
    ray (sigma) judges each screened result against the plain one; the
    network's own DA per ray (its predicted boundary) is reported beside
    them."""
    import torch
    from xtrack_gb300 import scan as sc
    from xtrack_gb300 import surrogate as sg
    from xtrack_gb300 import workloads
    from xtrack_gb300.batch import BatchTracker

    rank, world, local = _dist()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    turns = args.da_turns
    rng = np.random.default_rng(7)

    def counts(n, mean):
        return rng.integers(mean // 2, mean * 3 // 2 + 1, size=n)

    def features(scan):
        f = sg.da_features(scan)
        if args.da_features == "all":
            f = np.concatenate([f, scan.seed_features[scan.lattice_index]], axis=1)
        return f

    train_lines = [workloads.thick_ring(seed=100 + s) for s in range(args.da_train_seeds)]
    test_lines = [workloads.thick_ring(seed=200 + s) for s in range(args.da_test_seeds)]
    t0 = time.perf_counter()
    s_train = sc.build_scan(train_lines, counts(len(train_lines), args.da_train_particles),
                            r_max=args.da_rmax, device=dev, features=sg.seed_features)
    s_test = sc.build_scan(test_lines, counts(len(test_lines), args.da_particles),
                           r_max=args.da_rmax, device=dev, features=sg.seed_features)
    t_setup = time.perf_counter() - t0
    bt_train = BatchTracker(train_lines, device=dev, arith=args.arith)
    bt_test = BatchTracker(test_lines, device=dev, arith=args.arith)
    # one-warp blocks spread a small (screened) particle set over every SM
    # sub-partition; 12 KB chunks keep eight of them resident per SM
    for bt in (bt_train, bt_test):
        bt.set_tuning(compact_every=max(1, turns // 10), block_size=32, chunk_bytes=12288)

    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    st, at, _ = sc.run_scan(bt_train, s_train, turns, device=dev)
    t_train_scan = time.perf_counter() - t0
    surv, lt = sg.targets(st, at, turns)
    n_in = sg.N_DA_FEATURES + (sg.N_SEED_FEATURES if args.da_features == "all" else 0)
    net = sg.SurvivalMLP(n_in=n_in, seed=0, device=dev)
    t0 = time.perf_counter()
    hist = net.fit(features(s_train), surv, lt, epochs=args.da_epochs, batch=4096, lr=3e-3,
                   weight_decay=args.da_weight_decay)
    torch.cuda.synchronize(dev)
    t_fit = time.perf_counter() - t0

    # plain scan of the test seeds
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    st_p, at_p, _ = sc.run_scan(bt_test, s_test, turns, device=dev)
    t_plain = time.perf_counter() - t0
    surv_plain = sg.targets(st_p, at_p, turns)[0] > 0
    n_seeds = len(test_lines)
    da_plain = sc.da_table(s_test, surv_plain, n_seeds)
    ray = s_test.ray_index()

    def stats(da, seconds, tracked):
        err = np.abs(da - da_plain)
        return {"seconds": seconds, "speedup": t_plain / seconds,
                "tracked_fraction": float(tracked.mean()),
                "da_error_max_sigma": float(err.max()), "da_error_mean_sigma": float(err.mean()),
                "da_error_median_sigma": float(np.median(err)),
                "rays_exact": float(np.mean(err == 0.0))}

    def predict():
        p, _ = net.predict(features(s_test))
        return p

    if args.da_dump:
        # the scans' inputs and plain outcomes, for studying screening
        # strategies on the host (tracking is deterministic per particle)
        pt, lt_pred = net.predict(features(s_test))
        np.savez_compressed(args.da_dump, r=s_test.r, theta=s_test.theta,
                            delta_index=s_test.delta_index, lattice_index=s_test.lattice_index,
                            ray=ray, state=st_p, at_turn=at_p, p_survive=pt, logturn_pred=lt_pred,
                            x_test=features(s_test), seed_features_test=s_test.seed_features,
                            x_train=features(s_train), surv_train=surv, logturn_train=lt,
                            lattice_index_train=s_train.lattice_index, r_train=s_train.r,
                            ray_train=s_train.ray_index(), seed_features_train=s_train.seed_features,
                            turns=turns, t_plain=t_plain)

    # (1) the network's band alone, one pass
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    p = predict()
    track, audit = sg.screen_rays(p, s_test.r, ray, args.da_lo, args.da_hi, 0.0)
    st_s, at_s, _ = sc.run_scan(bt_test, s_test, turns, select=track, device=dev)
    t_band = time.perf_counter() - t0
    surv_band = sg.ray_outcome(p, s_test.r, ray, track, sg.targets(st_s, at_s, turns)[0] > 0,
                               hi=args.da_hi, audit_mask=audit)
    band = stats(sc.da_table(s_test, surv_band, n_seeds), t_band, track)

    # (2) sentinels + band, then brackets
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    p = predict()
    res = sc.screened_da_scan(bt_test, s_test, turns, p_survive=p, stride=args.da_stride,
                              lo=args.da_lo, hi=args.da_hi, band_stride=args.da_band_stride,
                              device=dev)
    t_net = time.perf_counter() - t0
    two_pass = stats(res.da, t_net, res.tracked)
    two_pass["pass_seconds"] = res.seconds
    two_pass["pass_fractions"] = [float(res.pass1.mean()), float(res.pass2.mean())]

    # (3) the same without the network
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    res0 = sc.screened_da_scan(bt_test, s_test, turns, p_survive=None, stride=args.da_stride,
                               device=dev)
    t_nonet = time.perf_counter() - t0
    no_net = stats(res0.da, t_nonet, res0.tracked)
    no_net["pass_seconds"] = res0.seconds
    no_net["pass_fractions"] = [float(res0.pass1.mean()), float(res0.pass2.mean())]

    # (4) three passes without the network: coarse sentinels, a fine window
    # below each ray's first coarse loss, brackets
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    res3 = sc.adaptive_da_scan(bt_test, s_test, turns, coarse=args.da_coarse, fine=args.da_stride,
                               window=args.da_window, device=dev)
    t_adapt = time.perf_counter() - t0
    adaptive = stats(res3.da, t_adapt, res3.tracked)
    adaptive["pass_seconds"] = res3.seconds
    adaptive["pass_fractions"] = [float(res3.pass1.mean()), float(res3.pass2.mean()),
                                  float(res3.pass3.mean())]

    # (5) two passes with the fine window placed by the network: coarse
    # sentinels + fine sentinels around the predicted boundary, brackets
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    p = predict()
    res5 = sc.guided_da_scan(bt_test, s_test, turns, p, coarse=args.da_coarse, fine=args.da_stride,
                             below=args.da_guide_below, above=args.da_guide_above, device=dev)
    t_guided = time.perf_counter() - t0
    guided = stats(res5.da, t_guided, res5.tracked)
    guided["pass_seconds"] = res5.seconds
    guided["pass_fractions"] = [float(res5.pass1.mean()), float(res5.pass2.mean())]

    # (6) the same two passes without the network: coarse sentinels, then
    # brackets of one coarse step
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    res6 = sc.guided_da_scan(bt_test, s_test, turns, np.ones(s_test.n), coarse=args.da_coarse,
                             fine=args.da_stride, below=0.0, above=-1.0, device=dev)
    t_blind = time.perf_counter() - t0
    blind = stats(res6.da, t_blind, res6.tracked)
    blind["pass_seconds"] = res6.seconds
    blind["pass_fractions"] = [float(res6.pass1.mean()), float(res6.pass2.mean())]

    # the network's own DA per ray (its predicted boundary) against plain tracking
    pred = sc.predicted_boundary(p, s_test)
    da_net = sc.da_table(s_test, s_test.r < pred, n_seeds)
    net_err = np.abs(da_net - da_plain)

    grid_step = float(np.max(np.diff(np.unique(s_test.r))))
    out = {"metric": "DA-scan time, surrogate vs plain", "value": t_plain / t_band,
           "unit": "x (plain time / screened time)", "higher_is_better": True, "n_gpus": 1,
           "dtype": "f64 tracking, bf16/f32 network", "data": "synthetic",
           "config": {"workload": "thick LHC-like ring seeds (6993 elements), polar grid "
                                  f"0-{args.da_rmax:g} sigma x 11 angles x delta in {{0, 2.7e-4}}",
                      "turns": turns, "screen_band": [args.da_lo, args.da_hi],
                      "sentinel_stride": args.da_stride, "band_stride": args.da_band_stride,
                      "adaptive_coarse_stride": args.da_coarse, "adaptive_window_sigma": args.da_window,
                      "guided_window_sigma": [args.da_guide_below, args.da_guide_above],
                      "train_seeds": len(train_lines), "test_seeds": n_seeds,
                      "train_particles": int(s_train.n), "test_particles": int(s_test.n),
                      "radial_step_sigma": grid_step, "arith": args.arith,
                      "features": args.da_features},
           "plain_s": t_plain, "screened_s": t_band,
           "da_error_sigma": band["da_error_max_sigma"],
           "da_error_mean_sigma": band["da_error_mean_sigma"],
           "tracked_fraction": band["tracked_fraction"],
           "methods": {"learned_band_one_pass": band, "sentinels_band_bracket": two_pass,
                       "sentinels_bracket_no_network": no_net,
                       "adaptive_three_pass_no_network": adaptive,
                       "guided_two_pass": guided, "coarse_bracket_two_pass_no_network": blind},
           "network_da_error_mean_sigma": float(net_err.mean()),
           "network_da_error_median_sigma": float(np.median(net_err)),
           "network_da_within_window": float(np.mean((da_net - da_plain <= args.da_guide_below)
                                                     & (da_plain - da_net <= args.da_guide_above))),
           "da_plain_mean_sigma": float(da_plain.mean()),
           "misclassification_all": float(np.mean((p >= 0.5) != surv_plain)),
           "train_scan_s": t_train_scan, "fit_s": t_fit, "fit_loss": [hist[0], hist[-1]],
           "fit_loss_curve": [float(h) for h in hist],
           "setup_s": t_setup}
    print(json.dumps(out))


def run_batch_scan(args):
    """Batched DA scan of many error seeds with uneven particle counts
    (uniform in [--batch-min, --batch-max] per seed) on the thick ring:
    all seeds in one persistent launch (BatchTracker, per-particle lattice
    index, autotuned launch shape) against the reference's way, one
    tracker and one tracking call per seed, run one after the other with
    the same launch shape. Both give bit-identical state / at_turn /
    at_element (checked). value = particle-turns/s of the batched scan."""
    import torch
    import xtrack_gb300 as xt
    from xtrack_gb300 import scan as sc
    from xtrack_gb300 import tuning as tu
    from xtrack_gb300 import workloads

    rank, world, local = _dist()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    turns = args.batch_turns
    rng = np.random.default_rng(11)
    n_seeds = args.batch_seeds
    counts = rng.integers(args.batch_min, args.batch_max + 1, size=n_seeds)
    lines = [workloads.thick_ring(seed=300 + s) for s in range(n_seeds)]
    t0 = time.perf_counter()
    scan = sc.build_scan(lines, counts, r_max=args.da_rmax, device=dev)
    t_setup = time.perf_counter() - t0
    bt = xt.BatchTracker(lines, device=dev, arith=args.arith)
    # the autotuner times its candidates on an evenly thinned copy of the
    # scan (every k-th particle, all seeds kept) when the scan is large
    k = max(1, int(np.ceil(scan.n / args.batch_tune_max)))
    sub = np.zeros(scan.n, dtype=bool)
    sub[::k] = True
    probe = sc.make_particles(scan, select=sub, device=dev)
    t0 = time.perf_counter()
    tuning, rep = tu.autotune(bt, probe, turns, probe_turns=2, repeats=1,
                              lattice_index=scan.lattice_index[sub])
    t_tune = time.perf_counter() - t0
    del probe

    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    st_b, at_b, ae_b = sc.run_scan(bt, scan, turns, device=dev)
    t_batch = time.perf_counter() - t0

    trackers = [ln.build_tracker(device=dev, arith=args.arith) for ln in lines]
    for tr in trackers:
        tr.set_tuning(**tuning)
    parts = [sc.make_particles(scan, select=scan.lattice_index == s, device=dev)
             for s in range(n_seeds)]
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for tr, p in zip(trackers, parts):
        tr._track(p, num_turns=turns)
    torch.cuda.synchronize(dev)
    t_seq = time.perf_counter() - t0
    same = True
    for s, p in enumerate(parts):
        sel = scan.lattice_index == s
        same &= bool(np.array_equal(p.state.cpu().numpy(), st_b[sel]) and
                     np.array_equal(p.at_turn.cpu().numpy(), at_b[sel]) and
                     np.array_equal(p.at_element.cpu().numpy(), ae_b[sel]))
    pt = float(np.sum(at_b))
    out = {"metric": "batched DA-scan particle-turns/s (60 seeds, one launch)",
           "value": pt / t_batch, "unit": "particle-turns/s", "higher_is_better": True,
           "n_gpus": 1, "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"{n_seeds} seeds of the thick ring (6993 elements), "
                                  f"{args.batch_min}-{args.batch_max} particles per seed on a "
                                  f"polar grid 0-{args.da_rmax:g} sigma x 11 angles x 2 deltas",
                      "turns": turns, "particles": int(scan.n), "arith": args.arith,
                      "seed_particles_min": int(counts.min()), "seed_particles_max": int(counts.max())},
           "batched_s": t_batch, "per_seed_s": t_seq, "speedup_vs_per_seed": t_seq / t_batch,
           "per_seed_particle_turns_per_s": pt / t_seq, "particle_turns": pt,
           "results_identical": same, "tuning": tuning, "autotune_s": t_tune,
           "autotune_candidates": len(rep.get("timings", [])), "autotune_particles": int(sub.sum()),
           "setup_s": t_setup}
    print(json.dumps(out))
    if not same:
        raise SystemExit("batched and per-seed results differ")


def run_monitor_hbm(args):
    """The turn-by-turn monitor's HBM regime: --particles protons (default
    3.2e7, the monitor-stress configuration's beam) through a one-drift
    line for --monitor-turns turns in one tracking call, with a
    ParticlesMonitor recording x, px, y, py, zeta, delta of every particle
    every turn in the reference's record layout (n_turns*(id - id0) +
    turn). Per call the push reads and writes the particle arrays once and
    writes 48 B per particle-turn of records: value = bytes moved / CUDA-event
    time of the call, against the measured HBM copy bandwidth."""
    import torch
    import xtrack_gb300 as xt
    from xtrack_gb300.monitors import ParticlesMonitor

    rank, world, local = _dist()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = args.particles if args.particles != 1_000_000 else 32_000_000
    turns = args.monitor_turns
    line = xt.Line(elements=[xt.Drift(length=1.0)])
    rng = np.random.default_rng(5)
    p = xt.Particles(device=dev, p0c=7e12, x=rng.normal(0, 1e-3, n), px=rng.normal(0, 1e-5, n),
                     y=rng.normal(0, 1e-3, n), py=rng.normal(0, 1e-5, n))
    line.build_tracker(device=dev, arith=args.arith)
    fields = ("x", "px", "y", "py", "zeta", "delta")
    times = []
    for rep in range(args.warmup + args.steps):
        mon = ParticlesMonitor(start_at_turn=rep * turns, stop_at_turn=(rep + 1) * turns,
                               num_particles=n, fields=fields, device=dev, auto_to_numpy=False)
        torch.cuda.synchronize(dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        line.track(p, num_turns=turns, turn_by_turn_monitor=mon)
        e1.record()
        torch.cuda.synchronize(dev)
        if rep >= args.warmup:
            times.append(e0.elapsed_time(e1) * 1e-3)
        del mon
    t = min(times)
    mon_bytes = n * turns * 48
    io_bytes = n * 152
    peak = _measured_hbm_gbs()
    gbs = (mon_bytes + io_bytes) / t / 1e9
    out = {"metric": "turn-by-turn monitor write bandwidth (GB/s)", "value": gbs, "unit": "GB/s",
           "higher_is_better": True, "n_gpus": 1, "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"{n:.3g} protons, one-drift line, {turns} turns per call, "
                                  "monitor of every particle (6 coordinates per turn)",
                      "arith": args.arith, "particles": n, "turns_per_call": turns},
           "seconds_per_call": t, "monitor_bytes_per_call": mon_bytes,
           "particle_io_bytes_per_call": io_bytes,
           "hbm_peak_gbs": peak, "frac": (gbs / peak) if peak else None,
           "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy, read+write)" if peak else None}
    print(json.dumps(out))


def run_mlp(args):
    """The surrogate's tensor-core contraction (tcgen05, TMA-staged BF16
    operands, FP32 accumulation in tensor memory): the forward product of
    one hidden layer, X[M, 256] W[256, 256]^T + b -> GELU, at M =
    --mlp-rows (2^20) rows, storing the BF16 activation only (the inference layer) and the
    FP32 pre-activation as well (the training layer); then one training
    step (forward, loss, backward, Adam) of the DA network at batch 4096
    and inference over 2^20 samples. Each timing is the best of --steps
    CUDA-event runs after --warmup. The layer moves 2*M*256*(2 + out) bytes
    against 2*M*256*256 FLOPs, so at this width the product is bound by
    HBM: the line reports both fractions against the measured peaks."""
    import ctypes

    import torch
    from xtrack_gb300 import _abi
    from xtrack_gb300 import surrogate as sg

    rank, world, local = _dist()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _abi.load_library()
    M, K, N = args.mlp_rows, 256, 256
    g = torch.Generator(device="cpu").manual_seed(3)
    X = torch.randn(M, K, generator=g).to(torch.bfloat16).to(dev)
    W = (torch.randn(N, K, generator=g) / 16).to(torch.bfloat16).to(dev)
    b = torch.randn(N, generator=g).to(dev)
    Z = torch.empty(M, N, device=dev)
    Y = torch.empty(M, N, dtype=torch.bfloat16, device=dev)
    stream = torch.cuda.current_stream(dev)
    st = ctypes.c_void_p(stream.cuda_stream)

    def best(fn):
        for _ in range(args.warmup):
            fn()
        ts = []
        for _ in range(args.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize(dev)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            ts.append(e0.elapsed_time(e1) * 1e-3)
        return min(ts)

    def layer(store_z):
        _abi.check_mlp(lib.xtg_mlp_gemm(sg._ptr(X), K, 1, sg._ptr(W), K, 1, M, N, K, sg._ptr(b),
                                        _abi.MLP_ACT_GELU, sg._ptr(Z) if store_z else None, N,
                                        sg._ptr(Y), N, None, 0, 0, st), lib)

    flops = 2.0 * M * N * K
    t_y = best(lambda: layer(False))
    t_zy = best(lambda: layer(True))
    bytes_y = M * K * 2 + N * K * 2 + M * N * 2
    bytes_zy = bytes_y + M * N * 4
    ref = torch.nn.functional.gelu(X[:4096].float() @ W.float().t() + b)
    layer(False)
    torch.cuda.synchronize(dev)
    err = float((Y[:4096].float() - ref).abs().max() / ref.abs().max())

    net = sg.SurvivalMLP(n_in=sg.N_DA_FEATURES + sg.N_SEED_FEATURES, seed=0, device=dev)
    rng = np.random.default_rng(1)
    Xs = rng.normal(size=(1 << 20, net.n_in)).astype(np.float32)
    net.set_normalisation(Xs)
    X16 = net.prepare_input(Xs)
    xb = X16[:4096].contiguous()
    sv = torch.from_numpy((rng.random(4096) < 0.5).astype(np.float32)).to(dev)
    lt = torch.from_numpy(rng.random(4096).astype(np.float32)).to(dev)

    def train_step():
        out = net.forward(xb, keep=True)
        _, dout, dout16 = net.loss_and_grad(out, sv, lt)
        net.backward(dout, dout16)
        net.adam_step(lr=1e-4)

    t_step = best(train_step)
    t_inf = best(lambda: net.forward(X16))
    _abi.check_mlp(lib.xtg_mlp_device_status(), lib)
    dims = net.dims
    flops_sample = 2.0 * sum(a * b_ for a, b_ in zip(dims[:-1], dims[1:]))
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    tf_peak = peaks.get("bf16_tflops")
    hbm = peaks.get("hbm_gbs")
    tf = flops / t_y / 1e12
    gbs_y = bytes_y / t_y / 1e9
    gbs_zy = bytes_zy / t_zy / 1e9
    out = {"metric": "surrogate contraction throughput (tcgen05, bf16 x bf16 -> f32)",
           "value": tf, "unit": "TFLOP/s", "higher_is_better": True, "n_gpus": 1,
           "dtype": "bf16", "data": "synthetic",
           "config": {"workload": f"hidden layer X[{M}, {K}] W[{N}, {K}]^T + b, GELU, bf16 store; "
                                  f"DA network {dims} training step at batch 4096 and inference "
                                  f"over {1 << 20} samples"},
           "layer_seconds": {"bf16_store": t_y, "f32_and_bf16_store": t_zy},
           "layer_gbs": {"bf16_store": gbs_y, "f32_and_bf16_store": gbs_zy},
           "roofline": {"bound": "hbm", "achieved": gbs_y, "peak": hbm, "unit": "GB/s",
                        "frac": (gbs_y / hbm) if hbm else None,
                        "tensor_frac": (tf / tf_peak) if tf_peak else None,
                        "peak_source": "MEASURED_PEAKS.json (hbm_gbs, bf16_tflops)"},
           "rel_error_vs_torch_fp32": err,
           "train_step_ms": t_step * 1e3,
           "inference_samples_per_s": (1 << 20) / t_inf,
           "inference_tflops": flops_sample * (1 << 20) / t_inf / 1e12}
    print(json.dumps(out))


def _measured_hbm_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(p))["hbm_gbs"])
    except Exception:
        return None


def run_toy_ring(args):
    """The toy thin ring (100 cells of drift, thin multipole, drift, thin
    multipole, LimitEllipse; one cavity; protons at 450 GeV): 10,000
    particles x 1000 turns through Line.track on the GPU (exact and fast
    arithmetic, CUDA-synchronised wall time of the whole call), and the
    oracle's port of the reference OpenMP path on all host cores over the
    same particles for --toy-cpu-turns turns. One JSON line."""
    import torch
    from xtrack_gb300 import workloads
    import pyoracle

    rank, world, local = _dist()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n, turns = args.toy_particles, args.toy_turns
    line = workloads.toy_ring()
    p0c = float(line.particle_ref.p0c[0])
    out = {"metric": "toy ring particle-turns/s", "unit": "particle-turns/s",
           "higher_is_better": True, "n_gpus": 1, "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"toy thin ring ({len(line.element_names)} elements), "
                                  f"{n} protons 450 GeV x {turns} turns", "particles": n,
                      "turns": turns}}
    for arith in ("exact", "fast"):
        tr = line.build_tracker(device=dev, arith=arith)
        warm = workloads.gaussian_beam(n, p0c, seed=1, device=dev)
        tr._track(warm, num_turns=10)
        p = workloads.gaussian_beam(n, p0c, seed=2, device=dev)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        tr._track(p, num_turns=turns)
        torch.cuda.synchronize(dev)
        dt = time.perf_counter() - t0
        pt = float(p.at_turn.sum().item())
        out[arith] = {"particle_turns_per_s": pt / dt, "seconds": dt,
                      "alive": int((p.state > 0).sum().item())}
    out["value"] = out["fast"]["particle_turns_per_s"]
    pyoracle.ensure_built(with_ref=False)
    recs = line._element_records()
    cpu_turns = min(turns, args.toy_cpu_turns)
    beam = pyoracle.host_arrays(workloads.gaussian_beam(n, p0c, seed=2, device="cpu").to_numpy())
    t0 = time.perf_counter()
    pyoracle.track(recs, beam, num_turns=cpu_turns, line_length=line.get_length(),
                   mode=pyoracle.MODE_OPENMP)
    dt = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": float(np.sum(beam["at_turn"])) / dt, "unit": "particle-turns/s",
                           "cores": pyoracle.max_threads(), "kind": "port",
                           "sample": f"{n} particles x {cpu_turns} turns ({dt:.1f} s, OpenMP)"}
    print(json.dumps(out))


# name: (fixture under tests/golden, description, beam sigmas of the bench's synthetic beam)
REAL_LATTICES = {
    "sps": (os.path.join("sps", "sps_thin_128p_20t.npz"), "thin SPS line",
            {"x": 6e-3, "px": 1.5e-4, "y": 5e-3, "py": 1.5e-4, "zeta": 0.05, "delta": 5e-4}),
    "psb": (os.path.join("psb", "psb_injection_128p_20t.npz"), "PS Booster injection line",
            {"x": 2e-3, "px": 2e-4, "y": 2e-3, "py": 2e-4, "zeta": 1.0, "delta": 1e-3}),
    "clic_dr": (os.path.join("clic_dr", "clic_dr_64p_5t.npz"), "CLIC damping ring",
                {"x": 5e-5, "px": 5e-6, "y": 1e-5, "py": 1e-6, "zeta": 1e-3, "delta": 1e-3}),
}


def run_real_lattice(args):
    """A real machine from the reference's test data, as packed records of
    a committed parity fixture (tests/golden): the thin SPS line (8200
    elements: drifts, thin multipoles, 1488 DipoleEdges, 1698 apertures,
    cavities), the PS Booster injection line (604 elements) or the CLIC
    damping ring (36954 elements, electrons). --particles particles around
    the fixture's particle with a Gaussian spread (on the SPS some are lost
    on the apertures), one turn per step, through the C-ABI
    (xtg_lattice_create / xtg_track) with CUDA events; the oracle's port of
    the reference OpenMP path on the host cores as the CPU baseline."""
    import ctypes

    import torch
    import xtrack_gb300 as xt
    from xtrack_gb300 import _abi
    import pyoracle

    rank, world, local = _dist()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    fixture, what, sig = REAL_LATTICES[args.lattice]
    d = np.load(os.path.join(ROOT, "tests", "golden", fixture))
    meta = json.loads(str(d["meta"]))
    recs = np.ascontiguousarray(d["records"])
    n_el, L = len(recs), float(meta["line_length"])
    p0 = {k[3:]: d[k] for k in d.files if k.startswith("in_")}
    rng = np.random.default_rng(16)
    base = {k: float(np.mean(p0[k])) for k in sig}

    def beam(n, device):
        kw = {k: base[k] + rng.normal(0.0, s, n) for k, s in sig.items()}
        return xt.Particles(device=device, p0c=float(p0["p0c"][0]), mass0=meta["mass0"],
                            q0=meta["q0"], **kw)

    lib = _abi.load_library()
    cfg = _abi.XtgConfig()
    cfg.has_global_xy_limit = 1
    cfg.global_xy_limit = 1.0
    cfg.arith = _abi.ARITH_FAST if args.arith == "fast" else _abi.ARITH_EXACT
    h = ctypes.c_void_p()
    _abi.check(lib.xtg_lattice_create(recs.ctypes.data_as(ctypes.c_void_p), n_el,
                                      ctypes.byref(cfg), ctypes.byref(h)), lib)
    nn, fl = ctypes.c_int64(), ctypes.c_double()
    _abi.check(lib.xtg_lattice_info(h, ctypes.byref(nn), 0, n_el, ctypes.byref(fl)), lib)
    flops_pt = fl.value
    p = beam(args.particles, dev)
    ps = p._xtg_struct()
    stream = torch.cuda.current_stream(dev)

    def step():
        _abi.check(lib.xtg_track(h, ctypes.byref(ps), 1, 0, n_el, 1, 1, 0, n_el, L, None, 0,
                                 ctypes.c_void_p(stream.cuda_stream)), lib)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    alive0 = int((p.state > 0).sum())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        e1.synchronize()
    _abi.check(lib.xtg_device_status(h), lib)
    ms = e0.elapsed_time(e1)
    alive1 = int((p.state > 0).sum())
    value = alive1 * args.steps / (ms * 1e-3)
    peak = ctypes.c_double()
    _abi.check(lib.xtg_measure_fp64_peak(ctypes.byref(peak)), lib)
    lib.xtg_lattice_destroy(h)
    # CPU: the oracle port on all host cores, one turn of a sample
    pyoracle.ensure_built(with_ref=False)
    n_cpu = max(1000, int(20000 * 8200 / n_el) // 1000 * 1000)
    arrs = pyoracle.host_arrays(beam(n_cpu, "cpu").to_numpy())
    t0 = time.perf_counter()
    pyoracle.track(recs, arrs, line_length=L, num_turns=1, q0=meta["q0"], mass0=meta["mass0"],
                   mode=pyoracle.MODE_OPENMP)
    dt = time.perf_counter() - t0
    cpu = float(np.sum(arrs["state"] > 0)) / dt
    achieved = value * flops_pt / 1e12
    out = {"metric": f"real-lattice particle-turns/s ({what})", "value": value,
           "unit": "particle-turns/s", "higher_is_better": True, "n_gpus": 1, "dtype": "f64",
           "data": "synthetic beam on a real lattice", "arith": args.arith,
           "config": {"workload": f"{what} of the reference's test data ({n_el} elements)",
                      "particles": args.particles, "turns_per_step": 1},
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
           "alive_before": alive0, "alive_after": alive1,
           "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak.value / 1e12,
                        "unit": "TFLOP/s", "frac": achieved / (peak.value / 1e12),
                        "flops_per_particle_turn": flops_pt},
           "cpu_baseline": {"value": cpu, "unit": "particle-turns/s",
                            "cores": pyoracle.max_threads(), "kind": "port",
                            "sample": f"{n_cpu} particles x 1 turn ({dt:.2f} s, OpenMP)"},
           "clocks": clk.summary()}
    print(json.dumps(out))


def run_sliced_ring(args):
    """The thick ring in its thin-sliced form: every magnet of the
    6993-element thick ring sliced with Teapot(8) by
    Line.slice_thick_elements (43,793 elements: thin kicks, drift slices,
    entry and exit edges, apertures, the cavity), 10^6 protons, one turn
    per step through the C-ABI (xtg_lattice_create / xtg_track) with CUDA
    events, in the --arith arithmetic; the oracle's port of the reference
    OpenMP path on the host cores as the CPU baseline."""
    import ctypes

    import torch
    import xtrack_gb300 as xt
    from xtrack_gb300 import _abi, workloads
    import pyoracle

    rank, world, local = _dist()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    line = workloads.thick_ring()
    line.slice_thick_elements([xt.Strategy(slicing=xt.Teapot(8))])
    recs = np.ascontiguousarray(line._element_records())
    n_el, L = len(recs), float(line.get_length())
    lib = _abi.load_library()
    cfg = _abi.XtgConfig()
    cfg.has_global_xy_limit = 1
    cfg.global_xy_limit = 1.0
    cfg.arith = _abi.ARITH_FAST if args.arith == "fast" else _abi.ARITH_EXACT
    h = ctypes.c_void_p()
    _abi.check(lib.xtg_lattice_create(recs.ctypes.data_as(ctypes.c_void_p), n_el,
                                      ctypes.byref(cfg), ctypes.byref(h)), lib)
    nn, fl = ctypes.c_int64(), ctypes.c_double()
    _abi.check(lib.xtg_lattice_info(h, ctypes.byref(nn), 0, n_el, ctypes.byref(fl)), lib)
    flops_pt = fl.value
    beam = workloads.gaussian_beam(args.particles, 7e12, device=dev, seed=7)
    ps = beam._xtg_struct()
    stream = torch.cuda.current_stream(dev)

    def step():
        _abi.check(lib.xtg_track(h, ctypes.byref(ps), 1, 0, n_el, 1, 1, 0, n_el, L, None, 0,
                                 ctypes.c_void_p(stream.cuda_stream)), lib)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    alive0 = int((beam.state > 0).sum())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        e1.synchronize()
    _abi.check(lib.xtg_device_status(h), lib)
    ms = e0.elapsed_time(e1)
    alive1 = int((beam.state > 0).sum())
    value = alive1 * args.steps / (ms * 1e-3)
    peak = ctypes.c_double()
    _abi.check(lib.xtg_measure_fp64_peak(ctypes.byref(peak)), lib)
    lib.xtg_lattice_destroy(h)
    out = {"metric": "FP64 particle-turns/s on the thick ring sliced thin (Teapot(8))",
           "value": value, "unit": "particle-turns/s", "higher_is_better": True, "n_gpus": 1,
           "dtype": "f64", "data": "synthetic", "arith": args.arith,
           "config": {"workload": f"thick LHC-like ring sliced with Teapot(8): {n_el} elements, "
                                  f"{args.particles:g} protons 7 TeV, 1 turn per step",
                      "particles": args.particles, "elements": n_el, "turns_per_step": 1},
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
           "alive_before": alive0, "alive_after": alive1,
           "roofline": {"bound": "fp64", "achieved": value * flops_pt / 1e12,
                        "peak": peak.value / 1e12, "unit": "TFLOP/s",
                        "frac": value * flops_pt / peak.value, "flops_per_particle_turn": flops_pt},
           "clocks": clk.summary()}
    if not args.no_cpu_baseline:
        pyoracle.ensure_built(with_ref=False)
        n_cpu = 20000
        arrs = pyoracle.host_arrays(workloads.gaussian_beam(n_cpu, 7e12, device="cpu", seed=8).to_numpy())
        t0 = time.perf_counter()
        pyoracle.track(recs, arrs, line_length=L, num_turns=1, mode=pyoracle.MODE_OPENMP)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": float(np.sum(arrs["state"] > 0)) / dt,
                               "unit": "particle-turns/s", "cores": pyoracle.max_threads(),
                               "kind": "port",
                               "sample": f"{n_cpu} particles x 1 turn ({dt:.2f} s, OpenMP)"}
    print(json.dumps(out))


def run_turn_latency(args):
    """Milliseconds per turn of the thick ring for particle counts from a
    fraction of one resident wave (8 warps per SM) to four waves, for
    several block sizes: where a small tracked set (a screened scan) stops
    being latency-bound. One JSON line per (count, block, chunk)."""
    import torch
    import xtrack_gb300 as xt
    from xtrack_gb300 import workloads

    rank, world, local = _dist()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    line = workloads.thick_ring(seed=1)
    tr = line.build_tracker(device=dev, arith=args.arith)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    rng = np.random.default_rng(0)
    for per_sm in (64, 128, 256, 512, 1024):
        n = per_sm * sms
        for block, chunk in ((32, 12288), (64, 16384), (256, 49152)):
            tr.set_tuning(block_size=block, compact_every=10, chunk_bytes=chunk, use_graph=0)
            best = None
            for _ in range(2):
                p = xt.Particles(device=dev, p0c=7e12, mass0=workloads.PROTON_MASS_EV,
                                 x=rng.normal(0, 1e-4, n), y=rng.normal(0, 1e-4, n))
                torch.cuda.synchronize(dev)
                t0 = time.perf_counter()
                tr._track(p, num_turns=10)
                torch.cuda.synchronize(dev)
                t = (time.perf_counter() - t0) / 10
                best = t if best is None else min(best, t)
            alive = int((p.state > 0).sum())
            print(json.dumps({"workload": "turn_latency", "particles": n, "per_sm": per_sm,
                              "block": block, "chunk_bytes": chunk, "ms_per_turn": 1e3 * best,
                              "alive": alive, "arith": args.arith}), flush=True)


def _traffic(arith):
    """DRAM bytes per launch of the track kernel in arithmetic `arith` from
    the committed ncu summary, when present."""
    p = os.path.join(ROOT, "profiles", "track_kernel_traffic.json")
    if os.path.exists(p):
        try:
            return json.load(open(p)).get(arith, {}).get("dram_bytes_per_launch")
        except Exception:
            return None
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--arith", default="exact", choices=["exact", "fast"])
    ap.add_argument("--no-alt", action="store_true",
                    help="skip the timing of the other arithmetic mode")
    ap.add_argument("--particles", type=int, default=1_000_000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--block-size", dest="block_size", type=int, default=None)
    ap.add_argument("--compact-every", dest="compact_every", type=int, default=None)
    ap.add_argument("--chunk-bytes", dest="chunk_bytes", type=int, default=None)
    ap.add_argument("--use-graph", dest="use_graph", type=int, default=None)
    ap.add_argument("--monitor-turns", dest="monitor_turns", type=int, default=8,
                    help="turns per call of the monitor_hbm workload")
    ap.add_argument("--monitor-first", dest="monitor_first", type=int, default=0,
                    help="record 6 coordinates per turn of the first N particles")
    ap.add_argument("--workload", default="thick_ring",
                    choices=["thick_ring", "da_screen", "turn_latency", "batch_scan", "toy_ring",
                             "real_lattice", "monitor_hbm", "mlp", "sliced_ring"])
    ap.add_argument("--lattice", default="sps", choices=sorted(REAL_LATTICES),
                    help="real_lattice workload: which fixture's line")
    ap.add_argument("--toy-particles", dest="toy_particles", type=int, default=10000)
    ap.add_argument("--toy-turns", dest="toy_turns", type=int, default=1000)
    ap.add_argument("--toy-cpu-turns", dest="toy_cpu_turns", type=int, default=1000)
    ap.add_argument("--batch-seeds", dest="batch_seeds", type=int, default=60)
    ap.add_argument("--batch-min", dest="batch_min", type=int, default=1000)
    ap.add_argument("--batch-max", dest="batch_max", type=int, default=20000)
    ap.add_argument("--batch-turns", dest="batch_turns", type=int, default=20)
    ap.add_argument("--batch-tune-max", dest="batch_tune_max", type=int, default=500000,
                    help="largest particle count the batch autotuner times candidates on")
    ap.add_argument("--da-turns", dest="da_turns", type=int, default=100)
    ap.add_argument("--da-train-particles", dest="da_train_particles", type=int, default=3200)
    ap.add_argument("--da-lo", dest="da_lo", type=float, default=0.02)
    ap.add_argument("--da-hi", dest="da_hi", type=float, default=0.98)
    ap.add_argument("--da-stride", dest="da_stride", type=int, default=34,
                    help="sentinel spacing of the screened DA scan, in grid amplitudes")
    ap.add_argument("--da-band-stride", dest="da_band_stride", type=int, default=4,
                    help="spacing of the tracked amplitudes inside the network's uncertain band")
    ap.add_argument("--da-rmax", dest="da_rmax", type=float, default=80.0,
                    help="largest amplitude of the grid (sigma); the synthetic ring at 7 TeV "
                         "keeps everything within 20 sigma, its DA lies near the aperture")
    ap.add_argument("--da-particles", dest="da_particles", type=int, default=100000,
                    help="mean particles per seed (uniform in [n/2, 3n/2])")
    ap.add_argument("--da-train-seeds", dest="da_train_seeds", type=int, default=120,
                    help="seeds of the training scan: the network carries a seed's DA to "
                         "unseen seeds only when it has seen many (24: 9.5 sigma off, 120: 0.94)")
    ap.add_argument("--da-test-seeds", dest="da_test_seeds", type=int, default=8)
    ap.add_argument("--da-epochs", dest="da_epochs", type=int, default=40)
    ap.add_argument("--da-features", dest="da_features", default="all",
                    choices=["all", "physics"],
                    help="all (the configuration's inputs): coordinates, tunes, orbit extremes, "
                         "the ray's linear aperture and the seed's 32 multipole-error features "
                         "(orders 0-10); physics: without the error features")
    ap.add_argument("--da-weight-decay", dest="da_weight_decay", type=float, default=0.0)
    ap.add_argument("--da-coarse", dest="da_coarse", type=int, default=272,
                    help="coarse sentinel stride of the three-pass scan")
    ap.add_argument("--da-window", dest="da_window", type=float, default=12.0,
                    help="sigma below the first coarse loss scanned at --da-stride")
    ap.add_argument("--mlp-rows", dest="mlp_rows", type=int, default=1 << 20,
                    help="rows of the mlp workload's layer product")
    ap.add_argument("--da-guide-below", dest="da_guide_below", type=float, default=6.0,
                    help="sigma below the network's predicted boundary scanned at --da-stride")
    ap.add_argument("--da-guide-above", dest="da_guide_above", type=float, default=2.0,
                    help="sigma above the network's predicted boundary scanned at --da-stride")
    ap.add_argument("--da-dump", dest="da_dump", default=None,
                    help="write the DA scans' inputs and plain outcomes to this .npz")
    args = ap.parse_args()
    if args.workload == "da_screen":
        run_da_screen(args)
    elif args.workload == "turn_latency":
        run_turn_latency(args)
    elif args.workload == "batch_scan":
        run_batch_scan(args)
    elif args.workload == "mlp":
        run_mlp(args)
    elif args.workload == "sliced_ring":
        run_sliced_ring(args)
    elif args.workload == "monitor_hbm":
        run_monitor_hbm(args)
    elif args.workload == "toy_ring":
        run_toy_ring(args)
    elif args.workload == "real_lattice":
        run_real_lattice(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

"""Benchmark: adaptive mixed-precision grain growth, 1024x1024, Q=8 (Fan-Chen,
gamma=1.5, kappa=2, L=1, dx=1, dt=0.05, periodic, eta_i ~ U[-1e-3, 1e-3]),
one bench step = one complete 10000-step run from the seeded initial state.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--sim-steps S]

Prints one JSON line.  `value` is Gcell-updates/s (cells x time steps / s)
with the initial state already in HBM; `e2e` is the same metric through the
C ABI from pinned host memory, including the host->device copy of the initial
fields and the device->host read of the final fields.  `plain_fp64` is the
plain-FP64 path on the same workload and `max_abs_err` the adaptive run's
error against it.  `roofline` covers the dominant update kernel, timed with
CUDA events on its launching stream during a profiled run.

--impl reference times the reference's FP64 update restated as a host
OpenMP loop (the oracle: the reference has no CPU implementation of its own)
on a bounded sample of the same workload, on all host cores.

Multi-GPU: the path does not shard (one grid per GPU); N ranks run N
independent replicas (weak scaling).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "graingrowth Fan-Chen Q=8 1024x1024 adaptive half/fp32/fp64, 10000 steps per run"
METRIC = "Gcell-updates/s"


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for k, n in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(n)
            except Exception:
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


TUNED = os.path.join(ROOT, "w3914777_gb300", "tuned", "graingrowth_1024_q8.json")


def load_tuned():
    """Monitor, thresholds and tile chosen by w3914777_gb300.autotune for this
    workload (file written by `python -m w3914777_gb300.autotune graingrowth`)."""
    try:
        with open(TUNED) as f:
            return json.load(f)["best"]
    except Exception:
        return None


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x, world, device="cpu"):
    """The largest of every rank's x (the job's time is its slowest rank's);
    x itself when there is one rank.  `device`: where the collective's tensor
    lives (the GPU for NCCL, the CPU for gloo)."""
    if world <= 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, cells, steps_per_run, runs, total_ms):
    """Whole-job Gcell-updates/s: every rank advances its own grid (weak
    scaling, replicas), timed by the slowest rank."""
    return world * cells * steps_per_run * runs / (total_ms * 1e-3) / 1e9


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def _oracle(threads):
    """The oracle's timed build (tests/oracle_bind.py, liboracle_fast.so: -O3,
    fused multiply-add, OpenMP over rows).  Loads no part of the product."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle_bind as ob
    return ob


def oracle_rate(nx, q, steps, threads):
    """The reference's FP64 grain-growth update (graingrowth/function.h:5-30,
    Q-general Fan-Chen form) as a host OpenMP loop: Gcell-updates/s over
    `steps` steps of the seeded nx^2 Q-field start."""
    ob = _oracle(threads)
    f0 = ob.gg_init_uniform(nx, nx, q, 1e-3, 1234)
    op = ob.gg_params(nx, nx, q=q, dx=1.0, dy=1.0, dt=0.05, mobil=1.0, grcoef=2.0, gamma=1.5)
    ob.gg_run(op, f0, 1, fast=True)  # warm the thread pool
    t0 = time.perf_counter()
    ob.gg_run(op, f0, steps, fast=True)
    dt = time.perf_counter() - t0
    return nx * nx * steps / dt / 1e9, dt


def oracle_rate_kobayashi(steps, threads, n=512):
    """The reference's FP64 Kobayashi update (snowflake/function.h:5-60) as a
    host OpenMP loop on the 512^2 plain-FP64 dendrite (zero flux, disc r^2 < 25
    at the centre, seeded noise 0.01): Gcell-updates/s over `steps` steps."""
    ob = _oracle(threads)
    phi, T = ob.kob_init_disc(n, n, n // 2, n // 2, 25.0)
    kp = ob.kob_params(n, n, bc=1, kappa=1.6, theta0=0.2, noise=0.01, seed=1234)
    ob.kob_run(kp, phi, T, 1, fast=True)
    t0 = time.perf_counter()
    ob.kob_run(kp, phi, T, steps, fast=True)
    dt = time.perf_counter() - t0
    return n * n * steps / dt / 1e9, dt


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    threads = cpu_threads()
    sample = args.ref_sample_steps
    rates = []
    for i in range(args.warmup + args.steps):
        r, dt = oracle_rate(1024, 8, sample, threads)
        if i >= args.warmup:
            rates.append((r, dt))
    value = statistics.median([r for r, _ in rates])
    ms = statistics.median([dt for _, dt in rates]) * 1e3
    kob, kdt = oracle_rate_kobayashi(args.ref_sample_steps, threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Gcell-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "nx": 1024, "ny": 1024, "Q": 8,
                   "sample": f"{sample} FP64 steps of the 1024^2 Q=8 grid per bench step (the rate of the "
                             "update; the GPU arm's run is 10000 adaptive steps)"},
        "cpu_baseline": {"value": value, "unit": "Gcell-updates/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} steps of 1024x1024 Q=8 FP64 (the oracle's restatement of "
                                   "graingrowth/function.h:5-30, built -O3 with fused multiply-add, "
                                   "OpenMP over rows)"},
        "e2e": {"value": value, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "configs": {"kobayashi_plain_fp64_512": {
            "value": kob, "unit": "Gcell-updates/s", "cores": threads,
            "sample": f"{args.ref_sample_steps} FP64 steps of the 512^2 zero-flux dendrite ({kdt:.2f} s)"}},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import w3914777_gb300 as w

    world, rank, local = dist_setup()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    S = args.sim_steps
    p = w.Params.preset("graingrowth", 0)
    tuned = load_tuned()
    if tuned:
        p = p.replace(**tuned["overrides"])
    if args.tile:
        p.tile = args.tile
    nf = p.num_fields
    cells = p.nx * p.ny
    host0 = torch.from_numpy(w.init_host(p, w.INIT_SEEDED)).pin_memory()
    dev0 = host0.to(dev)
    host_out = torch.empty_like(host0).pin_memory()
    stream = torch.cuda.Stream(device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # 256 MiB > L2

    sim = w.Simulation(p)
    sim.set_stream(stream.cuda_stream)

    def one_run_device():
        sim.set_fields_device(dev0.data_ptr())
        sim.run(S)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # warm-up (also captures the CUDA graph of a period)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            one_run_device()
    torch.cuda.synchronize()

    # ---- device-resident timing ----
    evs = []
    launches0 = sim.kernel_launches()
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_wall = time.perf_counter()
        with torch.cuda.stream(stream):
            for _ in range(args.steps):
                flush.zero_()
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                one_run_device()
                b.record(stream)
                evs.append((a, b))
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    barrier()
    # kernels the library launched in the timed region: the run loop's (steps,
    # classifications; counted by the library) plus, per run, the scatter of
    # the initial state and its classification
    timed_launches = sim.kernel_launches() - launches0 + 2 * args.steps
    ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = max_over_ranks(sum(ms), world, dev)
    value = job_rate(world, cells, S, args.steps, total_ms)
    stats = sim.stats()
    final_mixed = sim.fields()
    grains_mixed = sim.grains(threshold=0.5)

    # ---- end-to-end through the C ABI from pinned host memory ----
    e2e_ms = []
    for _ in range(max(1, args.steps)):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lib = w.lib()
        rc = lib.amps_set_fields(sim.h, ctypes.c_void_p(host0.data_ptr()), w.F64, 0)
        assert rc == 0
        sim.run(S)
        rc = lib.amps_get_fields(sim.h, ctypes.c_void_p(host_out.data_ptr()), w.F64, 0)
        assert rc == 0
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_total = max_over_ranks(sum(e2e_ms), world, dev)
    e2e = job_rate(world, cells, S, len(e2e_ms), e2e_total)
    bytes_io = nf * cells * 8

    # ---- profiled run: per-tier kernel durations for the roofline ----
    sim.set_fields_device(dev0.data_ptr())
    sim.set_profiling(True)
    sim.run(S)
    kms, klaunch, ktiles = sim.kernel_times()
    sim.set_profiling(False)
    T = p.tile
    tier_bytes = [2, 4, 8]
    # the grain-growth step is one fused kernel over every tier (index 3): its
    # algorithmic bytes per launch are the state each tier's tiles read and write
    algo_bytes = sum(ktiles[k] * T * T * nf * 2 * tier_bytes[k] for k in range(3))
    launches = max(klaunch[3], 1)
    per_launch_bytes = algo_bytes / launches
    per_launch_s = kms[3] * 1e-3 / launches
    achieved = per_launch_bytes / per_launch_s / 1e9 if per_launch_s > 0 else 0.0
    peak, peak_kind = peaks()
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            with open(tpath) as f:
                tr = json.load(f)
            # DRAM bytes per launch of the fused step kernel, from the ncu capture
            traffic = tr.get("gg_step_kernel_bytes_per_launch")
        except Exception:
            traffic = None
    # every step launch of the run: the fused all-tier kernel, and the staged
    # FP64 kernel for the warm-start period whose tiles are all FP64
    all_kernels = {"gg_step_kernel (fused, all tiers) + gg_step_f64_kernel (all-FP64 warm start)": {
                       "ms": kms[3], "launches": klaunch[3], "tile_steps_per_tier": ktiles[:3],
                       "us_per_launch": kms[3] * 1e3 / launches}}
    names = ["gg_step_kernel"]
    dom = 0

    # ---- plain FP64 path on the same workload + error of the adaptive run ----
    pf = p.replace(mode="purehigh", ref_order=0)
    with w.Simulation(pf) as s64:
        s64.set_stream(stream.cuda_stream)
        with torch.cuda.stream(stream):
            s64.set_fields_device(dev0.data_ptr())
            s64.run(10)
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            s64.set_fields_device(dev0.data_ptr())
            a.record(stream)
            s64.run(S)
            b.record(stream)
        torch.cuda.synchronize()
        fp64_ms = a.elapsed_time(b)
        final64 = s64.fields()
        grains64 = s64.grains(threshold=0.5)
        # per field: max-abs, RMS (L2 / sqrt(cells)) and the reference's error
        # metric, mean |a - b| over the grid (graingrowth/end2enderror.py:34)
        per_field = [s64.compare_all(f, final_mixed[f]) for f in range(nf)]
    mean_abs = max(e["mean_abs"] for e in per_field)
    plain = cells * S / (fp64_ms * 1e-3) / 1e9
    err = float(np.max(np.abs(final_mixed - final64)))

    # ---- all-FP32 path on the same workload (what the adaptive run is beside) ----
    p32 = p.replace(mode="purehigh", high_tier=w.TIER_FP32)
    with w.Simulation(p32) as s32:
        s32.set_stream(stream.cuda_stream)
        with torch.cuda.stream(stream):
            s32.set_fields_device(dev0.data_ptr())
            s32.run(2 * p.cadence)
            s32.set_fields_device(dev0.data_ptr())
            torch.cuda.synchronize()
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            s32.run(S)
            b.record(stream)
        torch.cuda.synchronize()
        fp32_ms = a.elapsed_time(b)
        err32 = float(np.max(np.abs(s32.fields() - final64)))
    all_fp32 = cells * S / (fp32_ms * 1e-3) / 1e9

    # ---- CPU baseline (oracle port on host cores), rank 0 only ----
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = cpu_threads()
        r, dt = oracle_rate(1024, 8, args.ref_sample_steps, threads)
        cpu = {"value": r, "unit": "Gcell-updates/s", "cores": threads, "kind": "port",
               "sample": f"{args.ref_sample_steps} FP64 steps of the 1024x1024 Q=8 grid ({dt:.1f} s; the "
                         "oracle's restatement of graingrowth/function.h:5-30 built -O3 with fused "
                         "multiply-add, OpenMP over rows)"}

    # tile-steps of one run (the profiled one); the warm start (first period,
    # every tile FP64, for the temporal and rate monitors) separated out
    ts = ktiles[:3]
    tot = max(sum(ts), 1)
    ntiles = (p.nx // T) * (p.ny // T)
    warm = p.cadence * ntiles if p.monitor != w.MONITOR_SPA else 0
    ts_after = [ts[0], ts[1], ts[2] - warm]
    tot_after = max(sum(ts_after), 1)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Gcell-updates/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f16+f32+f64 (per-tile adaptive)",
            "data": "synthetic (seeded uniform eta in [-1e-3,1e-3])",
            "config": {"workload": WORKLOAD, "nx": p.nx, "ny": p.ny, "Q": nf, "steps_per_run": S, "tile": T,
                       "monitor": {1: "spatial range", 2: "temporal change (snapshot)",
                                   3: "per-step change x cadence"}[p.monitor]
                                  + (", every cell" if p.monitor_samples else ", 4x4 lattice")
                                  + (", all fields" if p.monitor_field < 0 else f", field {p.monitor_field}")
                                  + f", every {p.cadence} steps",
                       "thresholds": [p.thr_lo, p.thr_hi], "tuned_by": "autotune" if tuned else "preset",
                       "l2": "flushed between runs (256 MiB write)",
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e, "unit": "Gcell-updates/s", "h2d_bytes_per_step": bytes_io,
                    "d2h_bytes_per_step": bytes_io, "ms_per_step": e2e_total / len(e2e_ms)},
            "plain_fp64": {"value": plain, "unit": "Gcell-updates/s", "ms_per_run": fp64_ms,
                           "arithmetic": "FP64 in fused multiply-add form (ref_order=0), equal to the oracle "
                                         "to <= 1e-12 relative (tests/test_gpu_parity.py)"},
            "all_fp32": {"value": all_fp32, "unit": "Gcell-updates/s", "ms_per_run": fp32_ms,
                         "max_abs_err_vs_fp64": err32},
            "speedup_vs_plain_fp64": value / plain,
            "max_abs_err_vs_fp64": err,
            "mean_abs_err_vs_fp64": mean_abs,
            "errors_vs_fp64_per_field": [{"field": f"eta{k + 1}", **per_field[k]} for k in range(nf)],
            "grains": {"adaptive": grains_mixed, "fp64": grains64,
                       "note": "connected regions of the dominant eta (>= 0.5), periodic"},
            "tier_mix": {"half": ts[0] / tot, "fp32": ts[1] / tot, "fp64": ts[2] / tot},
            "tier_mix_after_warm_start": {"half": ts_after[0] / tot_after, "fp32": ts_after[1] / tot_after,
                                          "fp64": ts_after[2] / tot_after,
                                          "note": f"the first {p.cadence} steps run every tile in FP64 "
                                                  "(the reference's warm start); the thresholds "
                                                  f"[{p.thr_lo:g}, {p.thr_hi:g}] promote no tile to FP64 "
                                                  "afterwards on this workload" if ts_after[2] == 0 else ""},
            "roofline": {"bound": "hbm", "l2_resident": True, "kernel": names[dom], "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                         "peak_source": f"{peak_kind} hbm_gbs",
                         "algorithmic_bytes_per_launch": per_launch_bytes,
                         "note": "algorithmic bytes = sum over tiers of tile-steps x tile^2 cells x Q fields x "
                                 "(read+write) x tier bytes; per launch = averaged over every step launch of "
                                 "the run (monitor steps and the FP64 warm start included); the 1024^2 state "
                                 "(16-64 MiB) stays L2-resident within a run"},
            "kernels": all_kernels,
            "gpu_launches": timed_launches,
            "clocks": clk.summary(),
            "wall_s_timed_region": t_wall,
        }
        if cpu:
            line["cpu_baseline"] = cpu
        if world == 1 and not args.no_hbm:
            line["roofline_hbm"] = run_roofline_hbm(p, peak, peak_kind)
        # single-GPU evidence: measured at N=1 only
        if world == 1 and not args.no_adjoint:
            line["adjoint"] = run_adjoint()
            line["adjoint"]["graingrowth"] = run_adjoint_gg()
        if world == 1 and not args.no_ensemble:
            line["ensemble"] = run_ensemble()
        if world == 1 and not args.no_configs:
            line["configs"] = run_configs()
        if world == 1 and not args.no_refcuda:
            line["reference_cuda"] = run_reference_cuda()
        print(json.dumps(line), flush=True)
    sim.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def run_reference_cuda(steps=2000):
    """The reference's own CUDA kernels on this GPU beside the library, at the
    reference's own configurations (its parameter files: 512^2, 16^2 tiles):
    grain growth para1 (Q = 2), the Kobayashi dendrite para2 and sintering
    para5 (two particles): plain FP64, AMSTENCIL at the sweep scripts'
    thresholds and (grain growth, Kobayashi) the all-half2 purelow runs.  The reference: its device
    code built from its sources for sm_103a (baseline/_ref/*.cubin), its host
    loops restated around driver-API launches (baseline/ref_cuda.cpp), timed
    by its own event window (step 5 to the end; one device synchronisation
    per step, as its programs do).  The library: amps_run of the same
    configuration (reference order, the same monitor and threshold; and, as
    `ours_mixed_fma_*`, the same run in the library's own arithmetic), wall
    clock around run + synchronize.  Rates in Gcell-updates/s."""
    import time
    from w3914777_gb300 import amps
    try:
        from baseline import refcuda
    except ImportError as e:
        return {"unavailable": f"baseline package: {e}"}
    if not (refcuda.available("graingrowth_pure") and refcuda.available("snowflake_pure")):
        return {"unavailable": "the reference's cubins (baseline/_ref) are not built: they need the reference tree"}
    n = 512 * 512
    total = steps + 5
    rate = lambda ms: n * steps / (ms * 1e-3) / 1e9  # noqa: E731

    def ours(p):
        with amps.Simulation(p, init=amps.INIT_REFERENCE) as s:
            s.run(10)
            s.synchronize()
            t0 = time.perf_counter()
            s.run(steps)
            s.synchronize()
            return n * steps / (time.perf_counter() - t0) / 1e9

    out = {"note": "reference: its own kernels and event window; ours: amps_run, wall clock; "
                   f"{steps} steps at the reference's configurations (512^2, 16^2 tiles)",
           "steps": steps}
    gg = {"ref_plain_fp64": rate(refcuda.gg_pure(total)[2]),
          "ours_plain_fp64_reference_order": ours(amps.Params.preset("graingrowth", 1, mode="purehigh", ref_order=1)),
          "ours_plain_fp64_fma": ours(amps.Params.preset("graingrowth", 1, mode="purehigh", ref_order=0))}
    for m, thr in ((2, 1e-4), (1, 0.5)):
        gg[f"ref_amstencil_monitor{m}_{thr:g}"] = rate(refcuda.gg_mix(total, thr, m)[3])
        gg[f"ours_mixed_monitor{m}_{thr:g}"] = ours(amps.Params.preset(
            "graingrowth", 1, mode="end2end_mix", monitor=m, monitor_samples=0, monitor_field=1, thr_lo=thr,
            thr_hi=thr, ref_order=1, half_arith=amps.HALF_REF, ref_snapshot=1))
        # the same run in the library's own arithmetic (FMA-form FP64 tiles,
        # float arithmetic on half tiles): the reference order keeps
        # pow(eta, 3) on the FP64 pipe, which paces the adaptive step
        gg[f"ours_mixed_fma_monitor{m}_{thr:g}"] = ours(amps.Params.preset(
            "graingrowth", 1, mode="end2end_mix", monitor=m, monitor_samples=0, monitor_field=1, thr_lo=thr,
            thr_hi=thr, ref_order=0))
    if refcuda.available("graingrowth_purelow"):
        gg["ref_purelow_half2"] = rate(refcuda.gg_purelow(total)[2])
        gg["ours_purelow"] = ours(amps.Params.preset("graingrowth", 1, mode="purelow"))
        gg["ours_purelow_half_ref"] = ours(amps.Params.preset("graingrowth", 1, mode="purelow",
                                                              half_arith=amps.HALF_REF))
    out["graingrowth_para1"] = gg
    kob = {"ref_plain_fp64": rate(refcuda.kob_pure(total)[2]),
           "ours_plain_fp64_reference_order": ours(amps.Params.preset("kobayashi", 2, mode="purehigh", ref_order=1)),
           "ours_plain_fp64_fma": ours(amps.Params.preset("kobayashi", 2, mode="purehigh", ref_order=0))}
    for m, thr in ((1, 0.5), (2, 1e-4)):
        kob[f"ref_amstencil_monitor{m}_{thr:g}"] = rate(refcuda.kob_mix(total, thr, m)[3])
        kob[f"ours_mixed_monitor{m}_{thr:g}"] = ours(amps.Params.preset(
            "kobayashi", 2, mode="end2end_mix", monitor=m, monitor_samples=0, monitor_field=0, thr_lo=thr,
            thr_hi=thr, ref_order=1))
        kob[f"ours_mixed_fma_monitor{m}_{thr:g}"] = ours(amps.Params.preset(
            "kobayashi", 2, mode="end2end_mix", monitor=m, monitor_samples=0, monitor_field=0, thr_lo=thr,
            thr_hi=thr, ref_order=0))
    if refcuda.available("snowflake_purelow"):
        kob["ref_purelow_half2"] = rate(refcuda.kob_purelow(total)[2])
        kob["ours_purelow"] = ours(amps.Params.preset("kobayashi", 2, mode="purelow"))
    out["kobayashi_para2"] = kob
    if refcuda.available("sintering_pure") and refcuda.available("sintering_mix"):
        f0 = amps.init_host(amps.Params.preset("sintering", 5, mode="purehigh", ref_order=1), amps.INIT_REFERENCE)
        sint = {"ref_plain_fp64": rate(refcuda.sint_pure(total, f0[0], f0[1], f0[2])[3]),
                "ours_plain_fp64_reference_order": ours(amps.Params.preset("sintering", 5, mode="purehigh",
                                                                           ref_order=1)),
                "ours_plain_fp64_fma": ours(amps.Params.preset("sintering", 5, mode="purehigh", ref_order=0))}
        for m, thr in ((2, 1e-4), (1, 0.5)):
            sint[f"ref_amstencil_monitor{m}_{thr:g}"] = rate(refcuda.sint_mix(total, thr, m, f0[0], f0[1], f0[2])[4])
            sint[f"ours_mixed_monitor{m}_{thr:g}"] = ours(amps.Params.preset(
                "sintering", 5, mode="end2end_mix", monitor=m, monitor_samples=0, monitor_field=0, thr_lo=thr,
                thr_hi=thr, ref_order=1, half_arith=amps.HALF_REF))
            sint[f"ours_mixed_fma_monitor{m}_{thr:g}"] = ours(amps.Params.preset(
                "sintering", 5, mode="end2end_mix", monitor=m, monitor_samples=0, monitor_field=0, thr_lo=thr,
                thr_hi=thr, ref_order=0))
        out["sintering_para5"] = sint
    return out


def run_roofline_hbm(p, peak, peak_kind, n=4096, warm=30, steps=200):
    """The headline step kernel where HBM, not L2, serves the state: the same
    tuned adaptive workload at 4096^2 (Q = 8: 512 MiB of FP32 state per
    parity, four times the L2).  After `warm` steps (the all-FP64 warm-start
    period and two more), `steps` profiled steps: each launch timed with CUDA
    events on its stream; algorithmic bytes per launch as in the headline."""
    import w3914777_gb300 as w
    q = p.replace(nx=n, ny=n)
    with w.Simulation(q, init=w.INIT_SEEDED) as s:
        s.run(warm)
        s.set_profiling(True)
        s.run(steps)
        kms, klaunch, ktiles = s.kernel_times()
        s.set_profiling(False)
    T, nf = q.tile, q.num_fields
    algo = sum(ktiles[k] * T * T * nf * 2 * (2, 4, 8)[k] for k in range(3))
    launches = max(klaunch[3], 1)
    per_launch_s = kms[3] * 1e-3 / launches
    achieved = algo / launches / per_launch_s / 1e9 if per_launch_s > 0 else 0.0
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            with open(tpath) as f:
                traffic = json.load(f).get("gg_step_kernel_4096_bytes_per_launch")
        except Exception:
            traffic = None
    tot = max(sum(ktiles[:3]), 1)
    return {"bound": "hbm", "kernel": "gg_step_kernel", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "peak_source": f"{peak_kind} hbm_gbs",
            "algorithmic_bytes_per_launch": algo / launches, "us_per_launch": per_launch_s * 1e6,
            "workload": f"the headline's tuned adaptive grain growth at {n}x{n}, Q={nf}: steps {warm + 1}.."
                        f"{warm + steps} (after the warm start), state {n * n * nf * 4 / 2**20:.0f} MiB per "
                        "parity in FP32 > L2",
            "tier_mix": {k: ktiles[i] / tot for i, k in enumerate(("half", "fp32", "fp64"))}}


def run_adjoint(steps=1000, segment=32, n=256):
    """Checkpointed adjoint on the 256^2 Kobayashi dendrite (zero-flux, noise),
    1000 FP32 steps, 32-step checkpoints; loss = L2 misfit of phi against the
    FP64 forward with delta = 0.04, K = 1.8.  Times the forward and backward
    sweeps (CUDA events, median of 3), the keep-every-state variant and one
    eager step of each; checks the FP32 gradients against FP64 ones and the
    FP64 delta-gradient against a central difference (h = 1e-4 delta)."""
    import torch
    from w3914777_gb300 import adjoint, amps

    p = amps.Params.preset(amps.KOBAYASHI, 0, nx=n, ny=n)
    x = amps.init_host(p, amps.INIT_REFERENCE)
    base = [p.delta, p.kappa, p.epsb]

    def med(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.median(ts)

    x64 = torch.tensor(x, device="cuda")
    tgt = adjoint.Rollout(p, steps, torch.float64, segment).forward(x64, [0.04, 1.8, p.epsb])[0]

    def grads(dtype, seg):
        run = adjoint.Rollout(p, steps, dtype, seg)
        pv = torch.tensor(base, dtype=torch.float64, requires_grad=True)
        x0 = torch.tensor(x, dtype=dtype, device="cuda", requires_grad=True)
        out = adjoint.rollout(x0, p, steps, param_values=pv, runner=run)
        loss = 0.5 * ((out[0].double() - tgt) ** 2).sum()
        loss.backward()
        g = torch.cat([pv.grad, x0.grad[1].double().flatten().cpu()])
        x0d = x0.detach()
        gf = torch.ones_like(x0d)
        tf = med(lambda: run.forward(x0d, base))
        tb = med(lambda: run.backward(gf))
        run.close()
        return g, tf, tb, float(loss.detach())

    g32, tf32, tb32, _ = grads(torch.float32, segment)
    _, tf_all, tb_all, _ = grads(torch.float32, 1)
    g64, tf64, tb64, _ = grads(torch.float64, segment)
    rel32 = float(((g32[:3] - g64[:3]).abs() / g64[:3].abs()).max())
    relT0 = float((g32[3:] - g64[3:]).norm() / g64[3:].norm())
    run64 = adjoint.Rollout(p, steps, torch.float64, segment)
    h = 1e-4 * p.delta
    lp = float(0.5 * ((run64.forward(x64, [p.delta + h, p.kappa, p.epsb])[0] - tgt) ** 2).sum())
    lm = float(0.5 * ((run64.forward(x64, [p.delta - h, p.kappa, p.epsb])[0] - tgt) ** 2).sum())
    fd = (lp - lm) / (2 * h)
    run64.close()
    st = adjoint.Stepper(p, torch.float32)
    xs = torch.tensor(x, dtype=torch.float32, device="cuda")
    ys, gs, gi = torch.empty_like(xs), torch.ones_like(xs), torch.empty_like(xs)
    gp = torch.zeros(3, dtype=torch.float64, device="cuda")
    t_sf = med(lambda: [st.forward(xs, 0, out=ys) for _ in range(50)]) / 50
    t_sa = med(lambda: [st.adjoint(xs, gs, 0, gp, grad_in=gi) for _ in range(50)]) / 50
    return {
        "workload": f"Kobayashi dendrite {n}x{n} zero-flux + noise, {steps} steps FP32, "
                    f"{segment}-step checkpoints; grads w.r.t. delta, K, epsb, T0",
        "forward_sweep_ms": tf32, "backward_sweep_ms": tb32, "ratio": tb32 / tf32,
        "step_forward_us": t_sf * 1e3, "step_adjoint_us": t_sa * 1e3, "step_ratio": t_sa / t_sf,
        "keep_all_states": {"forward_sweep_ms": tf_all, "backward_sweep_ms": tb_all, "ratio": tb_all / tf_all},
        "fp64": {"forward_sweep_ms": tf64, "backward_sweep_ms": tb64, "ratio": tb64 / tf64},
        "fp32_vs_fp64_param_grad_rel": rel32, "fp32_vs_fp64_T0_grad_rel_l2": relT0,
        "fp64_delta_grad_vs_central_difference_rel": abs(float(g64[0]) - fd) / abs(fd),
    }


def run_adjoint_gg(steps=200, n=1024, q=8):
    """Checkpointed adjoint of 200 grain-growth steps at 1024^2, Q = 8
    (sqrt(N)-step checkpoints) from the coarsening state after 1000 FP64
    steps of the seeded multi-grain start (the first steps amplify the
    start's noise, and with it rounding); loss = L2 misfit of all order parameters against
    the FP64 forward with L scaled by 1.1.  Times one eager step
    and its adjoint, and the forward and backward sweeps (CUDA events,
    median of 3), FP32 and FP64; checks the FP32 gradients against FP64 ones
    and the FP64 L-gradient against a central difference (h = 1e-4 L)."""
    import torch
    from w3914777_gb300 import adjoint, amps

    p = amps.Params.preset(amps.GRAINGROWTH, 0, nx=n, ny=n, nfields=q)
    base = [p.mobil, p.grcoef, p.gamma]

    def med(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.median(ts)

    warm = adjoint.Stepper(p, torch.float64)
    x64 = torch.tensor(amps.init_host(p, amps.INIT_SEEDED), device="cuda")
    nxt = torch.empty_like(x64)
    for i in range(1000):
        warm.forward(x64, i, out=nxt)
        x64, nxt = nxt, x64
    x = x64.cpu().numpy()
    run64 = adjoint.Rollout(p, steps, torch.float64)
    tgt = run64.forward(x64, [1.1 * p.mobil, p.grcoef, p.gamma]).clone()

    def loss_at(vals):
        return float(0.5 * ((run64.forward(x64, vals) - tgt) ** 2).sum())

    out = {"workload": f"grain growth {n}x{n}, Q={q}, {steps} steps from step 1000, sqrt(N)-step checkpoints; "
                       "grads w.r.t. L, kappa, gamma, eta0"}
    grads = {}
    for name, dtype in (("fp32", torch.float32), ("fp64", torch.float64)):
        run = run64 if dtype == torch.float64 else adjoint.Rollout(p, steps, dtype)
        pv = torch.tensor(base, dtype=torch.float64, requires_grad=True)
        x0 = torch.tensor(x, dtype=dtype, device="cuda", requires_grad=True)
        y = adjoint.rollout(x0, p, steps, param_values=pv, runner=run)
        (0.5 * ((y.double() - tgt) ** 2).sum()).backward()
        grads[name] = (pv.grad.clone(), x0.grad.double())
        x0d = x0.detach()
        gf = torch.ones_like(x0d)
        tf = med(lambda: run.forward(x0d, base))
        tb = med(lambda: run.backward(gf))
        st = adjoint.Stepper(p, dtype)
        ys, gi = torch.empty_like(x0d), torch.empty_like(x0d)
        gp = torch.zeros(3, dtype=torch.float64, device="cuda")
        t_sf = med(lambda: [st.forward(x0d, 0, out=ys) for _ in range(50)]) / 50
        t_sa = med(lambda: [st.adjoint(x0d, gf, 0, gp, grad_in=gi) for _ in range(50)]) / 50
        out[name] = {"forward_sweep_ms": tf, "backward_sweep_ms": tb, "ratio": tb / tf,
                     "step_forward_us": t_sf * 1e3, "step_adjoint_us": t_sa * 1e3, "step_ratio": t_sa / t_sf}
        if run is not run64:
            run.close()
    g32, g64 = grads["fp32"], grads["fp64"]
    out["fp32_vs_fp64_param_grad_rel"] = float(((g32[0] - g64[0]).abs() / g64[0].abs()).max())
    out["fp32_vs_fp64_eta0_grad_rel_l2"] = float((g32[1] - g64[1]).norm() / g64[1].norm())
    h = 1e-4 * p.mobil
    fd = (loss_at([p.mobil + h, p.grcoef, p.gamma]) - loss_at([p.mobil - h, p.grcoef, p.gamma])) / (2 * h)
    out["fp64_L_grad_vs_central_difference_rel"] = abs(float(g64[0][0]) - fd) / abs(fd)
    run64.close()
    return out


ENSEMBLE_TUNED = os.path.join(ROOT, "w3914777_gb300", "tuned", "ensemble_64.json")


def ensemble_overrides():
    """Tile, monitor and thresholds of the 64-member ensemble: the autotuner's
    choice for the ensemble itself (`python -m w3914777_gb300.autotune
    ensemble`), else the single-run workload's monitor and thresholds."""
    try:
        with open(ENSEMBLE_TUNED) as f:
            return dict(json.load(f)["best"]["overrides"]), "autotune (ensemble)"
    except Exception:
        tuned = load_tuned()
        ov = dict(tuned["overrides"]) if tuned else {}
        ov.pop("tile", None)
        return ov, "single-run tuning"


def run_ensemble(steps=5000, check_steps=1000, count=64, seed=2024):
    """64 grain-growth runs (any integer sides 128..1024, Q in {4,8,12,16}, kappa ~ U[1,3],
    L ~ U[0.5,2], per-member stable dt) advanced by one launch per group of
    members a step, at the autotuned monitor and thresholds.  Times `steps` steps of the
    ensemble; compares, over `check_steps` steps, the same members run one
    after another through amps_run, and the plain-FP64 ensemble (rate and
    per-member max-abs error)."""
    import torch
    from w3914777_gb300 import amps, ensemble

    ov, tuned_by = ensemble_overrides()
    params = ensemble.member_params(count=count, seed=seed, overrides=ov)
    cells = ensemble.cells(params)
    stream = torch.cuda.Stream()

    def timed(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b)

    def build(ps):
        sims = [amps.Simulation(p, init=amps.INIT_SEEDED) for p in ps]
        for sm in sims:
            sm.set_stream(stream.cuda_stream)
        ens = amps.Ensemble(sims)
        ens.set_stream(stream.cuda_stream)
        return sims, ens

    sims, ens = build(params)
    ens.run(10)  # warm-up period: captures the graphs
    ms = timed(lambda: ens.run(steps))
    ens.synchronize()
    stats = [sm.stats() for sm in sims]
    ens.close()
    for sm in sims:
        sm.close()
    # the same members, each through its own amps_run, one after another
    sims = [amps.Simulation(p, init=amps.INIT_SEEDED) for p in params]
    for sm in sims:
        sm.set_stream(stream.cuda_stream)
        sm.run(10)
    ms_seq = timed(lambda: [sm.run(check_steps) for sm in sims])
    for sm in sims:
        sm.close()
    # adaptive vs plain FP64 over check_steps
    sims, ens = build(params)
    ms_mix = timed(lambda: ens.run(check_steps))
    mixed = [sm.fields() for sm in sims]
    ens.close()
    for sm in sims:
        sm.close()
    p64 = [p.replace(mode=amps.PUREHIGH, high_tier=amps.TIER_FP64) for p in params]
    sims, ens = build(p64)
    ms_64 = timed(lambda: ens.run(check_steps))
    err = max(float(np.abs(sm.fields() - f).max()) for sm, f in zip(sims, mixed))
    ens.close()
    for sm in sims:
        sm.close()
    ts = np.sum([st["tile_steps"] for st in stats], axis=0)
    # algorithmic bytes a step: every member's cells x fields read and written
    # once, at the bytes of the tiers its tile-steps ran in (half 2, FP32 4, FP64 8)
    tb = np.array([2.0, 4.0, 8.0])
    alg = sum(p.nx * p.ny * p.nfields * 2 * float(np.dot(st["tile_steps"], tb)) / max(sum(st["tile_steps"]), 1)
              for p, st in zip(params, stats))
    peak, peak_src = peaks()
    achieved = alg * steps / (ms * 1e-3) / 1e9
    return {
        "workload": f"{count} grain-growth runs, square sides drawn log-uniformly in 128..1024 (any integer: "
                    f"{sum(p.nx % p.tile != 0 for p in params)} members have partial edge tiles), Q in {{4,8,12,16}}, "
                    f"kappa~U[1,3], L~U[0.5,2], dt=min(0.05, 0.9*2/(12 L kappa)), seeded eta~U[-1e-3,1e-3], "
                    f"{steps} steps, one launch per group of members a step (members of one occupancy "
                    f"class, parallel branches of the period's graph)",
        "members": count, "cells_per_step": cells,
        "value": cells * steps / (ms * 1e-3) / 1e9, "unit": "Gcell-updates/s", "ms": ms,
        "sequential_amps_run": {"value": cells * check_steps / (ms_seq * 1e-3) / 1e9, "steps": check_steps},
        "plain_fp64": {"value": cells * check_steps / (ms_64 * 1e-3) / 1e9, "steps": check_steps},
        "speedup_vs_plain_fp64": ms_64 / ms_mix,
        "max_abs_err_vs_fp64": err, "err_steps": check_steps,
        "tier_mix": {k: float(v) / float(ts.sum()) for k, v in zip(("half", "fp32", "fp64"), ts)},
        "roofline": {"bound": "hbm", "kernel": "gg_ens_kernel", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": f"{peak_src} hbm_gbs",
                     "algorithmic_bytes_per_step": alg,
                     "note": "whole run (warm-start FP64 period and monitor steps included); domain cells "
                             "only (a partial edge tile's padding is not counted); the ensemble's state "
                             "exceeds L2"},
        "tuned_by": tuned_by, "tile": params[0].tile, "thresholds": [params[0].thr_lo, params[0].thr_hi],
    }


def field_errors(a, b, names):
    """Per field: max |a - b|, RMS (the L2 norm over sqrt(cells)) and mean |a - b|."""
    out = {}
    for k, name in enumerate(names):
        d = np.abs(a[k] - b[k])
        out[name] = {"max_abs": float(d.max()), "rms": float(np.sqrt(np.mean(d * d))), "mean_abs": float(d.mean())}
    return out


def run_configs(kob_steps=2000, sint_steps=20000, cpu_sample=200):
    """The other two models' seeded workloads at their tuned settings
    (w3914777_gb300/tuned/*.json), each against its plain FP64 run from the
    same initial state: Kobayashi dendrite 512^2 zero-flux with noise, 2000
    steps (plus the all-FP32 run); sintering 1024^2 with 16 particles, 20000
    steps, with the conserved-mass drift and the neck widths.  Device-timed
    (CUDA events) graph replays; the states (4-34 MiB per tier) stay
    L2-resident."""
    import torch
    import w3914777_gb300 as w

    def tuned(name):
        with open(os.path.join(ROOT, "w3914777_gb300", "tuned", name)) as f:
            return json.load(f)["best"]["overrides"]

    stream = torch.cuda.Stream()

    def run(p, init, steps):
        with w.Simulation(p) as s:
            s.set_stream(stream.cuda_stream)
            s.set_fields(init)
            s.run(2 * p.cadence)  # captures the period graphs
            s.set_fields(init)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            s.run(steps)
            b.record(stream)
            s.synchronize()
            ms = a.elapsed_time(b)
            extra = {}
            if p.model == w.KOBAYASHI:
                extra["interface"] = s.interface(0, 0.5)
            if p.model == w.SINTERING:
                extra["mass"] = s.reduce(0, w.REDUCE_SUM)
                bl = s.boundary_lengths(0.5)
                iu = np.triu_indices(bl.shape[0], 1)
                necks = bl[iu][bl[iu] > 0]
                extra["necks"] = {"count": int(necks.size), "mean_width": float(necks.mean()) if necks.size else 0.0,
                                  "max_width": float(necks.max()) if necks.size else 0.0}
            st = s.stats()
            ts = st["tile_steps"]
            tot = max(sum(ts), 1)
            return ms, s.fields(), extra, [t / tot for t in ts]

    out = {}
    # Kobayashi dendrite (the FMA form throughout; the preset's reference-order
    # arithmetic is for parity with the reference)
    p = w.Params.preset("kobayashi", 0).replace(ref_order=0)
    init = w.init_host(p, w.INIT_SEEDED)
    ms_a, f_a, x_a, mix = run(p.replace(**tuned("kobayashi_512.json")), init, kob_steps)
    # plain runs in the FMA form (ref_order=0), as the adaptive run's FP64 tiles
    ms_64, f_64, x_64, _ = run(p.replace(mode=w.PUREHIGH, high_tier=w.TIER_FP64, ref_order=0), init, kob_steps)
    ms_32, f_32, _, _ = run(p.replace(mode=w.PUREHIGH, high_tier=w.TIER_FP32, ref_order=0), init, kob_steps)
    # the plain FP64 dendrite in the reference's expression order (snowflake/function.h:5-60,
    # no fused multiply-add): the 512^2, 2000-step FP64 configuration as the reference computes it
    ms_64r, f_64r, _, _ = run(p.replace(mode=w.PUREHIGH, high_tier=w.TIER_FP64, ref_order=1), init, kob_steps)
    # ... and on the host cores (the oracle's -O3 build), a bounded sample of the same steps
    kob_cpu, kob_cpu_s = oracle_rate_kobayashi(cpu_sample, cpu_threads())
    cells = p.nx * p.ny * kob_steps
    out["kobayashi"] = {
        "workload": f"Kobayashi dendrite {p.nx}x{p.ny} zero-flux, seeded noise, disc r^2<{p.init_r2:g} at the centre, "
                    f"{kob_steps} steps, tuned spatial monitor",
        "value": cells / (ms_a * 1e-3) / 1e9, "unit": "Gcell-updates/s",
        "plain_fp64": cells / (ms_64 * 1e-3) / 1e9, "all_fp32": cells / (ms_32 * 1e-3) / 1e9,
        "plain_fp64_reference_order": {
            "value": cells / (ms_64r * 1e-3) / 1e9, "unit": "Gcell-updates/s", "ms": ms_64r,
            "max_abs_vs_fma_form": float(np.abs(f_64r - f_64).max())},
        "cpu_baseline": {"value": kob_cpu, "unit": "Gcell-updates/s", "cores": cpu_threads(), "kind": "port",
                         "sample": f"{cpu_sample} FP64 steps of the same 512^2 dendrite ({kob_cpu_s:.2f} s; the "
                                   "oracle's restatement of snowflake/function.h:5-60 built -O3, OpenMP over rows)"},
        "speedup_vs_plain_fp64": ms_64 / ms_a,
        "max_abs_err_vs_fp64": float(np.abs(f_a - f_64).max()),
        "mean_abs_err_vs_fp64": float(np.abs(f_a - f_64).mean()),
        "errors_vs_fp64_per_field": field_errors(f_a, f_64, ("phi", "T")),
        "all_fp32_max_abs_err": float(np.abs(f_32 - f_64).max()),
        "interface": {"adaptive": x_a["interface"], "fp64": x_64["interface"]},
        "tier_mix": dict(zip(("half", "fp32", "fp64"), mix)),
    }
    # sintering
    p = w.Params.preset("sintering", 0)
    init = w.init_host(p, w.INIT_SEEDED)
    m0 = float(init[0].sum())
    ms_a, f_a, x_a, mix = run(p.replace(**tuned("sintering_1024_n16.json")), init, sint_steps)
    ms_64, f_64, x_64, _ = run(p.replace(mode=w.PUREHIGH, high_tier=w.TIER_FP64, ref_order=0), init, sint_steps)
    cells = p.nx * p.ny * sint_steps
    out["sintering"] = {
        "workload": f"sintering {p.nx}x{p.ny}, {p.nfields} particles (seeded non-overlapping discs), "
                    f"{sint_steps} steps, FP64 chemical-potential Laplacian, tuned spatial monitor",
        "value": cells / (ms_a * 1e-3) / 1e9, "unit": "Gcell-updates/s",
        "plain_fp64": cells / (ms_64 * 1e-3) / 1e9, "speedup_vs_plain_fp64": ms_64 / ms_a,
        "max_abs_err_vs_fp64": float(np.abs(f_a - f_64).max()),
        "mean_abs_err_vs_fp64": float(np.abs(f_a - f_64).mean()),
        "errors_vs_fp64_per_field": field_errors(f_a, f_64, ["c"] + [f"eta{k + 1}" for k in range(p.nfields)]),
        "mass_drift": {"adaptive": (x_a["mass"] - m0) / m0, "fp64": (x_64["mass"] - m0) / m0,
                       "note": "relative change of the FP64 sum of c; the reference clamps c to [0,1] after each "
                               "step (sintering/function.h:100-101), which removes mass in both runs"},
        "necks": {"adaptive": x_a["necks"], "fp64": x_64["necks"]},
        "tier_mix": dict(zip(("half", "fp32", "fp64"), mix)),
    }
    return out


def run_profile_case(args):
    """A short, untimed run of a tuned workload at nx^2 for ncu captures
    (`--profile-case 2048` puts a 256 MiB FP32 grain-growth state, larger than
    L2; `--profile-model kobayashi|sintering` the other models' tuned runs;
    `graingrowth-adjoint`: sim-steps FP32 step + adjoint-step pairs of the
    Q = 8 grain-growth module from the seeded state; `ensemble`: the first
    profile-case members of the 64-member ensemble workload)."""
    import torch
    import w3914777_gb300 as w
    torch.cuda.set_device(0)
    model = args.profile_model
    if model == "ensemble":
        from w3914777_gb300 import ensemble
        ov, _ = ensemble_overrides()
        params = ensemble.member_params(count=64, seed=2024, overrides=ov)[:args.profile_case]
        sims = [w.Simulation(p, init=w.INIT_SEEDED) for p in params]
        with w.Ensemble(sims) as ens:
            ens.run(args.sim_steps)
            ens.synchronize()
        for sm in sims:
            sm.close()
        print(json.dumps({"profile_case": args.profile_case, "steps": args.sim_steps, "model": model,
                          "cells_per_step": ensemble.cells(params)}))
        return
    if model == "graingrowth-adjoint":
        from w3914777_gb300 import adjoint
        p = w.Params.preset("graingrowth", 0, nx=args.profile_case, ny=args.profile_case)
        st = adjoint.Stepper(p, torch.float32)
        x = torch.tensor(w.init_host(p, w.INIT_SEEDED), dtype=torch.float32, device="cuda")
        y, g, gi = torch.empty_like(x), torch.ones_like(x), torch.empty_like(x)
        gp = torch.zeros(3, dtype=torch.float64, device="cuda")
        for i in range(args.sim_steps):
            st.forward(x, i, out=y)
            st.adjoint(x, g, i, gp, grad_in=gi)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": args.profile_case, "steps": args.sim_steps, "model": model,
                          "grad_in_norm": float(gi.norm())}))
        return
    p = w.Params.preset(model, 0, nx=args.profile_case, ny=args.profile_case)
    if model == "graingrowth":
        tuned = load_tuned()
    else:
        with open(os.path.join(ROOT, "w3914777_gb300", "tuned",
                               {"kobayashi": "kobayashi_512.json", "sintering": "sintering_1024_n16.json"}[model])) as f:
            tuned = json.load(f)["best"]
    if tuned:
        p = p.replace(**tuned["overrides"])
    with w.Simulation(p, init=w.INIT_SEEDED) as s:
        s.run(args.sim_steps)
        s.synchronize()
        st = s.stats()
    print(json.dumps({"profile_case": args.profile_case, "steps": args.sim_steps, "tile_steps": st["tile_steps"]}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--sim-steps", type=int, default=10000)
    ap.add_argument("--ref-sample-steps", type=int, default=500)
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-configs", action="store_true")
    ap.add_argument("--no-hbm", action="store_true")
    ap.add_argument("--no-refcuda", action="store_true")
    ap.add_argument("--profile-case", type=int, default=0)
    ap.add_argument("--profile-model", default="graingrowth",
                    choices=["graingrowth", "kobayashi", "sintering", "graingrowth-adjoint", "ensemble"])
    args = ap.parse_args()
    if args.profile_case:
        run_profile_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

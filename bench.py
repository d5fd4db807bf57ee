"""Benchmark: STA/TFM frames/s on GB300 (one JSON line on rank 0).

A step is one frame through the whole hot path: signal preparation
(upsampling, DC removal, Hilbert analytic signal) of every A-scan, then the
delay-and-sum with the coherence factor over every grid point.

Default workload (--workload cf2d): 64-element linear array, 4096 samples at
40 MHz, 8x upsampling, Blackman apodization, PCF, 512 x 512 grid, FP32; seeded
synthetic RF (32 point scatterers + 20 000 speckle scatterers).

  value  frames/s with the RF already resident in HBM (device entry point);
         4 RF buffers (4 x 67 MB) rotate between steps and every step writes
         and reads the 1.07 GB analytic tensor, so the inputs exceed L2.
  e2e    the same metric through the host entry points (usgb_submit_rf +
         usgb_process): RF copied host->device and the image device->host
         inside every step.
  --impl reference  times the CPU oracle (the C++ restatement of the
         reference processor) on the host cores instead.
Multi-GPU (torchrun): replicas, one frame stream per rank (weak scaling).
"""
from __future__ import annotations

import argparse
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

METRIC = "STA/TFM frames/s + p50/p99 latency, mixed-precision vs FP32 at ≤-60 dB error"


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def _workload(name: str, storage: str):
    from us_lab4a_gb300 import workloads
    if name == "cf2d":
        fr = workloads.cf2d()
        desc = "cf2d: 64-element linear array, 4096 samples @40 MHz, 8x upsampling, Blackman, PCF, 512x512 grid"
    elif name == "plain2d":
        fr = workloads.plain2d()
        desc = "plain2d: 32 elements, 2048 samples @40 MHz, 4x, rectangular apodization, no CF, 128x256 grid"
    elif name == "matrix3d":
        fr = workloads.matrix3d()
        desc = "matrix3d: 16x16 matrix array, 1024 samples @24 MHz, 4x, PCF, 64x64x128 voxels"
    else:
        raise SystemExit(f"unknown workload {name}")
    fr = workloads.with_storage(fr, storage)
    return fr, desc


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._proc = None
        self._thread = None
        self._mark = 0

    def start(self):
        cmd = ["nvidia-smi", "-i", str(self.index),
               "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
               "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
               "clocks_event_reasons.sw_power_cap",
               "--format=csv,noheader,nounits", "-lms", "50"]
        try:
            self._proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self._proc = None
            return

        def reader():
            for line in self._proc.stdout:
                self.samples.append([x.strip() for x in line.split(",")])
        self._thread = threading.Thread(target=reader, daemon=True)
        self._thread.start()
        # nvidia-smi takes a while to start: wait for its first sample so that
        # the samples taken from here on fall inside the timed region.
        t0 = time.time()
        while not self.samples and time.time() - t0 < 10.0 and self._proc.poll() is None:
            time.sleep(0.01)
        self._mark = len(self.samples)

    def stop(self):
        if self._proc is None:
            return None
        # A timed region shorter than the sampling interval may hold no
        # sample: then take the first one after it (flagged by in_region 0).
        n_region = len(self.samples) - self._mark
        if n_region == 0:
            t0 = time.time()
            while len(self.samples) <= self._mark and time.time() - t0 < 2.0 and self._proc.poll() is None:
                time.sleep(0.005)
        self.samples = self.samples[self._mark:]
        self._proc.terminate()
        try:
            self._proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self._proc.kill()
        if self._thread:
            self._thread.join(timeout=2)
        rows = [r for r in self.samples if len(r) >= 7]
        if not rows:
            return None
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[0]) for r in rows if num(r[0]) is not None]
        mx = [num(r[1]) for r in rows if num(r[1]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "in_region": n_region,
                "interval_ms": 50}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _oracle_spec(spec, threads):
    import oracle
    return oracle.OracleSpec(tx_xy=spec.tx_xy, rx_xy=spec.rx_xy, num_samples=spec.num_samples,
                             upsampling=4 if spec.real_path else spec.upsampling,
                             sampling_frequency=spec.sampling_frequency, propagation_speed=spec.propagation_speed,
                             center_frequency=spec.center_frequency, peak_offset=spec.peak_offset,
                             dead_zone_m=spec.dead_zone_m, rx_apod=spec.rx_apod,
                             cf={"none": 0, "pcf": 1, "scf": 2, "mf": 3}[spec.coherence], pcf_gamma=spec.pcf_gamma,
                             scf_p=spec.scf_p, real_path=spec.real_path, nthreads=threads)


def cpu_rf(frame) -> np.ndarray:
    """Host RF of the frame's shape for the CPU timings: the frame's point
    scatterers and noise, without its speckle background (synthesising 20 000
    speckle echoes on the host takes minutes; the oracle's cost does not
    depend on the sample values)."""
    from us_lab4a_gb300 import synth
    spec = frame.spec
    pts = frame.scatterers
    n = min(len(pts), 64)
    sub = synth.Scatterers(pts.x[:n], pts.y[:n], pts.z[:n], pts.amp[:n])
    return synth.synth_rf_numpy(spec.tx_xy, spec.rx_xy, sub, spec.sampling_frequency, spec.propagation_speed,
                                spec.center_frequency, spec.num_samples, np.random.default_rng(frame.seed + 1))


def time_oracle_frames(frame, rf: np.ndarray, threads: int, warmup: int, steps: int):
    """Whole frames through the FP32 oracle (the C++ restatement of the
    reference processor: preparation of every A-scan, delay-and-sum of every
    grid point, coherence factor), `warmup` untimed then `steps` timed runs,
    as the reference's ExecutionTimeMeasurement does (src/util/ExecutionTimeMeasurement.h:25,75-86).
    Returns the per-frame seconds of the timed runs."""
    import oracle
    spec = _oracle_spec(frame.spec, threads)
    times = []
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        oracle.process(spec, rf, frame.grid_xyz, dtype=np.float32)
        if i >= warmup:
            times.append(time.perf_counter() - t0)
    return times


def _stats(times):
    return {"mean_s": statistics.mean(times), "p50_s": float(np.percentile(times, 50)),
            "p99_s": float(np.percentile(times, 99)), "runs": len(times)}


def cpu_baseline(frame, threads: int, rf: np.ndarray, warmup: int = 1, steps: int = 2):
    """CPU baseline leg: whole frames through the FP32 oracle on the host cores."""
    times = time_oracle_frames(frame, rf, threads, warmup, steps)
    st = _stats(times)
    return {"value": 1.0 / st["mean_s"], "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": f"{steps} whole frames ({frame.spec.num_tx * frame.spec.num_rx} A-scans, {frame.npix} grid "
                      f"points each) after {warmup} warm-up, FP32 oracle on {threads} threads",
            **st}


def run_reference(args):
    """The reference arm: whole frames of the workload through the CPU oracle
    (the reference's CPU processor restated; the reference itself is a C++
    CMake/Qt project that does not install here), every host thread."""
    world, rank, _ = _dist()
    if rank != 0:
        return
    frame, desc = _workload(args.workload, "f32")
    threads = os.cpu_count() or 1
    rf = cpu_rf(frame)
    times = time_oracle_frames(frame, rf, threads, args.warmup, args.steps)
    st = _stats(times)
    value = 1.0 / st["mean_s"]
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * st["mean_s"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded point + speckle scatterers)",
            "config": _config(frame, desc, "f32"),
            "latency_ms": {"p50": 1e3 * st["p50_s"], "p99": 1e3 * st["p99_s"]},
            "cpu_baseline": {"value": value, "unit": "frames/s", "cores": threads, "kind": "port",
                             "sample": f"each step one whole frame ({frame.spec.num_tx * frame.spec.num_rx} A-scans, "
                                       f"{frame.npix} grid points) through the FP32 oracle on {threads} threads; RF of "
                                       "the frame's point scatterers and noise (speckle left out of the host input: "
                                       "the cost does not depend on sample values)"},
            "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _config(frame, desc: str, storage: str) -> dict:
    """The workload identification both arms print (implementation details go elsewhere)."""
    spec = frame.spec
    n_sig = spec.num_tx * spec.num_rx
    rf_mb = n_sig * spec.num_samples * 4 / 1e6
    tensor_gb = n_sig * spec.num_samples * spec.upsampling * {"f32": 8, "f16": 4, "bf16": 4}[storage] / 1e9
    return {"workload": desc, "storage": storage,
            "l2": f"inputs larger than L2 (129 MB) / the host's last-level cache: {rf_mb:.0f} MB RF in and a "
                  f"{tensor_gb:.2f} GB analytic tensor written and read per frame; GPU arm: 4 RF buffers rotate"}


def run_gpu(args):
    import torch
    from us_lab4a_gb300 import StaEngine, build
    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    build.build()
    frame, desc = _workload(args.workload, args.storage)
    spec = frame.spec
    eng = StaEngine(spec)
    if args.das == "plain":
        eng.set_das_variant(0)
    elif args.das in ("staged", "group", "group64", "group64x2") and not args.autotune:
        eng.set_das_variant({"staged": 1, "group": 2, "group64": 3, "group64x2": 4}[args.das], args.tile_rows,
                            args.stage_bytes, args.stages)
    stream = torch.cuda.Stream(device=dev)
    eng.set_stream(stream)
    with torch.cuda.stream(stream):
        rf0 = frame.make_rf_torch(dev)
        rfs = [rf0] + [rf0 * (1.0 + 0.01 * i) for i in range(1, 4)]  # 4 distinct resident inputs
        grid = torch.as_tensor(frame.grid_xyz, device=dev)
        value = torch.empty(frame.grid_xyz.shape[:2], device=dev)
        factor = torch.empty_like(value)
    stream.synchronize()
    eng.set_grid_device(grid)
    info = eng.signal_info()
    if args.das != "plain" and args.autotune:
        # Pick the delay-and-sum kernel and its tile / stage shape on this
        # frame (untimed): staged and receiver-group kernels, every shape
        # that fits, and the plain kernel.
        sig_t = torch.empty(info["signal_bytes"] // 4 + 1, dtype=torch.float32, device=dev)
        eng.prepare_signals_device(rf0, sig_t)
        eng.autotune_das(sig_t, value, factor, iterations=2)
        del sig_t
    das_cfg = eng.das_config()

    # A stream of frames: `pipeline` contexts, each on its own stream, take
    # the frames in turn, so one frame's preparation runs while the previous
    # frame's delay-and-sum finishes its last wave of tiles (SMs that would
    # idle). Every frame is prepared and imaged in full; the outputs of the
    # contexts are separate buffers.
    engines, streams, values, factors = [eng], [stream], [value], [factor]
    for _ in range(args.pipeline - 1):
        e = StaEngine(spec)
        st = torch.cuda.Stream(device=dev)
        e.set_stream(st)
        e.set_grid_device(grid)
        if das_cfg["variant"] == 0:
            e.set_das_variant(0)
        else:
            e.set_das_variant(das_cfg["variant"], das_cfg["tile_rows"], das_cfg["stage_bytes"], das_cfg["stages"])
        engines.append(e)
        streams.append(st)
        values.append(torch.empty_like(value))
        factors.append(torch.empty_like(factor))

    def step(i):
        k = i % len(engines)
        engines[k].process_device(rfs[i % len(rfs)], values[k], factors[k])

    for i in range(args.warmup):
        step(i)
    for st, e in zip(streams, engines):
        st.synchronize()
        e.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for st in streams[1:]:
        st.wait_event(t_start)
    for i in range(args.steps):
        st = streams[i % len(streams)]
        evs[i][0].record(st)
        step(i)
        evs[i][1].record(st)
    for st in streams[1:]:
        done = torch.cuda.Event()
        done.record(st)
        stream.wait_event(done)
    t_end.record(stream)
    stream.synchronize()
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    for e in engines:
        e.synchronize()
    for e in engines[1:]:
        e.close()
    del engines[1:], values[1:], factors[1:]
    total_ms = t_start.elapsed_time(t_end)
    per_step = [a.elapsed_time(b) for a, b in evs]
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())

    # Kernel-level timing of the two stages (roofline of the dominant kernel).
    sig = torch.empty(info["signal_bytes"] // 4 + 1, dtype=torch.float32, device=dev)
    kt = {"prep": [], "das": []}
    for i in range(args.warmup + 5):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        eng.prepare_signals_device(rfs[i % len(rfs)], sig)
        e1.record(stream)
        eng.delay_and_sum_device(sig, value, factor)
        e2.record(stream)
        stream.synchronize()
        if i >= args.warmup:
            kt["prep"].append(e0.elapsed_time(e1))
            kt["das"].append(e1.elapsed_time(e2))
    eng.synchronize()
    n_sig = spec.num_tx * spec.num_rx
    L = info["signal_length"]
    esize = {"f32": 8, "f16": 4, "bf16": 4}[spec.storage]
    prep_bytes = n_sig * spec.num_samples * 4 + n_sig * L * esize
    das_bytes = n_sig * L * esize + frame.npix * (12 + 8) + (spec.num_tx + spec.num_rx) * 8 + spec.num_rx * 4
    prep_ms, das_ms = statistics.median(kt["prep"]), statistics.median(kt["das"])
    peak, peak_kind = _peaks()
    top = ("das", das_ms, das_bytes) if das_ms >= prep_ms else ("prep", prep_ms, prep_bytes)
    achieved = top[2] / (top[1] * 1e-3) / 1e9
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tfile):
        tr = json.load(open(tfile)).get(args.workload + "/" + spec.storage + "/" + top[0])
        if tr:
            traffic = tr
    gathers = frame.npix * n_sig

    # On-chip roofline of the delay-and-sum (it is not HBM-bound): bytes
    # through the shared-memory pipe (window copies written + two taps read
    # per gather) against 152 SMs x 128 B/clk at the sampled SM clock, and
    # its algorithmic FP32 work (12 FLOP per gather) against the FP32 peak
    # (152 SMs x 128 lanes x 2 FLOP/clk).
    onchip = None
    if das_cfg["variant"] != 0:
        staged = staged_bytes_model(frame, 64 if das_cfg["variant"] >= 3 else 32,
                                    das_cfg["tile_rows"] * (2 if das_cfg["variant"] == 4 else 1), esize)
        tap_bytes = 2.0 * esize * gathers
        mhz = (clk or {}).get("sm_mhz") or 2070.0
        smem_peak = 152 * 128 * mhz * 1e6 / 1e9
        fp32_peak = 152 * 128 * 2 * mhz * 1e6 / 1e12
        smem_gbs = (staged + tap_bytes) / (das_ms * 1e-3) / 1e9
        tflops = 12.0 * gathers / (das_ms * 1e-3) / 1e12
        onchip = {"smem_bytes_per_launch": staged + tap_bytes, "staged_bytes_modelled": staged,
                  "tap_bytes": tap_bytes, "smem_achieved_gbs": smem_gbs, "smem_peak_gbs": smem_peak,
                  "smem_frac": smem_gbs / smem_peak, "fp32_tflops": tflops, "fp32_peak_tflops": fp32_peak,
                  "fp32_frac": tflops / fp32_peak, "clock_mhz": mhz}

    # End to end through the host entry points (host RF in, host image out).
    e2e = None
    if not args.no_e2e:
        # Host RF in, host image out, through usgb_process_rf: `pipeline`
        # host threads, each with its own context, take the frames in turn
        # (the native call releases the interpreter, so the frames overlap as
        # in the resident measurement); latency is per call.
        rf_host = rf0.cpu().numpy()
        hosts = [eng]
        for _ in range(args.pipeline - 1):
            e = StaEngine(spec)
            e.set_grid_device(grid)
            if das_cfg["variant"] == 0:
                e.set_das_variant(0)
            else:
                e.set_das_variant(das_cfg["variant"], das_cfg["tile_rows"], das_cfg["stage_bytes"], das_cfg["stages"])
            hosts.append(e)
        for e in hosts:
            for i in range(args.warmup):
                e.process_host(rf_host)
        lat = [[] for _ in hosts]
        failures = []
        start = threading.Barrier(len(hosts) + 1)

        def host_worker(k):
            start.wait()
            try:
                for i in range(k, args.steps, len(hosts)):
                    s0 = time.perf_counter()
                    hosts[k].process_host(rf_host)
                    lat[k].append(time.perf_counter() - s0)
            except Exception as ex:  # reported after the join: a failed frame is no frame
                failures.append(ex)

        workers = [threading.Thread(target=host_worker, args=(k,)) for k in range(len(hosts))]
        for w in workers:
            w.start()
        start.wait()
        t0 = time.perf_counter()
        for w in workers:
            w.join()
        e2e_s = time.perf_counter() - t0
        if failures:
            raise failures[0]
        for e in hosts[1:]:
            e.close()
        lat = [x for per in lat for x in per]
        e2e = {"value": world * args.steps / e2e_s if world == 1 else None, "unit": "frames/s",
               "h2d_bytes_per_step": int(rf_host.nbytes), "d2h_bytes_per_step": int(2 * frame.npix * 4),
               "host_threads": len(hosts),
               "p50_ms": 1e3 * float(np.percentile(lat, 50)), "p99_ms": 1e3 * float(np.percentile(lat, 99))}
        if world > 1:
            t = torch.tensor([e2e_s], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e["value"] = world * args.steps / float(t.item())

    cpu = None
    rf_host_full = rf0.cpu().numpy()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(frame, os.cpu_count() or 1, rf_host_full)

    configs = None
    if world == 1 and not args.no_configs:
        torch.cuda.empty_cache()
        configs = run_configs(dev)

    mixed = None
    if world == 1 and not args.no_mixed:
        eng.close()
        del rfs, rf0, value, factor, grid, sig
        torch.cuda.empty_cache()
        mixed = run_mixed(dev)

    single = None
    if world == 1 and not args.no_single:
        torch.cuda.empty_cache()
        single = run_single(dev)

    two_medium = None
    if world == 1 and not args.no_two_medium:
        torch.cuda.empty_cache()
        two_medium = run_two_medium(dev)

    if rank == 0:
        fps = world * args.steps / (total_ms * 1e-3)
        line = {
            "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": spec.storage if spec.storage != "f32" else "f32",
            "data": "synthetic (seeded point + speckle scatterers)",
            "config": _config(frame, desc, spec.storage),
            "implementation": {"das_kernel": ("plain" if das_cfg["variant"] == 0 else
                               ("staged" if das_cfg["variant"] == 1 else "receiver-group")
                               + f" (tile {64 if das_cfg['variant'] >= 3 else 32}x"
                               + f"{das_cfg['tile_rows'] * (2 if das_cfg['variant'] == 4 else 1)}, "
                               + f"{das_cfg['stages']} x {das_cfg['stage_bytes']} B stages"
                               + (", autotuned)" if args.autotune else ")")),
                               "frames_in_flight": f"{args.pipeline} contexts on {args.pipeline} streams take the "
                                                   "frames in turn",
                               "parallelism": f"replicas x{world}"},
            "voxels_per_s": fps * frame.npix,
            "latency_ms": {"p50": float(np.percentile(per_step, 50)), "p99": float(np.percentile(per_step, 99))},
            "kernels_ms": {"prep": prep_ms, "das": das_ms},
            "roofline": {"bound": "hbm", "kernel": top[0], "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                         "algorithmic_bytes": top[2]},
            "das_gathers_per_s": gathers / (das_ms * 1e-3),
            "das_onchip": onchip,
            "clocks": clk, "e2e": e2e, "gpu_launches": 2 * args.steps, "cpu_baseline": cpu,
            "configs": configs, "mixed": mixed, "single": single, "two_medium": two_medium,
        }
        line["summary"] = _summary(line)   # last key: the summary the record's tail keeps
        print(json.dumps(line), flush=True)
    eng.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def staged_bytes_model(frame, tile_cols: int, tile_rows: int, esize: int) -> float:
    """Bytes the staged delay-and-sum copies from L2 into shared memory per
    frame: for every pixel tile and (tx, rx) pair, the sample window
    [floor(min tx + min rx), floor(max tx + max rx) + 1] of the tile's
    delays, clipped to the A-scan, its start aligned down to 16 bytes and its
    length rounded up to 16 bytes (the producer's rule). Delays in FP32 as the
    kernel computes them."""
    spec = frame.spec
    L = spec.num_samples * spec.upsampling
    inv = np.float32(spec.sampling_frequency * spec.upsampling / spec.propagation_speed)
    off = np.float32(spec.sampling_frequency * spec.upsampling * spec.peak_offset / spec.center_frequency)
    g = frame.grid_xyz
    ncols, nrows = g.shape[0], g.shape[1]
    tx = np.asarray(spec.tx_xy, np.float32)
    rx = np.asarray(spec.rx_xy, np.float32)
    align = 16 // esize
    total = 0.0
    for c0 in range(0, ncols, tile_cols):
        for r0 in range(0, nrows, tile_rows):
            pts = g[c0:c0 + tile_cols, r0:r0 + tile_rows].reshape(-1, 3)

            def delays(el):
                d = np.sqrt((pts[None, :, 0] - el[:, None, 0]) ** 2 + (pts[None, :, 1] - el[:, None, 1]) ** 2
                            + pts[None, :, 2] ** 2).astype(np.float32) * inv
                return d.min(1), d.max(1)
            tmin, tmax = delays(tx)
            rmin, rmax = delays(rx)
            tmin, tmax = tmin + off, tmax + off
            lo = np.maximum(np.floor(tmin[:, None] + rmin[None, :]), 0)
            hi = np.minimum(np.floor(tmax[:, None] + rmax[None, :]) + 1, L - 1)
            ok = (lo <= L - 2) & (hi >= 1) & (hi >= lo)
            lo = (lo.astype(np.int64) // align) * align
            nbytes = ((hi.astype(np.int64) - lo + 1) * esize + 15) // 16 * 16
            total += float(nbytes[ok].sum())
    return total


def _summary(line: dict) -> dict:
    """Compact summary of the headline and the mixed-precision / batching /
    serving comparison (target: the FP16 batched serving form at >= 3x the
    frames/s of the plain FP32 GPU form at <= -60 dB against the FP64 oracle)."""
    out = {"cf2d_f32_frames_per_s": line["value"],
           "cf2d_e2e_frames_per_s": (line.get("e2e") or {}).get("value"),
           "kernels_ms": line["kernels_ms"],
           "das_hbm_frac": line["roofline"]["frac"] if line["roofline"]["kernel"] == "das" else None,
           "das_smem_pipe_frac": (line.get("das_onchip") or {}).get("smem_frac")}
    c = line.get("configs")
    if c:
        out["configs"] = {k: {"fps": v["frames_per_s"], "err_db": v["err_db_vs_fp64"]} for k, v in c.items()}
    m = line.get("mixed")
    if m:
        out["mixed_48"] = {
            "plain_f32_direct_kernel_fps": m["plain_f32"]["frames_per_s"],
            "default_f32_per_frame_fps": m["default_f32"]["frames_per_s"],
            "batched_f32_fps": m["batched_f32"]["frames_per_s"],
            "batched_f16_fps": m["batched_f16"]["frames_per_s"],
            "batched_f16_vs_plain_f32": m["speedup_vs_plain_f32"]["batched_f16"],
            "batched_f16_vs_default_f32": m["speedup_vs_default_f32"]["batched_f16"],
            "worst_err_db_f16": m["batched_f16"]["err_db"]}
        sv = m.get("serving")
        if sv:
            sat = {k: sv[k]["rates"][-1] for k in ("batched_f16", "plain_f32", "default_f32")}
            out["serving_2000_per_s"] = {
                k: {"fps": v["frames_per_s"], "p50_ms": v["p50_ms"], "p99_ms": v["p99_ms"]} for k, v in sat.items()}
            out["serving_f16_vs_plain_f32"] = sv["speedup_at_saturation"]
            out["serving_f16_vs_default_f32"] = sv["speedup_at_saturation_vs_default_f32"]
            out["serving_worst_err_db_f16"] = sat["batched_f16"].get("err_db")
    return out


def _db(err: float, peak: float) -> float:
    return float(20.0 * np.log10(max(err, 1e-30) / max(peak, 1e-30)))


def _sample_idx(img: np.ndarray, n_top: int, n_rand: int, seed: int) -> np.ndarray:
    """Flat indices of the n_top brightest points of an image and n_rand random ones."""
    flat = np.abs(img).reshape(-1)
    n_top = min(n_top, flat.size)
    top = np.argpartition(flat, -n_top)[-n_top:]
    rest = np.random.default_rng(seed).choice(flat.size, min(n_rand, flat.size), replace=False)
    return np.unique(np.concatenate([top, rest]))


def _fp64_refs(frames, rfs_host, images, threads, n_top=64, n_rand=192):
    """FP64 oracle values at sampled points of every frame: the brightest
    points of a GPU image of the frame and random ones (the oracle prepares
    every A-scan of the frame). Returns {i: (flat indices, values)}."""
    import oracle
    refs = {}
    for i, fr in enumerate(frames):
        idx = _sample_idx(images[i], n_top, n_rand, seed=100 + i)
        pts = fr.grid_xyz.reshape(-1, 3)[idx][:, None, :]
        v, _, _ = oracle.process(_oracle_spec(fr.spec, threads), rfs_host[i].astype(np.float64), pts,
                                 dtype=np.float64)
        refs[i] = (idx, v[:, 0])
    return refs


def _worst_db(refs, images) -> float:
    """Worst peak-relative error (dB) over every frame, at the sampled points."""
    worst = -1e9
    for i, (idx, ref) in refs.items():
        v = np.asarray(images[i], np.float64).reshape(-1)[idx]
        worst = max(worst, _db(float(np.abs(v - ref).max()), float(np.abs(ref).max())))
    return worst


def _time_frame(dev, frame, storage: str, reps: int):
    """One frame of the workload through usgb_process_device with the
    context's default kernels, RF resident: median ms per frame over `reps`
    CUDA-event-timed frames after 3 warm-up frames; returns (ms, image, host RF)."""
    import torch
    from us_lab4a_gb300 import StaEngine, workloads
    fr = workloads.with_storage(frame, storage) if storage != frame.spec.storage else frame
    rf = fr.make_rf_torch(dev)
    g = torch.as_tensor(fr.grid_xyz, device=dev)
    stream = torch.cuda.current_stream(dev)
    with StaEngine(fr.spec) as eng:
        eng.set_stream(stream)
        eng.set_grid_device(g)
        v = torch.empty(fr.grid_xyz.shape[:2], device=dev)
        f = torch.empty_like(v)
        for _ in range(3):
            eng.process_device(rf, v, f)
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            eng.process_device(rf, v, f)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        eng.synchronize()
        img = v.cpu().numpy()
    return statistics.median(ts), img, rf.cpu().numpy()


def run_configs(dev, reps: int = 10):
    """The other benchmark configurations at their full sizes, one frame at a
    time with the default kernels: the 32-element CPU configuration (FP32,
    whole image against the FP64 oracle, the CPU oracle timed on the whole
    frame) and the 16 x 16 matrix array (FP16 and BF16 storage against the
    FP64 oracle at sampled voxels; the oracle prepares all 65 536 A-scans)."""
    from us_lab4a_gb300 import workloads
    import oracle
    threads = os.cpu_count() or 1
    out = {}
    fr = workloads.plain2d()
    ms, img, rf = _time_frame(dev, fr, "f32", reps)
    t0 = time.perf_counter()
    ref, _, _ = oracle.process(_oracle_spec(fr.spec, threads), rf.astype(np.float64), fr.grid_xyz, dtype=np.float64)
    t_ref = time.perf_counter() - t0
    cpu = time_oracle_frames(fr, rf, threads, 1, 2)
    out["plain2d_f32"] = {
        "workload": "32-element linear array, 2048 samples @40 MHz, 4x, rectangular, no CF, 128x256 grid",
        "frames_per_s": 1e3 / ms, "ms_per_frame": ms, "voxels_per_s": 1e3 / ms * fr.npix,
        "err_db_vs_fp64": _db(float(np.abs(img.astype(np.float64) - ref).max()), float(np.abs(ref).max())),
        "err_points": "every grid point",
        "cpu_oracle": {"frames_per_s": 1.0 / statistics.mean(cpu), "cores": threads, "kind": "port",
                       "sample": "whole frames, FP32 oracle, 1 warm-up + 2 timed"},
        "fp64_oracle_s": t_ref}
    fr = workloads.matrix3d()
    idx = ref = None
    for storage in ("f16", "bf16"):
        ms, img, rf = _time_frame(dev, fr, storage, reps)
        if ref is None:   # the same sampled voxels for both storage types (the RF is the same)
            idx = _sample_idx(img, 256, 1792, seed=7)
            pts = fr.grid_xyz.reshape(-1, 3)[idx][:, None, :]
            ref, _, _ = oracle.process(_oracle_spec(fr.spec, threads), rf.astype(np.float64), pts, dtype=np.float64)
            ref = ref[:, 0]
        v = img.reshape(-1)[idx].astype(np.float64)
        out[f"matrix3d_{storage}"] = {
            "workload": "16x16 matrix array (pitch 0.3 mm), 1024 samples @24 MHz, 4x, PCF, 64x64x128 voxels",
            "frames_per_s": 1e3 / ms, "ms_per_frame": ms, "voxels_per_s": 1e3 / ms * fr.npix,
            "err_db_vs_fp64": _db(float(np.abs(v - ref).max()), float(np.abs(ref).max())),
            "err_points": f"{idx.size} voxels (the 256 brightest of the GPU image and random ones)"}
    return out


def run_mixed(dev, num_frames: int = 48, reps: int = 2):
    """The mixed-size workload: `num_frames` frames (elements {32, 64, 96,
    128}, samples {1024, 2048, 4096} at 40 MHz, grids {128x128, 256x256,
    512x1024}, PCF on or off, 4x upsampling), every frame's RF resident.

    plain_f32    frames/s of the plain FP32 form: one frame at a time, the
                 direct delay-and-sum kernel (one thread per grid point, both
                 taps gathered from global memory);
    default_f32  one frame at a time with the library's default FP32 kernels
                 (staged receiver-group delay-and-sum, tile shape chosen per
                 grid);
    batched_*    frames/s of all frames in one persistent preparation launch +
                 one persistent staged delay-and-sum launch, replayed from a
                 CUDA graph, tile shape autotuned on the batch;
    serving      run_serving(): the serving configuration (these frames plus
                 large ones as Poisson streams) through the continuous-batching
                 loop;
    err_db       worst peak-relative error over every frame against the FP64
                 oracle, at the 64 brightest and 192 random grid points of
                 each frame."""
    import torch
    from dataclasses import replace
    from us_lab4a_gb300 import StaEngine, workloads
    from us_lab4a_gb300.batch import Batch
    from us_lab4a_gb300.batch import BatchItem
    threads = os.cpu_count() or 1
    s = torch.cuda.Stream(device=dev)
    frames = workloads.mixed(num_frames, storage="f16")
    with torch.cuda.stream(s):
        rfs = [fr.make_rf_torch(dev) for fr in frames]
        grids = [torch.as_tensor(fr.grid_xyz, device=dev) for fr in frames]
    s.synchronize()
    gathers = sum(fr.npix * fr.spec.num_tx * fr.spec.num_rx for fr in frames)

    def items_for(storage, plain):
        items = []
        for fr, rf, g in zip(frames, rfs, grids):
            e = StaEngine(replace(fr.spec, storage=storage))
            e.set_stream(s)
            if plain:
                e.set_das_variant(0)
            e.set_grid_device(g)
            v = torch.empty(fr.grid_xyz.shape[:2], device=dev)
            items.append(BatchItem(e, rf, v, torch.empty_like(v)))
        return items

    def timed(fn):
        fn()
        s.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            fn()
        e1.record(s)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    def images(items):
        return [it.value.cpu().numpy() for it in items]

    out = {"workload": f"{num_frames} mixed-size frames (elements 32-128, 1024-4096 samples @40 MHz, 4x, "
                       f"grids 128x128 / 256x256 / 512x1024, PCF on/off), RF resident",
           "gathers": gathers}
    per_frame = lambda items: [it.engine.process_device(it.rf, it.value, it.factor) for it in items]
    plain = items_for("f32", plain=True)
    ms = timed(lambda: per_frame(plain))
    plain_img = images(plain)
    for it in plain:
        it.engine.close()
    del plain
    refs = _fp64_refs(frames, [rf.cpu().numpy() for rf in rfs], plain_img, threads)
    out["plain_f32"] = {"frames_per_s": num_frames * 1e3 / ms, "ms_per_pass": ms,
                        "err_db": _worst_db(refs, plain_img)}
    default = items_for("f32", plain=False)
    ms = timed(lambda: per_frame(default))
    out["default_f32"] = {"frames_per_s": num_frames * 1e3 / ms, "ms_per_pass": ms,
                          "err_db": _worst_db(refs, images(default))}
    for it in default:
        it.engine.close()
    del default
    best_f16 = None
    for storage in ("f32", "f16"):
        items = items_for(storage, plain=False)
        with Batch(num_frames, 128) as b:
            cfg, _ = b.autotune(items, s)
            ms = timed(lambda: b.run(items, s, use_graph=True))
            out[f"batched_{storage}"] = {"frames_per_s": num_frames * 1e3 / ms, "ms_per_pass": ms,
                                         "das_config": list(cfg), "err_db": _worst_db(refs, images(items))}
        for it in items:
            it.engine.close()
        if storage == "f16":
            best_f16 = cfg
    torch.cuda.synchronize(dev)
    out["err_db_frames"] = f"all {num_frames} frames, 64 brightest + 192 random grid points each, FP64 oracle"
    out["serving"] = run_serving(dev, frames, rfs, refs, best_f16, threads)
    base, dflt = out["plain_f32"]["frames_per_s"], out["default_f32"]["frames_per_s"]
    out["speedup_vs_plain_f32"] = {"batched_f16": out["batched_f16"]["frames_per_s"] / base,
                                   "batched_f32": out["batched_f32"]["frames_per_s"] / base,
                                   "default_f32": dflt / base}
    out["speedup_vs_default_f32"] = {"batched_f16": out["batched_f16"]["frames_per_s"] / dflt,
                                     "batched_f32": out["batched_f32"]["frames_per_s"] / dflt}
    return out


def run_serving(dev, frames, rfs, refs, das_config, threads, rates=(50.0, 200.0, 2000.0), n_large=5):
    """The serving configuration: the mixed-size frames plus ~10 % large frames
    (128 elements, 4096 samples, 8x, 1024 x 1024, Blackman, SCF) arriving as a
    Poisson stream at each rate in `rates`, RF in pinned host memory, images
    back in host memory, HBM budget 150 GB. The continuous-batching loop with
    FP16 storage and batched graph launches against the same loop serving the
    plain FP32 form (one frame at a time, direct kernel) and the per-frame
    FP32 form on the library's default kernels. Latency = arrival to image in
    host memory. err_db: worst over every frame (mixed and large) against the
    FP64 oracle at sampled points."""
    import torch
    from dataclasses import replace
    from us_lab4a_gb300 import StaEngine, workloads
    from us_lab4a_gb300.serving import Request, ServingLoop, poisson_arrivals
    large = [workloads.large_serving_frame(seed=1004 + i, storage="f16") for i in range(n_large)]
    allf = list(frames) + large
    large_rf = [fr.make_rf_torch(dev) for fr in large]
    host_rf = [rf.cpu().pin_memory() for rf in rfs] + [rf.cpu().pin_memory() for rf in large_rf]
    # FP64 oracle references of the large frames (sample points from an FP32 image of each).
    large_img = []
    for fr, rf in zip(large, large_rf):
        with StaEngine(replace(fr.spec, storage="f32")) as e:
            g = torch.as_tensor(fr.grid_xyz, device=dev)
            e.set_grid_device(g)
            v = torch.empty(fr.grid_xyz.shape[:2], device=dev)
            f = torch.empty_like(v)
            e.process_device(rf, v, f)
            e.synchronize()
            large_img.append(v.cpu().numpy())
    del large_rf
    lrefs = _fp64_refs(large, [h.numpy() for h in host_rf[len(frames):]], large_img, threads)
    all_refs = dict(refs)
    all_refs.update({len(frames) + i: r for i, r in lrefs.items()})
    order = np.random.default_rng(12).permutation(len(allf))  # large frames spread through the stream
    out = {"workload": f"{len(frames)} mixed-size frames + {n_large} frames of 128 elements, 4096 samples, 8x, "
                       f"1024x1024, SCF; Poisson arrivals; host RF in, host image out",
           "frames": len(allf), "hbm_budget_gb": 150}
    forms = (("batched_f16", "f16", False, False), ("plain_f32", "f32", True, False),
             ("default_f32", "f32", False, True))
    for name, storage, plain, per_frame in forms:
        loop = ServingLoop(hbm_budget_bytes=150 << 30, max_batch=len(allf), max_elements=128,
                           das_config=None if (plain or per_frame) else das_config, device=dev, plain=plain,
                           per_frame=per_frame)

        def requests(rate):
            arr = poisson_arrivals(len(allf), rate, seed=11)
            return [Request(int(i), replace(allf[i].spec, storage=storage), allf[i].grid_xyz, host_rf[i], float(t))
                    for i, t in zip(order, arr)]
        loop.run(requests(max(rates)), keep_images=False)  # resident slots, captured graphs
        per_rate = []
        for rate in rates:
            reqs = requests(rate)
            st = loop.run(reqs, keep_images=(rate == max(rates)))
            row = {"arrival_rate": rate, "frames_per_s": st["frames_per_s"], "p50_ms": st["p50_ms"],
                   "p99_ms": st["p99_ms"], "batches": st["batches"], "mean_batch": st["mean_batch"]}
            if rate == max(rates):
                by_id = {r.rid: r.value for r in reqs}
                row["err_db"] = _worst_db(all_refs, by_id)
            per_rate.append(row)
        out[name] = {"rates": per_rate, "peak_resident_gb": loop.peak_bytes / 1e9}
        loop.close()
    sat = {k: out[k]["rates"][-1] for k, _, _, _ in forms}
    out["speedup_at_saturation"] = sat["batched_f16"]["frames_per_s"] / sat["plain_f32"]["frames_per_s"]
    out["speedup_at_saturation_vs_default_f32"] = (sat["batched_f16"]["frames_per_s"]
                                                   / sat["default_f32"]["frames_per_s"])
    out["err_db_frames"] = f"all {len(allf)} frames at 2000 arrivals/s, 64 brightest + 192 random points each"
    return out


SINGLE_GRID = (96, 96, 192)   # x, y, z points over x, y in +-4 mm and z in 5-25 mm


def _single_case(dev, name: str, storage: str, reps: int, threads: int):
    """One single-term 3D workload: frames/s with the RF resident, terms/s,
    error against the FP64 oracle on three grid columns, and the FP32 oracle
    on those columns scaled to the frame (CPU baseline)."""
    import oracle
    import torch
    from us_lab4a_gb300 import SingleEngine, native, synth
    from us_lab4a_gb300.config import element_positions_matrix, tx_3d_focus_delay
    from us_lab4a_gb300.workloads import grid_xyz3
    fs, c, fc, ns, U = 40e6, 1540.0, 5e6, 2048, 4
    nx = 16 if name == "synthy" else 32
    el = element_positions_matrix(0.3e-3, nx, 0.0, 0.3e-3, nx, 0.0, np.float32)
    n = el.shape[0]
    gx, gy, gz = SINGLE_GRID
    grid = grid_xyz3(-4e-3, 4e-3, gx, -4e-3, 4e-3, gy, 5e-3, 25e-3, gz).astype(np.float32).reshape(gx * gy, gz, 3)
    rng = np.random.default_rng(2024)
    scat = synth.point_scatterers(rng, 40, (-4e-3, 4e-3), (6e-3, 24e-3), y_range=(-4e-3, 4e-3))
    nacq = 16 if name == "synthy" else 1
    mode = {"t1r1": native.USGB_SINGLE_T1R1_SAFT, "tnrn": native.USGB_SINGLE_TNRN,
            "synthy": native.USGB_SINGLE_SYNTH_Y_TNRN}[name]
    focus = (0.0, 0.0, -10e-3)
    if name == "t1r1":
        rfs = [synth.synth_rf_pairs_torch(el, el, scat, fs, c, fc, ns, 5, device=dev)]
        tx, apod, ys = el, None, [0.0]
    else:
        src = np.array([[focus[0], focus[1]]], np.float32)
        ys = [0.2e-3 * (a - (nacq - 1) / 2) for a in range(nacq)]
        rfs = [synth.synth_rf_torch(src, el + np.array([0.0, y], np.float32), scat, fs, c, fc, ns, 5 + a,
                                    device=dev)[0] for a, y in enumerate(ys)]
        tx, apod = el[:1], np.hanning(n + 2)[1:-1].astype(np.float32)
    delays = tx_3d_focus_delay(*focus, c, el) if name != "t1r1" else None
    eng = SingleEngine(mode, tx, el, ns, U, fs, c, fc, 1.5, 0.0, rx_apod=apod, coherence="pcf", pcf_gamma=1.0,
                       storage=storage, max_acquisitions=nacq if name == "synthy" else 0)
    if delays is not None:
        eng.set_tx_delays(*focus, delays)
    stream = torch.cuda.Stream()
    eng.set_stream(stream)
    eng.set_grid_device(torch.as_tensor(grid, device=dev))
    value = torch.empty(grid.shape[:2], device=dev)
    factor = torch.empty_like(value)

    added = []  # RF index of every acquisition added, in order

    def add(k):
        eng.add_acquisition_device(rfs[k % nacq], ys[k % nacq])
        added.append(k % nacq)

    def frame(k):
        if name == "synthy":
            # A new acquisition arrives and the window of the last nacq is imaged.
            add(k)
            last = len(added) - 1
            eng.process_window_device(last - nacq + 1, last, value, factor)
        else:
            eng.process_device(rfs[0], value, factor)

    with torch.cuda.stream(stream):
        if name == "synthy":
            for k in range(nacq):
                add(k)
        for k in range(3):
            frame(k)
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(reps):
            frame(k)
        e1.record(stream)
        e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    order = added[-nacq:] if name == "synthy" else [0]   # RF of each acquisition of the last window
    img = value.cpu().numpy()
    eng.close()
    cols = np.array([gx * gy // 2 + gy // 2, gx * gy // 3, 7 * gx * gy // 8])
    pts = grid[cols]
    rf_host = np.stack([rfs[a].cpu().numpy() for a in order])
    kw = dict(tx_xy=tx, rx_xy=el, num_samples=ns, upsampling=U, sampling_frequency=fs, propagation_speed=c,
              center_frequency=fc, peak_offset=1.5, rx_apod=apod, cf=1, pcf_gamma=1.0, nthreads=threads)
    if name != "t1r1":
        kw.update(focus=focus, first_tx_delay=float(delays[0]))
    if name == "synthy":
        kw["acq_y"] = np.asarray([ys[a] for a in order], np.float32)
    spec = oracle.SingleSpec(mode=mode, **kw)
    v64, _, _ = oracle.single(spec, rf_host, pts, dtype=np.float64)
    err_db = _db(float(np.abs(img[cols] - v64).max()), float(np.abs(v64).max()))
    # Preparation alone (one grid point), best of two; then preparation plus
    # 24 grid columns, enough points that the imaging part is most of the
    # second timing (a difference of two preparation-dominated timings is
    # noise).
    t_prep = float("inf")
    for _ in range(2):
        t0 = time.perf_counter()
        oracle.single(spec, rf_host, pts[:1, :1], dtype=np.float32)
        t_prep = min(t_prep, time.perf_counter() - t0)
    tcols = np.linspace(0, grid.shape[0] - 1, 24).astype(int)
    tpts = grid[tcols]
    t0 = time.perf_counter()
    oracle.single(spec, rf_host, tpts, dtype=np.float32)
    t_all = time.perf_counter() - t0
    t_das = max(t_all - t_prep, 0.5 * t_all) / (tpts.shape[0] * tpts.shape[1])
    npix = grid.shape[0] * grid.shape[1]
    # One frame of the CPU form prepares one acquisition and images the window.
    cpu_frame = t_prep / nacq + t_das * npix
    terms = npix * n * nacq
    return {"frames_per_s": 1e3 / ms, "ms_per_frame": ms, "terms_per_s": terms / (ms * 1e-3),
            "err_db_vs_fp64": err_db,
            "cpu_oracle": {"frames_per_s": 1.0 / cpu_frame, "cores": threads, "kind": "port",
                           "sample": f"FP32 oracle: preparation of {n * nacq} A-scans and {tpts.shape[0] * tpts.shape[1]}"
                                     f" grid points, scaled to {npix} points"}}


def run_single(dev, reps: int = 20):
    """The single-term 3D processors (T1R1 SAFT, TnRn, synthetic-y TnRn), PCF."""
    threads = os.cpu_count() or 1
    out = {"workload": ("T1R1 SAFT and TnRn (diverging, focus z = -10 mm): 32 x 32 matrix array (1024 elements); "
                        "synthetic y: 16 x 16 array, window of 16 acquisitions 0.2 mm apart in y; 2048 samples "
                        f"@40 MHz, 4x, PCF, grid {SINGLE_GRID[0]}x{SINGLE_GRID[1]}x{SINGLE_GRID[2]}; RF resident; "
                        "the prepared signals (<= 67 MB) stay in L2 between preparation and delay-and-sum")}
    for name in ("t1r1", "tnrn", "synthy"):
        for storage in ("f32", "f16"):
            out[f"{name}_{storage}"] = _single_case(dev, name, storage, reps, threads)
    return out


_TM_ORACLE = {}   # one_tx -> (FP64 oracle image of the sampled columns, CPU seconds per frame)


def _two_medium_case(dev, one_tx: bool, storage: str, reps: int, threads: int):
    """Two-medium imaging of the cylinder scene: GPU frames/s with the RF
    resident, error against the FP64 oracle on 8 columns, and the FP32 oracle
    (its fixed preparation cost plus the per-column cost scaled to the grid)
    as the CPU baseline."""
    import oracle
    import torch
    from us_lab4a_gb300 import TwoMediumEngine, TwoMediumSTAConfiguration, workloads
    sc = workloads.two_medium_scene(one_tx)
    cfg = TwoMediumSTAConfiguration(num_elements=sc.num_elements, num_elements_mux=sc.num_elements_mux,
                                    pitch=sc.pitch, center_frequency=sc.center_frequency,
                                    propagation_speed_1=sc.propagation_speed_1,
                                    propagation_speed_2=sc.propagation_speed_2,
                                    sampling_frequency=sc.sampling_frequency)
    eng = TwoMediumEngine(cfg, sc.rf.shape[0], sc.rf.shape[1], sc.num_samples, sc.upsampling, coherence="pcf",
                          max_fermat_block_size=sc.max_fermat_block_size, peak_offset=sc.peak_offset,
                          signal_start_offset=sc.signal_start_offset, storage=storage)
    stream = torch.cuda.Stream()
    eng.set_stream(stream)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a, np.float32), device=dev)
    rf, ifxz, apod, grid = t(sc.rf), t(sc.interface_xz), t(sc.rx_apod), t(sc.grid_xz)
    ncols, nrows = sc.grid_xz.shape[:2]
    out = torch.empty((ncols, nrows, 2), device=dev)
    with torch.cuda.stream(stream):
        for _ in range(3):
            eng.process_device(rf, sc.steps, ifxz, apod, grid, out)
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            eng.process_device(rf, sc.steps, ifxz, apod, grid, out)
        e1.record(stream)
        e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    img = out.cpu().numpy().view(np.complex64)[..., 0]
    eng.close()
    spec = oracle.TwoMediumSpec(
        num_elements=sc.num_elements, num_elements_mux=sc.num_elements_mux, pitch=sc.pitch,
        center_frequency=sc.center_frequency, propagation_speed_1=sc.propagation_speed_1,
        propagation_speed_2=sc.propagation_speed_2, sampling_frequency=sc.sampling_frequency,
        num_samples=sc.num_samples, upsampling=sc.upsampling, steps=sc.steps, interface_xz=sc.interface_xz,
        rx_apod=sc.rx_apod, max_fermat_block_size=sc.max_fermat_block_size, peak_offset=sc.peak_offset,
        signal_start_offset=sc.signal_start_offset, cf=1, pcf_gamma=1.0, nthreads=threads)
    cols = np.linspace(0, ncols - 1, 8).astype(int)
    sub = sc.grid_xz[cols]
    if one_tx not in _TM_ORACLE:
        ref64 = oracle.two_medium(spec, sc.rf, sub, dtype=np.float64)
        t0 = time.perf_counter()
        oracle.two_medium(spec, sc.rf, sc.grid_xz[:1, :2], dtype=np.float32)   # preparation (+ 2 points)
        t_prep = time.perf_counter() - t0
        t0 = time.perf_counter()
        oracle.two_medium(spec, sc.rf, sub, dtype=np.float32)
        t_cols = max(time.perf_counter() - t0 - t_prep, 1e-9) / len(cols)
        _TM_ORACLE[one_tx] = (ref64, t_prep + t_cols * ncols)
    ref64, cpu_frame = _TM_ORACLE[one_tx]
    err_db = _db(float(np.abs(img[cols] - ref64).max()), float(np.abs(ref64).max()))
    gathers = int(sum((s[3] - s[2] + 1) for s in sc.steps)) * sc.num_elements * ncols * nrows
    return {"frames_per_s": 1e3 / ms, "ms_per_frame": ms, "gathers_per_s": gathers / (ms * 1e-3),
            "err_db_vs_fp64": err_db,
            "cpu_oracle": {"frames_per_s": 1.0 / cpu_frame, "cores": threads, "kind": "port",
                           "sample": f"FP32 oracle: preparation of the {int(np.prod(sc.rf.shape[:3]))} A-scans and "
                                     f"{len(cols)} of {ncols} columns, scaled to the grid"}}


def run_two_medium(dev, reps: int = 10):
    """Two-medium imaging (VectorialCombinedTwoMediumImagingProcessor), PCF."""
    threads = os.cpu_count() or 1
    out = {"workload": ("cylinder scene: 64-element linear array (pitch 0.6 mm) in water (1480 m/s) over a "
                        "2700 m/s cylinder (radius 15 mm, top at 15 mm, interface sampled every lambda/4 over "
                        "-170..-10 degrees: 312 points); 32-element sub-aperture in 8 steps, one transmit element "
                        "(onetx) or STA (32 x 32) per step; 2000 samples @40 MHz, 4x, PCF; grid 128 x 256 "
                        "(x -8..8 mm, z 14..40 mm); RF resident; delay search, preparation and image per frame")}
    for one_tx in (True, False):
        for storage in ("f32", "f16"):
            out[("onetx" if one_tx else "sta") + "_" + storage] = _two_medium_case(dev, one_tx, storage, reps, threads)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cf2d", choices=["cf2d", "plain2d", "matrix3d"])
    ap.add_argument("--storage", default="f32", choices=["f32", "f16", "bf16"])
    ap.add_argument("--das", default="auto", choices=["auto", "plain", "staged", "group", "group64", "group64x2"],
                    help="delay-and-sum kernel; auto = autotuned over every kernel and shape")
    ap.add_argument("--tile-rows", type=int, default=4)
    ap.add_argument("--stage-bytes", type=int, default=32768)
    ap.add_argument("--stages", type=int, default=2)
    ap.add_argument("--no-autotune", dest="autotune", action="store_false")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--pipeline", type=int, default=2,
                    help="contexts (and streams) that take the resident frames in turn (1: one frame at a time)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the 48-frame mixed-size / serving section")
    ap.add_argument("--no-single", action="store_true", help="skip the single-term 3D processor section")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the section of the 32-element and 16 x 16 matrix-array configurations")
    ap.add_argument("--no-two-medium", action="store_true", help="skip the two-medium imaging section")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()

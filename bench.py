"""Benchmark: the fused colour chain on one 4096x4096 RGBA8 sRGB image.

Workload (the metric's configuration): sRGB -> linear -> XYZ D65 -> Bradford to
D50 -> Oklab -> L*1.1, C*0.9 -> back -> sRGB RGBA8, seeded gradient + uniform +-16
noise, random alpha.  One step = one pass of the compiled Program over one image.

  value     fused executor (one CUDA-graph-replayed kernel), inputs resident in HBM,
            Mpix/s of source pixels; 4 input/output buffer pairs are rotated (536 MB,
            larger than the 129 MB L2) so no step reads what the previous one left in L2
  e2e       same metric through Executable.run_host (C-ABI zs_run_host) from pinned host
            memory, every step moving the input host->device and the result device->host:
            zero copy (the chain kernel streams host memory over NVLink-C2C), with the staged
            form (H2D copy, kernel, D2H copy in row stripes) reported beside it; two host
            buffer pairs alternate (256 MiB > L2)
  plain     the same Program lowered as plain per-op FP32 CUDA kernels (and FP16)
  roofline  achieved HBM GB/s of the chain kernel (8 algorithmic bytes per pixel)
            against the measured copy bandwidth
  cpu_baseline  the plain per-op FP32 CPU pipeline (oracle port, OpenMP) on a bounded
            sample of the same image

--impl reference times the reference's CPU path restated in C (the oracle port,
all host threads) on the same workload, one bounded sample per step.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W = H = 4096
NPX = W * H
ALGO_BYTES = NPX * 8
METRIC = "Mpix/s fused+batched FP16-store vs plain per-op FP32 on GB300 at ≤1 LSB; %HBM peak"


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def max_over_ranks(dist, value: float, device: str = "cuda") -> float:
    """The slowest rank's figure: every rank contributes its own, every rank gets the max
    (no data path collective: only the timings are exchanged)."""
    if not dist:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seed(rank: int) -> int:
    """Each rank runs its own replica: a different seeded image of the same shape."""
    return 1 + rank


def aggregate_mpix(world: int, npx: int, seconds: float) -> float:
    """Whole-job throughput: the pixels all ranks processed per second of the slowest rank."""
    return world * npx / seconds / 1e6


def _best_of(fn, reps: int = 5) -> float:
    """Best wall time of `reps` runs of fn after one warm-up run."""
    fn()
    best = float("inf")
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        best = min(best, time.perf_counter() - t0)
    return best


def cpu_baseline():
    """The plain per-op FP32 CPU pipeline (oracle port of the reference's per-op shader math,
    one full pass per op): all host cores on the whole 4096x4096 image, and one core on a
    4096x256 band of it; best of 5 after a warm-up each."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle
    import pipelines as P
    from zosimos_gb300.synthetic import srgb_gradient_noise

    oracle.build()
    cores = oracle.max_threads()
    img = srgb_gradient_noise(W, H, seed=1)
    t_all = _best_of(lambda: P.oracle_chain(img, f32=True))
    band = img[:256]
    oracle.set_threads(1)
    try:
        t_one = _best_of(lambda: P.oracle_chain(band, f32=True))
    finally:
        oracle.set_threads(cores)
    return {"value": round(NPX / t_all / 1e6, 3), "unit": "Mpix/s", "cores": cores, "kind": "port",
            "sample": "the whole 4096x4096 RGBA8 image, plain per-op FP32 pipeline (oracle restatement of the "
                      "reference's per-op shader math, OpenMP over rows), best of 5 after a warm-up",
            "one_core": {"value": round(W * 256 / t_one / 1e6, 3), "unit": "Mpix/s", "cores": 1,
                         "sample": "4096x256 band of the same image, best of 5 after a warm-up"}}


def oracle_gate(outputs, img, rows=64):
    """Parity gate of the timed workload (checker only, outside every timed region): sampled
    rows of each 4096x4096 output against the FP64 oracle; returns the largest 8-bit
    difference of the colour channels and whether alpha was carried exactly."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import numpy as np
    import oracle
    import pipelines as P

    oracle.build()
    ys = np.linspace(0, H - 1, rows).astype(np.int64)
    ref = P.oracle_chain(np.ascontiguousarray(img[ys])).reshape(rows, W, 4)
    worst, alpha = 0, True
    for out in outputs:
        got = out.reshape(H, W, 4)[ys]
        worst = max(worst, int(np.abs(got[..., :3].astype(np.int16) - ref[..., :3].astype(np.int16)).max()))
        alpha = alpha and bool((got[..., 3] == img[ys][..., 3]).all())
    return worst, alpha


def run_reference(args, rank, world):
    """The reference's per-op pipeline restated on the CPU (the oracle port: FP32, one full
    pass per op), all host threads, the whole 4096x4096 image per step."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle
    import pipelines as P
    from zosimos_gb300.synthetic import srgb_gradient_noise

    oracle.build()
    cores = oracle.max_threads()
    img = srgb_gradient_noise(W, H, seed=1)
    for _ in range(args.warmup):
        P.oracle_chain(img, f32=True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        P.oracle_chain(img, f32=True)
    el = time.perf_counter() - t0
    mpix = args.steps * NPX / el / 1e6
    line = {"metric": METRIC, "value": round(mpix, 3), "unit": "Mpix/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(el / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "fused colour chain (sRGB->XYZ D65->Bradford D50->Oklab->L*1.1,C*0.9->back->sRGB), "
                                   "4096x4096 RGBA8 sRGB per step, seeded gradient+noise",
                       "pipeline": "plain per-op FP32 CPU (the reference's per-op shader math restated in C)"},
            "cpu_baseline": {"value": round(mpix, 3), "unit": "Mpix/s", "cores": cores, "kind": "port",
                             "sample": "the whole 4096x4096 RGBA8 image per step"},
            "e2e": {"value": round(mpix, 3), "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, dist):
    import ctypes

    import numpy as np
    import torch

    import zosimos_gb300 as zs
    from zosimos_gb300.synthetic import srgb_gradient_noise
    from zosimos_gb300.workloads import color_chain, rgba_bytes

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream()          # a real stream: graphs cannot capture the legacy default stream
    sh = stream.cuda_stream

    img = srgb_gradient_noise(W, H, seed=replica_seed(rank))
    host_in = rgba_bytes(img)

    def lowered(mode, zero_copy=True):
        c, _, _ = color_chain(W, H)
        return zs.Linker.from_included().compile(c).lower_to(
            zs.Capabilities(device=dev, mode=mode, use_graph=True, zero_copy=zero_copy))

    fused = lowered(zs.Mode.Fused)
    staged = lowered(zs.Mode.Fused, zero_copy=False)
    plain = lowered(zs.Mode.PerOpF32)
    plain16 = lowered(zs.Mode.PerOpF16)

    ROT = 4
    ins = [zs.DeviceBuffer(NPX * 4) for _ in range(ROT)]
    outs = [zs.DeviceBuffer(NPX * 4) for _ in range(ROT)]
    for b in ins:
        b.upload(host_in)

    if args.profile:
        # A short, fixed sequence for ncu: 2 warm-up launches then 3 profiled ones of the
        # fused chain, followed by one launch of the plain per-op FP32 program.
        for i in range(5):
            fused.run_device([ins[i % ROT].ptr], [outs[i % ROT].ptr], sh)
        plain.run_device([ins[0].ptr], [outs[1].ptr], sh)
        torch.cuda.synchronize()
        print("profile run done", flush=True)
        return

    # The autotuner times the chain kernel's block sizes on this very image and keeps the
    # fastest (every candidate computes the same bytes); the choice is reported below.
    chain_threads = fused.autotune([ins[0].ptr], [outs[0].ptr], sh, reps=10)
    tune_key = fused.tune_key(zs.Tune.ChainThreads)

    # Outputs of this very workload for the parity gate (checked against the FP64 oracle
    # after timing) and the fused-vs-plain comparison.
    fused.run_device([ins[0].ptr], [outs[0].ptr], sh)
    plain.run_device([ins[0].ptr], [outs[1].ptr], sh)
    torch.cuda.synchronize()
    a = outs[0].download(np.empty((H, W * 4), np.uint8))
    b = outs[1].download(np.empty((H, W * 4), np.uint8))
    max_lsb = int(np.abs(a.astype(np.int16) - b.astype(np.int16)).max())

    def timed(exe, steps, warmup):
        for i in range(warmup):
            exe.run_device([ins[i % ROT].ptr], [outs[i % ROT].ptr], sh)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        k0 = zs.kernel_launch_count()
        e0.record(stream)
        for i in range(steps):
            exe.run_device([ins[i % ROT].ptr], [outs[i % ROT].ptr], sh)
        e1.record(stream)
        torch.cuda.synchronize()
        launches = zs.kernel_launch_count() - k0
        ms = max_over_ranks(dist, e0.elapsed_time(e1))
        return ms / steps, launches

    with ClockSampler(dev) as clocks:
        ms_fused, launches = timed(fused, args.steps, args.warmup)
    ms_plain, _ = timed(plain, max(3, args.steps // 4), args.warmup)
    ms_plain16, _ = timed(plain16, max(3, args.steps // 4), args.warmup)

    # End to end through the C ABI with pinned host buffers: zs_run_host of the lone chain runs
    # zero copy (the kernel streams host memory over NVLink-C2C); the staged form (row stripes
    # of H2D copy, kernel, D2H copy on three streams) is timed beside it.
    lib = zs._lib()
    hins = [lib.zs_host_alloc(NPX * 4) for _ in range(2)]
    houts = [lib.zs_host_alloc(NPX * 4) for _ in range(2)]
    for hin in hins:
        ctypes.memmove(hin, host_in.ctypes.data, NPX * 4)
    inps = [(ctypes.c_void_p * 1)(hin) for hin in hins]
    outps = [(ctypes.c_void_p * 1)(hout) for hout in houts]

    def host_round_trips(exe):
        for i in range(args.warmup):
            zs._check(lib.zs_run_host(exe._h, inps[i % 2], 1, outps[i % 2], 1))
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for i in range(args.steps):
            zs._check(lib.zs_run_host(exe._h, inps[i % 2], 1, outps[i % 2], 1))
        return max_over_ranks(dist, (time.perf_counter() - t0) / args.steps)

    e2e_s = host_round_trips(fused)
    got = np.empty((H, W * 4), np.uint8)
    ctypes.memmove(got.ctypes.data, houts[0], NPX * 4)
    e2e_exact = bool((got == a).all())          # zero-copy result == device-resident result
    e2e_staged_s = host_round_trips(staged)
    for p in hins + houts:
        lib.zs_host_free(p)

    if rank != 0:
        return
    gate_lsb, gate_alpha = oracle_gate([a, got], img)
    if gate_lsb > 1 or not gate_alpha:
        raise SystemExit(f"parity gate failed: {gate_lsb} LSB against the FP64 oracle, alpha exact: {gate_alpha}")
    peak, peak_kind = _peaks()
    mpix = aggregate_mpix(world, NPX, ms_fused * 1e-3)
    achieved = ALGO_BYTES / (ms_fused * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": round(mpix, 1), "unit": "Mpix/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_fused, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (RGBA8 storage)", "data": "synthetic",
        "config": {"workload": "fused colour chain (sRGB->XYZ D65->Bradford D50->Oklab->L*1.1,C*0.9->back->sRGB), "
                               "4096x4096 RGBA8 sRGB per GPU, seeded gradient+noise",
                   "l2": "4 rotating input/output buffer pairs (536 MB) > 129 MB L2",
                   "parallelism": f"replicas x{world}",
                   "launch": "one kernel per step, launched directly with programmatic dependent launch "
                             "(multi-kernel executables replay CUDA graphs)",
                   "autotune": {"chain_threads_per_block": chain_threads,
                                "chain_vectors_per_iteration": fused.get_launch(zs.Tune.ChainVectors),
                                "key": tune_key}},
        "plain_per_op_fp32": {"value": round(aggregate_mpix(world, NPX, ms_plain * 1e-3), 1), "unit": "Mpix/s",
                              "ms_per_step": round(ms_plain, 4), "kernels": plain.kernel_count()},
        "per_op_fp16": {"value": round(aggregate_mpix(world, NPX, ms_plain16 * 1e-3), 1), "unit": "Mpix/s",
                        "ms_per_step": round(ms_plain16, 4), "kernels": plain16.kernel_count()},
        "speedup_vs_plain_fp32": round(ms_plain / ms_fused, 2),
        "parity": {"max_lsb_vs_fp64_oracle": gate_lsb, "alpha_exact": gate_alpha,
                   "sample": "64 evenly spaced rows of the timed 4096x4096 image, fused device-resident and "
                             "zero-copy host outputs", "max_lsb_vs_plain_fp32": max_lsb},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": ALGO_BYTES,
                     "traffic": None,
                     "traffic_source": "not measured in this run: DRAM bytes per launch come from a separate ncu "
                                       "capture (dram__bytes_read.sum + dram__bytes_write.sum over back-to-back "
                                       "launches), kept with the chain kernel's profile summary"},
        "e2e": {"value": round(aggregate_mpix(world, NPX, e2e_s), 1), "unit": "Mpix/s",
                "h2d_bytes_per_step": NPX * 4, "d2h_bytes_per_step": NPX * 4, "ms_per_step": round(e2e_s * 1e3, 3),
                "path": "zs_run_host, pinned host buffers, zero copy: the chain kernel loads and stores host "
                        "memory over NVLink-C2C",
                "equals_device_result": e2e_exact,
                "staged_copies": {"value": round(aggregate_mpix(world, NPX, e2e_staged_s), 1), "unit": "Mpix/s",
                                  "ms_per_step": round(e2e_staged_s * 1e3, 3),
                                  "path": "8 row stripes of H2D copy + kernel + D2H copy on 3 streams"}},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- secondary workloads
# (not the headline line: each prints its own JSON line with fused vs plain per-op FP32)


def _timer(stream):
    import torch

    def timed(fn, steps, warmup):
        for i in range(warmup):
            fn(i)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(steps):
            fn(i)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    return timed


def _clocked(timed, fn, steps, warmup):
    """timed(fn, steps, warmup) with nvidia-smi clocks sampled around it: (ms, clocks)."""
    import torch
    with ClockSampler(torch.cuda.current_device()) as ck:
        ms = timed(fn, steps, warmup)
    return ms, ck.summary()


def _line(name, src_px, algo_bytes, ms_fused, ms_plain, clocks, extra=None):
    """One secondary line: fused Mpix/s (source pixels), the HBM roofline of the fused launch
    (algorithmic bytes = inputs read once + outputs written once, CUDA-event time) and the
    plain per-op FP32 program beside it."""
    peak, kind = _peaks()
    achieved = algo_bytes / (ms_fused * 1e-3) / 1e9
    d = {"workload": name, "metric": "Mpix/s (source pixels)", "unit": "Mpix/s",
         "value": round(src_px / (ms_fused * 1e-3) / 1e6, 1), "ms_per_step": round(ms_fused, 4),
         "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                      "frac": round(achieved / peak, 4), "peak_kind": kind, "algorithmic_bytes_per_launch": algo_bytes,
                      "traffic": None},
         "clocks": clocks}
    if ms_plain is not None:
        d["plain_per_op_fp32"] = {"value": round(src_px / (ms_plain * 1e-3) / 1e6, 1), "ms_per_step": round(ms_plain, 4)}
        d["speedup_vs_plain_fp32"] = round(ms_plain / ms_fused, 2)
    if extra:
        d.update(extra)
    print(json.dumps(d), flush=True)


def workload_blend_resize(args, stream, sh):
    import zosimos_gb300 as zs
    from zosimos_gb300.synthetic import srgb_gradient_noise
    from zosimos_gb300.workloads import blend_resize, rgba_bytes
    timed = _timer(stream)
    c, _, _, _ = blend_resize()
    fused = zs.Linker.from_included().compile(c).lower_to(zs.Capabilities(mode=zs.Mode.Fused))
    plain = zs.Linker.from_included().compile(c).lower_to(zs.Capabilities(mode=zs.Mode.PerOpF32))
    rot = 64          # 64 input sets (268 MB) so the working set does not stay in L2
    a = rgba_bytes(srgb_gradient_noise(512, 512, seed=1, image=0))
    b = rgba_bytes(srgb_gradient_noise(512, 512, seed=1, image=1))
    ins = [(zs.DeviceBuffer(a.nbytes), zs.DeviceBuffer(b.nbytes)) for _ in range(rot)]
    outs = [zs.DeviceBuffer(384 * 384 * 4) for _ in range(rot)]
    for x, y in ins:
        x.upload(a)
        y.upload(b)
    run = lambda exe: (lambda i: exe.run_device([ins[i % rot][0].ptr, ins[i % rot][1].ptr], [outs[i % rot].ptr], sh))
    msf, clocks = _clocked(timed, run(fused), args.steps, args.warmup)
    msp = timed(run(plain), args.steps, args.warmup)
    _line("blend_resize 2x512^2 RGBA8 -> over -> bilinear 384^2 -> RGBA8", 2 * 512 * 512,
          2 * 512 * 512 * 4 + 384 * 384 * 4, msf, msp, clocks,
          {"fused_kernels": fused.kernel_count(), "plain_kernels": plain.kernel_count()})


def workload_resample(args, stream, sh):
    import numpy as np

    import zosimos_gb300 as zs
    from zosimos_gb300.synthetic import linear_gradient_gauss
    from zosimos_gb300.workloads import resample, rotation
    timed = _timer(stream)
    n = 4096 if args.profile else 8192
    img = np.ascontiguousarray(linear_gradient_gauss(n, n, seed=3)).view(np.uint8)
    src = zs.DeviceBuffer(img.nbytes)
    src.upload(img)
    if args.profile:
        # A short, fixed sequence for ncu (4096^2 RGBA16F source, 128 MiB > L2): one fused
        # launch each of Lanczos-3 /2, Lanczos-3 /8 and box /2, then one 17 degree rotation.
        import torch
        for filt, factor in ((zs.Filter.Lanczos3, 2.0), (zs.Filter.Lanczos3, 8.0), (zs.Filter.Box, 2.0)):
            ow = int(round(n / factor))
            c, _, _ = resample(n, n, ow, ow, filt)
            exe = zs.Linker.from_included().compile(c).lower_to(zs.Capabilities(mode=zs.Mode.Fused))
            dst = zs.DeviceBuffer(ow * ow * 8)
            exe.run_device([src.ptr], [dst.ptr], sh)
            torch.cuda.synchronize()
            dst.free()
        c, _, _, _ = rotation(n, n, 17.0)
        exe = zs.Linker.from_included().compile(c).lower_to(zs.Capabilities(mode=zs.Mode.Fused))
        dst = zs.DeviceBuffer(n * n * 8)
        exe.run_device([src.ptr], [dst.ptr], sh)
        torch.cuda.synchronize()
        dst.free()
        print("profile run done", flush=True)
        return
    steps = max(3, args.steps // 10)
    for filt, fname in ((zs.Filter.Lanczos3, "lanczos3"), (zs.Filter.Box, "box")):
        for factor in (2.0, 3.7, 8.0):
            ow = int(round(n / factor))
            c, _, _ = resample(n, n, ow, ow, filt)
            caps = [zs.Capabilities(mode=zs.Mode.Fused), zs.Capabilities(mode=zs.Mode.PerOpF32),
                    zs.Capabilities(mode=zs.Mode.Fused, simt_resample=True)]
            exes = [zs.Linker.from_included().compile(c).lower_to(cp) for cp in caps]
            dst = zs.DeviceBuffer(ow * ow * 8)
            tile = None
            if "tensor cores" in exes[0].describe():
                # the tile width of the tensor-core kernel, tuned on these buffers (outside the
                # timed region; every candidate computes the same bytes)
                exes[0].autotune([src.ptr], [dst.ptr], sh, reps=3)
                tile = exes[0].get_launch(zs.Tune.ResampleTile)
            ms0, clocks = _clocked(timed, lambda i, e=exes[0]: e.run_device([src.ptr], [dst.ptr], sh), steps,
                                   args.warmup)
            ms = [ms0] + [timed(lambda i, e=e: e.run_device([src.ptr], [dst.ptr], sh), steps, args.warmup)
                          for e in exes[1:]]
            tensor = "tensor cores" in exes[0].describe()
            _line(f"resample {fname} 8192^2 RGBA16F /{factor} -> {ow}^2", n * n, n * n * 8 + ow * ow * 8,
                  ms[0], ms[1], clocks,
                  {"kernel": "tcgen05 band MMA + TMEM epilogue" if tensor else "FP32 SIMT tiled",
                   "fused_simt_fp32_ms": round(ms[2], 4),
                   "autotune": {"tile_output_columns": tile}})
            dst.free()
    c, _, _, _ = rotation(n, n, 17.0)
    exes = [zs.Linker.from_included().compile(c).lower_to(zs.Capabilities(mode=m))
            for m in (zs.Mode.Fused, zs.Mode.PerOpF32)]
    dst = zs.DeviceBuffer(n * n * 8)
    ms0, clocks = _clocked(timed, lambda i, e=exes[0]: e.run_device([src.ptr], [dst.ptr], sh), steps, args.warmup)
    ms1 = timed(lambda i, e=exes[1]: e.run_device([src.ptr], [dst.ptr], sh), steps, args.warmup)
    _line("rotate 17 deg bilinear 8192^2 RGBA16F", n * n, 2 * n * n * 8, ms0, ms1, clocks)


def _thumbnail_parity(out, ws, hs, every=64):
    """Checker (outside the timed region): every 64th thumbnail of the timed batch against the
    FP64 oracle; the largest 8-bit difference."""
    import numpy as np
    import torch

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle
    import pipelines as P
    from zosimos_gb300.synthetic import srgb_gradient_noise

    oracle.build()
    torch.cuda.synchronize()
    got = out.download(np.empty((len(ws), 256, 1024), np.uint8))
    idx = list(range(0, len(ws), every))
    ref = P.oracle_thumbnails([srgb_gradient_noise(int(ws[i]), int(hs[i]), seed=4, image=i) for i in idx], 256)
    worst = max(int(np.abs(got[i].astype(np.int16) - r.astype(np.int16)).max()) for i, r in zip(idx, ref))
    if worst > 1:
        raise SystemExit(f"thumbnail parity failed: {worst} LSB against the FP64 oracle")
    return {"max_lsb_vs_fp64_oracle": worst, "sample": f"{len(idx)} of the {len(ws)} thumbnails of the timed batch"}


def workload_thumbnails(args, stream, sh):
    import numpy as np

    import zosimos_gb300 as zs
    from zosimos_gb300.synthetic import srgb_gradient_noise, thumbnail_sizes
    from zosimos_gb300.workloads import color_chain, rgba_bytes
    timed = _timer(stream)
    ws, hs = thumbnail_sizes(1024, seed=4)
    if args.profile:
        ws, hs = ws[:256], hs[:256]     # a short, fixed sequence for ncu: one batch of 256 images
    # Sources: 1024 independently seeded images (seed 4, image i), each in its own tight buffer.
    bufs = []
    for i, (w, h) in enumerate(zip(ws, hs)):
        b = zs.DeviceBuffer(int(w) * int(h) * 4)
        b.upload(rgba_bytes(srgb_gradient_noise(int(w), int(h), seed=4, image=i)))
        bufs.append(b)
    c, _, _ = color_chain(1, 1)
    exe = zs.Linker.from_included().compile(c).lower_to()
    out = zs.DeviceBuffer(1024 * 256 * 256 * 4)
    ptrs, wl, hl = [b.ptr for b in bufs], [int(w) for w in ws], [int(h) for h in hs]
    run = lambda i: exe.batch_thumbnails(ptrs, wl, hl, 256, out.ptr, sh)
    if args.profile:
        import torch
        run(0)
        torch.cuda.synchronize()
        print("profile run done", flush=True)
        return
    rows = exe.autotune_batch_thumbnails(ptrs, wl, hl, 256, out.ptr, sh, reps=2)
    ms, clocks = _clocked(timed, run, max(3, args.steps // 20), args.warmup)
    parity = _thumbnail_parity(out, ws, hs)
    # The same 1024 thumbnails without batching: one ordinary program per image (chain ->
    # box fit -> inscribe onto a transparent canvas -> sRGB8), fused and plain per-op FP32.
    # Each image's executable is timed alone (1 warm-up + 2 launches, CUDA events), so its
    # data is L2-resident when it fits: the per-image sums are lower bounds.
    from zosimos_gb300.workloads import thumbnail
    per = {}
    for mode, key in ((zs.Mode.Fused, "fused"), (zs.Mode.PerOpF32, "plain_fp32")):
        total, launches = 0.0, 0
        for k, (w, h) in enumerate(zip(wl, hl)):
            c, _, _ = thumbnail(w, h, 256)
            one = zs.Linker.from_included().compile(c).lower_to(zs.Capabilities(mode=mode))
            dst = out.ptr + k * 256 * 256 * 4
            total += timed(lambda i, e=one, p=ptrs[k], d=dst: e.run_device([p], [d], sh), 2, 1)
            launches += one.kernel_count()
            del one
        per[key] = (total, launches)
    src_px = int(sum(int(w) * int(h) for w, h in zip(ws, hs)))
    _line("thumbnails 1024 uneven RGBA8 -> colour chain -> box fit 256 -> centred 256^2", src_px,
          src_px * 4 + 1024 * 256 * 256 * 4, ms, per["plain_fp32"][0], clocks,
          {"images": 1024, "source_gpx": round(src_px / 1e9, 3), "launches_per_batch": 1,
           "autotune": {"rows_per_item": rows, "threads_per_block": exe.get_launch(zs.Tune.BatchThreads)}, "graph": "memset + kernel captured once, replayed per batch",
           "parity": parity,
           "plain": "one per-op FP32 program per image", "plain_launches": per["plain_fp32"][1],
           "per_image_fused_ms": round(per["fused"][0], 4), "per_image_fused_launches": per["fused"][1],
           "speedup_vs_per_image_fused": round(per["fused"][0] / ms, 2)})


def workload_loop(args, stream, sh):
    """The reference's one published figure (lib/zosimos/tests/loop.rs:60-98): a 157x151 RGBA8
    sRGB image inscribed onto a 512x512 one by a reused executable, each iteration writing both
    pool images from host memory (uploaded at launch), binding them, stepping to the end,
    retiring the output into the pool and reading it back to host memory.  Quoted there:
    "around 240 fps" (2021, unstated hardware).  Seeded synthetic images of the same sizes."""
    import time

    import zosimos_gb300 as zs
    from zosimos_gb300 import Rectangle
    from zosimos_gb300.synthetic import srgb_gradient_noise
    from zosimos_gb300.workloads import rgba_bytes
    bg = rgba_bytes(srgb_gradient_noise(512, 512, seed=1, image=0))
    fg = rgba_bytes(srgb_gradient_noise(157, 151, seed=1, image=1))
    pool = zs.Pool()
    kb, kf = pool.insert(zs.Descriptor.srgb_rgba8(512, 512), bg), pool.insert(zs.Descriptor.srgb_rgba8(157, 151), fg)
    c = zs.CommandBuffer()
    b, f = c.input(pool.descriptor(kb)), c.input(pool.descriptor(kf))
    o, _ = c.output(c.inscribe(b, Rectangle(0, 0, 157, 151), f))
    exe = zs.Linker.from_included().compile(c).lower_to()

    def once():
        pool.write(kb, bg)
        pool.write(kf, fg)
        env = exe.from_pool(pool)
        env.bind(b, kb)
        env.bind(f, kf)
        x = exe.launch(env)
        while x.is_running():
            x.step()
        k = x.retire_output(o)
        out = pool.read(k)
        pool.remove(k)
        return out

    for _ in range(max(3, args.warmup)):
        once()
    n = 200
    t0 = time.perf_counter()
    for _ in range(n):
        once()
    dt = (time.perf_counter() - t0) / n
    print(json.dumps({"workload": "loop.rs: inscribe 157x151 onto 512x512 RGBA8 sRGB, reused executable, "
                                  "host write + upload + readback per iteration",
                      "metric": "fps", "value": round(1.0 / dt, 1), "unit": "iterations/s",
                      "ms_per_iteration": round(dt * 1e3, 4), "iterations": n,
                      "output_mpix_s": round(512 * 512 / dt / 1e6, 1), "kernels": exe.kernel_count(),
                      "reference_published": {"value": 240, "unit": "fps", "hardware": "unstated (2021, wgpu/Vulkan)",
                                              "source": "lib/zosimos/tests/loop.rs:85-86"},
                      "ratio_vs_published": round(1.0 / dt / 240.0, 1)}), flush=True)


def workload_layers(args, stream, sh):
    import numpy as np

    import zosimos_gb300 as zs
    from zosimos_gb300.synthetic import layer_transforms, premultiplied_layer
    from zosimos_gb300.workloads import layer_stack
    timed = _timer(stream)
    n, w = (8, 4096) if args.profile else (32, 4096)
    distinct = n      # every input its own generated layer (4.3 GB of RGBA16F for 32)
    layers = []
    for i in range(distinct):
        img = np.ascontiguousarray(premultiplied_layer(w, w, seed=5, image=i)).view(np.uint8)
        b = zs.DeviceBuffer(img.nbytes)
        b.upload(img)
        layers.append(b)
    c, _, _ = layer_stack(w, w, layer_transforms(n, seed=5))
    exes = [zs.Linker.from_included().compile(c).lower_to(zs.Capabilities(mode=m))
            for m in (zs.Mode.Fused, zs.Mode.PerOpF32)]
    dst = zs.DeviceBuffer(w * w * 8)
    ins = [layers[i % distinct].ptr for i in range(n)]
    if args.profile:
        # A short, fixed sequence for ncu: one fused launch of an 8-layer stack (8 distinct
        # 4096^2 RGBA16F layers, 1 GiB > L2).
        import torch
        exes[0].run_device(ins, [dst.ptr], sh)
        torch.cuda.synchronize()
        print("profile run done", flush=True)
        return
    steps = max(3, args.steps // 40)
    ms0, clocks = _clocked(timed, lambda i, e=exes[0]: e.run_device(ins, [dst.ptr], sh), steps, args.warmup)
    ms1 = timed(lambda i, e=exes[1]: e.run_device(ins, [dst.ptr], sh), steps, args.warmup)
    _line("layer stack 32 distinct x 4096^2 premultiplied RGBA16F, affine + blend per layer", n * w * w,
          n * w * w * 8 + w * w * 8, ms0, ms1, clocks,
          {"fused_kernels": exes[0].kernel_count(), "plain_kernels": exes[1].kernel_count()})


def run_workloads(args):
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    stream = torch.cuda.Stream()
    names = ["blend_resize", "resample", "thumbnails", "layers", "loop"] if args.workload == "all" else [args.workload]
    for name in names:
        globals()["workload_" + name](args, stream, stream.cuda_stream)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", action="store_true", help="short fixed launch sequence for ncu captures")
    ap.add_argument("--workload", default="chain",
                    choices=["chain", "blend_resize", "resample", "thumbnails", "layers", "loop", "all"],
                    help="chain (default) is the headline line; the others print secondary lines")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.workload != "chain" and args.impl == "ours":
        run_workloads(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        td.init_process_group("nccl")
        dist = td
    try:
        run_ours(args, rank, world, dist)
    finally:
        if dist:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()

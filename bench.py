"""Benchmark of the impulse FFT path on GB300.

Workload (one "step"): the real-input FFT in packed halfcomplex layout
(impulse's ``fft(var openArray[float], forward)``, i.e. PocketFFT
``rfft_forward``) over seeded lengths 2^a 3^b 5^c 7^d 11^e in [64, 65536]
plus the primes 1009, 8191 and 65521 (Bluestein), each length batched to
about 2^24 real elements, values i.i.d. normal(0, 1).  Every length's batch
is one call of ``ig_rfft_exec_device``; a step is one forward transform of
every length.  The FP64 form is the headline; the FP32 form of the same
workload is reported beside it.

Metric: GB/s of algorithmic traffic (one read and one write of the real data
per transform: 2 * sizeof(real) * N bytes per line), with inputs resident in
HBM; ``e2e`` is the same metric through the host-memory C ABI
(``ig_rfft_exec_batch``: host->device copy, transform, device->host copy
inside the timed region).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED = 2
TOTAL_REALS = 1 << 24
PRIMES = [1009, 8191, 65521]


def smooth_numbers(lo, hi):
    out = []
    p2 = 1
    while p2 <= hi:
        p3 = p2
        while p3 <= hi:
            p5 = p3
            while p5 <= hi:
                p7 = p5
                while p7 <= hi:
                    p11 = p7
                    while p11 <= hi:
                        if p11 >= lo:
                            out.append(p11)
                        p11 *= 11
                    p7 *= 7
                p5 *= 5
            p3 *= 3
        p2 *= 2
    return sorted(out)


def workload_lengths(count=32):
    """32 log-uniform draws in [64, 65536] rounded (in log) to the nearest 11-smooth length, + 3 primes."""
    rng = np.random.default_rng(SEED)
    sm = np.array(smooth_numbers(64, 65536), dtype=np.float64)
    logs = np.log(sm)
    out = []
    for u in rng.uniform(math.log(64), math.log(65536), count):
        out.append(int(sm[np.argmin(np.abs(logs - u))]))
    return sorted(set(out)) + PRIMES


def batch_for(n):
    return max(1, int(round(TOTAL_REALS / n)))


def aggregate(ms_local, bytes_local, world, device=None):
    """Max step time over ranks and the whole-job throughput (weak scaling:
    every rank processes the full workload on its own GPU; no data-path
    collective)."""
    ms = float(ms_local)
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * bytes_local / (ms / 1e3) / 1e9


# --------------------------------------------------------------------------
# clocks sampled during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = self.smi_id(gpu_index)
        self.proc = None
        self.lines = []

    @staticmethod
    def smi_id(index):
        """nvidia-smi's --id for torch device `index`: the device UUID, so the
        sampled GPU is this process's even when CUDA_VISIBLE_DEVICES renumbers
        devices; else the physical index mapped through CUDA_VISIBLE_DEVICES."""
        try:
            import torch
            u = str(torch.cuda.get_device_properties(index).uuid)
            if u:
                return u if u.startswith("GPU-") else "GPU-" + u
        except Exception:
            pass
        vis = [v.strip() for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
        return vis[index] if index < len(vis) else str(index)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm), "gpu": self.gpu}


# --------------------------------------------------------------------------
# CPU side: the reference's algorithm restated (oracle port) on host threads
# --------------------------------------------------------------------------
def cpu_sample_run(lengths, min_seconds=10.0, max_passes=400):
    """Time the oracle's threaded halfcomplex transform on a bounded sample of the workload:
    each length at 1/64 of its batch, and at least two lines per host thread (the transform
    threads over lines, as PocketFFT does).  Returns (GB/s, threads, sample description,
    seconds per pass)."""
    from oracle import oracle as O  # CPU-baseline leg only
    if not os.path.exists(O.ORACLE_SO):
        O.build(ref=False)
    lib = O.lib()
    nth = os.cpu_count() or 1
    rng = np.random.default_rng(SEED)
    data = []
    for n in lengths:
        b = min(batch_for(n), max(2 * nth, batch_for(n) // 64))
        data.append((n, b, rng.standard_normal((b, n))))
    bytes_pass = sum(2 * 8 * n * b for n, b, _ in data)
    t0 = time.perf_counter()
    passes = 0
    while True:
        for n, b, x in data:
            # orthonormal scale keeps repeated in-place passes at unit magnitude
            lib.io_rfft_batch(n, b, x.ctypes.data_as(C.POINTER(C.c_double)), n, 1, 1.0 / math.sqrt(n), nth)
        passes += 1
        el = time.perf_counter() - t0
        if el >= min_seconds or passes >= max_passes:
            break
    gbs = bytes_pass * passes / el / 1e9
    sample = (f"{len(lengths)} lengths x max(1/64 of each batch, 2 lines per thread) "
              f"({bytes_pass / 2 / 8 / 1e6:.1f} M reals f64 per pass), {passes} passes, {el:.1f} s, oracle port "
              "(FP64 C restatement of PocketFFT's algorithm; 1.1-1.3x the time of PocketFFT built without SIMD "
              "on the same sample, measured in the build container)")
    return gbs, nth, sample, el / passes


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def run_ours(args, rank, world):
    import torch
    from impulse_gb300 import _lib as L
    from impulse_gb300 import fft as F

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    lib = L.load()
    stream = torch.cuda.current_stream(dev)
    sptr = C.c_void_p(stream.cuda_stream)
    lengths = workload_lengths()

    def make(dtype):
        dt = torch.float64 if dtype == "f64" else torch.float32
        code = L.IG_F64 if dtype == "f64" else L.IG_F32
        g = torch.Generator(device=dev)
        g.manual_seed(SEED)
        items = []
        for n in lengths:
            b = batch_for(n)
            x = torch.randn((b, n), generator=g, device=dev, dtype=dt)
            y = torch.empty_like(x)
            plan = lib.ig_make_rfft_plan(n, code)
            if not plan:
                raise RuntimeError(lib.ig_last_error_string().decode())
            items.append((n, b, x, y, plan))
        return items

    def step(items):
        for n, b, x, y, plan in items:
            rc = lib.ig_rfft_exec_device(plan, x.data_ptr(), y.data_ptr(), b, n, n, 1, 1.0, sptr)
            if rc:
                raise RuntimeError(lib.ig_last_error_string().decode())

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def timed(items, steps, warmup, per_length=False):
        for _ in range(warmup):
            step(items)
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        lib.ig_launch_count(1)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        per = None
        if per_length:
            per = [[torch.cuda.Event(enable_timing=True) for _ in range(len(items) + 1)] for _ in range(steps)]
        ev0.record(stream)
        for s in range(steps):
            if per_length:
                for i, it in enumerate(items):
                    per[s][i].record(stream)
                    step([it])
                per[s][-1].record(stream)
            else:
                step(items)
        ev1.record(stream)
        torch.cuda.synchronize()
        launches = lib.ig_launch_count(0)
        barrier()
        ms = ev0.elapsed_time(ev1)
        per_ms = None
        if per_length:
            per_ms = [sum(per[s][i].elapsed_time(per[s][i + 1]) for s in range(steps)) / steps
                      for i in range(len(items))]
        return ms, launches, per_ms

    def max_over_ranks(v):
        return aggregate(v, 0.0, world, dev)[0]

    # per-length autotuning (outside every timed region): radix order, elements per
    # thread, lines per CTA and the four-step split, kept for the plans made below
    tune_s = None
    if not args.no_autotune:
        t0 = time.perf_counter()
        for code in (L.IG_F64, L.IG_F32):
            for n in lengths:
                F.autotune(n, code, 1)
        torch.cuda.synchronize()
        tune_s = round(time.perf_counter() - t0, 2)

    result = {}
    items64 = make("f64")
    bytes64 = sum(2 * 8 * n * b for n, b, *_ in items64)
    clk = ClockSampler(dev.index)
    clk.start()
    ms64, launches, per_ms = timed(items64, args.steps, args.warmup, per_length=True)
    clocks = clk.stop()
    ms64, _ = aggregate(ms64, bytes64, world, dev)
    step_ms = ms64 / args.steps
    value = world * bytes64 / (step_ms / 1e3) / 1e9

    # FP32 form of the same workload, and its error against the FP64 result
    items32 = make("f32")
    ms32, _, per32 = timed(items32, args.steps, args.warmup, per_length=True)
    ms32 = max_over_ranks(ms32)
    errs = []
    for (n, b, x64, y64, _), (_, _, x32, y32, _) in zip(items64, items32):
        # same seeded input in FP64 for the FP32 error: transform x32 upcast with the FP64 path
        xr = x32[:4].double().contiguous()
        yr = torch.empty_like(xr)
        rc = lib.ig_rfft_exec_device(items64[[i[0] for i in items64].index(n)][4], xr.data_ptr(), yr.data_ptr(),
                                     xr.shape[0], n, n, 1, 1.0, sptr)
        assert rc == 0
        torch.cuda.synchronize()
        d = (y32[:4].double() - yr)
        errs.append((n, float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(yr))))
    bytes32 = sum(2 * 4 * n * b for n, b, *_ in items32)

    # end to end through the host-memory C ABI (pinned host buffers)
    e2e = None
    if not args.no_e2e:
        host = []
        for n, b, x, y, plan in items64:
            h = torch.empty((b, n), dtype=torch.float64, pin_memory=True)
            h.copy_(x.cpu())
            host.append((n, b, h))
        plans = {n: F.FFTPlanReal(n, L.IG_F64) for n, _, _ in host}
        e_steps = max(1, min(args.steps, 5))
        for _ in range(1):
            for n, b, h in host:
                L.check(lib.ig_rfft_exec_batch(plans[n].pocket, h.data_ptr(), b, n, 1, 1.0))
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        for _ in range(e_steps):
            for n, b, h in host:
                L.check(lib.ig_rfft_exec_batch(plans[n].pocket, h.data_ptr(), b, n, 1, 1.0))
        torch.cuda.synchronize()
        el = max_over_ranks(time.perf_counter() - t0)
        hb = sum(8 * n * b for n, b, _ in host)
        e2e = {"value": round(world * bytes64 * e_steps / el / 1e9, 3), "unit": "GB/s",
               "h2d_bytes_per_step": hb, "d2h_bytes_per_step": hb, "steps": e_steps,
               "api": "ig_rfft_exec_batch (host memory, in place)"}

    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    peak = peaks.get("hbm_gbs")
    peak_kind = "measured"
    if not peak:
        peak, peak_kind = 6800.0, "fallback"
    # roofline of the dominant kernel: the lengths whose call is one k_fft_smem
    # launch (counted live); algorithmic bytes / event-timed launch durations
    single = []
    for i, it in enumerate(items64):
        lib.ig_launch_count(1)
        step([it])
        torch.cuda.synchronize()
        if lib.ig_launch_count(0) == 1:
            single.append(i)
    sb = sum(2 * 8 * items64[i][0] * items64[i][1] for i in single)
    st = sum(per_ms[i] for i in single)
    achieved = sb / (st / 1e3) / 1e9 if single else 0.0
    workload_achieved = bytes64 / (sum(per_ms) / 1e3) / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "traffic_ratio.txt")
    if os.path.exists(prof) and single:
        for ln in open(prof):
            if ln.startswith("dram_bytes_per_algorithmic_byte:"):
                traffic = round(float(ln.split(":")[1]) * sb / len(single))
    # compute (issue) roofline of the same kernel: thread instructions per complex point from the
    # ncu capture in profiles/ x complex points per second, against the SM issue peak (4
    # schedulers x 32 lanes per SM per clock) at the sampled SM clock
    compute = None
    ipp = os.path.join(ROOT, "profiles", "instr_per_point.txt")
    if os.path.exists(ipp) and single and clocks.get("sm_mhz"):
        for ln in open(ipp):
            if ln.startswith("df_halfcomplex_4096:"):
                inst = float(ln.split(":")[1])
                sms = torch.cuda.get_device_properties(dev).multi_processor_count
                peak_ti = sms * 4 * 32 * clocks["sm_mhz"] * 1e6 / 1e12
                ach_ti = inst * (achieved * 1e9 / 32.0) / 1e12  # 32 bytes (16 in, 16 out) per complex point
                compute = {"bound": "instruction issue (double-float arithmetic on the FP32 pipes)",
                           "instr_per_complex_point": inst, "achieved": round(ach_ti, 2),
                           "peak": round(peak_ti, 2), "unit": "T thread-instructions/s",
                           "frac": round(ach_ti / peak_ti, 3)}
    slow = [(n, round(2 * 8 * n * b / (t / 1e3) / 1e9, 1)) for (n, b, *_), t in zip(items64, per_ms)]
    result = {
        "metric": "FFT GB/s (halfcomplex real FFT, algorithmic bytes) vs HBM peak",
        "value": round(value, 2),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(step_ms, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded normal(0,1))",
        "config": {"workload": "real-input FFT, packed halfcomplex, f64: "
                               f"{len(lengths)} lengths 2^a3^b5^c7^d11^e in [64,65536] + primes 1009/8191/65521, "
                               "~2^24 reals per length, out of place",
                   "lengths": lengths, "reals_per_step": int(bytes64 / 16),
                   "l2": f"inputs larger than L2 (128 MiB per length, {len(lengths)} lengths per step)",
                   "arith": "double-float butterflies on FP64 data",
                   "autotune_s": tune_s},
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clocks,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "kernel": f"double-float line kernels (k_fft_line halfcomplex, else k_fft_smem), one launch per length ({len(single)} of {len(items64)} lengths)",
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                     else "fallback 6.8 TB/s",
                     "workload_achieved": round(workload_achieved, 1),
                     "compute_roofline": compute,
                     "note": "achieved = algorithmic bytes of the single-launch lengths / their event-timed "
                             "launch durations; traffic = ncu DRAM bytes per algorithmic byte x bytes per launch; "
                             "workload_achieved covers every length, multi-pass ones included"},
        "fp32": {"value": round(world * bytes32 / (ms32 / args.steps / 1e3) / 1e9, 2), "unit": "GB/s",
                 "ms_per_step": round(ms32 / args.steps, 4),
                 "speedup_vs_f64": round(ms64 / ms32, 3),
                 "max_rel_l2_vs_f64": max(e for _, e in errs),
                 "bound_1e-6_log2N": all(e <= 1e-6 * math.log2(n) for n, e in errs),
                 "per_length_gbs": [(n, round(2 * 4 * n * b / (t / 1e3) / 1e9, 1))
                                    for (n, b, *_), t in zip(items32, per32)]},
        "per_length_gbs": slow,
    }
    keep = [] if (rank == 0 and world == 1 and not args.no_cpu) else None
    if not args.no_extra:
        result.update(run_nd(lib, dev, args, peak, keep))
        result["uneven"] = run_uneven(lib, dev, world, args)
        result["conv"] = run_conv(dev, args, peak)
    if rank == 0 and world == 1 and not args.no_cpu:
        gbs, nth, sample, _ = cpu_sample_run(lengths, min_seconds=args.cpu_seconds)
        result["cpu_baseline"] = {"value": round(gbs, 3), "unit": "GB/s", "cores": nth, "kind": "port",
                                  "sample": sample}
        if keep:
            result["cpu_baseline"]["configs_1_3"] = cpu_nd_check(keep)
    return result


def run_uneven(lib, dev, world, args):
    """20,000 complex transforms of uneven lengths (log-uniform, 90 % 7-smooth,
    10 % prime, ~2^28 elements): FP32 through the captured work-list graph vs
    the per-transform launch loop, and FP64 (double-float) through the graph."""
    import torch
    from impulse_gb300 import _lib as L
    from impulse_gb300.batch import MultiFFT, uneven_lengths
    lengths = uneven_lengths()
    tot = sum(lengths)
    s = torch.cuda.Stream(dev)
    g = torch.Generator(device=dev)
    g.manual_seed(4)
    out = {"transforms": len(lengths), "elements": tot}

    def timed(plan, x, y, mode, reps):
        with torch.cuda.stream(s):
            for _ in range(2):
                plan.run(x.data_ptr(), y.data_ptr(), s.cuda_stream, mode)
            s.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s)
            for _ in range(reps):
                plan.run(x.data_ptr(), y.data_ptr(), s.cuda_stream, mode)
            e1.record(s)
            s.synchronize()
        return e0.elapsed_time(e1) / reps

    x32 = torch.complex(torch.randn(tot, generator=g, device=dev), torch.randn(tot, generator=g, device=dev))
    y32 = torch.empty_like(x32)
    t0 = time.perf_counter()
    p32 = MultiFFT(lengths, L.IG_F32)
    out["plan_s_fp32"] = round(time.perf_counter() - t0, 2)
    out["paths"] = p32.info
    ms32 = timed(p32, x32, y32, "graph", max(3, args.steps // 2))
    ms32_loop = timed(p32, x32, y32, "loop", 2)

    def part_ms(plan, x, y, parts, reps=3):
        with torch.cuda.stream(s):
            plan.run_part(x.data_ptr(), y.data_ptr(), parts, s.cuda_stream)
            s.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s)
            for _ in range(reps):
                plan.run_part(x.data_ptr(), y.data_ptr(), parts, s.cuda_stream)
            e1.record(s)
            s.synchronize()
        return round(e0.elapsed_time(e1) / reps, 3)

    # per-path device time of the FP32 plan (each part alone, not in a graph)
    out["fp32_path_ms"] = {"worklist_phase0": part_ms(p32, x32, y32, 1), "worklist_phase1": part_ms(p32, x32, y32, 2),
                           "general": part_ms(p32, x32, y32, 4)}
    x64 = x32.to(torch.complex128)
    y64 = torch.empty_like(x64)
    p64 = MultiFFT(lengths, L.IG_F64)
    ms64 = timed(p64, x64, y64, "graph", max(3, args.steps // 2))
    err = float(torch.linalg.vector_norm(y32.to(torch.complex128) - y64) / torch.linalg.vector_norm(y64))
    out.update({
        "fp32_graph_ms": round(ms32, 3), "fp32_graph_gbs": round(2 * 8 * tot / (ms32 / 1e3) / 1e9, 1),
        "fp32_loop_ms": round(ms32_loop, 3), "graph_vs_loop_speedup": round(ms32_loop / ms32, 2),
        "fp64_graph_ms": round(ms64, 3), "fp64_graph_gbs": round(2 * 16 * tot / (ms64 / 1e3) / 1e9, 1),
        "fp32_vs_fp64_speedup": round(ms64 / ms32, 3),
        "rel_l2_fp32_vs_fp64": err, "bound_1e-6_log2_maxN": err <= 1e-6 * math.log2(max(lengths)),
    })
    del p32, p64, x32, y32, x64, y64
    torch.cuda.empty_cache()
    return out


def run_conv(dev, args, peak):
    """64 images 2048x2048 f32 convolved ('same') with 31x31 filters (one per
    image), zero padded to 4096x4096: forward + backward (adjoints wrt image and
    filter, spectra recomputed)."""
    import torch
    from impulse_gb300.fftconv import FFTConv2d
    B, H, K, P = 64, 2048, 31, 4096
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    x = torch.rand((B, H, H), generator=g, device=dev)
    k = torch.randn((B, K, K), generator=g, device=dev)
    k = k / k.abs().sum(dim=(1, 2), keepdim=True)
    gy = torch.randn((B, H, H), generator=g, device=dev)
    op = FFTConv2d(B, H, H, K, B, torch.float32, recompute=True, pad=(P, P))
    for _ in range(2):
        op.forward(x, k)
        op.backward(gy)
    torch.cuda.synchronize()
    reps = 3
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e2 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        op.forward(x, k)
    e1.record()
    for _ in range(reps):
        op.backward(gy)
    e2.record()
    torch.cuda.synchronize()
    fwd = e0.elapsed_time(e1) / reps
    bwd = e1.elapsed_time(e2) / reps
    io_bytes = 2 * 4 * B * H * H + 4 * B * K * K  # images in, result out, filters
    # FFT-pipeline bytes of one forward call, per image: pad (image in, padded
    # out), 2-D r2c of the padded image and of the padded filter (row pass:
    # reals in, half spectrum out; column pass: half spectrum in and out), the
    # spectrum product (two spectra in, one out), 2-D c2r (column pass, then
    # row pass: half spectrum in, reals out), crop (region in and out)
    real_p, half_p = 4 * P * P, 8 * P * (P // 2 + 1)
    r2c2d = (real_p + half_p) + 2 * half_p
    per_image = (4 * H * H + real_p) + r2c2d + real_p + r2c2d + 3 * half_p + r2c2d + 2 * 4 * H * H
    pipe_gbs = B * per_image / (fwd / 1e3) / 1e9
    del op, x, k, gy
    torch.cuda.empty_cache()
    return {"workload": "64 x 2048^2 f32, 31x31 filter per image, padded to 4096^2", "forward_ms": round(fwd, 2),
            "backward_ms": round(bwd, 2), "images_per_s_fwd_bwd": round(B / ((fwd + bwd) / 1e3), 1),
            "forward_io_gbs": round(io_bytes / (fwd / 1e3) / 1e9, 1),
            "forward_pipeline_bytes": B * per_image, "forward_pipeline_gbs": round(pipe_gbs, 1),
            "forward_pipeline_frac": round(pipe_gbs / peak, 4)}


def _nd_call(lib, kind, code, x, y, axes, fwd, fct, stream):
    """ig_{kind}_device on torch tensors (byte strides from the tensors)."""
    shp = list(y.shape) if kind == "c2r" else list(x.shape)
    si = [st * x.element_size() for st in x.stride()]
    so = [st * y.element_size() for st in y.stride()]
    arr = lambda t, v: (t * len(v))(*v)
    rc = getattr(lib, f"ig_{kind}_device")(code, len(shp), arr(C.c_size_t, shp), arr(C.c_ssize_t, si),
                                           arr(C.c_ssize_t, so), len(axes), arr(C.c_size_t, list(axes)), int(fwd),
                                           x.data_ptr(), y.data_ptr(), float(fct), stream)
    if rc:
        raise RuntimeError(lib.ig_last_error_string().decode())


def _event_ms(fn, reps, stream):
    import torch
    for _ in range(2):
        fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def run_nd(lib, dev, args, peak, keep=None):
    """Configs 1 and 3 through the N-d device entry points (pocketfft::c2c / r2c
    mirrors), device-resident, event-timed.  GB/s counts one read and one write
    of the whole array per call whatever the number of axes (a call that makes
    P passes over HBM is capped at 1/P of the roofline); `launches` is the
    engine's kernel count per call.  `keep` collects (name, input, output,
    axes, kind) on the host for the oracle check of the CPU leg."""
    import torch
    from impulse_gb300 import _lib as L
    stream = torch.cuda.current_stream(dev)
    sp = C.c_void_p(stream.cuda_stream)
    reps = max(3, args.steps)
    g = torch.Generator(device=dev)
    g.manual_seed(1)
    out = {}
    if not args.no_autotune:
        # the complex lengths of configs 1 and 3, tuned like the halfcomplex ones
        from impulse_gb300 import fft as F
        for n, code in ((4096, L.IG_F64), (4096, L.IG_F32), (256, L.IG_F32)):
            F.autotune(n, code, 0)
        F.autotune(4096, L.IG_F32, 1)

    def uniform_c(shape, dt):
        rdt = torch.float64 if dt == torch.complex128 else torch.float32
        return torch.complex(torch.rand(shape, generator=g, device=dev, dtype=rdt) * 2 - 1,
                             torch.rand(shape, generator=g, device=dev, dtype=rdt) * 2 - 1)

    # config 1: c128, N = 4096, 1024 lines (both axis orders) and 16384 lines (2^26 elements)
    c1 = {}
    for name, shape, axes in (("4096x1024_axes0", (4096, 1024), [0]), ("1024x4096_axes1", (1024, 4096), [1]),
                              ("16384x4096_axes1", (16384, 4096), [1])):
        x = uniform_c(shape, torch.complex128)
        y = torch.empty_like(x)
        z = torch.empty_like(x)
        nb = 2 * 16 * x.numel()
        _nd_call(lib, "c2c", L.IG_F64, x, y, axes, True, 1.0, sp)  # plans built outside the count
        torch.cuda.synchronize()
        lib.ig_launch_count(1)
        _nd_call(lib, "c2c", L.IG_F64, x, y, axes, True, 1.0, sp)
        torch.cuda.synchronize()
        launches = int(lib.ig_launch_count(0))
        tf = _event_ms(lambda: _nd_call(lib, "c2c", L.IG_F64, x, y, axes, True, 1.0, sp), reps, stream)
        tb = _event_ms(lambda: _nd_call(lib, "c2c", L.IG_F64, y, z, axes, False, 1.0 / 4096, sp), reps, stream)
        rt = float(torch.linalg.vector_norm(z - x) / torch.linalg.vector_norm(x))
        gf, gb = nb / tf / 1e6, nb / tb / 1e6
        c1[name] = {"forward_ms": round(tf, 4), "backward_ms": round(tb, 4), "forward_gbs": round(gf, 1),
                    "backward_gbs": round(gb, 1), "frac_forward": round(gf / peak, 4),
                    "frac_backward": round(gb / peak, 4), "launches": launches,
                    "round_trip_rel_l2": rt, "round_trip_ok_1e-10": rt <= 1e-10}
        if keep is not None and name != "16384x4096_axes1":
            keep.append(("config1_" + name, x.cpu().numpy(), y.cpu().numpy(), axes, "c2c"))
        del x, y, z
        torch.cuda.empty_cache()
    out["config1"] = {"dtype": "c128 (double-float butterflies)", "api": "ig_c2c_device", **c1}

    # config 3: multi-axis
    c3 = {}
    for name, shape, axes, dt in (("c128_4096x4096_axes01", (4096, 4096), [0, 1], torch.complex128),
                                  ("c64_4096x4096_axes01", (4096, 4096), [0, 1], torch.complex64),
                                  ("c64_256x256x256_axes012", (256, 256, 256), [0, 1, 2], torch.complex64)):
        code = L.IG_F64 if dt == torch.complex128 else L.IG_F32
        x = uniform_c(shape, dt)
        y = torch.empty_like(x)
        nb = 2 * x.element_size() * x.numel()
        _nd_call(lib, "c2c", code, x, y, axes, True, 1.0, sp)
        torch.cuda.synchronize()
        lib.ig_launch_count(1)
        _nd_call(lib, "c2c", code, x, y, axes, True, 1.0, sp)
        torch.cuda.synchronize()
        launches = int(lib.ig_launch_count(0))
        t = _event_ms(lambda: _nd_call(lib, "c2c", code, x, y, axes, True, 1.0, sp), reps, stream)
        c3[name] = {"ms": round(t, 4), "gbs": round(nb / t / 1e6, 1), "frac": round(nb / t / 1e6 / peak, 4),
                    "launches": launches}
        if keep is not None:
            keep.append(("config3_" + name, x.cpu().numpy(), y.cpu().numpy(), axes, "c2c"))
        del x, y
        torch.cuda.empty_cache()
    x = torch.rand((4096, 4096), generator=g, device=dev) * 2 - 1
    y = torch.empty((4096, 2049), dtype=torch.complex64, device=dev)
    z = torch.empty_like(x)
    nb = 4 * x.numel() + 8 * y.numel()
    _nd_call(lib, "r2c", L.IG_F32, x, y, [0, 1], True, 1.0, sp)
    torch.cuda.synchronize()
    lib.ig_launch_count(1)
    _nd_call(lib, "r2c", L.IG_F32, x, y, [0, 1], True, 1.0, sp)
    torch.cuda.synchronize()
    launches = int(lib.ig_launch_count(0))
    t = _event_ms(lambda: _nd_call(lib, "r2c", L.IG_F32, x, y, [0, 1], True, 1.0, sp), reps, stream)
    tb = _event_ms(lambda: _nd_call(lib, "c2r", L.IG_F32, y, z, [0, 1], False, 1.0 / 4096 ** 2, sp), reps, stream)
    rt = float(torch.linalg.vector_norm(z - x) / torch.linalg.vector_norm(x))
    c3["r2c_f32_4096x4096_axes01"] = {"ms": round(t, 4), "gbs": round(nb / t / 1e6, 1),
                                      "frac": round(nb / t / 1e6 / peak, 4), "launches": launches,
                                      "c2r_ms": round(tb, 4), "c2r_gbs": round(nb / tb / 1e6, 1),
                                      "round_trip_rel_l2": rt}
    if keep is not None:
        keep.append(("config3_r2c_f32_4096x4096_axes01", x.cpu().numpy(), y.cpu().numpy(), [0, 1], "r2c"))
    del x, y, z
    torch.cuda.empty_cache()
    out["config3"] = {"api": "ig_c2c_device / ig_r2c_device / ig_c2r_device",
                      "note": "one read + one write of the array credited per call; a call of P passes is "
                              "capped at 1/P of the roofline", **c3}
    return out


def cpu_nd_check(keep):
    """CPU-baseline leg of configs 1 and 3: the oracle on the same inputs on
    all host cores -- its time (GB/s on the same algorithmic bytes) and the
    GPU result's relative L2 error against it."""
    from oracle import oracle as O  # CPU-baseline leg only
    nth = os.cpu_count() or 1
    res = {}
    for name, x, y, axes, kind in keep:
        t0 = time.perf_counter()
        if kind == "c2c":
            want = O.c2c(x.astype(np.complex128), axes, True, nthreads=nth)
        else:
            want = O.r2c(x.astype(np.float64), axes, True, nthreads=nth)
        el = time.perf_counter() - t0
        nb = x.nbytes + y.nbytes
        res[name] = {"cpu_gbs": round(nb / el / 1e9, 3), "cpu_cores": nth, "kind": "port",
                     "gpu_rel_l2_vs_oracle": O.rel_l2(y, want)}
    return res


PROFILE_CASES = {
    # name: (kind, dtype, length, batch)
    "rfft4096_f64": ("r", "f64", 4096, 16384),
    "rfft4096_f32": ("r", "f32", 4096, 32768),
    "c2c4096_f64": ("c", "f64", 4096, 8192),
    "c2c4096_f32": ("c", "f32", 4096, 16384),
    "rfft2205_f64": ("r", "f64", 2205, 7609),
    "rfft52272_f64": ("r", "f64", 52272, 321),
    "rfft52272_f32": ("r", "f32", 52272, 642),
    "c2c4096x4096_f32_axes01": ("n", "f32", 4096, 4096),
    "rfft1009_f64": ("r", "f64", 1009, 16628),
    "rfft65521_f64": ("r", "f64", 65521, 256),
    "rfft65521_f32": ("r", "f32", 65521, 512),
    "rfft8191_f64": ("r", "f64", 8191, 2048),
    # autotuned plans (the benchmark's): wide 8-element core, Rader row convolution
    "rfft10000_f64_tuned": ("r", "f64", 10000, 1677, "tune"),
    "rfft8191_f64_tuned": ("r", "f64", 8191, 2048, "tune"),
    "rfft65521_f64_tuned": ("r", "f64", 65521, 256, "tune"),
    "rfft65521_f32_tuned": ("r", "f32", 65521, 512, "tune"),
    "rfft8191_f32_tuned": ("r", "f32", 8191, 4096, "tune"),
    "rfft29403_f32_tuned": ("r", "f32", 29403, 1141, "tune"),
    # every 10th transform of the uneven-length workload (FP32, work-list graph)
    "uneven_tenth_f32": ("u", "f32", 0, 10),
    # FFT convolution forward, 4 images 2048^2 f32, 31x31 filters, padded to 4096^2
    "conv4_f32": ("v", "f32", 2048, 4),
}


def run_case(name):
    """One launch sequence of a small named case, for profiler captures.  Plans
    and inputs are made first; only the transform runs between
    cudaProfilerStart and cudaProfilerStop (ncu --profile-from-start off
    captures just that)."""
    import torch
    from impulse_gb300 import _lib as L
    kind, dt, n, b = PROFILE_CASES[name][:4]
    tune = PROFILE_CASES[name][4:] == ("tune",)
    lib = L.load()
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    code = L.IG_F64 if dt == "f64" else L.IG_F32
    prof = torch.cuda.cudart()
    if kind == "u":
        from impulse_gb300.batch import MultiFFT, uneven_lengths
        lengths = uneven_lengths()[::b]
        tot = sum(lengths)
        x = torch.complex(torch.randn(tot, device="cuda"), torch.randn(tot, device="cuda"))
        y = torch.empty_like(x)
        plan = MultiFFT(lengths, code)
        cs = torch.cuda.Stream()  # graph capture needs a created stream
        plan.run(x.data_ptr(), y.data_ptr(), cs.cuda_stream, "graph")  # graph captured and instantiated here
        torch.cuda.synchronize()
        prof.cudaProfilerStart()
        plan.run(x.data_ptr(), y.data_ptr(), cs.cuda_stream, "graph")
        torch.cuda.synchronize()
        prof.cudaProfilerStop()
        print(json.dumps({"case": name, "ok": True, "transforms": len(lengths), "elements": tot}))
        return
    if kind == "v":
        from impulse_gb300.fftconv import FFTConv2d
        K = 31
        x = torch.rand((b, n, n), device="cuda")
        k = torch.randn((b, K, K), device="cuda")
        op = FFTConv2d(b, n, n, K, b, torch.float32, recompute=True, pad=(2 * n, 2 * n))
        op.forward(x, k)
        torch.cuda.synchronize()
        prof.cudaProfilerStart()
        op.forward(x, k)
        torch.cuda.synchronize()
        prof.cudaProfilerStop()
        print(json.dumps({"case": name, "ok": True}))
        return
    if kind == "n":
        # multi-axis c2c of an n x b array over axes [0, 1]
        x = torch.randn((n, b), device="cuda", dtype=torch.complex128 if dt == "f64" else torch.complex64)
        y = torch.empty_like(x)
        torch.cuda.synchronize()
        _nd_call(lib, "c2c", code, x, y, [0, 1], True, 1.0, s)
        torch.cuda.synchronize()
        prof.cudaProfilerStart()
        _nd_call(lib, "c2c", code, x, y, [0, 1], True, 1.0, s)
        torch.cuda.synchronize()
        prof.cudaProfilerStop()
        print(json.dumps({"case": name, "ok": True}))
        return
    if tune:
        ms = C.c_double(0.0)
        L.check(lib.ig_autotune(code, n, 1 if kind == "r" else 0, C.byref(ms)))
    if kind == "r":
        x = torch.randn((b, n), device="cuda", dtype=torch.float64 if dt == "f64" else torch.float32)
        plan = lib.ig_make_rfft_plan(n, code)
        fn = lib.ig_rfft_exec_device
    else:
        x = torch.randn((b, n), device="cuda", dtype=torch.complex128 if dt == "f64" else torch.complex64)
        plan = lib.ig_make_cfft_plan(n, code)
        fn = lib.ig_cfft_exec_device
    y = torch.empty_like(x)
    torch.cuda.synchronize()
    L.check(fn(plan, x.data_ptr(), y.data_ptr(), b, n, n, 1, 1.0, s))
    torch.cuda.synchronize()
    prof.cudaProfilerStart()
    L.check(fn(plan, x.data_ptr(), y.data_ptr(), b, n, n, 1, 1.0, s))
    torch.cuda.synchronize()
    prof.cudaProfilerStop()
    print(json.dumps({"case": name, "ok": True}))


def run_reference(args, rank, world):
    """Reference arm: the reference's algorithm on the host cores (the compiled
    PocketFFT cannot travel to the GPU host, so the oracle port stands in)."""
    if rank != 0:
        return None
    lengths = workload_lengths()
    # warmup
    for _ in range(args.warmup):
        cpu_sample_run(lengths, min_seconds=0.0, max_passes=1)
    vals = []
    t0 = time.perf_counter()
    sample = ""
    nth = os.cpu_count() or 1
    # each step: passes over the bounded sample for at least 2 s of CPU work
    for _ in range(args.steps):
        gbs, nth, sample, _ = cpu_sample_run(lengths, min_seconds=2.0, max_passes=400)
        vals.append(gbs)
    el = time.perf_counter() - t0
    value = statistics.mean(vals)
    return {
        "metric": "FFT GB/s (halfcomplex real FFT, algorithmic bytes) vs HBM peak",
        "impl": "reference",
        "value": round(value, 3),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(el / args.steps * 1e3, 2),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded normal(0,1))",
        "config": {"workload": "real-input FFT, packed halfcomplex, f64 (bounded CPU sample: max(1/64 of each batch, 2 lines per thread))",
                   "lengths": lengths},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": nth, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-autotune", action="store_true", help="use the default plan heuristics")
    ap.add_argument("--no-extra", action="store_true", help="skip the uneven-batch and convolution measurements")
    ap.add_argument("--case", default=None, choices=sorted(PROFILE_CASES), help="run one small case once and exit")
    args = ap.parse_args()
    if args.case:
        run_case(args.case)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        if args.warmup < 3:
            args.warmup = 3
        res = run_ours(args, rank, world)
    if rank == 0 and res is not None:
        print(json.dumps(res))
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

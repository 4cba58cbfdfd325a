"""Benchmark of the fft3d hot path: 512^3 complex<float> forward (scale::full)
+ backward on one GB300, heFFTe speed3d semantics (benchmarks/speed3d.h:162-258):
GFLOP/s = 5 N log2(N) per transform, two transforms per step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--size 512] [--prec single|double] [--tc]

--impl reference times the reference's CPU algorithm for the same workload on
the host cores: the C restatement of heFFTe's stock backend in oracle/port
(the reference tree itself is not available on the GPU host), all threads.

One JSON line on rank 0.  With torchrun (N > 1) every rank runs an
independent replica (the single-rank fft3d path does not shard; no
collective on the data path) and `value` sums the replicas ("scaling": "weak").
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--prec", default="single", choices=["single", "double"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="", help="report other configurations: a name, a comma list or 'all'")
    ap.add_argument("--kernel-variant", type=int, default=0,
                    help="--workload lines: kernel family (heffte_gb300_set_kernel_variant; 3 = lengths that "
                         "are not powers of two on the runtime radix plan)")
    return ap.parse_args()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def metric_name():
    return "512^3 c2c fp32 GFLOP/s & %HBM roofline, TC vs plain FP32 at rel-L2<=1e-6"


def workload_string(n, prec):
    """config.workload of both arms (the same string, so the lines compare)."""
    return f"c2c {n}^3 complex<{'float' if prec == 0 else 'double'}> fwd(scale::full)+bwd"


def flops_per_transform(n_total):
    return 5.0 * n_total * math.log2(n_total)


# --------------------------------------------------------------------------
# clocks sampled during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [p.strip() for p in l.split(",")]
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
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------
# CPU baseline: the C port of the reference stock backend, all host threads
# --------------------------------------------------------------------------
def cpu_run(n, prec, steps, warmup, threads):
    from oracle import heffte_oracle as O
    if O.load_port() is None:
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "port")], check=True)
    size = (n, n, n)
    N = n ** 3
    rng = np.random.default_rng(512)
    dt = np.complex64 if prec == 0 else np.complex128
    x = (rng.uniform(-1, 1, N) + 1j * rng.uniform(-1, 1, N)).astype(dt)
    times = []
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        y = O.port_fft3d_c2c(x, size, 0, O.SCALE_FULL, threads=threads)
        O.port_fft3d_c2c(y, size, 1, O.SCALE_NONE, threads=threads)
        t1 = time.perf_counter()
        if i >= warmup:
            times.append(t1 - t0)
    sec = float(np.sum(times))
    value = 2 * steps * flops_per_transform(N) / sec / 1e9
    return value, sec / steps


def reference_arm(args, rank, world):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    prec = 0 if args.prec == "single" else 1
    value, sec = cpu_run(args.size, prec, args.steps, args.warmup, threads)
    line = {
        "metric": metric_name(), "value": value, "unit": "GFLOP/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64" if prec == 0 else "c128", "data": "synthetic",
        "config": {"workload": workload_string(args.size, prec), "global_batch": 1, "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": "GFLOP/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} x (forward+backward) of the full {args.size}^3 box, "
                                   f"C restatement of the heFFTe stock backend, {threads} OpenMP threads"},
        "e2e": {"value": value, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# our arm
# --------------------------------------------------------------------------
def e2e_streamed(gb, box, prec, cdt, N, x, args):
    """Per-step time of the streamed end-to-end loop (see the caller) and the
    largest round-trip error of the results that came back to the host."""
    import torch
    s_cmp, s_h2d, s_d2h = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    plan = gb.fft3d(box, box, stream=s_cmp)
    hx = torch.empty(N, dtype=cdt, pin_memory=True)
    hx.copy_(x.cpu())
    hz = [torch.empty(N, dtype=cdt, pin_memory=True) for _ in range(2)]
    xin = [torch.empty_like(x) for _ in range(2)]
    yb = [torch.empty_like(x) for _ in range(2)]
    zb = [torch.empty_like(x) for _ in range(2)]
    work = torch.empty(max(plan.size_workspace(), 1), dtype=cdt, device="cuda")
    h2d_done = [torch.cuda.Event() for _ in range(2)]
    cmp_done = [torch.cuda.Event() for _ in range(2)]
    d2h_done = [torch.cuda.Event() for _ in range(2)]
    used = [False, False]

    def step(k):
        b = k % 2
        if used[b]:
            s_h2d.wait_event(cmp_done[b])      # xin[b] was read by step k-2
        with torch.cuda.stream(s_h2d):
            xin[b].copy_(hx, non_blocking=True)
            h2d_done[b].record(s_h2d)
        s_cmp.wait_event(h2d_done[b])
        if used[b]:
            s_cmp.wait_event(d2h_done[b])      # zb[b] was read back by step k-2
        plan.forward_ptr(prec, xin[b].data_ptr(), yb[b].data_ptr(), work.data_ptr(), gb.scale.full)
        plan.backward_ptr(prec, yb[b].data_ptr(), zb[b].data_ptr(), work.data_ptr(), gb.scale.none)
        cmp_done[b].record(s_cmp)
        s_d2h.wait_event(cmp_done[b])
        with torch.cuda.stream(s_d2h):
            hz[b].copy_(zb[b], non_blocking=True)
            d2h_done[b].record(s_d2h)
        used[b] = True

    for k in range(2):
        step(k)
    torch.cuda.synchronize()
    # three timed runs of e_steps steps each; the host link's throughput
    # varies from run to run, the median is reported
    e_steps = max(4, min(args.steps, 12))
    cur = torch.cuda.current_stream()
    runs, k = [], 2
    for _ in range(3):
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(cur)
        for s_ in (s_cmp, s_h2d, s_d2h):
            s_.wait_event(start)
        for _ in range(e_steps):
            step(k)
            k += 1
        for s_ in (s_cmp, s_h2d, s_d2h):
            cur.wait_stream(s_)
        end.record(cur)
        torch.cuda.synchronize()
        runs.append(start.elapsed_time(end) / e_steps)
    rt = max(float(np.abs(h.numpy() - hx.numpy()).max()) for h in hz)
    return float(np.median(runs)), rt, runs


def combine_replicas(ms_step, world, flops_per_step, dist=None, device="cpu"):
    """Replicas only (the single-rank path does not shard): the step time is
    the maximum over ranks and the value the whole job's work (every replica's
    steps) over that time.  dist: torch.distributed (None on one rank)."""
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([ms_step], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
    return ms_step, world * flops_per_step / (ms_step / 1e3) / 1e9

def ours(args, rank, world, local_rank):
    import torch
    import heffte_gb300 as gb

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
    n = args.size
    N = n ** 3
    prec = 0 if args.prec == "single" else 1
    cdt = torch.complex64 if prec == 0 else torch.complex128
    esize = 8 if prec == 0 else 16
    stream = torch.cuda.current_stream()
    box = gb.box3d((0, 0, 0), (n - 1, n - 1, n - 1))
    plan = gb.fft3d(box, box, stream=stream)

    gen = torch.Generator(device="cuda")
    gen.manual_seed(1234 + rank)
    re = torch.rand(N, device="cuda", generator=gen, dtype=torch.float64 if prec else torch.float32) * 2 - 1
    im = torch.rand(N, device="cuda", generator=gen, dtype=re.dtype) * 2 - 1
    x = torch.complex(re, im).to(cdt)
    del re, im
    y = torch.empty_like(x)
    z = torch.empty_like(x)
    work = torch.empty(max(plan.size_workspace(), 1), dtype=cdt, device="cuda")

    def step():
        plan.forward_buffered(x, y, work, gb.scale.full)
        plan.backward_buffered(y, z, work, gb.scale.none)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # accuracy of this very workload: round trip and forward vs an FP64 check on a sample
    rt_err = float((z - x).abs().max().item())

    clocks = ClockSampler(local_rank)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    if dist:
        dist.barrier()
    clk = clocks.stop()
    ms_step = ms / args.steps
    ms_step, value = combine_replicas(ms_step, world, 2 * flops_per_transform(N), dist, "cuda")

    # dominant kernel: one strided pass (k_c2c column layout, the y and z
    # passes) and the contiguous x pass, each timed on its own with events
    per_launch = {}
    for d in range(3):
        ex = gb.executor(gb.kind.c2c, box, [d])
        for _ in range(2):
            ex.forward(prec, y, y, stream=stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 5
        e0.record(stream)
        for _ in range(reps):
            ex.forward(prec, y, y, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        per_launch[d] = e0.elapsed_time(e1) / reps
    pass_bytes = 2.0 * N * esize
    dom = max(per_launch, key=lambda d: per_launch[d])
    peak, peak_kind = peaks()
    achieved = pass_bytes / (per_launch[dom] / 1e3) / 1e9
    step_bytes = 6 * pass_bytes   # algorithmic: 3 passes x read+write, forward and backward

    # end-to-end through the C ABI with host buffers, every step: H2D of its
    # input from pinned memory, forward(scale::full) + backward, D2H of its
    # result.  Streamed: step k's H2D (copy stream) and step k-1's D2H (a
    # second copy stream) run while step k-1 / k compute on the plan's stream
    # (two device buffer sets, events order every reuse of a buffer).
    e2e_ms, rt_host, e2e_runs = e2e_streamed(gb, box, prec, cdt, N, x, args)
    e2e_val = world * 2 * flops_per_transform(N) / (e2e_ms / 1e3) / 1e9

    tc = tensor_core_form(gb, box, x, y, z, work, stream, args, ms_step, world) if prec == 0 else None

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        cv, csec = cpu_run(n, prec, 1, 0, threads)
        # single-core latency: the reference's stock backend is single-threaded
        sv, ssec = cpu_run(n, prec, 1, 0, 1)
        cpu = {"value": cv, "unit": "GFLOP/s", "cores": threads, "kind": "port",
               "sample": f"1 x (forward+backward) of the full {n}^3 box, C restatement of the heFFTe stock "
                         f"backend, {threads} OpenMP threads ({csec:.2f} s)",
               "single_core": {"value": sv, "unit": "GFLOP/s", "cores": 1, "ms_per_step": ssec * 1e3,
                               "sample": f"1 x (forward+backward) of the full {n}^3 box on one thread "
                                         f"({ssec:.2f} s)"}}
    line = {
        "metric": metric_name(),
        "value": value, "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64" if prec == 0 else "c128", "data": "synthetic",
        "config": {"workload": workload_string(n, prec), "placement": "out of place, caller workspace",
                   "global_batch": world, "parallelism": f"replicas x{world}",
                   "l2": f"inputs {N * esize / 2**30:.2f} GiB > 129 MB L2 (no flush needed)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "peak_nominal": NOMINAL_HBM_GBS, "frac_nominal": achieved / NOMINAL_HBM_GBS,
                     # DRAM read+write bytes per launch of the column pass kernel: not measured
                     # in this run, but taken from one ncu capture of this command
                     # (profiles/k_pipe_c2c_512cube_fp32.md); traffic_source says so in the line
                     "traffic": 2.086e9 if (n == 512 and prec == 0) else None,
                     "traffic_source": ("ncu capture of this command (dram__bytes_read.sum + "
                                        "dram__bytes_write.sum per launch), profiles/k_pipe_c2c_512cube_fp32.md; "
                                        "not measured in this run") if (n == 512 and prec == 0) else None,
                     "kernel": "k_pipe " + ("column" if dom else "line") + f" pass along dim {dom}",
                     "algorithmic_bytes_per_launch": pass_bytes,
                     "per_pass_ms": {str(d): per_launch[d] for d in per_launch},
                     "step_bytes": step_bytes, "step_gbs": step_bytes / (ms_step / 1e3) / 1e9,
                     "step_frac": step_bytes / (ms_step / 1e3) / 1e9 / peak},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_val, "unit": "GFLOP/s", "h2d_bytes_per_step": N * esize, "d2h_bytes_per_step": N * esize,
                "ms_per_step": e2e_ms, "api": "heffte_gb300_forward/backward (C ABI), pinned host buffers",
                "pipeline": "streamed: H2D of step k and D2H of step k-1 overlap the plan's compute "
                            "(copy streams + plan stream, two device buffer sets)",
                "ms_per_step_runs": e2e_runs},
        "gpu_launches": 6 * args.steps,
        "clocks": clk,
        "accuracy": {"roundtrip_max_abs": rt_err, "roundtrip_max_abs_e2e": rt_host},
        "tensor_cores": tc,
    }
    print(json.dumps(line), flush=True)


NOMINAL_HBM_GBS = 7900.0   # GB300 HBM3e nominal bandwidth


def fp64_host(kind, size, x, y=None, conv=False):
    """FP64 result for the input x (a device tensor of the box in order
    (0, 1, 2)), computed on the host by pocketfft (scipy.fft, all host
    threads) with heFFTe's conventions: the unscaled forward transform of kind
    c2c, r2c (along dimension 0) or cos (DCT-II = REDFT10 along every
    dimension, scipy's type-2 DCT); conv: the circular convolution of x and y
    (y None: x with itself), i.e. backward(forward(x) .* forward(y)) with
    scale::full.  Outside every timed region."""
    import scipy.fft as sf
    w = os.cpu_count() or 1
    shape = (size[2], size[1], size[0])       # numpy axes: dimension 2, 1, 0

    def host(t, dt):
        return t.cpu().numpy().reshape(shape).astype(dt)
    if conv:
        if kind == "r2c":
            fx = sf.rfftn(host(x, np.float64), workers=w)
            fy = fx if y is None else sf.rfftn(host(y, np.float64), workers=w)
            return sf.irfftn(fx * fy, s=shape, workers=w)
        fx = sf.fftn(host(x, np.complex128), workers=w)
        fy = fx if y is None else sf.fftn(host(y, np.complex128), workers=w)
        return sf.ifftn(fx * fy, workers=w)
    if kind == "c2c":
        return sf.fftn(host(x, np.complex128), workers=w)
    if kind == "r2c":
        return sf.rfftn(host(x, np.float64), workers=w)
    return sf.dctn(host(x, np.float64), type=2, workers=w)


def rel_l2_host(got, ref, chunk=1 << 24):
    """||got - ref|| / ||ref|| in float64 (got: device tensor), in chunks."""
    g = got.cpu().numpy().ravel()
    r = np.asarray(ref).ravel()
    num = den = 0.0
    for i in range(0, r.size, chunk):
        gi, ri = g[i:i + chunk].astype(r.dtype), r[i:i + chunk]
        num += float(np.sum(np.abs(gi - ri) ** 2))
        den += float(np.sum(np.abs(ri) ** 2))
    return float(np.sqrt(num / den))


def fp64_check(gb, box, x, stream, forms, kind="c2c"):
    """rel-L2 of the forward transform of x by each plan in `forms` against
    the host FP64 transform of the same input (fp64_host)."""
    import torch
    ref = fp64_host(kind, box.size, x)
    out = {}
    single = x.dtype in (torch.float32, torch.complex64)
    for name, p in forms.items():
        if kind == "cos":
            odt = torch.float32 if single else torch.float64
        else:
            odt = torch.complex64 if single else torch.complex128
        y = torch.empty(p.size_outbox(), dtype=odt, device=x.device)
        p.forward(x, y)
        out[name] = rel_l2_host(y, ref)
        del y
    return out


def tensor_core_form(gb, box, x, y, z, work, stream, args, ms_fp32, world):
    """The same workload with the radix-16 stages as split-BF16 DFT contractions
    on the tensor cores (plan.set_tensor_cores), timed over the same steps."""
    import torch
    plan_tc = gb.fft3d(box, box, stream=stream)
    plan_tc.set_tensor_cores(True)

    def step():
        plan_tc.forward_buffered(x, y, work, gb.scale.full)
        plan_tc.backward_buffered(y, z, work, gb.scale.none)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    n_total = box.count()
    plan_fp32 = gb.fft3d(box, box, stream=stream)
    acc = fp64_check(gb, box, x, stream, {"fp32": plan_fp32, "tensor_cores": plan_tc})
    step_bytes = 6 * 2.0 * n_total * 8
    peak, _ = peaks()
    return {"form": "radix-16 stages as 16-point DFT contractions on tcgen05, operands in three fixed-point "
                    "BF16 slices, exact FP32 group sums in TMEM",
            "value": world * 2 * flops_per_transform(n_total) / (ms / 1e3) / 1e9, "unit": "GFLOP/s",
            "ms_per_step": ms, "speedup_vs_fp32": ms_fp32 / ms,
            "step_gbs": step_bytes / (ms / 1e3) / 1e9, "step_frac": step_bytes / (ms / 1e3) / 1e9 / peak,
            "rel_l2_forward_vs_fp64": acc["tensor_cores"], "rel_l2_forward_vs_fp64_plain_fp32": acc["fp32"],
            "fp64_reference": "pocketfft FP64 (scipy.fft) of the same input on the host"}


WORKLOADS = {
    # name: (kind, size, precision) — the other configurations of the metric's
    # table, reported by --workload (parity cases; not the contract line)
    "c2c512": ("c2c", (512, 512, 512), 0),
    "r2c512": ("r2c", (512, 512, 512), 0),
    "dct256": ("cos", (256, 256, 256), 0),
    "z2z512": ("c2c", (512, 512, 512), 1),
    # the same with each arithmetic form of the complex<double> passes forced
    "z2z512fp64": ("c2c", (512, 512, 512), 1, False, "fp64"),
    "z2z512df": ("c2c", (512, 512, 512), 1, False, "double-float"),
    "c2c1024x1024x512": ("c2c", (1024, 1024, 512), 0),
    # lengths that are not powers of two (runtime-radix pipelined passes)
    "c2c384": ("c2c", (384, 384, 384), 0),
    "c2c448": ("c2c", (448, 448, 448), 0),
    "c2c480": ("c2c", (480, 480, 480), 0),
    "c2c640x640x320": ("c2c", (640, 640, 320), 0),
    # the same two c2c float boxes with the radix-16 stages on the tensor cores
    "c2c512tc": ("c2c", (512, 512, 512), 0, True),
    "c2c1024x1024x512tc": ("c2c", (1024, 1024, 512), 0, True),
    # small case (256 MiB, above L2) for ncu captures of the tensor-core kernel
    "c2c512x512x128tc": ("c2c", (512, 512, 128), 0, True),
    "z2z64": ("c2c", (64, 64, 64), 1),
    # small case (256 MiB complex<double>, above L2) for ncu captures of the FP64 pass kernels
    "z2z256": ("c2c", (256, 256, 256), 1),
    "z2z256fp64": ("c2c", (256, 256, 256), 1, False, "fp64"),
    "z2z256df": ("c2c", (256, 256, 256), 1, False, "double-float"),
    # small case (256 MiB, above L2) of the 512-point double-float passes, for ncu captures
    "z2z512x512x64df": ("c2c", (512, 512, 64), 1, False, "double-float"),
    # the FP64 rate of this GPU: cuBLAS DGEMM 8192^3 through torch (burst)
    "fp64peak": ("fp64peak", None, 1),
    # small case (256 MiB, above L2) for ncu captures of the c2c pass kernels
    "c2c512x512x128": ("c2c", (512, 512, 128), 0),
    # small case (256 MiB real input, above L2) for ncu captures of the r2c line pass
    "r2c512x512x256": ("r2c", (512, 512, 256), 0),
    # 256 r2c float boxes, sides i.i.d. from {16, 24, ..., 128} (seed 256), one persistent launch
    "batch256": ("batch", None, 0),
    # the same after autotuning the radix plan / tile size of every side length
    "batch256tuned": ("batch", "tuned", 0),
    # the same with each CTA's next tile copied ahead into shared memory
    "batch256prefetch": ("batch", "prefetch", 0),
    # the same queued in groups of 16 MB of boxes, each group's passes two groups apart (L2-resident)
    "batch256grouped": ("batch", "grouped", 0),
    # the same with 8 values per thread (radix plans up to 8; the default holds 16)
    "batch256values8": ("batch", "values8", 0),
    # the same boxes as a loop over one fft3d_r2c plan per box (how the reference runs them)
    "batch256loop": ("batch", "loop", 0),
    # learned plan selection on the 2000 measured shapes (tests/golden/selector_timings.npz)
    "selector2000": ("selector", None, 0),
    # the step of the reference's convolution benchmark on 512^3 complex<float>
    # (in place: forward, X .* X, backward) through plan.convolve; fused route,
    # the unfused route (the reference's order of operations), and two inputs
    "conv512": ("conv", (512, 512, 512), 0, "self"),
    "conv512unfused": ("conv", (512, 512, 512), 0, "self-unfused"),
    "conv512xy": ("conv", (512, 512, 512), 0, "xy"),
    # the same on real data through an r2c plan (the product on the half spectrum)
    "conv512r2c": ("conv", (512, 512, 512), 0, "r2c-self"),
    "conv512r2cunfused": ("conv", (512, 512, 512), 0, "r2c-self-unfused"),
    # the location layer (transpose_unpack for the five non-identity maps,
    # direct_pack / direct_unpack of a 384x512x512 sub-box, scale_data) on a
    # 512^3 complex<float> array
    "location512": ("location", (512, 512, 512), 0),
    # small case (256 MiB, above L2) for ncu captures of the fused convolution
    # pass on 512-point columns
    "conv256x256x512": ("conv", (256, 256, 512), 0, "self"),
}

BATCH_SIDES = [16, 24, 32, 40, 48, 64, 80, 96, 128]


def batch_sizes(nboxes=256, seed=256):
    rng = np.random.default_rng(seed)
    return [tuple(int(v) for v in rng.choice(BATCH_SIDES, 3)) for _ in range(nboxes)]


def run_batch_loop(name, sizes, steps, warmup):
    import torch
    import heffte_gb300 as gb
    stream = torch.cuda.current_stream()
    plans, xs, ys, zs = [], [], [], []
    gen = torch.Generator(device="cuda")
    gen.manual_seed(7)
    for s in sizes:
        box = gb.box3d((0, 0, 0), [v - 1 for v in s])
        p = gb.fft3d_r2c(box, box.r2c(0), 0, stream=stream)
        plans.append(p)
        xs.append(torch.randn(p.size_inbox(), device="cuda", generator=gen))
        ys.append(torch.empty(p.size_outbox(), dtype=torch.complex64, device="cuda"))
        zs.append(torch.empty(p.size_inbox(), device="cuda"))

    def step():
        for p, x, y, z in zip(plans, xs, ys, zs):
            p.forward(x, y, gb.scale.full)
            p.backward(y, z, gb.scale.none)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    flops = sum(2 * flops_per_transform(s[0] * s[1] * s[2]) for s in sizes)
    byts = sum(2 * algorithmic_bytes("r2c", s, 0) for s in sizes)
    peak, _ = peaks()
    return {"workload": name, "boxes": len(sizes), "ms_per_step": ms, "gflops": flops / (ms / 1e3) / 1e9,
            "gbs": byts / (ms / 1e3) / 1e9, "hbm_frac": byts / (ms / 1e3) / 1e9 / peak,
            "launches_per_step": 6 * len(sizes)}


def run_batch_workload(name, steps, warmup, tune_cache=None):
    import torch
    import heffte_gb300 as gb
    sizes = batch_sizes()
    stream = torch.cuda.current_stream()
    if tune_cache == "loop":
        return run_batch_loop(name, sizes, steps, warmup)
    # launch shapes other than the default (prefetch, tile KB, group MB)
    fixed = {"prefetch": (1, 48, 0, 0), "grouped": (0, 48, 16, 0), "values8": (0, 48, 0, 8)}.get(tune_cache)
    if fixed:
        tune_cache = None
    plans = None
    if tune_cache is not None:
        gb.tune(0, BATCH_SIDES, tune_cache, stream=stream)
        plans = {}
        for n in BATCH_SIDES:
            rad, tpb, us = gb.tuned_choice(0, n)
            plans[str(n)] = {"radices": rad, "tpb": tpb, "us_per_tuning_batch": us}
    b = gb.boxbatch(gb.kind.r2c, sizes, 0, stream=stream)
    if fixed:
        b.configure(*fixed)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(7)
    x = torch.randn(b.input_size(), device="cuda", generator=gen)
    y = torch.empty(b.output_size(), dtype=torch.complex64, device="cuda")
    z = torch.empty_like(x)
    w = torch.empty(b.workspace_size(), dtype=torch.complex64, device="cuda")

    shape = None
    if tune_cache is not None:
        # the launch shape (prefetch, tile bound, queue groups) timed on these buffers
        pf, kb, gm, vals, tms = b.autotune(x, y, z, w, reps=5)
        shape = {"prefetch": pf, "tile_kb": kb, "group_mb": gm, "values": vals, "ms_at_tuning": tms}

    def step():
        b.forward(x, y, gb.scale.full)
        b.backward(y, z, w, gb.scale.none)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    err = float((z - x).abs().max().item())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    flops = sum(2 * flops_per_transform(s[0] * s[1] * s[2]) for s in sizes)
    byts = sum(2 * algorithmic_bytes("r2c", s, 0) for s in sizes)
    peak, _ = peaks()
    return {"workload": name, "boxes": len(sizes), "ms_per_step": ms, "gflops": flops / (ms / 1e3) / 1e9,
            "gbs": byts / (ms / 1e3) / 1e9, "hbm_frac": byts / (ms / 1e3) / 1e9 / peak,
            "roundtrip_max_abs": err, "launches_per_step": 2, "tuned": tune_cache is not None,
            "launch_shape": dict(zip(("prefetch", "tile_kb", "group_mb", "values"), b.config())),
            **({"tuned_plans": plans} if plans else {}), **({"tuned_shape": shape} if shape else {})}


def algorithmic_bytes(kind, size, prec):
    """Bytes of the three passes of one transform (read + write per pass)."""
    N = size[0] * size[1] * size[2]
    rs, cs = (4, 8) if prec == 0 else (8, 16)
    if kind == "c2c":
        return 3 * 2 * N * cs
    if kind == "r2c":
        nc = (size[0] // 2 + 1) * size[1] * size[2]
        return N * rs + nc * cs + 4 * nc * cs
    return 3 * 2 * N * rs


def run_selector_workload(name):
    """Trains the selector (this library's CUDA kernels) on 80% of the measured
    shapes, and reports its held-out regret against exhaustive search, the
    default plan's and the best fixed candidate's, the training time and the
    time of one selection."""
    import time
    import torch
    from heffte_gb300 import selector
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "selector_timings.npz"))
    X, T = d["X"], selector.filled(d["T"])
    idx = np.random.default_rng(0).permutation(len(X))
    tr, te = idx[:int(0.8 * len(X))], idx[int(0.8 * len(X)):]
    net = selector.Selector(hidden=64, seed=1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss = net.train(X[tr], selector.targets(T[tr]), steps=4000, lr=2e-3)
    train_s = time.perf_counter() - t0
    choice = net.choose(X[te])
    fixed = int(np.argmin(np.log(T[tr] / T[tr].min(axis=1, keepdims=True)).mean(axis=0)))
    shapes = selector.sample_shapes(len(X), seed=int(d["seed"]))
    t0 = time.perf_counter()
    for i in te[:100]:
        net.select(*shapes[i])
    sel_us = (time.perf_counter() - t0) / 100 * 1e6
    return {"workload": name, "shapes": int(len(X)), "train_shapes": int(len(tr)), "heldout_shapes": int(len(te)),
            "regret_selector": selector.regret(T[te], choice),
            "regret_default_plan": selector.regret(T[te], np.zeros(len(te), dtype=int)),
            "regret_best_fixed_candidate": selector.regret(T[te], np.full(len(te), fixed)),
            "train_s": train_s, "train_steps": 4000, "final_loss": loss, "select_us": sel_us,
            "network": "18-64-64-16 ReLU, FP32, full-batch Adam (CUDA kernels of this library)",
            "dataset_device": str(d["device"])}


def run_conv_workload(name, steps, warmup):
    """plan.convolve on a c2c (or r2c) box: time per convolution, GFLOP/s
    counting its transforms (5 N log2 N each: 2 for x .* x, 3 for x .* y), the
    bytes of its passes against the HBM peak, and the result against the host
    FP64 convolution of the same input (fp64_host)."""
    import torch
    import heffte_gb300 as gb
    _, size, prec, form = WORKLOADS[name]
    N = size[0] * size[1] * size[2]
    real = form.startswith("r2c")
    two = form == "xy"
    stream = torch.cuda.current_stream()
    box = gb.box3d((0, 0, 0), [s - 1 for s in size])

    def make_plan():
        return gb.fft3d_r2c(box, box.r2c(0), 0, stream=stream) if real else gb.fft3d(box, box, stream=stream)
    plan = make_plan()
    if form.endswith("unfused"):
        plan.set_convolution_fusion(False)
    rdt = torch.float32 if prec == 0 else torch.float64
    gen = torch.Generator(device="cuda")
    gen.manual_seed(99)

    def rand():
        if real:
            return torch.randn(N, device="cuda", generator=gen, dtype=rdt)
        return torch.complex(torch.rand(N, device="cuda", generator=gen, dtype=rdt) * 2 - 1,
                             torch.rand(N, device="cuda", generator=gen, dtype=rdt) * 2 - 1)
    x = rand()
    y = rand() if two else None
    # out of place: the benchmark's in-place loop feeds each result back in,
    # which under- or overflows after a few steps; the passes are the same
    out = torch.empty_like(x)
    cdt = torch.complex64 if prec == 0 else torch.complex128
    work = torch.empty(plan.convolve_workspace(), dtype=cdt, device="cuda")
    route = plan.convolve_route(prec, two)

    def step():
        plan.convolve(x, y, out, gb.scale.full, workspace=work)

    for _ in range(warmup):
        step()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    ntrans = 3 if two else 2
    rs, cs = (4, 8) if prec == 0 else (8, 16)
    if real:
        # r2c: the real passes read / write N reals, the complex ones move the
        # (unpadded) half spectrum Nc; fused: r2c, c2c, fused, c2c, c2r;
        # unfused: r2c, 2 c2c, product, 2 c2c, c2r
        nc = (size[0] // 2 + 1) * size[1] * size[2]
        b = 2 * N * rs + (8 if route >= 0 else 12) * nc * cs
    else:
        # passes over the box in units of N complex values moved (read or
        # write): fused self 5 passes (10); fused xy 2 + 2 forward passes, the
        # fused pass (2 reads, 1 write), 2 backward passes (15); unfused self
        # 3 + 3 transform passes and the product's read + write (14; 18 with
        # y's forward and read)
        units = (15 if two else 10) if route >= 0 else (18 if two else 14)
        b = units * N * cs
    peak, _ = peaks()
    del work
    err = rel_l2_host(out, fp64_host("r2c" if real else "c2c", size, x, y, conv=True))
    return {"workload": name, "form": form, "fused_dim": route, "ms_per_step": ms,
            "gflops": ntrans * flops_per_transform(N) / (ms / 1e3) / 1e9,
            "bytes_per_step": b, "gbs": b / (ms / 1e3) / 1e9, "hbm_frac": b / (ms / 1e3) / 1e9 / peak,
            "rel_l2_vs_fp64": err}


def run_location_workload(name, steps, warmup):
    """The location layer of the reference's GPU backends (transpose_unpack,
    direct_pack / direct_unpack, scale_data) through this library's C ABI on a
    512^3 complex<float> array (1 GiB, above L2): per operation the device time
    per call and the bytes read + written against the HBM peak."""
    import torch
    import heffte_gb300 as gb
    _, size, prec = WORKLOADS[name][:3]
    n0, n1, n2 = size
    N = n0 * n1 * n2
    stream = torch.cuda.current_stream()
    gen = torch.Generator(device="cuda")
    gen.manual_seed(5)
    x = torch.complex(torch.randn(N, device="cuda", generator=gen), torch.randn(N, device="cuda", generator=gen))
    y = torch.empty_like(x)
    cf = 2                                      # complex<float> (dtype code of the C ABI)
    sub = (384, n1, n2)                         # sub-box of the pack / unpack
    nsub = sub[0] * sub[1] * sub[2]
    buf = torch.empty(nsub, dtype=torch.complex64, device="cuda")
    ops = []
    for mp in ((1, 0, 2), (0, 2, 1), (2, 1, 0), (1, 2, 0), (2, 0, 1)):
        ops.append(("transpose_unpack map " + "".join(map(str, mp)),
                    lambda mp=mp: gb.transpose_unpack(cf, n0, n1, n2, n0, n0 * n1, n0, n0 * n1, mp, x, y, stream=stream),
                    2 * N * 8))
    ops.append(("direct_pack 384x512x512 of 512^3",
                lambda: gb.direct_pack(cf, sub[0], sub[1], sub[2], n0, n0 * n1, x, buf, stream=stream), 2 * nsub * 8))
    ops.append(("direct_unpack 384x512x512 into 512^3",
                lambda: gb.direct_unpack(cf, sub[0], sub[1], sub[2], n0, n0 * n1, buf, y, stream=stream), 2 * nsub * 8))
    ops.append(("scale_data 2^28 floats in place", lambda: gb.scale_data(0, 2 * N, x, 1.0, stream=stream), 2 * N * 8))
    peak, _ = peaks()
    out = {"workload": name, "ops": []}
    for label, fn, b in ops:
        for _ in range(warmup):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        gbs = b / (ms / 1e3) / 1e9
        out["ops"].append({"op": label, "ms": ms, "bytes": b, "gbs": gbs, "hbm_frac": gbs / peak})
    return out


def run_fp64_peak(name, steps, warmup):
    """FP64 throughput of this GPU, the denominator of the complex<double>
    transforms: cuBLAS DGEMM of 8192^3 through torch.matmul (2 n^3 flops per
    product), best of `steps` timed products after `warmup`, CUDA events."""
    import torch
    n = 8192
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    a = torch.randn(n, n, device="cuda", dtype=torch.float64, generator=g)
    b = torch.randn(n, n, device="cuda", dtype=torch.float64, generator=g)
    for _ in range(max(1, warmup)):
        c = a @ b
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(max(1, steps)):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        c = a @ b
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del c
    return {"workload": name, "method": "cuBLAS DGEMM 8192^3 (torch.matmul float64), best of %d" % max(1, steps),
            "ms": best, "fp64_tflops": 2.0 * n ** 3 / (best / 1e3) / 1e12}


def run_workload(name, steps, warmup):
    import torch
    import heffte_gb300 as gb
    kind, size, prec = WORKLOADS[name][:3]
    if kind == "fp64peak":
        return run_fp64_peak(name, steps, warmup)
    if kind == "selector":
        return run_selector_workload(name)
    if kind == "conv":
        return run_conv_workload(name, steps, warmup)
    if kind == "location":
        return run_location_workload(name, steps, warmup)
    tc = len(WORKLOADS[name]) > 3 and WORKLOADS[name][3]
    arith = WORKLOADS[name][4] if len(WORKLOADS[name]) > 4 else None
    if arith is not None:
        old = gb.set_double_arithmetic(gb.FP64 if arith == "fp64" else gb.DOUBLE_FLOAT)
        try:
            out = run_workload_plain(name, steps, warmup, kind, size, prec, tc)
        finally:
            gb.set_double_arithmetic(old)
        out["double_arithmetic"] = arith
        return out
    if kind == "batch":
        cache = size if size in ("loop", "prefetch", "grouped", "values8") else None
        if size == "tuned":
            import tempfile
            cache = os.path.join(tempfile.mkdtemp(), "tune.tsv")
        return run_batch_workload(name, steps, warmup, cache)
    return run_workload_plain(name, steps, warmup, kind, size, prec, tc)


def run_workload_plain(name, steps, warmup, kind, size, prec, tc):
    """One transform workload (c2c / r2c / cos) timed over forward+backward steps."""
    import torch
    import heffte_gb300 as gb
    N = size[0] * size[1] * size[2]
    stream = torch.cuda.current_stream()
    box = gb.box3d((0, 0, 0), [s - 1 for s in size])
    rdt = torch.float32 if prec == 0 else torch.float64
    cdt = torch.complex64 if prec == 0 else torch.complex128
    gen = torch.Generator(device="cuda")
    gen.manual_seed(99)
    if kind == "c2c":
        plan = gb.fft3d(box, box, stream=stream)
        if tc:
            plan.set_tensor_cores(True)
        x = torch.complex(torch.rand(N, device="cuda", generator=gen, dtype=rdt) * 2 - 1,
                          torch.rand(N, device="cuda", generator=gen, dtype=rdt) * 2 - 1)
        y, z = torch.empty_like(x), torch.empty_like(x)
        wdt = cdt
    elif kind == "r2c":
        plan = gb.fft3d_r2c(box, box.r2c(0), 0, stream=stream)
        x = torch.randn(N, device="cuda", generator=gen, dtype=rdt)
        y = torch.empty(plan.size_outbox(), device="cuda", dtype=cdt)
        z = torch.empty_like(x)
        wdt = cdt
    else:
        plan = gb.rtransform(gb.kind.cos, box, box, stream=stream)
        x = torch.randn(N, device="cuda", generator=gen, dtype=rdt)
        y, z = torch.empty_like(x), torch.empty_like(x)
        wdt = rdt
    work = torch.empty(max(plan.size_workspace(), 1), dtype=wdt, device="cuda")

    def step():
        plan.forward_buffered(x, y, work, gb.scale.full)
        plan.backward_buffered(y, z, work, gb.scale.none)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    err = float((z - x).abs().max().item())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    b = 2 * algorithmic_bytes(kind, size, prec)
    peak, _ = peaks()
    out = {"workload": name, "ms_per_step": ms, "gflops": 2 * flops_per_transform(N) / (ms / 1e3) / 1e9,
           "gbs": b / (ms / 1e3) / 1e9, "hbm_frac": b / (ms / 1e3) / 1e9 / peak, "roundtrip_max_abs": err}
    del y, z, work
    out["rel_l2_forward_vs_fp64"] = fp64_check(gb, box, x, stream, {"p": plan}, kind)["p"]
    if tc:
        out["tensor_cores"] = True
    return out


def main():
    args = parse()
    if args.workload:
        if args.kernel_variant:
            import heffte_gb300 as gb
            gb.set_kernel_variant(args.kernel_variant)
        for name in (WORKLOADS if args.workload == "all" else args.workload.split(",")):
            out = run_workload(name, args.steps, args.warmup)
            if args.kernel_variant:
                out["kernel_variant"] = args.kernel_variant
            print(json.dumps(out), flush=True)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    ours(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

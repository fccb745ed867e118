"""Benchmark: batched mixed-size C2C FFT, forward + VJP, on one GB300.

Workload (the batched configuration of the reference's headline metric):
4096 Complex Float32 transforms, lengths n_i = round(exp(U[ln 16, ln 65536]))
(seed 4); a second seeded draw snaps 50% to the nearest 2^a 3^b 5^c, 25% to
the next prime >= n_i and leaves 25% raw; data i.i.d. N(0,1) (seed 5);
spectral weights w ~ U[0,1] (seed 6).  One step = forward transform of every
signal (the reference's Planned.transform forward), the cotangent
g = 2 w (.) X of loss sum w|X|^2, and the VJP DFT^H g.  Algorithmic bytes per
step: 16 N per transform application (read + write), i.e. 32 sum(n_i).

Arms: `--impl ours` (default) runs libaf; `--impl reference` times the CPU
restatement of the reference algorithm (the oracle; the Haskell reference
cannot be built here) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "accelerate-fourier_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "C2C FFT GB/s & % HBM roofline (fwd+VJP, batched mixed N) vs plain; err vs FP64"
UNIT = "GB/s"
COUNT = 4096
TRAFFIC_PROFILE = os.path.join("profiles", "fast_kernel_workload_traffic.md")


def profiled_traffic():
    """DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one step's
    persistent launches of the default workload, with the commit the ncu
    capture was taken at, from the committed profile summary; None when the
    summary is absent."""
    import re
    path = os.path.join(ROOT, TRAFFIC_PROFILE)
    if not os.path.exists(path):
        return None, None
    txt = open(path).read()
    m = re.search(r"traffic_bytes_per_step:\s*([0-9.e+]+)", txt)
    c = re.search(r"profiled_at_commit:\s*([0-9a-f]+)", txt)
    return (float(m.group(1)) if m else None), (c.group(1) if c else None)


# ----------------------------------------------------------------- workload
def smooth235_sorted(limit=1 << 18):
    vals = []
    p2 = 1
    while p2 <= limit:
        p3 = p2
        while p3 <= limit:
            p5 = p3
            while p5 <= limit:
                vals.append(p5)
                p5 *= 5
            p3 *= 3
        p2 *= 2
    return np.array(sorted(vals))


def is_prime(n: int) -> bool:
    if n < 2:
        return False
    if n % 2 == 0:
        return n == 2
    r = int(math.isqrt(n))
    for p in range(3, r + 1, 2):
        if n % p == 0:
            return False
    return True


def next_prime(n: int) -> int:
    while not is_prime(n):
        n += 1
    return n


CATEGORIES = ("all", "smooth", "prime", "raw")


def workload_sizes(count: int = COUNT, seed: int = 4, category: str = "all"):
    """The workload's lengths; `category` keeps only those drawn as 5-smooth,
    as the next prime, or left raw (profiling cases: one category's time)."""
    rng = np.random.default_rng(seed)
    base = np.round(np.exp(rng.uniform(math.log(16), math.log(65536), count))).astype(np.int64)
    cat = rng.uniform(size=count)
    sm = smooth235_sorted()
    out = []
    for n, c in zip(base, cat):
        n = int(n)
        if c < 0.5:
            i = int(np.searchsorted(sm, n))
            lo = sm[max(i - 1, 0)]
            hi = sm[min(i, len(sm) - 1)]
            n = int(lo if (n - lo) <= (hi - n) else hi)
            kind = "smooth"
        elif c < 0.75:
            n = next_prime(n)
            kind = "prime"
        else:
            kind = "raw"
        if category in ("all", kind):
            out.append(n)
    return np.array(out, dtype=np.int64)


def parse_lengths(spec: str):
    """Lengths given on the command line, e.g. "4096*2048,30011*64" (length*count)."""
    out = []
    for part in spec.split(","):
        n, _, k = part.partition("*")
        out += [int(n)] * int(k or 1)
    return np.array(out, dtype=np.int64)


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int = 0):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        """Starts sampling and returns once the first sample has arrived (at
        most a few seconds), so that the samples taken after it fall inside
        the timed region that follows."""
        self.mark = 0
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        deadline = time.time() + 5.0
        while not self.lines and time.time() < deadline and self.proc.poll() is None:
            time.sleep(0.01)
        self.mark = len(self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # the samples taken while the timed region ran; the last one before it
        # when the region was shorter than the sampling interval
        window = self.lines[self.mark:] or self.lines[-1:]
        for ln in window:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- CPU leg
def cpu_baseline(ns, budget_s: float = 12.0, threads: int = 0):
    """Oracle (CPU restatement of the reference algorithm) in FP32 on the
    host cores: forward + inverse-sign transform of a bounded prefix sample of
    the workload.  Returns (GB/s, cores, sample description)."""
    from oracle import oracle as O
    nthreads = threads or O.lib().or_max_threads()
    fwd = O.Mixed(ns, -1)
    inv = O.Mixed(ns, +1)
    rng = np.random.default_rng(5)
    x = (rng.standard_normal(fwd.total) + 1j * rng.standard_normal(fwd.total)).astype(np.complex64)
    X = np.empty_like(x)
    G = np.empty_like(x)
    # grow the prefix until one fwd+inv pass takes ~budget/3, then time it
    count = 64
    while True:
        t0 = time.perf_counter()
        fwd.exec_f32(x, X, 0, count, nthreads)
        inv.exec_f32(X, G, 0, count, nthreads)
        dt = time.perf_counter() - t0
        if dt > budget_s / 3 or count >= len(ns):
            break
        count = min(len(ns), int(count * max(2.0, (budget_s / 3) / max(dt, 1e-3))))
    reps = max(1, int((budget_s * 2 / 3) / max(dt, 1e-3)))
    t0 = time.perf_counter()
    for _ in range(reps):
        fwd.exec_f32(x, X, 0, count, nthreads)
        inv.exec_f32(X, G, 0, count, nthreads)
    dt = (time.perf_counter() - t0) / reps
    nbytes = 32 * int(ns[:count].sum())
    sample = f"first {count} of {len(ns)} transforms (sum n = {int(ns[:count].sum())}), fwd + inverse-sign, {reps} reps"
    return nbytes / dt / 1e9, nthreads, sample


# ----------------------------------------------------------------- GPU arm
class PlainRunner:
    """The plain one-launch-per-size GPU path: the same transforms laid out
    grouped by length (one contiguous [count, n] block per distinct n), one
    af_exec_c2c and one af_vjp_c2c per distinct length over its whole block,
    and the cotangent g = 2 w X with the loss sum w |X|^2 as elementwise
    device kernels.  The step is captured in a CUDA graph, so no host work
    is timed."""

    def __init__(self, ns):
        from accelerate_fourier import _lib
        ns = np.asarray(ns, dtype=np.int64)
        offs = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int64)
        order = np.argsort(ns, kind="stable")
        # gather index: grouped position -> natural position
        self.gather = np.concatenate([np.arange(offs[i], offs[i] + ns[i]) for i in order]).astype(np.int64)
        self.groups = []  # (plan, start element, count)
        pos = 0
        for n in sorted(set(int(v) for v in ns)):
            k = int(np.sum(ns == n))
            self.groups.append((_lib.Plan(n, -1, "auto"), pos, k))
            pos += n * k
        self.launches_per_step = sum(2 * p.launches(k) for p, _, k in self.groups) + 3

    def step(self, xg, wg, Xg, gradg, loss, stream):
        import torch
        xp, Xp, dp = xg.data_ptr(), Xg.data_ptr(), gradg.data_ptr()
        for plan, start, k in self.groups:
            plan.exec_ptr(xp + 8 * start, None, Xp + 8 * start, None, k, stream)
        loss.copy_(torch.sum(wg * (Xg.real * Xg.real + Xg.imag * Xg.imag)).double().reshape(1))
        Xg.mul_(2.0 * wg)
        for plan, start, k in self.groups:
            plan.exec_ptr(Xp + 8 * start, None, dp + 8 * start, None, k, stream, vjp=True)


class BatchRunner:
    """The batched executor: af_batch_forward_cotangent (forward transform of
    every signal with the fused epilogue g = 2 w X, loss = sum w |X|^2) and
    af_batch_vjp (grad = DFT^H g)."""

    def __init__(self, ns, tune=True, cache=None):
        import tempfile
        from accelerate_fourier import _lib
        t0 = time.perf_counter()
        # planner choices timed on this GPU (af_batch_create_tuned); the cache
        # lives in a fresh temporary file, so every run tunes, unless a cache
        # file is given (profiling runs reuse the choice of an earlier run)
        if tune and not cache:
            cache = os.path.join(tempfile.mkdtemp(prefix="af_tune_"), "tune.jsonl")
        self.batch = _lib.Batch(ns, -1, tune=tune, tune_cache=cache)
        self.create_s = time.perf_counter() - t0
        self.describe = self.batch.describe()
        self.launches_per_step = 2 * self.batch.launches()  # persistent launches (the loss reset is a memset)

    def step(self, x, w, cot, grad, loss, stream):
        self.batch.forward_cotangent_ptr(x.data_ptr(), w.data_ptr(), cot.data_ptr(), loss.data_ptr(), stream)
        self.batch.vjp_ptr(cot.data_ptr(), grad.data_ptr(), stream)


def max_over_ranks(v: float, dist=None) -> float:
    """The largest value over all ranks (the job's time is its slowest
    rank's); v itself when not distributed."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return v
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def time_steps(fn, steps, warmup, torch, dist=None):
    """CUDA-event time per step on the launching stream, after `warmup`
    untimed steps, with a barrier and a device synchronize on both sides of
    the timed region; the maximum over ranks."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    if dist is not None and dist.is_initialized():
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    if dist is not None and dist.is_initialized():
        dist.barrier()
    return max_over_ranks(e0.elapsed_time(e1) / steps, dist)


def time_e2e(sets, xpin, wpin, gpins, lpins, steps, warmup, torch, dist=None):
    """Per-step time of the pipelined end-to-end loop (H2D on one stream, the
    captured step on the compute stream, D2H on a third), from an event
    before the first copy to one after the last read-back, max over ranks."""
    comp = torch.cuda.current_stream()
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    ev = {k: [torch.cuda.Event() for _ in range(2)] for k in ("in", "done", "read")}

    def run(n, start=None):
        for k in range(n):
            b = k % 2
            xb, wb, _, gb, lb, gr = sets[b]
            if k == 0 and start is not None:
                s_in.wait_event(start)
            if k >= 2:
                s_in.wait_event(ev["done"][b])  # step k-2 has read x_b, w_b
            with torch.cuda.stream(s_in):
                xb.copy_(xpin, non_blocking=True)
                wb.copy_(wpin, non_blocking=True)
            ev["in"][b].record(s_in)
            comp.wait_event(ev["in"][b])
            if k >= 2:
                comp.wait_event(ev["read"][b])  # grad_b of step k-2 has been read back
            gr.replay()
            ev["done"][b].record(comp)
            s_out.wait_event(ev["done"][b])
            with torch.cuda.stream(s_out):
                gpins[b].copy_(gb, non_blocking=True)
                lpins[b].copy_(lb, non_blocking=True)
            ev["read"][b].record(s_out)
        for b in range(min(n, 2)):
            comp.wait_event(ev["read"][b])

    run(warmup)
    torch.cuda.synchronize()
    if dist is not None and dist.is_initialized():
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(comp)
    run(steps, e0)
    e1.record(comp)
    torch.cuda.synchronize()
    if dist is not None and dist.is_initialized():
        dist.barrier()
    return max_over_ranks(e0.elapsed_time(e1) / steps, dist)


def dist_setup(torch):
    """One process per GPU under torchrun (RANK / LOCAL_RANK / WORLD_SIZE);
    the collectives only synchronize the timing: the transforms are replicas
    with no exchange."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local if world > 1 else 0)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        return rank, world, dist
    return 0, 1, None


def run_ours(args):
    import torch
    rank, world, dist = dist_setup(torch)
    ns = parse_lengths(args.lengths) if args.lengths else workload_sizes(args.count, category=args.category)
    total = int(ns.sum())
    nbytes = 32 * total
    rng = np.random.default_rng(5)
    xh = (rng.standard_normal(total) + 1j * rng.standard_normal(total)).astype(np.complex64)
    wh = np.random.default_rng(6).uniform(0, 1, total).astype(np.float32)
    x = torch.from_numpy(xh).cuda()
    w = torch.from_numpy(wh).cuda()
    cot = torch.empty_like(x)
    grad = torch.empty_like(x)
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    runner = BatchRunner(ns, cache=args.tune_cache)

    def step():
        runner.step(x, w, cot, grad, loss, torch.cuda.current_stream().cuda_stream)

    # capture one step in a CUDA graph (plans and workspaces exist already)
    for _ in range(2):
        step()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        step()
    torch.cuda.synchronize()

    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    ms = time_steps(graph.replay, args.steps, args.warmup, torch, dist)
    clk = clocks.stop()

    # per-launch timing of the two halves (forward+cotangent, VJP)
    ms_fwd = time_steps(lambda: runner.batch.forward_cotangent_ptr(
        x.data_ptr(), w.data_ptr(), cot.data_ptr(), loss.data_ptr(), torch.cuda.current_stream().cuda_stream),
        args.steps, 2, torch, dist)
    ms_vjp = time_steps(lambda: runner.batch.vjp_ptr(cot.data_ptr(), grad.data_ptr(),
                                                     torch.cuda.current_stream().cuda_stream), args.steps, 2, torch,
                        dist)

    # end to end: every step copies its inputs (x, w) from pinned host memory
    # and reads its gradient and loss back.  Two device buffer sets let the
    # input copy of step k+1 and the read-back of step k-1 overlap the
    # transforms of step k (copy engines and SMs work at once).
    xpin = torch.from_numpy(xh).pin_memory()
    wpin = torch.from_numpy(wh).pin_memory()
    sets = [(x, w, cot, grad, loss, graph)]
    x1, w1 = torch.empty_like(x), torch.empty_like(w)
    cot1, grad1 = torch.empty_like(cot), torch.empty_like(grad)
    loss1 = torch.zeros_like(loss)
    for _ in range(2):
        runner.step(x1, w1, cot1, grad1, loss1, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    graph1 = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph1):
        runner.step(x1, w1, cot1, grad1, loss1, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    sets.append((x1, w1, cot1, grad1, loss1, graph1))
    gpins = [torch.empty_like(xpin).pin_memory() for _ in range(2)]
    lpins = [torch.zeros(1, dtype=torch.float64).pin_memory() for _ in range(2)]
    ms_e2e = time_e2e(sets, xpin, wpin, gpins, lpins, args.steps, 2, torch, dist)

    # plain path (one launch per distinct length, graph-captured) for the
    # "vs plain" ratio, timed like the batched step
    ms_plain = plain_launches = None
    if not args.skip_plain and world == 1:
        plain = PlainRunner(ns)
        gidx = torch.from_numpy(plain.gather).cuda()
        xg, wg = x[gidx].contiguous(), w[gidx].contiguous()
        Xg, gg = torch.empty_like(xg), torch.empty_like(xg)
        lossg = torch.zeros(1, dtype=torch.float64, device="cuda")

        def plain_step():
            plain.step(xg, wg, Xg, gg, lossg, torch.cuda.current_stream().cuda_stream)

        for _ in range(2):
            plain_step()
        torch.cuda.synchronize()
        pgraph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(pgraph):
            plain_step()
        torch.cuda.synchronize()
        ms_plain = time_steps(pgraph.replay, args.steps, args.warmup, torch)
        plain_launches = plain.launches_per_step
        # the plain path computes the same gradient
        pgraph.replay()
        step()
        torch.cuda.synchronize()
        plain_err = float((gg - grad[gidx]).norm() / grad[gidx].norm())
        del pgraph, xg, wg, Xg, gg

    if rank != 0:
        dist.barrier()
        dist.destroy_process_group()
        return
    # accuracy vs the FP64 oracle on a sample of transforms
    from oracle import oracle as O
    step()
    torch.cuda.synchronize()
    ch = cot.cpu().numpy()
    offs = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int64)
    errs = []
    for i in range(0, len(ns), 128):
        n, o = int(ns[i]), int(offs[i])
        X = O.planned(xh[o:o + n].astype(np.complex128)[None], -1)[0]
        ref = 2 * wh[o:o + n] * X
        errs.append(np.linalg.norm(ch[o:o + n] - ref) / np.linalg.norm(ref))

    # whole-job throughput: every rank transforms its own copy of the workload
    value = world * nbytes / (ms * 1e-3) / 1e9
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    # the dominant kernel is the tile kernel (every launch of the step); its
    # algorithmic bytes per step: read x, read w, write g, read g, write grad
    alg_bytes = total * (8 + 4 + 8 + 8 + 8)
    achieved = alg_bytes / ((ms_fwd + ms_vjp) * 1e-3) / 1e9
    # DRAM bytes of one step's persistent launches, from the committed ncu
    # summary (with the commit it was taken at, so that a stale figure shows)
    full = args.count == COUNT and not args.lengths and args.category == "all"
    traffic, traffic_commit = profiled_traffic() if full else (None, None)
    cpu = None
    if not args.no_cpu and world == 1:
        v, cores, sample = cpu_baseline(ns)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 (fp32)", "data": "synthetic",
        "config": {"workload": "4096 mixed-size C2C transforms, n log-uniform [16, 65536] "
                               "(50% 5-smooth, 25% prime, 25% raw), fwd + cotangent + VJP"
                               + ("" if full else f" [profiling case: {args.lengths or args.category}, "
                                  f"{len(ns)} transforms]"),
                   "sum_n": total, "path": "af_batch_* (one persistent launch per direction), CUDA graph",
                   "parallelism": f"replicas x{world} (no exchange)",
                   "l2": "inputs (267 MB) larger than L2",
                   "bytes_credited_per_step": "32 * sum(n) (16 N per transform application)",
                   "ms_forward_cotangent": ms_fwd, "ms_vjp": ms_vjp,
                   "plain_ms_per_step": ms_plain, "speedup_vs_plain": (ms_plain / ms) if ms_plain else None,
                   "autotune": runner.describe.get("autotune"), "tuning": runner.describe.get("tuning"),
                   "batch_create_s": runner.create_s,
                   "plain": "one af_exec_c2c + one af_vjp_c2c per distinct length over its length-grouped "
                            "block, cotangent and loss as elementwise kernels, CUDA graph, same steps",
                   "plain_launches_per_step": plain_launches,
                   "plain_grad_rel_diff": plain_err if ms_plain else None},
        "e2e": {"value": world * nbytes / (ms_e2e * 1e-3) / 1e9, "unit": UNIT,
                "note": "pinned H2D of x and w, the step, D2H of grad and loss, every step; double-buffered "
                        "so that copies overlap the neighbouring steps' transforms",
                "h2d_bytes_per_step": int(xh.nbytes + wh.nbytes), "d2h_bytes_per_step": int(xh.nbytes + 8)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "traffic_source": f"{TRAFFIC_PROFILE} (ncu at commit {traffic_commit})" if traffic else None,
                     "note": "the persistent kernel (every launch of the step): algorithmic 36 B per point "
                             "(x, w read, g written; g read, grad written) / its two launches' time "
                             "(CUDA events); peak = measured copy bandwidth (MEASURED_PEAKS.json); "
                             "traffic = DRAM bytes per step"},
        "cpu_baseline": cpu,
        "gpu_launches": runner.launches_per_step * args.steps * world,
        "clocks": clk,
        "err_vs_fp64": {"max_rel_l2": float(max(errs)), "median_rel_l2": float(np.median(errs)),
                        "sample": f"{len(errs)} transforms"},
        "loss": float(loss.item()),
    }
    print(json.dumps(out))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


# ----------------------------------------------------------------- configs 1, 2, 3, 5
def _peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    return json.load(open(path)).get("hbm_gbs", 6800.0) if os.path.exists(path) else 6800.0


def _err(y, ref):
    y = np.asarray(y, dtype=np.complex128)
    ref = np.asarray(ref, dtype=np.complex128)
    return float(np.linalg.norm(y - ref) / np.linalg.norm(ref)), float(np.max(np.abs(y - ref)))


def _cpu_c2c(ns, budget_s=8.0):
    """The oracle (CPU restatement of the reference algorithm) in FP32 on the
    host cores: forward + inverse-sign transforms of these lengths, repeated
    for about budget_s."""
    from oracle import oracle as O
    nth = O.lib().or_max_threads()
    ns = np.asarray(ns, dtype=np.int64)
    fwd, inv = O.Mixed(ns, -1), O.Mixed(ns, +1)
    rng = np.random.default_rng(5)
    x = (rng.standard_normal(fwd.total) + 1j * rng.standard_normal(fwd.total)).astype(np.complex64)
    X, G = np.empty_like(x), np.empty_like(x)
    reps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s or reps == 0:
        fwd.exec_f32(x, X, 0, len(ns), nth)
        inv.exec_f32(X, G, 0, len(ns), nth)
        reps += 1
    dt = (time.perf_counter() - t0) / reps
    return {"value": 32 * int(ns.sum()) / dt / 1e9, "unit": UNIT, "cores": nth, "kind": "port",
            "sample": f"{len(ns)} transforms (sum n = {int(ns.sum())}), fwd + inverse-sign, {reps} reps"}


def _line(cfg, workload, value, ms, steps, warmup, extra, alg_bytes, cpu, e2e_ms=None, h2d=0, d2h=0,
          launches=None, clk=None, dtype="c64 (fp32)"):
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic", "config": dict({"config": cfg, "workload": workload}, **extra),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": _peak(), "unit": "GB/s",
                         "frac": achieved / _peak(), "traffic": None},
            "e2e": {"value": alg_bytes / (e2e_ms * 1e-3) / 1e9 if e2e_ms else None, "unit": UNIT,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "cpu_baseline": cpu, "gpu_launches": launches, "clocks": clk}


def _e2e(torch, fn, host_in, dev_in, dev_out, host_out, steps):
    """Per-step time of: pinned H2D of the inputs, the call, D2H of the output."""
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        for h, d in zip(host_in, dev_in):
            d.copy_(h, non_blocking=True)
        fn()
        host_out.copy_(dev_out, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def run_config(args):
    import torch
    from accelerate_fourier import _lib, convolution, planned, real
    from oracle import oracle as O
    torch.cuda.set_device(0)
    st = lambda: torch.cuda.current_stream().cuda_stream
    steps, warm = args.steps, args.warmup
    clocks = ClockSampler(0)
    cfg = args.config
    if cfg == 1:
        n, B = 1024, 64
        rng = np.random.default_rng(1)
        xh = (rng.uniform(-1, 1, (B, n)) + 1j * rng.uniform(-1, 1, (B, n))).astype(np.complex64)
        x = torch.from_numpy(xh).cuda()
        X, y = torch.empty_like(x), torch.empty_like(x)
        pf, pi = _lib.Plan(n, -1, "auto"), _lib.Plan(n, +1, "auto")

        def step():
            pf.exec_ptr(x.data_ptr(), None, X.data_ptr(), None, B, st())
            pi.exec_ptr(X.data_ptr(), None, y.data_ptr(), None, B, st())
            _lib.check(_lib.load().af_scale_down(0, y.data_ptr(), None, n, B, st()))

        clocks.start()
        ms = time_steps(step, steps, warm, torch)
        clk = clocks.stop()
        step()
        torch.cuda.synchronize()
        ref = O.planned(xh.astype(np.complex128), -1)
        ef, mf = _err(X.cpu().numpy(), ref)
        er, mr = _err(y.cpu().numpy(), xh)
        xp, yp = torch.from_numpy(xh).pin_memory(), torch.empty_like(torch.from_numpy(xh)).pin_memory()
        e2e = _e2e(torch, step, [xp], [x], y, yp, steps)
        out = _line(1, "C2C N=1024 x 64, forward then inverse x 1/N (af_exec_c2c, af_scale_down)",
                    32 * n * B / (ms * 1e-3) / 1e9, ms, steps, warm,
                    {"rel_l2_forward_vs_fp64": ef, "max_abs_forward": mf, "rel_l2_round_trip": er,
                     "max_abs_round_trip": mr, "bound": 4 * 2 ** -24 * 10, "note": "512 KB: launch-bound"},
                    32 * n * B, _cpu_c2c([n] * B, 5.0), e2e, xh.nbytes, xh.nbytes,
                    (pf.launches(B) + pi.launches(B) + 1) * steps, clk)
    elif cfg == 2:
        sizes = [1 << 20, 3 ** 12, 1001 * 1024, 65537, 1000003]
        rng = np.random.default_rng(2)
        per, tot_ms, tot_b, launches = [], 0.0, 0, 0
        clocks.start()
        for n in sizes:
            xh = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
            x = torch.from_numpy(xh).cuda()
            X = torch.empty_like(x)
            p = _lib.Plan(n, -1, "auto")
            f = lambda: p.exec_ptr(x.data_ptr(), None, X.data_ptr(), None, 1, st())
            ms = time_steps(f, steps, warm, torch)
            f()
            torch.cuda.synchronize()
            e, m = _err(X.cpu().numpy(), O.planned(xh.astype(np.complex128)[None], -1)[0])
            per.append({"n": n, "plan": p.describe()[:60], "ms": ms, "GBs": 16 * n / (ms * 1e-3) / 1e9,
                        "rel_l2_vs_fp64": e, "max_abs": m, "bound_4eps_log2n": 4 * 2 ** -24 * np.log2(n)})
            tot_ms += ms
            tot_b += 16 * n
            launches += p.launches(1) * steps
        clk = clocks.stop()
        out = _line(2, "single large C2C transforms, batch 1 each: 2^20, 3^12, 1001*1024, 65537, 1000003 "
                       "(af_exec_c2c)", tot_b / (tot_ms * 1e-3) / 1e9, tot_ms, steps, warm, {"sizes": per},
                    tot_b, _cpu_c2c(sizes, 8.0), launches=launches, clk=clk)
    elif cfg == 3:
        rng = np.random.default_rng(3)
        res = {}
        clocks.start()
        # R2C 2^24 x 8 through the half-length complex plan (Real.toSpectrum)
        N, B = 1 << 24, 8
        xr = rng.standard_normal((B, N)).astype(np.float32)
        xd = torch.from_numpy(xr).cuda()
        half = planned.transform(-1, N // 2)
        ms_r = time_steps(lambda: real.toSpectrum(half, xd), steps, warm, torch)
        spec = real.toSpectrum(half, xd)
        torch.cuda.synchronize()
        e, m = _err(spec[0].cpu().numpy(), O.to_spectrum(xr[:1].astype(np.float64))[0])
        res["r2c"] = {"n": N, "batch": B, "ms": ms_r, "GBs": 12 * N * B / (ms_r * 1e-3) / 1e9,
                      "bytes_per_point": "4 read + 8 written (full spectrum, as the reference)",
                      "rel_l2_vs_fp64_row0": e, "max_abs_row0": m}
        del xd, spec
        # cyclic convolution of two length-2^20 signals (Planned.convolveCyclic, complex)
        n = 1 << 20
        a = rng.standard_normal(n) + 0j
        b = rng.standard_normal(n) + 0j
        ad = torch.from_numpy(a.astype(np.complex64)[None]).cuda()
        bd = torch.from_numpy(b.astype(np.complex64)[None]).cuda()
        conv = planned.convolveCyclic(n)
        ms_c = time_steps(lambda: conv(ad, bd), steps, warm, torch)
        z = conv(ad, bd)
        torch.cuda.synchronize()
        e, m = _err(z[0].cpu().numpy(), O.convolve_cyclic(a[None], b[None])[0])
        res["cyclic_convolution"] = {"n": n, "ms": ms_c, "GBs": 24 * n / (ms_c * 1e-3) / 1e9,
                                     "bytes_per_point": "two c64 inputs read, one c64 output written",
                                     "rel_l2_vs_fp64": e, "max_abs": m}
        # Karatsuba, Int32 4096 -> Int64, bit-exact
        L = 4096
        xi = rng.integers(-1000, 1001, (1, L)).astype(np.int32)
        yi = rng.integers(-1000, 1001, (1, L)).astype(np.int32)
        xk, yk = torch.from_numpy(xi).cuda(), torch.from_numpy(yi).cuda()
        ms_k = time_steps(lambda: convolution.karatsuba(xk, yk), steps, warm, torch)
        zk = convolution.karatsuba(xk, yk).cpu().numpy()
        exact = np.convolve(xi[0].astype(np.int64), yi[0].astype(np.int64))
        res["karatsuba"] = {"L": L, "ms": ms_k, "leaf_mults_per_s": 3 ** 12 / (ms_k * 1e-3),
                            "bit_exact_vs_int64": bool(np.array_equal(zk[0], exact)),
                            "bit_exact_vs_oracle": bool(np.array_equal(zk, O.karatsuba(xi, yi)))}
        clk = clocks.stop()
        tot_ms = ms_r + ms_c
        tot_b = 12 * N * B + 24 * n
        t0 = time.perf_counter()
        O.to_spectrum(xr[:1].astype(np.float64))
        O.convolve_cyclic(a[None], b[None])
        dt = time.perf_counter() - t0
        cpu = {"value": (12 * N + 24 * n) / dt / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "one 2^24 R2C signal (of 8) and the 2^20 cyclic convolution, FP64 oracle, once"}
        out = _line(3, "R2C 2^24 x 8 (af_to_spectrum), cyclic convolution 2^20 (af_convolve_cyclic), "
                       "Karatsuba Int32 4096 -> Int64 (af_karatsuba_i32_i64)",
                    tot_b / (tot_ms * 1e-3) / 1e9, tot_ms, steps, warm, res, tot_b, cpu, clk=clk)
    else:  # 5: loss sum w |FFT x|^2, forward + VJP
        res = {}
        clocks.start()
        tot_ms, tot_b = 0.0, 0
        for label, n, B in (("c2c 2^16", 1 << 16, 256), ("bluestein 99991", 99991, 32)):
            rng = np.random.default_rng(5)
            xh = (rng.standard_normal((B, n)) + 1j * rng.standard_normal((B, n))).astype(np.complex64)
            wh = rng.uniform(0, 1, (B, n)).astype(np.float32)
            x, w = torch.from_numpy(xh).cuda(), torch.from_numpy(wh).cuda()
            cot, grad = torch.empty_like(x), torch.empty_like(x)
            loss = torch.zeros(1, dtype=torch.float64, device="cuda")
            bt = _lib.Batch([n] * B, -1)

            def step():
                bt.forward_cotangent_ptr(x.data_ptr(), w.data_ptr(), cot.data_ptr(), loss.data_ptr(), st())
                bt.vjp_ptr(cot.data_ptr(), grad.data_ptr(), st())

            ms = time_steps(step, steps, warm, torch)
            step()
            bt.status(st())
            g = grad.cpu().numpy()
            errs = []
            for i in range(0, B, max(1, B // 4)):
                X = np.fft.fft(xh[i].astype(np.complex128))
                gref = np.fft.ifft(2 * wh[i] * X) * n  # 2 F^H (w . F x)
                errs.append(_err(g[i], gref)[0])
            res[label] = {"n": n, "batch": B, "ms": ms, "GBs": 32 * n * B / (ms * 1e-3) / 1e9,
                          "grad_rel_l2_vs_fp64": max(errs), "launches_per_step": 2 * bt.launches()}
            tot_ms += ms
            tot_b += 32 * n * B
            del x, w, cot, grad
        # real FFT 2^18 x 32: toSpectrum forward, g = 2 w S, the toSpectrum VJP
        n, B = 1 << 18, 32
        rng = np.random.default_rng(5)
        xr = rng.standard_normal((B, n)).astype(np.float32)
        wr = rng.uniform(0, 1, (B, n)).astype(np.float32)
        xd, wd = torch.from_numpy(xr).cuda(), torch.from_numpy(wr).cuda()
        half = planned.transform(-1, n // 2)

        def rstep():
            S = real.toSpectrum(half, xd)
            return real.toSpectrum_vjp(half, S * (2 * wd))

        ms = time_steps(rstep, steps, warm, torch)
        gr = rstep().cpu().numpy()
        X = np.fft.fft(xr[0].astype(np.float64))
        gref = np.real(np.fft.ifft(2 * wr[0] * X) * n)
        res["real 2^18"] = {"n": n, "batch": B, "ms": ms, "GBs": 24 * n * B / (ms * 1e-3) / 1e9,
                            "bytes_per_point": "4 read + 8 spectrum (forward), 8 + 4 (VJP)",
                            "grad_rel_l2_vs_fp64_row0": _err(gr[0], gref)[0]}
        tot_ms += ms
        tot_b += 24 * n * B
        clk = clocks.stop()
        res["fd_check"] = "FP64 central finite differences: tests/test_gpu_grad.py"
        out = _line(5, "loss sum w |FFT x|^2, forward + VJP: 256 x 2^16 and 32 x 99991 (af_batch_*), "
                       "32 x real 2^18 (af_to_spectrum + af_vjp_to_spectrum)",
                    tot_b / (tot_ms * 1e-3) / 1e9, tot_ms, steps, warm, res, tot_b,
                    _cpu_c2c([1 << 16] * 8, 6.0), clk=clk)
    print(json.dumps(out))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    ns = workload_sizes()
    vals = []
    # each step is a bounded sample of the workload; the whole run stays
    # near a minute of CPU time whatever --steps is
    for _ in range(args.warmup):
        cpu_baseline(ns, budget_s=min(3.0, 10.0 / max(args.warmup, 1)))
    for _ in range(args.steps):
        v, cores, sample = cpu_baseline(ns, budget_s=min(6.0, 60.0 / max(args.steps, 1)))
        vals.append(v)
    v = float(np.median(vals))
    out = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 (fp32)", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": "4096 mixed-size C2C transforms, n log-uniform [16, 65536] "
                               "(50% 5-smooth, 25% prime, 25% raw), fwd + VJP",
                   "sum_n": int(ns.sum())},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--skip-plain", action="store_true", help="skip the plain-path comparison (profiling runs)")
    ap.add_argument("--count", type=int, default=COUNT, help="transforms in the workload (profiling runs use fewer)")
    ap.add_argument("--tune-cache", default="", help="planner-choice cache file to reuse (profiling runs: no tuning "
                    "launches once an earlier run with the same file has tuned)")
    ap.add_argument("--lengths", default="", help='profiling cases: "n*count,..." in place of the workload')
    ap.add_argument("--category", default="all", choices=CATEGORIES,
                    help="profiling cases: only the workload's 5-smooth, prime or raw lengths")
    ap.add_argument("--config", type=int, default=4, choices=[1, 2, 3, 4, 5],
                    help="4: the batched mixed-size headline (default); 1, 2, 3, 5: the other configurations")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.config != 4:
        run_config(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

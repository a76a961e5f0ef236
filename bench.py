#!/usr/bin/env python3
"""Benchmark: exact negacyclic products/s at N=65536, W=1747 (L=55, P=114).

A step is one batch of B=128 products sharing one seeded 1747-bit modulus
(the batched point of the reference, native-batched/solve.cu; its published
figure is 1,427.8 products/s whole-call on an RTX PRO 6000).  Inputs are
seeded synthetic operands uniform in [0, q) standing in for the FHERMA
challenge cases: 16 distinct products repeated to B, all larger than L2
together (no L2 flush needed).

  value   : device-resident products/s (inputs already in HBM): each step is
            one launch of the batch's CUDA graph (bcg_batch_run); K timed
            steps bracketed by barrier + synchronize, CUDA events on the
            launching stream, max over ranks.
  e2e     : the same batch through the public host API (bcg_multiply) from
            pinned host memory, H2D + compute + D2H inside the timed region.
  plain   : one product per call (device-resident and host buffers).
  uneven  : 96 products of two geometries and six moduli in one graph.
  served  : the request loop (bcg_server_*) under seeded Poisson arrivals at
            swept offered load: sustained products/s, p50/p99 latency.

One JSON line on rank 0.  Under torchrun each rank runs its own batch on its
own GPU (products shard with no collective: weak scaling).

--impl reference times the reference algorithm on the host cores (the CPU
restatement in oracle/, multithreaded) on the same workload.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

N, W, B = 65536, 1747, 128
DISTINCT = 16
METRIC = "exact products/s N=65536 W=1747: batched+served vs plain; p50/p99 latency"
PUBLISHED_BATCHED = 1427.8   # products/s: the reference's published B=128 whole-call figure (RTX PRO 6000)


def dist_info():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # nvidia-smi's start-up (NVML initialisation) stalls the GPU's work for
            # some 20 ms: the timed region starts once it samples.
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.005)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_inputs(pkg, seed_base: int):
    import numpy as np
    q = pkg.inputs.modulus(W, 2025)
    L = (W + 31) // 32
    a = np.empty((DISTINCT, N, L), np.uint32)
    b = np.empty((DISTINCT, N, L), np.uint32)
    for i in range(DISTINCT):
        a[i] = pkg.inputs.uniform(q, N, seed_base + 2 * i)
        b[i] = pkg.inputs.uniform(q, N, seed_base + 2 * i + 1)
    return q, a, b


def host_link(h_in, d_in, h_out, d_out, reps: int = 3) -> dict:
    """Copy-engine rates of the host link between pinned host memory and this
    GPU: H2D alone, D2H alone, and both directions at once (GB/s each way).
    The buffers are the e2e step's own pinned and device tensors, so the copies
    rewrite them with the contents they already hold."""
    import torch
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()

    def timed(pairs) -> float:
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s_in)
        s_out.wait_stream(s_in)
        for _ in range(reps):
            for dst, src, st in pairs:
                with torch.cuda.stream(st):
                    dst.copy_(src, non_blocking=True)
        s_in.wait_stream(s_out)
        e1.record(s_in)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1000.0 / reps

    nb_in, nb_out = h_in.numel() * h_in.element_size(), h_out.numel() * h_out.element_size()
    t_in = timed([(d_in, h_in, s_in)])
    t_out = timed([(h_out, d_out, s_out)])
    t_both = timed([(d_in, h_in, s_in), (h_out, d_out, s_out)])
    return {"h2d_gbs": nb_in / t_in / 1e9, "d2h_gbs": nb_out / t_out / 1e9,
            "both_gbs": (nb_in + nb_out) / t_both / 1e9, "bytes": [nb_in, nb_out],
            "method": "cudaMemcpyAsync on two streams, pinned host memory, %d reps" % reps}


def best_link(x: dict, y: dict) -> dict:
    """Per direction, the higher of two host_link() measurements."""
    out = dict(x)
    for k in ("h2d_gbs", "d2h_gbs", "both_gbs"):
        out[k] = max(x[k], y[k])
    out["method"] = x["method"] + "; best of one run before and one after the e2e window"
    return out


def link_bound(link: dict, in_bytes: int, out_bytes: int) -> float:
    """Products/s the host link allows at most when each product moves in_bytes
    in and out_bytes out: no schedule beats the slowest of the three measured
    capacities (H2D alone, D2H alone, both directions together)."""
    t = max(in_bytes / (link["h2d_gbs"] * 1e9), out_bytes / (link["d2h_gbs"] * 1e9),
            (in_bytes + out_bytes) / (link["both_gbs"] * 1e9))
    return 1.0 / t


def link_model_even_split(link: dict, in_bytes: int, out_bytes: int) -> float:
    """Products/s if, while both directions run, each gets half of the two-way
    rate and the rest of the larger direction then runs alone (how the probe's
    equal-size two-way copies behaved); a model, not a bound."""
    both = link["both_gbs"] * 1e9 / 2
    shared = min(in_bytes, out_bytes)
    t = shared / both + (in_bytes - shared) / (link["h2d_gbs"] * 1e9) + (out_bytes - shared) / (link["d2h_gbs"] * 1e9)
    return 1.0 / t


def tile_to(t, count):
    import torch
    reps = (count + t.shape[0] - 1) // t.shape[0]
    return t.repeat(reps, 1, 1)[:count].contiguous()


def algorithmic(info):
    """Algorithmic bytes and modular multiplies per product for each stage."""
    P, L = info.P, info.L
    plane = 4 * P * N
    io = 4 * N * L
    return {
        "encode": 2 * io + 2 * plane,
        "column": 4 * plane,
        "row": 3 * plane,
        "column_inverse": 2 * plane,
        "crt": plane + io,
    }


def load_traffic():
    path = os.path.join(REPO, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def load_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


def load_tensor_peak():
    """Sustained dense bf16 TFLOP/s (the kernels are timed inside a long step);
    fp16 tcgen05 MMAs run at the bf16 rate."""
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["bf16_tflops_sustained"]), "measured (sustained)"
    except (OSError, ValueError, KeyError):
        return 1700.0, "fallback (sustained)"


def rooflines(info, stage_us, sm_count, sm_mhz):
    """HBM, tensor and INT32-issue fractions per stage from the live stage times.

    tensor: fp16 digit-MMA FLOPs actually issued (padded K and N) per product;
    int32 issue: warp instructions per product from the ncu capture of the
    same kernel (profiles/traffic.json) x 32 lanes, against the SMs' issue
    peak (4 warp instructions per clock per SM) at the sampled SM clock."""
    P, L = info.P, info.L
    hbm_peak, hbm_src = load_peaks()
    tc_peak, tc_src = load_tensor_peak()
    alg = algorithmic(info)
    flops = {"encode": 2.0 * 2 * N * info.enc_k * info.enc_cols, "crt": 2.0 * N * info.crt_k * info.crt_n}
    insts = load_traffic().get("warp_instructions_per_product", {})
    issue_peak = sm_count * 4 * 32 * sm_mhz * 1e6          # thread instructions / s
    out = {"hbm_peak_gbs": hbm_peak, "hbm_peak_source": hbm_src, "tensor_peak_tflops": tc_peak,
           "tensor_peak_source": tc_src, "issue_peak_tinst_per_s": issue_peak / 1e12, "stages": {}}
    for s, us in stage_us.items():
        e = {"us_per_product": us, "hbm_gbs": alg[s] / us / 1e3, "hbm_frac": alg[s] / us / 1e3 / hbm_peak}
        if s in flops:
            e["tensor_tflops"] = flops[s] / us / 1e6
            e["tensor_frac"] = e["tensor_tflops"] / tc_peak
        if s in insts:
            e["issue_tinst_per_s"] = insts[s] * 32 / us / 1e6
            e["issue_frac"] = insts[s] * 32 / (us * 1e-6) / issue_peak
        out["stages"][s] = e
    total_us = sum(stage_us.values())
    out["whole_chain"] = {"us_per_product": total_us, "hbm_gbs": sum(alg.values()) / total_us / 1e3,
                          "hbm_frac": sum(alg.values()) / total_us / 1e3 / hbm_peak}
    return out


def host_cpu() -> dict:
    """The host cores a CPU leg runs on: model, logical CPUs, the affinity mask
    and the physical cores in it (Linux /proc and /sys)."""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":")[0].strip().lower()
                if key in ("model name", "cpu model", "hardware") and ":" in line:
                    model = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    if model is None:   # Arm: the implementer and part codes (0x41/0xd4f: Arm Neoverse V2, as in Grace)
        codes = {}
        try:
            with open("/proc/cpuinfo") as f:
                for line in f:
                    if ":" in line:
                        k, v = (x.strip() for x in line.split(":", 1))
                        if k in ("CPU implementer", "CPU part") and k not in codes:
                            codes[k] = v
        except OSError:
            pass
        names = {("0x41", "0xd4f"): "Arm Neoverse V2", ("0x41", "0xd40"): "Arm Neoverse V1",
                 ("0x41", "0xd0c"): "Arm Neoverse N1"}
        key = (codes.get("CPU implementer"), codes.get("CPU part"))
        model = names.get(key) or (f"implementer {key[0]} part {key[1]}" if key[0] else platform.machine())
    mask = sorted(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else list(range(os.cpu_count() or 1))
    cores = set()
    for cpu in mask:
        base = f"/sys/devices/system/cpu/cpu{cpu}/topology/"
        try:
            with open(base + "core_id") as f1, open(base + "physical_package_id") as f2:
                cores.add((f2.read().strip(), f1.read().strip()))
        except OSError:
            cores.add(("?", str(cpu)))
    span = f"{mask[0]}-{mask[-1]}" if mask and mask == list(range(mask[0], mask[-1] + 1)) else ",".join(map(str, mask))
    return {"model": model, "nproc": os.cpu_count(), "affinity": span, "physical_cores_in_mask": len(cores),
            "arch": platform.machine()}


def cpu_baseline(pkg, q, a, b, sample: int):
    from oracle import oracle
    o = oracle.Oracle(N, W, q)
    o.multiply(a[0], b[0])            # warm (page-in, thread pool)
    t0 = time.perf_counter()
    for i in range(sample):
        o.multiply(a[i % a.shape[0]], b[i % b.shape[0]])
    dt = time.perf_counter() - t0
    cpu = host_cpu()
    threads = oracle.max_threads()
    return {"value": sample / dt, "unit": "products/s", "cores": min(threads, cpu["physical_cores_in_mask"]),
            "threads": threads, "kind": "port", "host": cpu,
            "sample": f"{sample} products of N=65536/W=1747 (oracle RNS-NTT-CRT restatement, OpenMP)"}


def run_reference(args):
    world, rank, _ = dist_info()
    if rank != 0:
        return
    pkg = importlib.import_module("fherma-bytecrt_gb300")
    import numpy as np
    from oracle import oracle
    q = pkg.inputs.modulus(W, 2025)
    a = np.stack([pkg.inputs.uniform(q, N, 1), pkg.inputs.uniform(q, N, 3)])
    b = np.stack([pkg.inputs.uniform(q, N, 2), pkg.inputs.uniform(q, N, 4)])
    o = oracle.Oracle(N, W, q)
    per_step = 1
    for i in range(args.warmup):
        o.multiply(a[i % 2], b[i % 2])
    t0 = time.perf_counter()
    for i in range(args.steps):
        o.multiply(a[i % 2], b[i % 2])
    dt = time.perf_counter() - t0
    value = args.steps * per_step / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "products/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded uniform operands in [0,q), seeded odd 1747-bit q)",
        "config": {"workload": "N=65536 W=1747 L=55 P=114 exact negacyclic product, CPU, "
                               f"{per_step} product per step (bounded sample of the B=128 batch)",
                   "global_batch": per_step},
        "cpu_baseline": {"value": value, "unit": "products/s",
                         "cores": min(oracle.max_threads(), host_cpu()["physical_cores_in_mask"]),
                         "threads": oracle.max_threads(), "kind": "port", "host": host_cpu(),
                         "sample": f"{per_step} product per step, {args.steps} steps",
                         "reference_py": "not timed here: the reference checkout (reference.py) is not on this "
                                         "machine; it checks the CRT only and has no product path"},
        "e2e": {"value": value, "unit": "products/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    line["gpu_kernels"] = reference_gpu_kernels()
    print(json.dumps(line), flush=True)


def reference_gpu_kernels():
    """The reference's own encode_mma32 and g1_crt32 kernels (compiled unmodified from its
    sources into oracle/_ref/ref_kernels.cubin), checked against the oracle and timed on this
    GPU, one product per launch as the reference launches them; None where the cubin or a GPU
    is missing."""
    try:
        import torch
        from oracle import ref_kernels
        if not (ref_kernels.available() and torch.cuda.is_available()):
            return None
        return [ref_kernels.run(n, w) for n, w in ((65536, 1747), (32768, 868))]
    except Exception as e:          # reported, never fatal for the CPU arm
        return {"error": str(e)[:200]}


def e2e_in_worker(args, local: int, rank: int, knobs: dict | None) -> dict:
    """Runs run_e2e_worker in a child process and returns its JSON (or an error)."""
    cmd = [sys.executable, os.path.abspath(__file__), "--e2e-worker", "--e2e-device", str(local),
           "--e2e-seed", str(1000 + 97 * rank), "--steps", str(args.steps), "--warmup", str(args.warmup)]
    if knobs is not None:
        cmd += ["--e2e-tuning", json.dumps(knobs)]
    elif args.autotune:
        cmd.append("--e2e-autotune")
    try:
        worker = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
        return json.loads(worker.stdout.strip().splitlines()[-1])
    except subprocess.TimeoutExpired:
        return {"error": "the worker ran past 600 s"}
    except (IndexError, ValueError):
        return {"error": (worker.stderr or worker.stdout)[-300:]}


def run_native(args):
    world, rank, local = dist_info()
    # With one GPU the e2e window runs first, before this process loads torch
    # at all (see the e2e section below); with several, after the ranks meet.
    early = e2e_in_worker(args, local, rank, None) if world == 1 else None
    import numpy as np
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    torch.cuda.set_device(local)
    pkg = importlib.import_module("fherma-bytecrt_gb300")
    q, a_np, b_np = make_inputs(pkg, 1000 + 97 * rank)
    L = (W + 31) // 32
    m = pkg.Multiplier(N, W, q, device=local)
    # The autotuner picks this geometry's kernel shapes; the batch's contexts
    # (same geometry) start from its result.
    tuning = m.autotune(max_group=32) if args.autotune else None
    if args.group:
        m.set_group(args.group)
    group = m.get_tuning("group")
    info = m.info

    a_dev = tile_to(torch.from_numpy(a_np.view(np.int32)).cuda(), B)
    b_dev = tile_to(torch.from_numpy(b_np.view(np.int32)).cuda(), B)
    c_dev = torch.empty_like(a_dev)
    # A dedicated stream: the kernels and the timing events share it (a NULL
    # stream handle would select the library's own stream instead).
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def max_over_ranks(x: float) -> float:
        if world == 1:
            return x
        t = torch.tensor([x], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        return float(t.item())

    def timed(fn, steps):
        barrier()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(steps):
            fn()
        e.record(stream)
        torch.cuda.synchronize()
        barrier()
        return max_over_ranks(s.elapsed_time(e))

    # ---- batched B=128, one CUDA graph per step (the headline value).
    batch = pkg.Batch(local)
    batch.add(N, W, q, a_dev, b_dev, c_dev, B)
    batch.set_lanes(args.lanes)
    batch.profile(every=0)            # the timed graph carries no stage events
    for _ in range(args.warmup):
        batch.run(stream.cuda_stream)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        ms = timed(lambda: batch.run(stream.cuda_stream), args.steps)
    binfo = batch.info()
    # Stage times for the rooflines: the same graph re-captured with CUDA events
    # around every stage of every profile_every-th chain (about 1% slower), on
    # one branch so that each stage's events bracket that stage's kernels only.
    batch.set_lanes(1)
    batch.profile(every=args.profile_every)
    batch.run(stream.cuda_stream)
    torch.cuda.synchronize()
    batch.read_profile()
    for _ in range(max(4, args.steps // 4)):
        batch.run(stream.cuda_stream)
    torch.cuda.synchronize()
    prof = batch.read_profile()
    value = world * B * args.steps / (ms / 1000.0)
    c0 = c_dev[0].cpu()
    assert torch.equal(c0, c_dev[DISTINCT].cpu()), "repeated inputs gave different products"

    # ---- the same batch issued as stream launches (no graph), for comparison.
    for _ in range(2):
        m.multiply_device(a_dev, b_dev, c_dev, B, stream=stream.cuda_stream)
    stream_ms = timed(lambda: m.multiply_device(a_dev, b_dev, c_dev, B, stream=stream.cuda_stream),
                      max(3, args.steps // 2))
    stream_value = world * B * max(3, args.steps // 2) / (stream_ms / 1000.0)
    assert torch.equal(c_dev[0].cpu(), c0), "graph and stream launches disagree"

    # ---- plain single product (the per-product baseline).
    plain_iters = max(3, args.steps)
    for _ in range(2):
        m.multiply_device(a_dev, b_dev, c_dev, 1, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    s2, e2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s2.record(stream)
    for i in range(plain_iters):
        m.multiply_device(a_dev[i % DISTINCT], b_dev[i % DISTINCT], c_dev[i % DISTINCT], 1,
                          stream=stream.cuda_stream)
    e2.record(stream)
    torch.cuda.synchronize()
    plain_ms = s2.elapsed_time(e2) / plain_iters

    # ---- end to end through the host API from pinned memory.  The timed window runs in a worker process
    # that does not load torch (run_e2e_worker): calls from a process that has loaded torch stall now and
    # then (every ~0.5 s, 7-150 ms), and the same calls from a torch-free process do not; with one GPU the
    # worker runs before this process loads torch at all.  This process keeps its own window beside it as
    # `in_process_torch`.
    a_h = torch.empty((B, N, L), dtype=torch.int32).pin_memory()
    b_h = torch.empty((B, N, L), dtype=torch.int32).pin_memory()
    c_h = torch.empty((B, N, L), dtype=torch.int32).pin_memory()
    a_h.copy_(a_dev.cpu())
    b_h.copy_(b_dev.cpu())
    for _ in range(max(1, args.warmup)):
        m.multiply_into(a_h, b_h, c_h, B)
    link_before = host_link(a_h, a_dev, c_h, c_dev)
    knobs = {k: m.get_tuning(k) for k in ("group", "crt_tiles", "crt_persistent", "row_local", "row_rows",
                                           "row_bits", "row_pass", "encode_scalar")}
    barrier()
    w = early if early is not None else e2e_in_worker(args, local, rank, knobs)
    barrier()
    with ClockSampler(local) as e2e_clocks:
        t0 = time.perf_counter()
        in_steps = []
        for _ in range(args.steps):
            ts = time.perf_counter()
            m.multiply_into(a_h, b_h, c_h, B)
            in_steps.append(1000.0 * (time.perf_counter() - ts))
        in_s = time.perf_counter() - t0
    assert torch.equal(c_h[0], c0), "host path and device path disagree"
    for _ in range(2):
        m.multiply_into(a_h[0], b_h[0], c_h[0], 1)
    t0 = time.perf_counter()
    for i in range(plain_iters):
        m.multiply_into(a_h[i % DISTINCT], b_h[i % DISTINCT], c_h[i % DISTINCT], 1)
    in_plain_ms = 1000 * (time.perf_counter() - t0) / plain_iters
    # The link is shared with the rest of the host: its rate moves between runs, so the bound takes the
    # better of a measurement just before and one just after the e2e window.
    link = best_link(link_before, host_link(a_h, a_dev, c_h, c_dev))
    del a_h, b_h, c_h
    import hashlib
    want_hashes = [hashlib.sha256(c_dev[i].cpu().numpy().tobytes()).hexdigest() for i in range(DISTINCT)]
    in_process = {"value": B * args.steps / in_s, "plain_ms_per_product": in_plain_ms,
                  "step_ms": {"min": min(in_steps), "median": sorted(in_steps)[len(in_steps) // 2],
                              "max": max(in_steps), "each": [round(t, 2) for t in in_steps]},
                  "clocks": e2e_clocks.summary()}
    if "seconds" in w:
        if w.get("hashes") != want_hashes:
            raise AssertionError("the e2e worker's products differ from the device path's")
        e2e_s = max_over_ranks(w["seconds"])
        e2e_steps, plain_e2e_ms, e2e_clock = w["step_ms"], w["plain_ms_per_product"], w.get("clocks")
        e2e_where = ("a worker process without torch (pinned buffers from bcg_host_alloc)"
                     + (", run before this process loaded torch" if early is not None else "")
                     + "; every distinct product's sha256 equals the device path's")
    else:
        e2e_s = max_over_ranks(in_s)
        e2e_steps, plain_e2e_ms, e2e_clock = in_steps, in_plain_ms, in_process["clocks"]
        e2e_where = "this process (the torch-free worker failed: " + str(w.get("error"))[:200] + ")"
    e2e_value = world * B * args.steps / e2e_s

    uneven = run_uneven(pkg, args, stream, local) if args.uneven else None
    encode_kernels = run_encode_kernels(pkg, stream, local) if args.encode_kernels and rank == 0 else None
    served = None
    if args.served:
        # Like the e2e window, the request loop runs in a worker that does not load torch.
        cmd = [sys.executable, os.path.abspath(__file__), "--served-worker", "--e2e-device", str(local),
               "--served-batched", repr(value / world), "--served-e2e", repr(e2e_value / world)]
        for flag in ("served_loads", "served_seconds", "served_requests", "served_slots", "served_max_batch",
                     "served_p99_ms", "served_bisect"):
            cmd += ["--" + flag.replace("_", "-"), str(getattr(args, flag))]
        if not args.autotune:
            cmd.append("--no-autotune")
        try:
            sw = subprocess.run(cmd, capture_output=True, text=True, timeout=1800)
            served = json.loads(sw.stdout.strip().splitlines()[-1])
            served["measured_in"] = "a worker process without torch (pinned buffers from bcg_host_alloc)"
        except subprocess.TimeoutExpired:
            served = {"error": "the served worker ran past 1800 s"}
        except (IndexError, ValueError):
            served = {"error": (sw.stderr or sw.stdout)[-300:]}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # ---- roofline of the dominant kernel, from the CUDA events inside the graph.
    alg = algorithmic(info)
    per_launch = {s: prof["ms"][s] / prof["timed"][s] for s in prof["ms"] if prof["timed"][s]}
    launches = prof["launches"]
    dominant = max(per_launch, key=lambda s: per_launch[s] * launches[s])
    per_launch_ms = per_launch[dominant]
    products_per_launch = B / max(1, launches[dominant])
    alg_bytes = alg[dominant] * products_per_launch
    achieved = alg_bytes / (per_launch_ms / 1000.0) / 1e9
    peak, peak_kind = load_peaks()
    traffic = load_traffic().get(dominant)
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
        "traffic": traffic * products_per_launch if traffic else None,
        "kernel": dominant, "peak_source": peak_kind,
        "algorithmic_bytes_per_launch": alg_bytes, "avg_launch_ms": per_launch_ms,
        "products_per_launch": products_per_launch,
        "stage_ms_per_product": {s: per_launch[s] * launches[s] / B for s in per_launch},
        "timed_launches": prof["timed"][dominant], "profile_every": args.profile_every,
    }
    clock = clocks.summary()
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    stage_us = {s: 1000 * per_launch[s] * launches[s] / B for s in per_launch}
    all_rooflines = rooflines(info, stage_us, sm_count, clock["sm_mhz"] or 2070.0)
    # The NTT passes are bound by integer multiplies, not HBM: for them the INT32 issue rate (warp
    # instructions x 32 / time against 4 warp instructions per clock per SM) sits beside the HBM figure.
    dom = all_rooflines["stages"].get(dominant, {})
    if dominant in ("column", "row", "column_inverse") and "issue_frac" in dom:
        roofline["binding"] = {"resource": "INT32 issue", "frac": dom["issue_frac"],
                               "achieved_tinst_per_s": dom["issue_tinst_per_s"],
                               "peak_tinst_per_s": all_rooflines["issue_peak_tinst_per_s"]}
    cpu = cpu_baseline(pkg, q, a_np, b_np, sample=args.cpu_sample) if args.cpu_sample > 0 else None
    plugin = run_plugin(pkg, args, local) if args.plugin else None
    # The reference's published figure is a whole call through its batched plugin at B=128
    # (pack, H2D, compute, D2H, owned output): compared with the same whole call here.
    plugin_b128 = (plugin or {}).get("solution_batched") or {}
    vs_baseline = (plugin_b128["products_per_s"] / PUBLISHED_BATCHED
                   if plugin_b128.get("products_per_s") and plugin_b128.get("B") == B else None)
    line = {
        "metric": METRIC, "value": value, "unit": "products/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": vs_baseline,
        "vs_baseline_basis": "whole call through the batched plugin (solution_batched, B=128) against the "
                             "reference's published B=128 whole call, 1,427.8 products/s on an RTX PRO 6000 "
                             "(PCIe): cross-hardware",
        "dtype": "u32",
        "data": "synthetic (seeded uniform operands in [0,q), seeded odd 1747-bit q; 16 distinct products repeated)",
        "config": {"workload": "batched B=128 exact negacyclic products, N=65536 W=1747 L=55 P=114, one q, "
                               "one CUDA graph per step",
                   "global_batch": B * world, "per_gpu_batch": B, "group": group, "graph_lanes": args.lanes or "automatic (one branch for one group)",
                   "tuning": {k: m.get_tuning(k) for k in ("crt_tiles", "crt_persistent", "row_local", "row_rows", "row_bits",
                                                           "row_pass")},
                   "autotune": tuning,
                   "l2": "inputs larger than L2 (3.7 GB per step), no flush", "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": "products/s", "h2d_bytes_per_step": 2 * B * N * L * 4,
                "d2h_bytes_per_step": B * N * L * 4, "api": "bcg_multiply (host buffers, pinned)",
                "link_bound": link_bound(link, 2 * N * L * 4, N * L * 4),
                "link_frac": e2e_value / world / link_bound(link, 2 * N * L * 4, N * L * 4),
                "link_model_even_split": link_model_even_split(link, 2 * N * L * 4, N * L * 4),
                "step_ms": {"min": min(e2e_steps), "median": sorted(e2e_steps)[len(e2e_steps) // 2],
                            "max": max(e2e_steps), "each": [round(t, 2) for t in e2e_steps]},
                "clocks": e2e_clock, "measured_in": e2e_where, "in_process_torch": in_process,
                "median_call_products_per_s": world * B / (sorted(e2e_steps)[len(e2e_steps) // 2] / 1000.0),
                "median_call_note": "B / the median call's time: the rate without the calls that stall on the "
                                    "device's page faults on the host buffers (their number grows over a box's "
                                    "life); `value` above is the whole window, stalls included",
                "host_link": link},
        "stream_launch": {"products_per_s": stream_value, "ms_per_step": stream_ms / max(3, args.steps // 2)},
        "plain": {"device_ms_per_product": plain_ms, "device_products_per_s": 1000.0 / plain_ms,
                  "e2e_ms_per_product": plain_e2e_ms, "e2e_products_per_s": 1000.0 / plain_e2e_ms,
                  "batched_over_plain_device": value / world / (1000.0 / plain_ms),
                  "batched_over_plain_e2e": e2e_value / world / (1000.0 / plain_e2e_ms)},
        "uneven": uneven,
        "encode_kernels": encode_kernels,
        "served": served,
        "plugin": plugin,
        "roofline": roofline,
        "rooflines": all_rooflines,
        "cpu_baseline": cpu,
        "clocks": clock,
        "gpu_launches": binfo["launches"] * args.steps,
    }
    print(json.dumps(line), flush=True)
    batch.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def run_e2e_worker(args):
    """The e2e window of run_native, in a process that does not load torch:
    B=128 products per bcg_multiply call from pinned host buffers
    (bcg_host_alloc), W warm-up calls, K timed calls, then one product per
    call; prints one JSON line with each call's time and the sha256 of each
    distinct product."""
    import ctypes
    import hashlib
    import numpy as np
    pkg = importlib.import_module("fherma-bytecrt_gb300")
    q, a_np, b_np = make_inputs(pkg, args.e2e_seed)
    L = (W + 31) // 32
    m = pkg.Multiplier(N, W, q, device=args.e2e_device)
    if args.e2e_autotune:
        m.autotune(max_group=32)
    for k, v in json.loads(args.e2e_tuning or "{}").items():
        m.set_tuning(k, v)
    words = N * L
    nbytes = B * words * 4
    pa, pb, pc = (pkg.native.host_alloc(nbytes, args.e2e_device) for _ in range(3))
    try:
        idx = np.arange(B) % DISTINCT
        for ptr, x in ((pa, a_np), (pb, b_np)):
            src = np.ascontiguousarray(x[idx])
            ctypes.memmove(ptr, src.ctypes.data, nbytes)
        for _ in range(max(1, args.warmup)):
            m.multiply_into(pa, pb, pc, B)
        steps = []
        with ClockSampler(args.e2e_device) as clocks:
            t0 = time.perf_counter()
            for _ in range(args.steps):
                ts = time.perf_counter()
                m.multiply_into(pa, pb, pc, B)
                steps.append(1000.0 * (time.perf_counter() - ts))
            seconds = time.perf_counter() - t0
        out = np.ctypeslib.as_array((ctypes.c_uint32 * (B * words)).from_address(pc))
        hashes = [hashlib.sha256(out[i * words:(i + 1) * words].tobytes()).hexdigest() for i in range(DISTINCT)]
        plain_iters = max(3, args.steps)
        for _ in range(2):
            m.multiply_into(pa, pb, pc, 1)
        t0 = time.perf_counter()
        for i in range(plain_iters):
            off = (i % DISTINCT) * words * 4
            m.multiply_into(pa + off, pb + off, pc + off, 1)
        plain_ms = 1000 * (time.perf_counter() - t0) / plain_iters
    finally:
        for ptr in (pa, pb, pc):
            pkg.native.host_free(ptr)
    print(json.dumps({"seconds": seconds, "step_ms": steps, "plain_ms_per_product": plain_ms, "hashes": hashes,
                      "clocks": clocks.summary()}), flush=True)


def run_served_worker(args):
    """run_served in a process that does not load torch (see run_native); prints its result as one JSON line."""
    pkg = importlib.import_module("fherma-bytecrt_gb300")
    out = run_served(pkg, args, args.e2e_device, args.served_batched, args.served_e2e or None)
    print(json.dumps(out), flush=True)


def run_encode_kernels(pkg, stream, device=0):
    """The two encode kernels at the points where the CUDA-core one applies
    (L <= 32): microseconds per product for the encode alone, with one product
    per launch and with the point's default chain length, and for the whole
    chain through each.  Both encoders' whole products are checked equal."""
    import numpy as np
    import torch
    out = {}
    for n, w in ((1024, 64), (4096, 200), (16384, 434), (32768, 868)):
        q = pkg.inputs.modulus(w, 5)
        m = pkg.Multiplier(n, w, q, device=device)
        group = m.get_tuning("group")
        cw, pw = n * m.L, m.plane_words
        a = torch.from_numpy(np.stack([pkg.inputs.uniform(q, n, 10 + i) for i in range(group)]).view(np.int32)).cuda()
        b = torch.from_numpy(np.stack([pkg.inputs.uniform(q, n, 50 + i) for i in range(group)]).view(np.int32)).cuda()
        pa = torch.empty(group * pw, dtype=torch.int32, device="cuda")
        pb = torch.empty_like(pa)
        c = torch.empty((group, n, m.L), dtype=torch.int32, device="cuda")
        row = {"N": n, "W": w, "L": m.L, "P": m.P, "group": group}
        products = {}
        for kind in ("tcgen05", "scalar"):
            m.set_tuning("encode_scalar", 1 if kind == "scalar" else 0)

            def per_product(fn, count, iters):
                for _ in range(3):
                    fn()
                s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s.record(stream)
                for _ in range(iters):
                    fn()
                e.record(stream)
                torch.cuda.synchronize()
                return 1000.0 * s.elapsed_time(e) / (iters * count)

            cs = stream.cuda_stream
            row[kind] = {
                "encode_us_1": per_product(lambda: m.encode_device(a, b, pa, pb, pw, 1, stream=cs), 1, 50),
                "encode_us_chain": per_product(lambda: m.encode_device(a, b, pa, pb, pw, group, stream=cs),
                                               group, 20),
                "chain_us": per_product(lambda: m.multiply_device(a, b, c, group, stream=cs), group, 10),
            }
            m.synchronize()
            products[kind] = c.cpu()
        row["same_products"] = bool(torch.equal(products["tcgen05"], products["scalar"]))
        out[f"{n}/{w}"] = row
        m.close()
    return out


def run_plugin(pkg, args, device=0):
    """The drop-in path as the challenge harness drives it: the `solution` and
    `solution_batched` binaries (the reference's wire format and per-case timer
    around fherma_run, with caller-owned pageable std::vector operands and an
    owned output vector) on N=65536/W=1747 cases: one product per call, and
    B=128 per call (the reference's published batched measure).  Milliseconds
    per product, median of the cases after the first.  Operands are 16
    distinct seeded products repeated to B; every output of the first case is
    compared with the same product from a device-resident context."""
    import shutil
    import subprocess
    import tempfile
    import numpy as np
    import torch
    pkg_dir = os.path.dirname(os.path.abspath(pkg.__file__))
    q = pkg.inputs.gap_modulus(W, 0x9E3779B1)
    L = len(q)
    distinct = 16
    a16 = np.stack([pkg.inputs.uniform(q, N, 7000 + 2 * j) for j in range(distinct)])
    b16 = np.stack([pkg.inputs.uniform(q, N, 7001 + 2 * j) for j in range(distinct)])
    m = pkg.Multiplier(N, W, q, device=device)
    want = torch.empty((distinct, N, L), dtype=torch.int32, device=f"cuda:{device}")
    m.multiply_device(torch.from_numpy(a16.view(np.int32)).cuda(device),
                      torch.from_numpy(b16.view(np.int32)).cuda(device), want, distinct)
    m.synchronize()
    want = want.cpu().numpy().view(np.uint32)
    m.close()
    out = {"point": f"N={N} W={W} q=2^{W}-2654435761, pageable host vectors"}
    for name, B, cases in (("solution", 1, 6), ("solution_batched", 128, args.plugin_cases)):
        exe = os.path.join(pkg_dir, name)
        if not os.path.exists(exe):
            out[name] = None
            continue
        need = (2 + cases) * B * N * L * 4 + (1 << 30)
        base = tempfile.gettempdir()
        if shutil.disk_usage(base).free < need:
            out[name] = {"error": f"needs {need >> 30} GiB free in {base}"}
            continue
        root = tempfile.mkdtemp(prefix="bcg_plugin_")
        try:
            man = {"N": N, "W": W, "L": L, "cases": cases}
            if name.endswith("batched"):
                man["B"] = B
            os.makedirs(os.path.join(root, "point"))
            with open(os.path.join(root, "manifest.json"), "w") as f:
                json.dump(man, f)
            q.astype("<u4").tofile(os.path.join(root, "point", "q.bin"))
            idx = np.arange(B) % distinct
            for i in range(cases):
                d = os.path.join(root, "cases", f"{i:06d}")
                os.makedirs(d)
                for tag, x in (("a", a16), ("b", b16)):
                    if B == 1:
                        x[i % distinct][None].astype("<u4").tofile(os.path.join(d, f"{tag}.bin"))
                    elif i == 0:
                        x[idx].astype("<u4").tofile(os.path.join(d, f"{tag}.bin"))
                    else:   # every batched case holds the same operands
                        os.symlink(os.path.join(root, "cases", f"{0:06d}", f"{tag}.bin"), os.path.join(d, f"{tag}.bin"))
            r = subprocess.run([exe, root], capture_output=True, text=True, timeout=900)
            res = json.load(open(os.path.join(root, "out", "results.json")))
            ms = [1000.0 * c["seconds"] / B for c in res["cases"] if c.get("status") == "ok"]
            warm = sorted(ms[1:]) if len(ms) > 1 else ms
            got = np.fromfile(os.path.join(root, "out", f"{0:06d}", "c.bin"), dtype="<u4").reshape(B, N, L)
            mism = int(sum(0 if np.array_equal(got[k], want[idx[k] if B > 1 else 0]) else 1 for k in range(B)))
            out[name] = {"B": B, "cases": cases, "ms_per_product": warm[len(warm) // 2] if warm else None,
                         "products_per_s": 1000.0 / warm[len(warm) // 2] if warm else None,
                         "ms_per_call": warm[len(warm) // 2] * B if warm else None,
                         "first_case_ms_per_product": ms[0] if ms else None, "rc": r.returncode,
                         "verified": B, "mismatches": mism}
        except Exception as e:          # reported, never fatal for the bench line
            out[name] = {"error": str(e)[:200]}
        finally:
            shutil.rmtree(root, ignore_errors=True)
    single, batched = out.get("solution") or {}, out.get("solution_batched") or {}
    if single.get("products_per_s") and batched.get("products_per_s"):
        # The reference's own batched/plain figure (2.39x) is this ratio: both whole calls.
        out["batched_over_plain_whole_call"] = batched["products_per_s"] / single["products_per_s"]
    out["reference_published"] = {"plain_whole_call_ms": [1.56, 1.67], "batched_B128_ms_per_call": 89.6,
                                  "batched_B128_products_per_s": PUBLISHED_BATCHED, "hardware": "RTX PRO 6000 (PCIe)"}
    return out


def autotune_geometries(pkg, args, device, geometries):
    """Runs the autotuner once per geometry; later contexts of it start tuned."""
    if not args.autotune:
        return None
    out = {}
    for n, w in geometries:
        m = pkg.Multiplier(n, w, pkg.inputs.modulus(w, 1), device=device)
        r = m.autotune(max_group=32)
        out[f"{n}/{w}"] = {k: r[k] for k in ("group", "crt_tiles", "crt_persistent", "row_local", "row_rows", "row_bits",
                                             "row_pass", "us_per_product_tuned")}
        m.close()
    return out


def run_uneven(pkg, args, stream, device):
    """96 products in one graph: 58 at N=32768/W=868 and 38 at N=65536/W=1747,
    three seeded moduli per geometry, four distinct operand pairs per modulus."""
    import numpy as np
    import torch
    tuned = autotune_geometries(pkg, args, device, [(32768, 868), (65536, 1747)])
    batch = pkg.Batch(device)
    keep = []
    total_bytes = 0
    for (n, w), counts in (((32768, 868), (20, 19, 19)), ((65536, 1747), (13, 13, 12))):
        for k, count in enumerate(counts):
            q = pkg.inputs.modulus(w, 4000 + 10 * k + w)
            a = np.stack([pkg.inputs.uniform(q, n, 7000 + 2 * i) for i in range(4)])
            b = np.stack([pkg.inputs.uniform(q, n, 7001 + 2 * i) for i in range(4)])
            ad = tile_to(torch.from_numpy(a.view(np.int32)).cuda(), count)
            bd = tile_to(torch.from_numpy(b.view(np.int32)).cuda(), count)
            cd = torch.empty_like(ad)
            batch.add(n, w, q, ad, bd, cd, count)
            keep.append((n, w, q, ad, bd, cd, count))
            total_bytes += 3 * ad.numel() * 4
    batch.set_lanes(args.lanes)
    for _ in range(args.warmup):
        batch.run(stream.cuda_stream)
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(stream)
    for _ in range(args.steps):
        batch.run(stream.cuda_stream)
    e.record(stream)
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / args.steps
    info = batch.info()
    # Every one of the 96 outputs of the last timed run against the same product run alone
    # (a context of its own, one product per call), compared on the device.
    verified = mismatches = 0
    for n, w, q, ad, bd, cd, count in keep:
        m = pkg.Multiplier(n, w, q, device=device)
        for i in range(min(4, count)):
            alone = torch.empty_like(ad[i])
            m.multiply_device(ad[i], bd[i], alone, 1, stream=stream.cuda_stream)
            torch.cuda.synchronize()
            for k in range(i, count, 4):
                verified += 1
                mismatches += 0 if torch.equal(cd[k], alone) else 1
        m.close()
    batch.close()
    return {"workload": "96 products: 58 at N=32768/W=868, 38 at N=65536/W=1747, 3 moduli per geometry, "
                        "one CUDA graph per step, device-resident",
            "products_per_s": 96 / (ms / 1000.0), "ms_per_step": ms, "groups": info["groups"], "autotune": tuned,
            "chains": info["chains"], "launches": info["launches"], "io_bytes": total_bytes,
            "verified": verified, "mismatches": mismatches,
            "verify": "every output of the last timed run equals the same product run alone"}


def run_served(pkg, args, device, batched_value, e2e_value=None):
    """Served request loop: seeded Poisson arrivals at swept offered load, 30%
    N=16384/W=434, 40% N=32768/W=868, 30% N=65536/W=1747 over 5 moduli; half
    the requests reuse a resident left operand.  Latency is submission to
    completion (host clock) including H2D, compute and D2H from pinned memory.

    Each offered load runs twice with the same seeded stream: a timed pass
    (latencies, sustained rate) and a verification replay, off the latency
    clock, in which every response is compared with the same product run
    alone.  Beside the sweep, the offered load is bisected for the highest
    sustained rate whose p99 meets --served-p99-ms."""
    from concurrent.futures import ThreadPoolExecutor
    import ctypes
    import numpy as np
    autotune_geometries(pkg, args, device, [(16384, 434), (32768, 868), (65536, 1747)])
    pinned = []

    def pinned_array(shape):
        """A uint32 numpy array over pinned host memory from bcg_host_alloc."""
        count = int(np.prod(shape))
        addr = pkg.native.host_alloc(count * 4, device)
        pinned.append(addr)
        return np.ctypeslib.as_array((ctypes.c_uint32 * count).from_address(addr)).reshape(shape)

    srv = pkg.Server(device, slots=args.served_slots, max_batch=args.served_max_batch)
    mix = [((16384, 434), 0.3, 1), ((32768, 868), 0.4, 2), ((65536, 1747), 0.3, 2)]
    points = []   # (n, w, q, pid, a pool, b pool, resident ids, out ring)
    for (n, w), share, nq in mix:
        for k in range(nq):
            q = pkg.inputs.modulus(w, 9000 + 17 * k + w)
            pid = srv.add_point(n, w, q)
            l = (w + 31) // 32
            pool = pinned_array((8, n, l))
            for i in range(8):
                pool[i] = pkg.inputs.uniform(q, n, 100 * k + i)
            res = [srv.add_operand(pid, pool[i]) for i in (0, 1)]
            ring = pinned_array((48, n, l))
            points.append(dict(n=n, w=w, q=q, pid=pid, pool=pool, res=res, ring=ring, share=share / nq,
                               slot=0, owner=[None] * 48))
    shares = np.array([p["share"] for p in points])
    # Work per product relative to N=65536 (N * P, P ~ N * W): capacity estimate for the sweep.
    rel = np.array([(p["n"] * (2 * p["w"] + 20)) / (65536 * 3514.0) for p in points])
    capacity_device = batched_value / float((shares * rel).sum())
    # Every request also crosses the host link: operand b, operand a unless
    # resident (half of them), and c.  The batched end-to-end rate gives the
    # link's bytes/s (3 coefficient arrays per N=65536/W=1747 product).
    capacity, basis = capacity_device, "device"
    if e2e_value:
        link_bytes_s = e2e_value * 3 * 65536 * 55 * 4
        req_bytes = np.array([2.5 * p["n"] * ((p["w"] + 31) // 32) * 4 for p in points])
        capacity_link = link_bytes_s / float((shares / shares.sum() * req_bytes).sum())
        if capacity_link < capacity_device:
            capacity, basis = capacity_link, "host link"
    # Alone results for the combinations a request can draw (operand a from pool[0..1]
    # resident or pool[2..3] sent, operand b from pool[4..7]), for verification.
    alone = {}
    for pi, p in enumerate(points):
        mult = pkg.Multiplier(p["n"], p["w"], p["q"], device=device)
        for ai in range(4):
            for bi in range(4, 8):
                alone[(pi, ai, bi)] = mult.multiply(p["pool"][ai], p["pool"][bi])
        mult.close()
    compare = ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4))

    def draw(rate, seed):
        """The seeded request stream of one offered load (arrival gaps, points, operands)."""
        r = np.random.default_rng(seed)
        count = int(min(args.served_requests, max(200, rate * args.served_seconds)))
        gaps = r.exponential(1.0 / rate, size=count)
        which = r.choice(len(points), size=count, p=shares / shares.sum())
        use_res = r.random(count) < 0.5
        ai = np.where(use_res, r.integers(2, size=count), 2 + r.integers(2, size=count))
        bi = 4 + r.integers(4, size=count)
        return count, gaps, which, use_res, ai, bi

    def drive(stream, verify: bool):
        """Submits the stream at its arrival times; returns (elapsed s, latencies ms,
        verified, mismatches).  With verify, every response is compared (on worker
        threads) with its alone result before its ring slot is reused."""
        count, gaps, which, use_res, ai, bi = stream
        pending = {}      # request id -> (point index, ai, bi, ring slot)
        checks = {}       # (point index, ring slot) -> comparison in flight
        lat = []
        tally = [0, 0]    # verified, mismatches

        def finish(rid):
            pi, a_i, b_i, slot = pending.pop(rid)
            lat.append(srv.wait(rid))
            if verify:
                got = points[pi]["ring"][slot]
                checks[(pi, slot)] = compare.submit(np.array_equal, got, alone[(pi, a_i, b_i)])

        def settle(key):
            f = checks.pop(key, None)
            if f is not None:
                tally[0] += 1
                tally[1] += 0 if f.result() else 1

        t_start = time.perf_counter()
        t_next = t_start
        for i in range(count):
            t_next += gaps[i]
            while True:   # wait for the arrival time (sleep, then spin the last half millisecond)
                left = t_next - time.perf_counter()
                if left <= 0:
                    break
                if left > 0.0005:
                    time.sleep(0.0002)
            pi = int(which[i])
            p = points[pi]
            slot = p["slot"]
            p["slot"] = (slot + 1) % len(p["owner"])
            owner = p["owner"][slot]
            if owner is not None:   # ring slot still in use: that request must finish first
                finish(owner)
            settle((pi, slot))
            a_i, b_i = int(ai[i]), int(bi[i])
            if use_res[i]:
                rid = srv.submit(p["pid"], p["pool"][b_i], p["ring"][slot], operand=p["res"][a_i])
            else:
                rid = srv.submit(p["pid"], p["pool"][b_i], p["ring"][slot], a=p["pool"][a_i])
            p["owner"][slot] = rid
            pending[rid] = (pi, a_i, b_i, slot)
        for rid in list(pending):
            finish(rid)
        elapsed = time.perf_counter() - t_start
        for key in list(checks):
            settle(key)
        for p in points:
            p["owner"] = [None] * len(p["owner"])
        return elapsed, lat, tally[0], tally[1]

    def run_load(frac, seed):
        rate = frac * capacity
        stream = draw(rate, seed)
        srv_before = srv.stats()
        elapsed, lat, _, _ = drive(stream, verify=False)
        batches = srv.stats()["batches"] - srv_before["batches"]
        _, _, verified, mismatches = drive(stream, verify=True)
        lat_ms = np.array(lat)
        count = stream[0]
        return {"offered_fraction": frac, "offered_per_s": rate, "requests": count,
                "sustained_per_s": count / elapsed,
                "p50_ms": float(np.percentile(lat_ms, 50)), "p99_ms": float(np.percentile(lat_ms, 99)),
                "mean_batch": count / max(1, batches), "verified": verified, "mismatches": mismatches}

    loads = [float(x) for x in args.served_loads.split(",")]
    results = [run_load(frac, 77 + k) for k, frac in enumerate(loads)]
    # Bisect the offered load for the highest sustained rate whose p99 meets the target.
    target = args.served_p99_ms
    bisect = []
    meets = [r for r in results if r["p99_ms"] <= target]
    misses = [r for r in results if r["p99_ms"] > target]
    lo = max((r["offered_fraction"] for r in meets), default=0.0)
    hi = min((r["offered_fraction"] for r in misses if r["offered_fraction"] > lo), default=None)
    for k in range(args.served_bisect if hi is not None else 0):
        mid = 0.5 * (lo + hi)
        r = run_load(mid, 177 + k)
        bisect.append(r)
        if r["p99_ms"] <= target:
            lo = mid
        else:
            hi = mid
    stats = srv.stats()
    srv.close()
    compare.shutdown()
    for addr in pinned:
        pkg.native.host_free(addr)
    every = results + bisect
    saturated = max(every, key=lambda r: r["sustained_per_s"])
    at_target = max((r for r in every if r["p99_ms"] <= target), key=lambda r: r["sustained_per_s"], default=None)
    head = at_target or saturated
    return {"workload": "Poisson arrivals; 30% N=16384/W=434, 40% N=32768/W=868, 30% N=65536/W=1747; "
                        "5 moduli (1/2/2); 50% reuse a resident left operand; host buffers (pinned)",
            "capacity_estimate_per_s": capacity, "capacity_basis": basis,
            "capacity_device_per_s": capacity_device, "sweep": results, "bisect": bisect,
            "p99_target_ms": target, "meets_target": at_target is not None,
            "sustained_per_s": head["sustained_per_s"], "p50_ms": head["p50_ms"], "p99_ms": head["p99_ms"],
            "saturated": {k: saturated[k] for k in ("offered_per_s", "sustained_per_s", "p50_ms", "p99_ms")},
            "verified": sum(r["verified"] for r in every), "requests": sum(r["requests"] for r in every),
            "mismatches": sum(r["mismatches"] for r in every),
            "verify": "per offered load, a replay of the same seeded stream compares every response with the "
                      "same product run alone",
            "memory_budget": stats["memory_budget"], "memory_peak": stats["memory_peak"],
            "rejected": stats["rejected"], "failed": stats["failed"]}


def run_profile_case(args):
    """Small case for ncu: `count` products of N=65536/W=1747 (or --profile-point
    N,W) through the device path, once to warm up and `steps` more times (inputs
    + planes of 2 products at N=65536, or 32 at N=16384, exceed L2; a few hundred
    MB on the device).  --profile-encoder picks the encode kernel."""
    import numpy as np
    import torch
    pkg = importlib.import_module("fherma-bytecrt_gb300")
    n, w = (int(x) for x in args.profile_point.split(",")) if args.profile_point else (N, W)
    q = pkg.inputs.modulus(w, 2025)
    count = args.profile_count
    a = np.stack([pkg.inputs.uniform(q, n, 2 * i) for i in range(count)])
    b = np.stack([pkg.inputs.uniform(q, n, 2 * i + 1) for i in range(count)])
    m = pkg.Multiplier(n, w, q)
    m.set_group(count)
    if args.profile_encoder == "scalar":
        m.set_tuning("encode_scalar", 1)
    da = torch.from_numpy(a.view(np.int32)).cuda()
    db = torch.from_numpy(b.view(np.int32)).cuda()
    dc = torch.empty_like(da)
    for _ in range(1 + args.steps):
        m.multiply_device(da, db, dc, count)
    m.synchronize()
    print(json.dumps({"profile_case": f"{count} products N={n} W={w}, {args.profile_encoder} encoder",
                      "launches": m.read_profile()["launches"]}))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["native", "reference"], default="native")
    ap.add_argument("--cpu-sample", type=int, default=24,
                    help="products in the CPU baseline sample, about 10 s on 16 Arm cores (0: skip)")
    ap.add_argument("--profile-case", action="store_true", help="run the small ncu case and exit")
    ap.add_argument("--profile-count", type=int, default=2)
    ap.add_argument("--profile-point", default="", help="N,W of the profile case (default 65536,1747)")
    ap.add_argument("--profile-encoder", choices=("tcgen05", "scalar"), default="tcgen05",
                    help="encode kernel of the profile case")
    ap.add_argument("--group", type=int, default=0, help="products per launch chain (0: library default)")
    ap.add_argument("--profile-every", type=int, default=2,
                    help="time the stages of every k-th launch chain with CUDA events")
    ap.add_argument("--no-uneven", dest="uneven", action="store_false", help="skip the uneven 96-product batch")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false", help="keep the default kernel shapes")
    ap.add_argument("--lanes", type=int, default=0, choices=(0, 1, 2),
                    help="parallel branches of the timed batch graphs that launch chains alternate over (0: the "
                         "library's choice, two for batches of several geometry/modulus groups; the profiled pass "
                         "for the rooflines always runs one branch)")
    ap.add_argument("--no-served", dest="served", action="store_false", help="skip the served sweep")
    ap.add_argument("--no-encode-kernels", dest="encode_kernels", action="store_false",
                    help="skip comparing the tcgen05 and CUDA-core encoders at small-L points")
    ap.add_argument("--no-plugin", dest="plugin", action="store_false",
                    help="skip timing the plugin harness binaries")
    ap.add_argument("--plugin-cases", type=int, default=5, help="cases of the B=128 plugin run")
    ap.add_argument("--served-loads", default="0.25,0.5,0.75,0.9",
                    help="offered loads as fractions of the estimated capacity")
    ap.add_argument("--served-seconds", type=float, default=1.5, help="arrival window per offered load")
    ap.add_argument("--served-requests", type=int, default=20000, help="cap on requests per offered load")
    ap.add_argument("--served-slots", type=int, default=3, help="server batches in flight")
    ap.add_argument("--served-max-batch", type=int, default=0,
                    help="server products per batch (0: each point's launch-chain length)")
    ap.add_argument("--served-p99-ms", type=float, default=5.0,
                    help="p99 latency target: the served figure is the highest sustained rate that meets it")
    ap.add_argument("--served-bisect", type=int, default=3,
                    help="offered-load bisection steps toward the p99 target")
    ap.add_argument("--e2e-worker", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--served-worker", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--served-batched", type=float, default=0.0, help=argparse.SUPPRESS)
    ap.add_argument("--served-e2e", type=float, default=0.0, help=argparse.SUPPRESS)
    ap.add_argument("--e2e-device", type=int, default=0, help=argparse.SUPPRESS)
    ap.add_argument("--e2e-seed", type=int, default=1000, help=argparse.SUPPRESS)
    ap.add_argument("--e2e-tuning", default="", help=argparse.SUPPRESS)
    ap.add_argument("--e2e-autotune", action="store_true", help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.e2e_worker:
        run_e2e_worker(args)
    elif args.served_worker:
        run_served_worker(args)
    elif args.profile_case:
        run_profile_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_native(args)


if __name__ == "__main__":
    main()

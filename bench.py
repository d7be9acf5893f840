#!/usr/bin/env python3
"""Benchmark of the GB300 concrete-fft hot path.

Headline workload: negacyclic u64 polynomial products, N = 2048 (folded to a
1024-point c64 unordered FFT), 8192 products per launch, A uniform u64, B
signed digits uniform in [-2^7, 2^7) pre-transformed and resident on the
device (one operand per product).  One step = one launch over 8192 products.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference's algorithm on the host cores (the CPU
restatement under oracle/: the Rust crate cannot be built here) on the same
workload, using every host thread.  Prints one JSON line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "concrete-fft_gb300")

N_POLY = 2048
COUNT = 8192
ALGO_NAMES = ["Dif2", "Dit2", "Dif4", "Dit4", "Dif8", "Dit8", "Dif16", "Dit16"]
BASE_SEED = 2  # the workload's index in the benchmark table
BYTES_PER_PRODUCT = 3 * N_POLY * 8  # A + Bhat + out: 16 KiB each
METRIC = "N=2048 negacyclic u64 polymul/s"


def fp64_ops_per_transform(n, base_n, algo):
    """FP64 instructions (DADD/DMUL/DFMA, one each) of one unordered transform
    of n points with the given base, counted from the butterfly code."""
    core = {2: 4, 4: 16, 8: 56, 16: 168}
    ops = 0
    m = n
    while m > base_n:  # outer levels: core + (r-1) twiddle products of 4 ops
        r = 2 if m == 2 * base_n else (4 if m == 4 * base_n else 8)
        ops += (n // r) * (core[r] + 4 * (r - 1))
        m //= r
    R = 2 << (algo // 2)
    rem, passes = base_n, 0
    while rem > R:
        rem //= R
        passes += 1
    ops += passes * (n // R) * (core[R] + 4 * (R - 1))
    ops += (n // rem) * core[rem]
    return ops


def fp64_ops_per_product(N, base_n, algo):
    n = N // 2
    return 2 * fp64_ops_per_transform(n, base_n, algo) + 3 * 4 * n  # twist, pointwise, untwist


class ClockSampler:
    """nvidia-smi sampling during the timed region (SM clock, throttle reasons)."""
    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index, interval_ms=200):
        self.index = index
        self.interval_ms = interval_ms
        self.proc = None
        self.lines = []
        self.window = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", str(self.interval_ms)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi's start-up (NVML initialisation) takes driver locks: let it finish
            # before the timed region, so that it does not stall the first timed launches
            deadline = time.time() + 3.0
            while not self.lines and time.time() < deadline and self.proc.poll() is None:
                time.sleep(0.01)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def mark(self, t0, t1):
        self.window = (t0, t1)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ts, ln in self.lines:
            if self.window and not (self.window[0] - 0.25 <= ts <= self.window[1] + 0.25):
                continue
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 10:
                continue
            try:
                sm.append(float(f[2]))
                mx = float(f[3])
            except ValueError:
                continue
            for name, v in zip(names, f[6:10]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def profiled_traffic(name):
    """DRAM bytes per launch from a committed ncu summary (profiles/<name>.json), if any."""
    try:
        with open(os.path.join(ROOT, "profiles", name + ".json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def make_inputs(count, seed):
    import numpy as np
    rng = np.random.default_rng(seed)
    a = rng.integers(0, 2 ** 64, (count, N_POLY), dtype=np.uint64)
    b = rng.integers(-2 ** 7, 2 ** 7, (count, N_POLY), dtype=np.int64)
    return a, b


_CPU_ALGO = {}


def cpu_fastest_algo(threads):
    """Method::Measure on the host: the fastest (base algorithm, base size) of the
    reference's candidates for n = 1024 (src/unordered.rs:553-640: bases 512 and 1024,
    the 8 algorithms), timed on the restated pipeline with `threads` threads."""
    if threads in _CPU_ALGO:
        return _CPU_ALGO[threads]
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    sample = max(64, 8 * threads)
    a, b = make_inputs(sample, 7)
    best = None
    for base in (512, 1024):
        for algo in range(8):
            bhat = pyoracle.u64_prepare(N_POLY, algo, base, b)
            pyoracle.u64_product(N_POLY, algo, base, a, bhat, nthreads=threads)
            t0 = time.perf_counter()
            for _ in range(3):
                pyoracle.u64_product(N_POLY, algo, base, a, bhat, nthreads=threads)
            el = time.perf_counter() - t0
            if best is None or el < best[0]:
                best = (el, algo, base)
    _CPU_ALGO[threads] = best[1:]
    return best[1:]


def cpu_product_rate(threads, seconds, seed):
    """Products/s of the oracle's restatement of the reference pipeline on the host cores,
    with the algorithm the reference's Method::Measure would pick there."""
    for p in (os.path.join(ROOT, "oracle"),):
        sys.path.insert(0, p)
    import numpy as np
    import pyoracle
    algo, base = cpu_fastest_algo(threads)
    sample = 256 if threads == 1 else max(256, 64 * threads)
    a, b = make_inputs(sample, seed + 1000)
    bhat = pyoracle.u64_prepare(N_POLY, algo, base, b)
    pyoracle.u64_product(N_POLY, algo, base, a[:threads], bhat[:threads], nthreads=threads)  # warm
    done, t0 = 0, time.perf_counter()
    while True:
        pyoracle.u64_product(N_POLY, algo, base, a, bhat, nthreads=threads)
        done += sample
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return done / el, done, el


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    import numpy as np
    algo, base = cpu_fastest_algo(threads)
    sample = 256 * threads  # large enough per step that thread start-up does not show in the rate
    a, b = make_inputs(sample, BASE_SEED)
    bhat = pyoracle.u64_prepare(N_POLY, algo, base, b)
    for _ in range(args.warmup):  # full-size steps, so that caches and clocks settle as in the timed ones
        pyoracle.u64_product(N_POLY, algo, base, a, bhat, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pyoracle.u64_product(N_POLY, algo, base, a, bhat, nthreads=threads)
    el = time.perf_counter() - t0
    value = args.steps * sample / el
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "products/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded numpy PCG64)",
        "config": {"workload": "u64 negacyclic product N=2048 (CPU), %s base %d (fastest on this host)"
                               % (ALGO_NAMES[algo], base),
                   "products_per_step": sample, "threads": threads},
        "cpu_baseline": {"value": value, "unit": "products/s", "cores": threads, "kind": "port",
                         "sample": "%d products per step of the N=2048 workload" % sample},
        "e2e": {"value": value, "unit": "products/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def exact_u64_products(np, a, b, rows):
    """The exact products a[r] * b[r] mod (X^N + 1, 2^64) of the sampled rows, computed here with
    wrapping uint64 numpy arithmetic (independent of the oracle)."""
    n = a.shape[-1]
    out = np.zeros((len(rows), n), dtype=np.uint64)
    for i, r in enumerate(rows):
        conv = np.convolve(a[r].astype(np.uint64), b[r].astype(np.int64).view(np.uint64))  # wraps mod 2^64
        out[i] = conv[:n]
        out[i, : n - 1] -= conv[n:]  # X^N = -1
    return out


def headline_accuracy(np, got, a, b, algo, base_n, sample=64):
    """Torus error of `sample` products of the timed launch (spread over it) against the exact
    product, beside the restated reference pipeline's error on the same products: with the same
    base algorithm as the GPU plan, and with the algorithm the reference's Method::Measure picks
    on this host."""
    po = _oracle()
    threads = host_threads()
    count, N = a.shape
    rows = np.linspace(0, count - 1, sample).astype(np.int64)
    exact = exact_u64_products(np, a, b, rows)
    gbits, gex = torus_bits_u64(got[rows], exact)
    ref = po.u64_product(N, algo, base_n, a[rows], po.u64_prepare(N, algo, base_n, b[rows]), nthreads=threads)
    rbits, rex = torus_bits_u64(ref, exact)
    calgo, cbase = cpu_fastest_algo(threads)
    ref_h = po.u64_product(N, calgo, cbase, a[rows], po.u64_prepare(N, calgo, cbase, b[rows]), nthreads=threads)
    hbits, hex_ = torus_bits_u64(ref_h, exact)
    return {"sample_products": sample, "max_torus_error_bits": gbits, "exact_coefficient_fraction": gex,
            "reference_pipeline_same_algo": {"max_torus_error_bits": rbits, "exact_coefficient_fraction": rex,
                                             "algo": "%s base %d" % (ALGO_NAMES[algo], base_n),
                                             "gpu_bit_identical": bool(np.array_equal(got[rows], ref))},
            "reference_pipeline_host_measure": {"max_torus_error_bits": hbits, "exact_coefficient_fraction": hex_,
                                                "algo": "%s base %d" % (ALGO_NAMES[calgo], cbase)},
            "gpu_bits_le_reference_bits": gbits <= min(rbits, hbits),
            "against": "exact wrapping-integer negacyclic product (numpy, uint64)"}


def run_gb300(args):
    import numpy as np
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    sys.path.insert(0, PKG)
    import concrete_fft as cf
    from concrete_fft import replicas
    lib = cf.load()
    cf.check(lib.cfft_device_check())

    count = args.count or COUNT
    if args.base_algo is not None:
        plan = cf.product.U64ProductPlan(N_POLY, cf.FftAlgo[args.base_algo], args.base_n)
    else:
        plan = cf.product.U64ProductPlan(N_POLY, measure_seconds=0.002)
    if args.int_adds is not None:
        plan.set_int_adds(args.int_adds)
    algo, base_n = plan.algo()
    int_adds = plan.int_adds()
    a_np, b_np = make_inputs(count, BASE_SEED + rank)
    a = torch.from_numpy(a_np.view(np.int64)).cuda()
    b = torch.from_numpy(b_np).cuda()
    bhat = torch.empty((count, N_POLY // 2), dtype=torch.complex128, device="cuda")
    plan.prepare_operand(b, bhat)
    out = torch.empty_like(a)
    stream = torch.cuda.current_stream()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    if args.profile_case:  # one warm-up and one measured launch for ncu, nothing else
        plan.product(a, bhat, out)
        plan.product(a, bhat, out)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "u64 product N=2048", "products": count, "base_algo": algo.name,
                          "base_n": base_n}))
        return
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        time.sleep(0.5)  # let the sampler start before the timed region
        for _ in range(args.warmup):
            plan.product(a, bhat, out)
        barrier()
        t_start = time.time()
        e0.record(stream)
        for _ in range(args.steps):
            plan.product(a, bhat, out)
        e1.record(stream)
        barrier()
        clk.mark(t_start, time.time())
    ms = replicas.max_over_ranks(e0.elapsed_time(e1), "cuda")
    per_launch_s = ms * 1e-3 / args.steps
    accuracy = headline_accuracy(np, out.cpu().numpy().view(np.uint64), a_np, b_np, int(algo), base_n)
    value = world * count * args.steps / (ms * 1e-3)

    # one product alone: the automatic path (five launches for a lone product of this plan),
    # the fused kernel on one CTA, and the five launches on a caller-held workspace
    a1, bh1, o1 = a[:1].clone(), bhat[:1].clone(), out[:1].clone()
    ms_one_auto, _ = timed(torch, lambda: plan.product(a1, bh1, o1), 50, 5, local, world)
    plan.set_cluster_size(1)
    ms_one, _ = timed(torch, lambda: plan.product(a1, bh1, o1), 50, 5, local, world)
    plan.set_cluster_size(0)
    z1 = torch.empty((1, N_POLY // 2), dtype=torch.complex128, device="cuda")
    ms_one_u, _ = timed(torch, lambda: plan.product_unfused(a1, bh1, o1, z1), 50, 5, local, world)
    # the plain Plan path on the same products: five launches (fold+twist, forward FFT, pointwise,
    # inverse FFT, untwist+round) per batch, and per product (one launch per transform)
    z = torch.empty((count, N_POLY // 2), dtype=torch.complex128, device="cuda")
    out_plain = torch.empty_like(out)
    plain_steps = max(3, args.steps // 20)
    ms_pb, _ = timed(torch, lambda: plan.product_unfused(a, bhat, out_plain, z), plain_steps, 2, local, world)
    plain_ok = bool(torch.equal(out_plain, out))
    sample = 256

    def per_product():
        for i in range(sample):
            plan.product_unfused(a[i:i + 1], bhat[i:i + 1], out_plain[i:i + 1], z[i:i + 1])
    ms_pp, _ = timed(torch, per_product, 2, 1, local, world)
    # device time of one product (20 calls in a CUDA graph): the automatic path (a cluster of
    # CTAs on the base's residue classes), one CTA, the five launches
    one_dev = {"auto": graph_device_us(torch, lambda: plan.product(a1, bh1, o1))}
    plan.set_cluster_size(1)
    one_dev["one_cta"] = graph_device_us(torch, lambda: plan.product(a1, bh1, o1))
    plan.set_cluster_size(0)
    one_dev["five_launches"] = graph_device_us(torch, lambda: plan.product_unfused(a1, bh1, o1, z1))
    plain = {"batched_5_launches_products_per_s": world * count * plain_steps / (ms_pb * 1e-3),
             "per_product_5_launches_products_per_s": world * sample * 2 / (ms_pp * 1e-3),
             "per_product_sample": sample, "matches_fused_result": plain_ok,
             "one_product_us": round(ms_one_auto * 1e3 / 50, 2), "one_product_us_fused": round(ms_one * 1e3 / 50, 2),
             "one_product_us_5_launches": round(ms_one_u * 1e3 / 50, 2),
             "one_product_device_us": {k: round(v, 2) for k, v in one_dev.items()},
             "one_product_note": "one_product_us*: 50 calls from Python between CUDA events (host launch cost "
                                 "included); one_product_device_us: 20 calls in a CUDA graph"}

    # end to end: pinned host A in, pinned host result out, through the C ABI host entry point
    # (A crosses by copy; the kernels store the results into the page-locked `hout` over the link)
    ha = torch.from_numpy(a_np.view(np.int64)).pin_memory()
    hout = torch.empty_like(ha).pin_memory()
    for _ in range(max(1, args.warmup // 2)):
        plan.product(ha, bhat, hout)
    barrier()
    t0 = time.perf_counter()
    e2e_steps = max(3, args.steps // 10)
    for _ in range(e2e_steps):
        plan.product(ha, bhat, hout)
    e2e_s = replicas.max_over_ranks(time.perf_counter() - t0, "cuda")
    e2e = world * count * e2e_steps / e2e_s
    ok = bool(np.array_equal(hout.numpy(), out.cpu().numpy()))
    # the copies alone (pinned host <-> device, one direction at a time): the e2e ceiling
    copy_gbs = {}
    for name, (dst_t, src_t) in {"h2d": (a, ha), "d2h": (hout, out)}.items():
        dst_t.copy_(src_t, non_blocking=True)
        torch.cuda.synchronize()
        c0 = time.perf_counter()
        for _ in range(3):
            dst_t.copy_(src_t, non_blocking=True)
        torch.cuda.synchronize()
        copy_gbs[name] = 3 * src_t.numel() * 8 / (time.perf_counter() - c0) / 1e9
    # both directions at once on two streams (what the pipelined e2e path does)
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    torch.cuda.synchronize()
    c0 = time.perf_counter()
    for _ in range(3):
        with torch.cuda.stream(s_in):
            a.copy_(ha, non_blocking=True)
        with torch.cuda.stream(s_out):
            hout.copy_(out, non_blocking=True)
    torch.cuda.synchronize()
    copy_gbs["both_directions_total"] = 3 * 2 * ha.numel() * 8 / (time.perf_counter() - c0) / 1e9

    peaks, peak_kind = measured_peaks()
    achieved_gbs = BYTES_PER_PRODUCT * count / per_launch_s / 1e9
    traffic = profiled_traffic("u64_product_n2048")
    rates = fp64_rates(cf)
    fp64_peak = max(rates.values())
    fp64_ops = fp64_ops_per_product(N_POLY, base_n, int(algo))
    fp64_achieved = fp64_ops * count / per_launch_s

    del z, out_plain, ha, hout
    # the other benchmark configurations, each with its own clocks, roofline, e2e, accuracy and
    # CPU baseline (one GPU only)
    configs = None
    if world == 1 and not args.no_configs:
        configs = {}
        for name, fn in (("ordered_c64_n1024", lambda: measure_ordered(torch, cf, 50, 3, local, world)),
                         ("u128_product", lambda: measure_u128(torch, cf, 10, 3, local, world)),
                         ("mixed_batch_100k", lambda: measure_mixed(torch, cf, 3, 3, local, world)),
                         ("serving_20k_req_s", lambda: measure_serving(torch, cf, local, world)),
                         ("reference_bench_cases", lambda: measure_reference_cases(torch, cf, local, world)),
                         ("one_call_latency", lambda: measure_latency(torch, cf, local, world))):
            t_cfg = time.perf_counter()
            try:
                configs[name] = fn()
            except Exception as exc:  # recorded in the line, not hidden
                configs[name] = {"error": "%s: %s" % (type(exc).__name__, exc)}
            configs[name]["wall_s"] = round(time.perf_counter() - t_cfg, 1)
            torch.cuda.empty_cache()
    if rank != 0:
        return
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, done, el = cpu_product_rate(threads, args.cpu_seconds, BASE_SEED)
        calgo, cbase = cpu_fastest_algo(threads)
        rate1, done1, el1 = cpu_product_rate(1, args.cpu_seconds / 5, BASE_SEED)
        cpu = {"value": rate, "unit": "products/s", "cores": threads, "kind": "port",
               "single_thread_us_per_product": el1 / done1 * 1e6,
               "sample": "%d products (N=2048) in %.1f s on %d host threads, %s base %d (Method::Measure's pick "
                         "there); one thread: %d products in %.1f s"
                         % (done, el, threads, ALGO_NAMES[calgo], cbase, done1, el1)}
    line = {
        "metric": METRIC, "value": value, "unit": "products/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded numpy PCG64)",
        "config": {"workload": "u64 negacyclic product N=2048 (1024-point unordered c64 FFT), 8192 products "
                               "per launch, distinct resident Bhat per product",
                   "base_algo": algo.name, "base_n": base_n, "int_adds_eighths": int_adds,
                   "products_per_step": count,
                   "l2": "inputs 384 MiB > L2 (no flush needed)", "parallelism": "replicas" if world > 1 else "1 GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                     "frac": achieved_gbs / peaks.get("hbm_gbs"), "peak_kind": peak_kind,
                     "traffic": traffic.get("dram_bytes_per_launch") if traffic else None,
                     "algorithmic_bytes_per_launch": BYTES_PER_PRODUCT * count,
                     "fp64": {"achieved_ops_per_s": fp64_achieved, "peak_ops_per_s": fp64_peak,
                              "frac": fp64_achieved / fp64_peak, "ops_per_product": fp64_ops,
                              "microbenchmark_rates": rates,
                              "note": "binding roof: FP64 pipe (best DFMA/DADD/DMUL/mix issue rate, measured live)"}},
        "plain_path": plain,
        "cpu_baseline": cpu,
        "accuracy": accuracy,
        "e2e": {"value": e2e, "unit": "products/s", "h2d_bytes_per_step": count * N_POLY * 8,
                "d2h_bytes_per_step": count * N_POLY * 8, "steps": e2e_steps, "matches_device_result": ok,
                "copy_only_gbs": copy_gbs},
        "clocks": clk.summary(),
        "gpu_launches": args.steps,
        "configs": configs,
    }
    print(json.dumps(line))


# ---------------------------------------------------------------- other workloads
def fp64_ops_ordered(n, algo):
    return fp64_ops_per_transform(n, n, algo)


def gpu_setup():
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    sys.path.insert(0, PKG)
    import concrete_fft as cf
    cf.check(cf.load().cfft_device_check())
    return torch, cf, rank, world, local


def timed(torch, fn, steps, warmup, local, world):
    """CUDA-event time of `steps` calls of fn (after warm-up), max over ranks, with clocks."""
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        time.sleep(0.5)
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        t0 = time.time()
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        clk.mark(t0, time.time())
    from concrete_fft import replicas
    return replicas.max_over_ranks(e0.elapsed_time(e1), "cuda"), clk.summary()


def graph_device_us(torch, call, calls=20, replays=10):
    """Device time of one call: `calls` calls captured in a CUDA graph, replayed `replays`
    times between CUDA events (no host launch cost between the calls)."""
    call()  # outside the capture: one-time kernel attributes and launch shapes
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        for _ in range(calls):
            call()
    graph.replay()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(replays):
        graph.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) * 1e3 / (calls * replays)


def fp64_rates(cf):
    """FP64 thread-instruction rates of the DFMA, DADD, DMUL and mixed microbenchmarks."""
    import ctypes
    r = (ctypes.c_double * 4)()
    cf.check(cf.load().cfft_diag_fp64_rates(r))
    return dict(zip(("dfma", "dadd", "dmul", "mix_2add_1fma_1mul"), list(r)))


def fp64_peak(cf):
    """The FP64 roof: the best of the microbenchmark rates."""
    return max(fp64_rates(cf).values())


def _oracle():
    p = os.path.join(ROOT, "oracle")
    if p not in sys.path:
        sys.path.insert(0, p)
    import pyoracle
    return pyoracle


def host_threads():
    return os.cpu_count() or 1


def rel_l2(got, want):
    import numpy as np
    got, want = np.asarray(got), np.asarray(want)
    den = float(np.linalg.norm(want.ravel()))
    return float(np.linalg.norm((got - want).ravel())) / den if den else 0.0


def same_bits(got, want):
    import numpy as np
    return bool(np.array_equal(np.ascontiguousarray(got).view(np.uint64), np.ascontiguousarray(want).view(np.uint64)))


def cpu_loop(fn, seconds, min_reps=2):
    """Calls fn until `seconds` have passed (at least min_reps times); returns (reps, elapsed)."""
    fn()  # warm
    reps, t0 = 0, time.perf_counter()
    while True:
        fn()
        reps += 1
        el = time.perf_counter() - t0
        if el >= seconds and reps >= min_reps:
            return reps, el


_CPU_MEASURE = {}


def cpu_measure_ordered(po, n):
    """ordered::Plan's Method::Measure on the host (src/ordered.rs:99-180): the fastest of the 8
    algorithms for one n-point forward transform, single-threaded, on the restatement."""
    key = ("o", n)
    if key not in _CPU_MEASURE:
        import numpy as np
        x = np.random.default_rng(n).uniform(-1, 1, (max(1, 4096 // n), n)).astype(np.complex128)
        best = None
        for algo in range(8):
            w, _ = po.ordered_twiddles(po.radix(algo), n)
            reps, el = cpu_loop(lambda: po.ordered_batch_inplace(1, algo, x, w, 1), 0.02)
            if best is None or el / reps < best[0]:
                best = (el / reps, algo)
        _CPU_MEASURE[key] = best[1]
    return _CPU_MEASURE[key]


def cpu_measure_unordered(po, n):
    """unordered::Plan's Method::Measure on the host (src/unordered.rs:553-640): n <= 256 takes
    the ordered winner at n; otherwise bases 512 and 1024 (<= n), each with the ordered winner at
    the base, and the faster forward transform wins."""
    key = ("u", n)
    if key not in _CPU_MEASURE:
        import numpy as np
        if n <= 256:
            _CPU_MEASURE[key] = (cpu_measure_ordered(po, n), n)
        else:
            best = None
            for base in (512, 1024):
                if n < base:
                    break
                algo = cpu_measure_ordered(po, base)
                w, _ = po.unordered_twiddles(n, base, algo)
                x = np.random.default_rng(n).uniform(-1, 1, (max(1, 8192 // n), n)).astype(np.complex128)
                reps, el = cpu_loop(lambda: po.unordered_batch_inplace(1, algo, base, x, w, 1), 0.03)
                if best is None or el / reps < best[0]:
                    best = (el / reps, algo, base)
            _CPU_MEASURE[key] = best[1:]
    return _CPU_MEASURE[key]


def torus_bits_u128(got, exact):
    """Largest |got - exact| mod 2^128 (as a signed 128-bit difference) in bits, and the
    fraction of exact coefficients; arrays (..., N, 2) uint64 holding (lo, hi)."""
    import numpy as np
    g = np.ascontiguousarray(got, dtype=np.uint64).reshape(-1, 2)
    e = np.ascontiguousarray(exact, dtype=np.uint64).reshape(-1, 2)
    lo = g[:, 0] - e[:, 0]
    borrow = (g[:, 0] < e[:, 0]).astype(np.uint64)
    hi = (g[:, 1] - e[:, 1] - borrow).view(np.int64)
    small_pos = hi == 0
    small_neg = hi == -1
    mag = np.where(small_pos, lo.astype(np.float64), 0.0)
    mag = np.where(small_neg, (np.uint64(0) - lo).astype(np.float64), mag)
    big = ~(small_pos | small_neg)
    mag = np.where(big, np.abs(hi.astype(np.float64) + lo.astype(np.float64) / 2.0 ** 64) * 2.0 ** 64, mag)
    worst = float(mag.max()) if mag.size else 0.0
    exact_frac = float(((lo == 0) & (hi == 0)).mean()) if mag.size else 1.0
    return (float(np.log2(worst)) if worst > 0 else 0.0), exact_frac


def torus_bits_u64(got, exact):
    import numpy as np
    diff = (np.ascontiguousarray(got, dtype=np.uint64) - np.ascontiguousarray(exact, dtype=np.uint64)).view(np.int64)
    worst = float(np.abs(diff.astype(np.float64)).max()) if diff.size else 0.0
    return (float(np.log2(worst)) if worst > 0 else 0.0), float((diff == 0).mean()) if diff.size else 1.0


# ---------------------------------------------------------------- config 1: ordered c64
def measure_ordered(torch, cf, steps, warmup, local, world, full=False, cpu_seconds=2.0, cpu=True):
    """ordered::Plan n = 1024, forward then inverse: batch 256 (throughput) and batch 1
    (latency), accuracy against the oracle and numpy, e2e through the host entry points on a
    page-locked buffer, and the reference's CPU algorithm on the host cores."""
    import numpy as np
    po = _oracle()
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, (256, 1024)) + 1j * rng.uniform(-1, 1, (256, 1024))
    plan = cf.ordered.Plan(1024, cf.ordered.Method.Measure(0.002))
    algo = plan.algo()
    d = torch.from_numpy(x).cuda()
    # accuracy: one forward and one inverse of all 256 transforms against the oracle's
    # restatement of the same algorithm, and the forward against numpy's FFT
    plan.fwd(d)
    got_f = d.cpu().numpy()
    plan.inv(d)
    got_i = d.cpu().numpy()
    want_f = po.ordered_fwd(int(algo), x)
    want_i = po.ordered_inv(int(algo), want_f)
    accuracy = {"sample_transforms": 256, "rel_l2_fwd_vs_oracle": rel_l2(got_f, want_f),
                "rel_l2_inv_vs_oracle": rel_l2(got_i, want_i),
                "bit_identical_to_oracle": same_bits(got_f, want_f) and same_bits(got_i, want_i),
                "rel_l2_fwd_vs_numpy_fft": rel_l2(got_f, np.fft.fft(x, axis=-1)),
                "roundtrip_rel_l2": rel_l2(got_i / 1024, x),
                "bound": "c64 relative L2 <= 1e-13 against the reference (the oracle: same algorithm, same bits)"}
    d.copy_(torch.from_numpy(x))  # fwd+inv multiplies by n each step: start from the inputs
    one = d[:1].clone()

    def step256():
        plan.fwd(d)
        plan.inv(d)

    def step1():
        plan.fwd(one)
        plan.inv(one)

    ms256, clocks = timed(torch, step256, steps, warmup, local, world)
    d.copy_(torch.from_numpy(x))
    ms1, _ = timed(torch, step1, steps, warmup, local, world)
    # device-side batch-1 latency: 20 fwd+inv pairs in one CUDA graph (no host call between)
    graph20 = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph20):
        for _ in range(20):
            step1()
    reps20 = max(5, steps // 10)
    ms1g20, _ = timed(torch, graph20.replay, reps20, warmup, local, world)
    per = ms256 * 1e-3 / steps
    ops = 256 * 2 * fp64_ops_ordered(1024, int(algo))
    peak = fp64_peak(cf)
    peaks, peak_kind = measured_peaks()
    bytes_step = 256 * 2 * 32768  # each of the 512 calls reads and writes 16 KiB
    prof = profiled_traffic("split_kernel_ordered_n1024_b256") or {}
    # end to end through the host entry points on a page-locked buffer (in place across the link)
    h = torch.from_numpy(x.copy()).pin_memory()
    plan.fwd(h)
    plan.inv(h)
    h.copy_(torch.from_numpy(x))
    e2e_steps = max(3, steps // 5)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        plan.fwd(h)
        plan.inv(h)
    e2e = world * 512 * e2e_steps / (time.perf_counter() - t0)
    entry = {
        "metric": "ordered c64 n=1024 transforms/s (batch 256, fwd then inv)",
        "value": world * 512 * steps / (ms256 * 1e-3), "unit": "transforms/s", "steps": steps, "warmup": warmup,
        "ms_per_step": ms256 / steps, "higher_is_better": True, "dtype": "f64",
        "config": {"workload": "ordered::Plan n=1024, batch 256 and batch 1, fwd then inv (in place)",
                   "algo": algo.name, "l2": "8 MiB batch, L2-resident between calls (as in the reference's loop)",
                   "batch1_us_per_fwd_inv": ms1 * 1e3 / steps,
                   "batch1_us_per_fwd_inv_device": ms1g20 * 1e3 / (reps20 * 20)},
        "roofline": {"bound": "hbm", "achieved": bytes_step / per / 1e9, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": bytes_step / per / 1e9 / peaks["hbm_gbs"], "peak_kind": peak_kind,
                     "traffic": prof.get("dram_bytes_per_launch"),
                     "algorithmic_bytes_per_launch": 256 * 32768,
                     "fp64": {"achieved_ops_per_s": ops / per, "peak_ops_per_s": peak, "frac": ops / per / peak,
                              "ops_per_transform": fp64_ops_ordered(1024, int(algo)),
                              "note": "binding roof: FP64 pipe"}},
        "e2e": {"value": e2e, "unit": "transforms/s", "h2d_bytes_per_step": 2 * 256 * 1024 * 16,
                "d2h_bytes_per_step": 2 * 256 * 1024 * 16, "steps": e2e_steps,
                "path": "cfft_ordered_fwd_host / _inv_host on a page-locked buffer, in place"},
        "accuracy": accuracy, "clocks": clocks, "gpu_launches": 2 * steps,
    }
    if full:
        entry["config"].update(ordered_sweeps(torch, cf, plan, d, one, step1, steps, warmup, local, world, rng))
    if cpu and world == 1:
        threads = host_threads()
        calgo = cpu_measure_ordered(po, 1024)
        w, wi = po.ordered_twiddles(po.radix(calgo), 1024)
        x1 = np.ascontiguousarray(x[:1])

        def one_call():
            po.ordered_batch_inplace(1, calgo, x1, w, 1)
            po.ordered_batch_inplace(0, calgo, x1, wi, 1)
        reps1, el1 = cpu_loop(one_call, cpu_seconds / 4)
        xb = np.ascontiguousarray(np.tile(x, (max(1, threads // 4), 1)))

        def all_core():
            po.ordered_batch_inplace(1, calgo, xb, w, threads)
            po.ordered_batch_inplace(0, calgo, xb, wi, threads)
        repsb, elb = cpu_loop(all_core, cpu_seconds)
        entry["cpu_baseline"] = {
            "value": 2 * xb.shape[0] * repsb / elb, "unit": "transforms/s", "cores": threads, "kind": "port",
            "single_thread_us_per_fwd_inv": el1 / reps1 * 1e6,
            "single_thread_transforms_per_s": 2 * reps1 / el1, "algo": ALGO_NAMES[calgo],
            "sample": "%d x (fwd+inv of %d transforms, n=1024) on %d threads in %.1f s; batch 1 on one thread "
                      "(%s: Method::Measure's pick on this host, scalar restatement)"
                      % (repsb, xb.shape[0], threads, elb, ALGO_NAMES[calgo])}
    return entry


def ordered_sweeps(torch, cf, plan, d, one, step1, steps, warmup, local, world, rng):
    """The ordered workload's diagnostics: caller-captured graph replay, unordered batch-1
    latency by n, and the CTAs-per-transform sweep."""
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        step1()
    ms1g, _ = timed(torch, graph.replay, steps, warmup, local, world)
    large = {}
    for lgn in (12, 13, 14, 15):
        up = cf.unordered.Plan(1 << lgn, cf.unordered.Method.UserProvided(cf.FftAlgo.Dif4, 1024))
        u1 = torch.from_numpy(rng.uniform(-1, 1, (1, 1 << lgn)) + 0j).cuda()

        def stepu():
            up.fwd(u1)
            up.inv(u1)
        row = {}
        for ctas, name in ((0, "split"), (1, "one_cta_or_levels")):
            up.set_cluster_size(ctas)
            msu, _ = timed(torch, stepu, max(10, steps // 4), warmup, local, world)
            row[name] = round(msu * 1e3 / max(10, steps // 4), 2)
        large[1 << lgn] = row
    sweep = {}
    for aname in ("Dit4", "Dif4"):
        sp = cf.ordered.Plan(1024, cf.ordered.Method.UserProvided(cf.FftAlgo[aname]))
        sweep[aname] = {}
        for batch in (1, 16, 64, 256):
            sub = d[:batch].clone()

            def step_b():
                sp.fwd(sub)
                sp.inv(sub)
            row = {}
            for ctas in (0, 1, 2, 4, 8):
                sp.set_cluster_size(ctas)
                ms_b, _ = timed(torch, step_b, max(10, steps // 4), warmup, local, world)
                row["auto" if ctas == 0 else ctas] = round(ms_b * 1e3 / max(10, steps // 4), 2)
            sweep[aname][batch] = row
    # the same at batch 256 without spreading one-wave grids over every SM (cfft_diag_set_spread)
    lib = cf.load()
    no_spread = {}
    lib.cfft_diag_set_spread(0)
    try:
        for aname in ("Dit4", "Dif4"):
            sp = cf.ordered.Plan(1024, cf.ordered.Method.UserProvided(cf.FftAlgo[aname]))
            sub = d[:256].clone()

            def step_b():
                sp.fwd(sub)
                sp.inv(sub)
            row = {}
            for ctas in (0, 1, 2, 4, 8):
                sp.set_cluster_size(ctas)
                ms_b, _ = timed(torch, step_b, max(10, steps // 4), warmup, local, world)
                row["auto" if ctas == 0 else ctas] = round(ms_b * 1e3 / max(10, steps // 4), 2)
            no_spread[aname] = row
    finally:
        lib.cfft_diag_set_spread(1)
    return {"batch1_us_per_fwd_inv_graph_replay": ms1g * 1e3 / steps,
            "batch256_us_per_fwd_inv_without_spread": no_spread,
            "unordered_batch1_us_per_fwd_inv_by_n": large,
            "us_per_fwd_inv_by_batch_and_ctas_per_transform": sweep}


# ---------------------------------------------------------------- config 3: mixed batch
def mixed_items(cf, count, seed):
    import numpy as np
    rng = np.random.default_rng(seed)
    log2n = rng.integers(8, 17, count)
    kind = rng.integers(0, 2, count)
    kind = np.where(log2n > 10, 1, kind)  # the reference has no ordered plan above 1024 points
    sizes = (1 << log2n).astype(np.int64)
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.uint64)
    items = np.zeros(count, dtype=cf.batch.ITEM_DTYPE)
    items["offset"], items["log2n"], items["kind"], items["direction"] = offs, log2n, kind, 3
    return items, log2n, kind, sizes, offs, rng


def measure_mixed(torch, cf, steps, warmup, local, world, count=100000, tune_seconds=0.0005, seed=3,
                  cpu_seconds=3.0, cpu=True, e2e_steps=3):
    """100,000 c64 transforms, sizes 2^k with k uniform in 8..16, half ordered and half unordered,
    forward then inverse, one persistent launch per step (CUDA graph replay)."""
    import numpy as np
    po = _oracle()
    items, log2n, kind, sizes, offs, rng = mixed_items(cf, count, seed)
    total = int(sizes.sum())
    t0 = time.perf_counter()
    b = cf.batch.Batch(items, tune_seconds=tune_seconds)
    tune_s = time.perf_counter() - t0
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    data = (torch.rand((total, 2), dtype=torch.float64, device="cuda", generator=g) * 2 - 1)
    sample = rng.choice(count, 64, replace=False)
    saved = {int(i): data[int(offs[i]):int(offs[i]) + int(sizes[i])].clone() for i in sample}
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        ms, clocks = timed(torch, lambda: b.run(data), steps, warmup, local, world)
        # accuracy: the sampled items from their inputs again, one launch, against the oracle
        for i, v in saved.items():
            data[int(offs[i]):int(offs[i]) + int(sizes[i])].copy_(v)
        b.run(data)
        torch.cuda.current_stream().synchronize()
    worst_rel, identical, rt = 0.0, True, 0.0
    for i, v in saved.items():
        n = int(sizes[i])
        xs = v.cpu().numpy()
        xi = xs[:, 0] + 1j * xs[:, 1]
        got = data[int(offs[i]):int(offs[i]) + n].cpu().numpy()
        got = got[:, 0] + 1j * got[:, 1]
        algo, base, _ = b.schedule(int(kind[i]), int(log2n[i]), 3)
        if kind[i] == 0:
            want = po.ordered_inv(int(algo), po.ordered_fwd(int(algo), xi))
        else:
            want = po.unordered_inv(int(algo), base, po.unordered_fwd(int(algo), base, xi))
        worst_rel = max(worst_rel, rel_l2(got, want))
        identical = identical and same_bits(got, want)
        rt = max(rt, rel_l2(got / n, xi))
    accuracy = {"sample_items": len(saved), "max_rel_l2_vs_oracle": worst_rel, "bit_identical_to_oracle": identical,
                "max_roundtrip_rel_l2": rt,
                "against": "oracle restatement of the reference's ordered/unordered plans with the scheduled algorithm"}
    transforms = 2 * count
    value = world * transforms * steps / (ms * 1e-3)
    per_launch = ms * 1e-3 / steps
    ops = 0
    sched = {}
    for k in range(8, 17):
        for kd in (0, 1):
            sel = (log2n == k) & (kind == kd)
            if not sel.any():
                continue
            algo, base, tpc = b.schedule(kd, k, 3)
            sched["%s%d" % ("o" if kd == 0 else "u", k)] = [algo.name, base, tpc]
            ops += int(sel.sum()) * 2 * fp64_ops_per_transform(1 << k, base, int(algo))
    peak = fp64_peak(cf)
    bytes_alg = total * 32 * 2  # forward and inverse each read and write every point
    peaks, peak_kind = measured_peaks()
    prof = profiled_traffic("batch_kernel_mixed") or {}
    # end to end: pinned host data in and out, chunks of items pipelined (cfft_batch_run_host)
    host = data.cpu().pin_memory()
    with torch.cuda.stream(stream):
        b.run_host(host, data)  # builds the chunk tables
        torch.cuda.current_stream().synchronize()
        t1 = time.perf_counter()
        for _ in range(e2e_steps):
            b.run_host(host, data)
        torch.cuda.current_stream().synchronize()
    e2e_s = time.perf_counter() - t1
    del host, data
    entry = {
        "metric": "mixed-size c64 transforms/s (100k items, n=2^8..2^16, fwd then inv)", "value": value,
        "unit": "transforms/s", "steps": steps, "warmup": warmup, "ms_per_step": ms / steps,
        "higher_is_better": True, "dtype": "f64",
        "config": {"workload": "mixed batch, %d items, %d points, one persistent launch per step (graph)"
                               % (count, total),
                   "schedule": sched, "units": b.units(), "tune_seconds_total": tune_s,
                   "ordered_items": int((kind == 0).sum()), "l2": "23 GB of data > L2"},
        "roofline": {"bound": "hbm", "achieved": bytes_alg / per_launch / 1e9, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": bytes_alg / per_launch / 1e9 / peaks["hbm_gbs"], "peak_kind": peak_kind,
                     "traffic": (prof.get("dram_bytes_per_point") * total) if prof.get("dram_bytes_per_point") else None,
                     "algorithmic_bytes_per_launch": bytes_alg,
                     "fp64": {"achieved_ops_per_s": ops / per_launch, "peak_ops_per_s": peak,
                              "frac": ops / per_launch / peak, "note": "binding roof: FP64 pipe"}},
        "e2e": {"value": world * transforms * e2e_steps / e2e_s, "unit": "transforms/s",
                "h2d_bytes_per_step": total * 16, "d2h_bytes_per_step": total * 16, "steps": e2e_steps,
                "path": "cfft_batch_run_host from page-locked host memory, 16 pipelined chunks"},
        "accuracy": accuracy, "clocks": clocks, "gpu_launches": steps,
    }
    if cpu and world == 1:
        entry["cpu_baseline"] = cpu_mixed_rate(po, log2n, kind, cpu_seconds)
    return entry


def cpu_mixed_rate(po, log2n, kind, seconds):
    """The reference's CPU path over the mixed items, in item order, on every host thread (one
    Python thread per core driving the single-threaded restatement; ctypes releases the GIL),
    each size with the algorithm Method::Measure picks on this host."""
    import numpy as np
    from concurrent.futures import ThreadPoolExecutor
    threads = host_threads()
    tables = {}
    for k in range(8, 17):
        for kd in (0, 1):
            n = 1 << k
            if kd == 0 and k <= 10:
                a = cpu_measure_ordered(po, n)
                tables[(kd, k)] = (a, n, *po.ordered_twiddles(po.radix(a), n))
            elif kd == 1:
                a, base = cpu_measure_unordered(po, n)
                tables[(kd, k)] = (a, base, *po.unordered_twiddles(n, base, a))
    rng = np.random.default_rng(11)
    bufs = {k: rng.uniform(-1, 1, (threads, 1 << k)).astype(np.complex128) for k in range(8, 17)}
    stop_at = [None]
    done = [0] * threads

    def worker(t):
        i = t
        while time.perf_counter() < stop_at[0]:
            k, kd = int(log2n[i % len(log2n)]), int(kind[i % len(kind)])
            a, base, w, wi = tables[(kd, k)]
            buf = bufs[k][t:t + 1]
            if kd == 0:
                po.ordered_batch_inplace(1, a, buf, w, 1)
                po.ordered_batch_inplace(0, a, buf, wi, 1)
            else:
                po.unordered_batch_inplace(1, a, base, buf, w, 1)
                po.unordered_batch_inplace(0, a, base, buf, wi, 1)
            buf *= 1.0 / (1 << k)
            done[t] += 1
            i += threads
    t0 = time.perf_counter()
    stop_at[0] = t0 + seconds
    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(worker, range(threads)))
    el = time.perf_counter() - t0
    items_done = sum(done)
    return {"value": 2 * items_done / el, "unit": "transforms/s", "cores": threads, "kind": "port",
            "sample": "the first %d items of the 100k list (same size/kind mix), fwd+inv each, %d host threads, "
                      "%.1f s; per size the algorithm Method::Measure picks on this host (scalar restatement)"
                      % (items_done, threads, el),
            "host_algorithms": {("o%d" % k if kd == 0 else "u%d" % k): [ALGO_NAMES[v[0]], v[1]]
                                for (kd, k), v in sorted(tables.items())}}


# ---------------------------------------------------------------- config 4: u128 products
def measure_u128(torch, cf, steps, warmup, local, world, full=False, cpu_seconds=2.0, cpu=True, sample=64):
    """u128 negacyclic products N = 1024 and 4096, 2048 per launch, A uniform u128, B digits in
    [-2^15, 2^15); per N: device rate, accuracy on `sample` products against the exact
    wrapping-u128 schoolbook beside the restated reference pipeline's, and the CPU rate."""
    import numpy as np
    po = _oracle()
    threads = host_threads()
    by_n = {}
    clocks = None
    e2e = None
    count = 2048
    for N in (1024, 4096):
        plan = cf.product.U128ProductPlan(N)
        rng = np.random.default_rng(4)
        a_np = rng.integers(0, 2 ** 64, (count, N, 2), dtype=np.uint64)
        b_np = rng.integers(-2 ** 15, 2 ** 15, (count, N))
        a = torch.from_numpy(a_np.view(np.int64)).cuda()
        b = torch.from_numpy(b_np).cuda()
        bhat = torch.empty((count, 4, N // 2), dtype=torch.float64, device="cuda")
        plan.prepare_operand(b, bhat)
        out = torch.empty_like(a)
        ms, clk = timed(torch, lambda: plan.product(a, bhat, out), steps, warmup, local, world)
        clocks = clocks or clk
        a1, b1, o1 = a[:1].clone(), bhat[:1].clone(), out[:1].clone()
        ms1, _ = timed(torch, lambda: plan.product(a1, b1, o1), max(10, steps), warmup, local, world)
        rows = np.linspace(0, count - 1, sample).astype(np.int64)
        got = out.cpu().numpy().view(np.uint64)[rows]
        exact = po.schoolbook_batch(a_np[rows], b_np[rows], threads)
        ref = po.u128_product(N, a_np[rows], po.u128_prepare(N, b_np[rows]), nthreads=threads)
        gbits, gex = torus_bits_u128(got, exact)
        rbits, rex = torus_bits_u128(ref, exact)
        row = {"products_per_s": world * count * steps / (ms * 1e-3), "ms_per_launch": ms / steps,
               "one_product_us": round(ms1 * 1e3 / max(10, steps), 2),
               "accuracy": {"sample_products": sample, "gpu_max_torus_error_bits": gbits,
                            "gpu_exact_coefficient_fraction": gex,
                            "reference_pipeline_max_torus_error_bits": rbits,
                            "reference_pipeline_exact_coefficient_fraction": rex,
                            "gpu_equals_reference_pipeline": bool(np.array_equal(got, ref)),
                            "gpu_bits_le_reference_bits": gbits <= rbits,
                            "against": "exact wrapping-u128 schoolbook (oracle, unsigned __int128)"}}
        if N == 1024:  # end to end: pinned host A in and results out through the host entry point
            ha = a.cpu().pin_memory()
            hout = torch.empty_like(ha).pin_memory()
            plan.product(ha, bhat, hout)
            e2e_steps = max(3, steps // 3)
            t0 = time.perf_counter()
            for _ in range(e2e_steps):
                plan.product(ha, bhat, hout)
            e2e = {"value": world * count * e2e_steps / (time.perf_counter() - t0), "unit": "products/s",
                   "h2d_bytes_per_step": count * N * 16, "d2h_bytes_per_step": count * N * 16, "steps": e2e_steps,
                   "matches_device_result": bool(torch.equal(hout, out.cpu())), "N": N,
                   "path": "cfft_u128_product_host, page-locked A and result"}
        if cpu and world == 1:
            cs = max(64, 8 * threads)
            ca, cb = a_np[:cs], po.u128_prepare(N, b_np[:cs])
            reps, el = cpu_loop(lambda: po.u128_product(N, ca, cb, nthreads=threads), cpu_seconds / 2)
            reps1, el1 = cpu_loop(lambda: po.u128_product(N, ca[:1], cb[:1], nthreads=1), cpu_seconds / 8)
            row["cpu_products_per_s"] = cs * reps / el
            row["cpu_single_thread_us_per_product"] = el1 / reps1 * 1e6
            row["cpu_sample"] = "%d x %d products on %d threads in %.1f s" % (reps, cs, threads, el)
        by_n[N] = row
        del a, b, bhat, out
    prof = profiled_traffic("u128_product_n1024") or {}
    peak = fp64_peak(cf)
    peaks, peak_kind = measured_peaks()
    v = by_n[1024]["products_per_s"]
    fp64 = None
    if prof.get("fp64_thread_inst_per_product"):
        ach = prof["fp64_thread_inst_per_product"] * v
        fp64 = {"achieved_ops_per_s": ach, "peak_ops_per_s": peak, "frac": ach / peak,
                "ops_per_product": prof["fp64_thread_inst_per_product"],
                "note": "DADD/DFMA/DMUL per product counted by ncu (N=1024); the FP64 pipe also issues the "
                        "double-double code's comparisons and conversions"}
    # fft128::Plan itself at n = 512 (batch 4096 and batch 1), GPU and the host's restatement
    plans128 = {}
    for n, batch in (((512, 4096), (2048, 1024), (4096, 512), (16384, 128)) if full else ((512, 4096),)):
        fp = cf.fft128.Plan(n)
        bufs = [torch.rand((batch, n), dtype=torch.float64, device="cuda") for _ in range(4)]

        def step128():
            fp.fwd(*bufs)
            fp.inv(*bufs)
        s128 = max(5, steps)
        ms128, _ = timed(torch, step128, s128, warmup, local, world)
        one = [bb[:1].clone() for bb in bufs]

        def step1():
            fp.fwd(*one)
            fp.inv(*one)
        ms1, _ = timed(torch, step1, max(10, steps), warmup, local, world)
        row = {"transforms_per_s": world * 2 * batch * s128 / (ms128 * 1e-3), "batch": batch,
               "batch1_us_per_fwd_inv": round(ms1 * 1e3 / max(10, steps), 2)}
        if cpu and world == 1 and n == 512:
            t = po.f128_twiddles(n)
            rng = np.random.default_rng(12)
            hb = [rng.uniform(-1, 1, (4 * threads, n)) for _ in range(4)]

            def cpu_all():
                po.f128_batch_inplace(1, hb, t, threads)
                po.f128_batch_inplace(0, hb, t, threads)
                for v_ in hb:
                    v_ *= 1.0 / n
            reps, el = cpu_loop(cpu_all, cpu_seconds / 2)
            h1 = [v_[:1].copy() for v_ in hb]

            def cpu_one():
                po.f128_batch_inplace(1, h1, t, 1)
                po.f128_batch_inplace(0, h1, t, 1)
                for v_ in h1:
                    v_ *= 1.0 / n
            reps1, el1 = cpu_loop(cpu_one, cpu_seconds / 8)
            row["cpu_transforms_per_s"] = 2 * 4 * threads * reps / el
            row["cpu_single_thread_us_per_fwd_inv"] = el1 / reps1 * 1e6
        plans128[n] = row
        del bufs
    entry = {
        "metric": "u128 negacyclic polymul/s (double-double), N=1024", "value": v, "unit": "products/s",
        "steps": steps, "warmup": warmup, "ms_per_step": by_n[1024]["ms_per_launch"], "higher_is_better": True,
        "dtype": "f64x2 (double-double)",
        "config": {"workload": "u128 products N=1024 and N=4096, 2048 per launch, A uniform u128, "
                               "B digits in [-2^15, 2^15)", "by_N": by_n, "fft128_plan_fwd_inv_by_n": plans128,
                   "l2": "N=1024: 96 MiB per launch (A, Bhat, out); N=4096: 384 MiB"},
        "roofline": {"bound": "hbm", "achieved": v * 49152 / 1e9, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": v * 49152 / 1e9 / peaks["hbm_gbs"], "peak_kind": peak_kind,
                     "traffic": prof.get("dram_bytes_per_launch"),
                     "algorithmic_bytes_per_launch": 49152 * count, "fp64": fp64,
                     "note": "N=1024: 49,152 algorithmic bytes per product; bound by the FP64 pipe"},
        "e2e": e2e,
        "accuracy": {"N%d" % N: r["accuracy"] for N, r in by_n.items()},
        "clocks": clocks, "gpu_launches": 4 * steps,
    }
    if cpu and world == 1:
        entry["cpu_baseline"] = {
            "value": by_n[1024]["cpu_products_per_s"], "unit": "products/s", "cores": threads, "kind": "port",
            "N4096_products_per_s": by_n[4096]["cpu_products_per_s"],
            "single_thread_us_per_product": {N: r["cpu_single_thread_us_per_product"] for N, r in by_n.items()},
            "fft128_n512": {k: plans128[512][k] for k in ("cpu_transforms_per_s", "cpu_single_thread_us_per_fwd_inv")},
            "sample": "N=1024: %s; restated reference pipeline (fft128 double-double, scalar)"
                      % by_n[1024]["cpu_sample"]}
    return entry


# ---------------------------------------------------------------- the reference's own bench cases
def reference_case_tables(torch, cf, local, world, cpu=True, cpu_seconds=0.04):
    """The cases of the reference's benches/fft.rs, one call each as criterion times them:
    ordered fwd (n <= 1024), unordered fwd, unordered inv and fwd_monomial for n = 2^8..2^16
    (plans from Method::Measure), and fft128 negacyclic fwd/inv for n = 64..16384.  Per case:
    the GPU's device time per call (20 calls of one transform replayed from a CUDA graph, so no
    host call sits between them), the time per call through the host-slice entry point on a
    pageable buffer (what a caller of the slice API pays, Python's call overhead included),
    the GPU's batched rate (2^22 points per call), and the restated reference's time per call
    on one host core with the algorithm its Method::Measure picks there."""
    import numpy as np
    po = _oracle()
    stream = torch.cuda.current_stream()

    def events_ms(fn, steps, warmup):  # CUDA events on the launching stream (clocks: the configs' samplers)
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    def device_us(call):
        call()  # first call outside the capture (one-time kernel attributes and launch shapes)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            for _ in range(20):
                call()
        return events_ms(graph.replay, 10, 2) * 1e3 / 200

    def host_us(call, reps=20):
        call()
        t0 = time.perf_counter()
        for _ in range(reps):
            call()
        return (time.perf_counter() - t0) * 1e6 / reps

    def batched_per_s(call, count):
        return count * 5 / (events_ms(call, 5, 2) * 1e-3)

    rows = {}
    rng = np.random.default_rng(13)
    for k in range(8, 17):
        n = 1 << k
        batch = max(1, (1 << 22) // n)
        one = torch.from_numpy(rng.uniform(-1, 1, (1, n)) + 1j * rng.uniform(-1, 1, (1, n))).cuda()
        many = torch.empty((batch, n), dtype=torch.complex128, device="cuda").normal_()
        host = (rng.uniform(-1, 1, (1, n)) + 1j * rng.uniform(-1, 1, (1, n))).astype(np.complex128)
        up = cf.unordered.Plan(n, cf.unordered.Method.Measure(0.002))
        ua, ub = up.algo()
        row = {"gpu_unordered_plan": "%s/%d" % (ua.name, ub)}
        cases = [("unordered_fwd", lambda b: up.fwd(b)), ("unordered_inv", lambda b: up.inv(b)),
                 ("fwd_monomial", lambda b: up.fwd_monomial(n // 3, b))]
        if n <= 1024:
            op = cf.ordered.Plan(n, cf.ordered.Method.Measure(0.002))
            row["gpu_ordered_plan"] = op.algo().name
            cases.insert(0, ("ordered_fwd", lambda b: op.fwd(b)))
        for name, fn in cases:
            r = {"gpu_device_us": round(device_us(lambda: fn(one)), 3),
                 "host_slice_api_us": round(host_us(lambda: fn(host)), 2)}
            if name != "fwd_monomial":
                r["gpu_batched_transforms_per_s"] = batched_per_s(lambda: fn(many), batch)
            rows.setdefault(n, row)[name] = r
        if cpu and world == 1:
            ca, cb = cpu_measure_unordered(po, n)
            row["cpu_unordered_plan"] = "%s/%d" % (ALGO_NAMES[ca], cb)
            row["unordered_fwd"]["cpu_one_core_us"] = round(po.bench_call(1, n, ca, cb, cpu_seconds) * 1e6, 2)
            row["unordered_inv"]["cpu_one_core_us"] = round(po.bench_call(2, n, ca, cb, cpu_seconds) * 1e6, 2)
            row["fwd_monomial"]["cpu_one_core_us"] = round(po.bench_call(3, n, 0, cb, cpu_seconds) * 1e6, 3)
            if n <= 1024:
                oa = cpu_measure_ordered(po, n)
                row["cpu_ordered_plan"] = ALGO_NAMES[oa]
                row["ordered_fwd"]["cpu_one_core_us"] = round(po.bench_call(0, n, oa, 0, cpu_seconds) * 1e6, 2)
        rows[n] = row
        del one, many
    f128rows = {}
    for k in range(6, 15):
        n = 1 << k
        batch = max(1, (1 << 20) // n)
        fp = cf.fft128.Plan(n)
        one = [torch.rand((1, n), dtype=torch.float64, device="cuda") for _ in range(4)]
        many = [torch.rand((batch, n), dtype=torch.float64, device="cuda") for _ in range(4)]
        host = [np.random.default_rng(k).uniform(-1, 1, (1, n)) for _ in range(4)]
        row = {}
        for name, fn in (("fwd", fp.fwd), ("inv", fp.inv)):
            row[name] = {"gpu_device_us": round(device_us(lambda: fn(*one)), 3),
                         "host_slice_api_us": round(host_us(lambda: fn(*host)), 2),
                         "gpu_batched_transforms_per_s": batched_per_s(lambda: fn(*many), batch)}
            if cpu and world == 1:
                row[name]["cpu_one_core_us"] = round(po.bench_call(4 if name == "fwd" else 5, n, 0, 0, cpu_seconds)
                                                     * 1e6, 2)
        f128rows[n] = row
        del one, many
    return rows, f128rows


def measure_reference_cases(torch, cf, local, world, cpu=True, cpu_seconds=0.04):
    """reference_case_tables under an nvidia-smi clock sampler."""
    with ClockSampler(local) as clk:
        t0 = time.time()
        rows, f128rows = reference_case_tables(torch, cf, local, world, cpu, cpu_seconds)
        clk.mark(t0, time.time())
    return {"c64": rows, "fft128": f128rows, "clocks": clk.summary(),
            "cpu": "restated reference, one host thread, scalar (the reference's own Scalar backend on this Arm "
                   "host), each call timed in a loop in C as criterion does",
            "gpu_device": "20 calls of one transform in a CUDA graph, replayed 10 times, CUDA events",
            "host_slice_api": "cfft_*_fwd_host / _inv_host / fwd_monomial_host on a pageable numpy buffer, from "
                              "Python (staged copies in and out)"}


# ---------------------------------------------------------------- config 5: serving
SERVE_SIZES = [10, 11, 12, 13, 14]


def measure_serving(torch, cf, local, world, rate=20000.0, seconds=1.0, operand_gb=8, full=False, cpu=True,
                    cpu_seconds=2.0, seed=5, check_requests=64):
    """Poisson stream of (k+1)*l-product requests, N in 2^10..2^14, 8 GiB of resident Fourier
    operands: continuous batching against the plain one-launch-per-step loop on the same
    seeded stream, and a sample of served results against the same requests run alone."""
    import numpy as np
    eng = cf.serving.ProductEngine(SERVE_SIZES)
    t0 = time.perf_counter()
    srv = cf.serving.Server(eng, SERVE_SIZES, operand_bytes=operand_gb << 30, seed=seed)
    setup_s = time.perf_counter() - t0
    # warm-up as long as the timed run: a process's first runs show a longer tail, and the
    # timed run's results then land in output-ring pages the device has written before
    srv.run(srv.config(rate=rate, duration_s=seconds))
    cfg = srv.config(rate=rate, duration_s=seconds)
    with ClockSampler(local, interval_ms=1000) as clk:
        time.sleep(0.5)  # the sampler's start-up (a process on the host) stays out of the timed run
        t1 = time.time()
        batched = srv.run(cfg)
        clk.mark(t1, time.time())
    # the same stream again, keeping every 50th request's results for the check (copying
    # results out in the serving thread delays the requests behind them: not timed)
    cfg_rec = srv.config(rate=rate, duration_s=seconds, record_every=50)
    srv.run(cfg_rec)
    ids = srv.recorded_ids()[:check_requests]
    same = all(np.array_equal(srv.recorded_output(cfg_rec, int(r)), srv.run_alone(cfg_rec, int(r))) for r in ids)
    extra = {}
    if full:
        extra["batched_without_clusters"] = srv.run(srv.config(rate=rate, duration_s=seconds, cluster_log2N=32))
        extra["batched_staged_io"] = srv.run(srv.config(rate=rate, duration_s=seconds, staged_io=True))
        extra["batched_via_queue"] = srv.run(srv.config(rate=rate, duration_s=seconds, via_queue=True))
        # the memory gate on a fixed stand-in budget instead of cudaMemGetInfo readings (its cost)
        extra["batched_gate_without_readings"] = srv.run(srv.config(rate=rate, duration_s=seconds,
                                                                    mem_free_override=1 << 50))
        extra["batched_repeat"] = srv.run(srv.config(rate=rate, duration_s=seconds))  # the first run, again
        sweep = {}
        for r in (50000.0, 100000.0, 150000.0, 200000.0):
            st = srv.run(srv.config(rate=r, duration_s=0.5))
            sweep["%d" % r] = {k: st[k] for k in ("products_per_s", "p50_ms", "p99_ms", "max_ms", "launches",
                                                  "mean_batch", "deferred_admissions") if k in st}
        extra["capacity_sweep_req_per_s"] = sweep
    # the comparator last: it saturates and queues for seconds
    plain = srv.run(srv.config(rate=rate, duration_s=seconds, plain=True))
    out_bytes = batched.get("output_bytes", 0)
    entry = {
        "metric": "serving: products/s and p50/p99 latency, Poisson %g req/s" % rate,
        "value": batched["products_per_s"], "unit": "products/s", "steps": 1, "warmup": 1,
        "higher_is_better": True, "dtype": "f64",
        "config": {"workload": "serving, (k+1)*l products per request, k in 1..2, l in 1..4, N in 2^10..2^14, "
                               "digits b in 4..10 bits, resident operands %d GiB" % operand_gb,
                   "duration_s": seconds, "resident_setup_s": setup_s},
        "value_note": "the offered load is served in full: products/s equals the arrival rate's products; the "
                      "serving workload's capacity sweep gives the loop's ceiling",
        "p50_ms": batched["p50_ms"], "p99_ms": batched["p99_ms"],
        "plain_p50_ms": plain["p50_ms"], "plain_p99_ms": plain["p99_ms"],
        "p99_speedup_vs_plain": plain["p99_ms"] / batched["p99_ms"] if batched["p99_ms"] else None,
        "batched": batched, "plain": plain,
        "accuracy": {"checked_requests": len(ids), "same_alone_and_in_the_mix": bool(same),
                     "against": "each recorded request of a second run of the same stream recomputed alone "
                                "(outside any mix), bit for bit"},
        "e2e": {"value": batched["products_per_s"], "unit": "products/s", "h2d_bytes_per_step": batched.get("input_bytes"),
                "d2h_bytes_per_step": out_bytes,
                "path": "requests admitted on the host as they arrive; item records read from and results stored "
                        "into page-locked host memory by the kernels; latency from arrival to completion on the "
                        "host clock"},
        "clocks": clk.summary(), "gpu_launches": batched["launches"],
    }
    entry.update(extra)
    if cpu and world == 1:
        entry["cpu_baseline"] = cpu_serving_rate(srv, cfg, cpu_seconds)
    del srv, eng
    return entry


def cpu_serving_rate(srv, cfg, seconds):
    """The restated reference pipeline on the host cores over the served requests' products
    (each request's digit rows times its Fourier operands, per size with the plan's algorithm),
    in request order until `seconds` have passed: products/s."""
    import numpy as np
    from concurrent.futures import ThreadPoolExecutor
    po = _oracle()
    threads = host_threads()
    reqs = []
    for rid in range(4096):
        lN, npd = srv.shape(cfg, rid)
        digits, bhat = srv.inputs(cfg, rid)
        algo, base = srv.engine.algo(lN)
        reqs.append((1 << lN, algo, base, digits.view(np.uint64), bhat))
    stop_at = [None]
    done = [0] * threads

    def worker(t):
        i = t
        while time.perf_counter() < stop_at[0]:
            N, algo, base, a, bh = reqs[i % len(reqs)]
            po.u64_product(N, algo, base, a, bh, nthreads=1)
            done[t] += a.shape[0]
            i += threads
    t0 = time.perf_counter()
    stop_at[0] = t0 + seconds
    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(worker, range(threads)))
    el = time.perf_counter() - t0
    return {"value": sum(done) / el, "unit": "products/s", "cores": threads, "kind": "port",
            "sample": "%d products of the first 4096 requests of the same seeded stream (N in 2^10..2^14), in "
                      "request order and repeated, on %d host threads in %.1f s, the restated reference pipeline "
                      "with each size's plan algorithm; a capacity (all requests present), not a served rate"
                      % (sum(done), threads, el)}


def print_line(entry, world, data="synthetic (seeded)"):
    line = {"metric": entry["metric"], "value": entry["value"], "unit": entry["unit"], "n_gpus": world,
            "steps": entry.get("steps"), "warmup": entry.get("warmup"), "ms_per_step": entry.get("ms_per_step"),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": entry.get("dtype", "f64"),
            "data": data}
    line.update({k: v for k, v in entry.items() if k not in line})
    print(json.dumps(line))


def autotune_check(torch, cf, schedule, local, world, points=1 << 24):
    """Whether the persistent kernel's per-size schedule (Dif4 / Dif8, bases 512 / 1024) is the best
    of every candidate the reference's Method::Measure considers: per size, the standalone plan
    of each (algorithm, base) times forward+inverse over 2^24 points of that size, and the best
    is compared with the algorithm and base the mixed batch scheduled (same FP64 work per
    transform, so the standalone ranking carries over)."""
    rows = {}
    for k in range(8, 17):
        n = 1 << k
        batch = points // n
        x = torch.empty((batch, n, 2), dtype=torch.float64, device="cuda")
        cands = {}
        bases = [n] if n <= 512 else [bb for bb in (512, 1024) if bb <= n]
        for base in bases:
            for a in range(8):
                algo = cf.FftAlgo(a)
                plan = cf.unordered.Plan(n, cf.unordered.Method.UserProvided(algo, base))
                x.uniform_(-1, 1)  # six forward+inverse steps grow the data by at most n^6 <= 2^96

                def step():
                    plan.fwd(x)
                    plan.inv(x)
                ms, _ = timed(torch, step, 4, 2, local, world)
                cands["%s/%d" % (algo.name, base)] = ms * 1e3 / 4 / (2 * batch)
        best = min(cands, key=cands.get)
        sched = schedule.get("u%d" % k)
        sname = "%s/%d" % (sched[0], sched[1]) if sched else None
        rows[n] = {"best": best, "best_us_per_transform": round(cands[best], 4), "scheduled": sname,
                   "scheduled_us_per_transform": round(cands[sname], 4) if sname in cands else None,
                   "gap_pct": round(100 * (cands[sname] / cands[best] - 1), 2) if sname in cands else None,
                   "fp64_ops_per_point": {c: fp64_ops_per_transform(n, int(c.split("/")[1]),
                                                                    int(cf.FftAlgo[c.split("/")[0]])) / n
                                          for c in (best, sname) if c},
                   "fastest_candidates_us": {c: round(v, 4) for c, v in sorted(cands.items(), key=lambda kv: kv[1])[:6]}}
        del x
    return rows


def run_mixed(args):
    """The mixed-size batch (100,000 items) as its own JSON line, with the check of the
    persistent kernel's per-size schedule against every Method::Measure candidate."""
    torch, cf, rank, world, local = gpu_setup()
    if args.profile_case:  # for ncu: two persistent launches over --mixed-items items of the same mix
        items, log2n, kind, sizes, offs, rng = mixed_items(cf, args.mixed_items, 3)
        b = cf.batch.Batch(items, tune_seconds=args.tune_seconds)
        total = int(sizes.sum())
        data = torch.rand((total, 2), dtype=torch.float64, device="cuda") * 2 - 1
        for _ in range(2):
            b.run(data)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "mixed batch x2", "items": args.mixed_items, "points": total}))
        return
    entry = measure_mixed(torch, cf, args.steps, args.warmup, local, world, count=args.mixed_items,
                          tune_seconds=args.tune_seconds, seed=3 + rank, cpu=not args.no_cpu_baseline and rank == 0,
                          cpu_seconds=args.cpu_seconds)
    torch.cuda.empty_cache()
    entry["autotune_check"] = autotune_check(torch, cf, entry["config"]["schedule"], local, world)
    if rank == 0:
        print_line(entry, world)


def run_ordered(args):
    """ordered::Plan n = 1024 with the full set of latency diagnostics, as its own JSON line."""
    import numpy as np
    torch, cf, rank, world, local = gpu_setup()
    if args.profile_case:  # for ncu: 4 forward calls of batch 256 split over 4 CTAs per transform
        rng = np.random.default_rng(1)
        x = rng.uniform(-1, 1, (256, 1024)) + 1j * rng.uniform(-1, 1, (256, 1024))
        d = torch.from_numpy(x).cuda()
        algo = cf.FftAlgo[args.base_algo] if args.base_algo else cf.FftAlgo.Dit4
        plan = cf.ordered.Plan(1024, cf.ordered.Method.UserProvided(algo))
        plan.set_cluster_size(args.cluster_size if args.cluster_size is not None else 4)
        for _ in range(4):
            plan.fwd(d)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "ordered n=1024 batch 256", "algo": algo.name}))
        return
    entry = measure_ordered(torch, cf, args.steps, args.warmup, local, world, full=True,
                            cpu=not args.no_cpu_baseline and rank == 0, cpu_seconds=args.cpu_seconds)
    if rank == 0:
        print_line(entry, world)


def run_u128(args):
    """u128 negacyclic products N = 1024 and 4096 and the fft128 plan, as its own JSON line."""
    torch, cf, rank, world, local = gpu_setup()
    if args.profile_case:  # for ncu: four forward calls of the fft128 plan (n = 512, batch 4096),
        # then two launches of 2048 u128 products at N = 1024 (the timed shape)
        import numpy as np
        fp = cf.fft128.Plan(512)
        bufs = [torch.rand((4096, 512), dtype=torch.float64, device="cuda") for _ in range(4)]
        for _ in range(4):
            fp.fwd(*bufs)
        N, count = 1024, 2048
        plan = cf.product.U128ProductPlan(N)
        rng = np.random.default_rng(4)
        a = torch.from_numpy(rng.integers(0, 2 ** 64, (count, N, 2), dtype=np.uint64).view(np.int64)).cuda()
        b = torch.from_numpy(rng.integers(-2 ** 15, 2 ** 15, (count, N))).cuda()
        bhat = torch.empty((count, 4, N // 2), dtype=torch.float64, device="cuda")
        plan.prepare_operand(b, bhat)
        out = torch.empty_like(a)
        for _ in range(2):
            plan.product(a, bhat, out)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "fft128 plan n=512 batch 4096 forward x4; u128 products N=1024 x2048 x2"}))
        return
    entry = measure_u128(torch, cf, args.steps, args.warmup, local, world, full=True,
                         cpu=not args.no_cpu_baseline and rank == 0, cpu_seconds=args.cpu_seconds)
    if rank == 0:
        print_line(entry, world)


def run_product_sum(args):
    """External-product shape: groups of T = 8 products N = 2048 summed in the Fourier domain
    (one inverse per group), 1024 groups per launch; reported as products/s (8192 per launch)."""
    import numpy as np
    torch, cf, rank, world, local = gpu_setup()
    N, T, groups = 2048, 8, 1024
    plan = cf.product.U64ProductPlan(N, cf.FftAlgo.Dif4, 1024)
    rng = np.random.default_rng(6 + rank)
    a = torch.from_numpy(rng.integers(0, 2 ** 64, (groups, T, N), dtype=np.uint64).view(np.int64)).cuda()
    b = torch.from_numpy(rng.integers(-2 ** 7, 2 ** 7, (groups * T, N))).cuda()
    bhat = torch.empty((groups, T, N // 2), dtype=torch.complex128, device="cuda")
    plan.prepare_operand(b, bhat)
    out = torch.empty((groups, N), dtype=torch.int64, device="cuda")
    if args.profile_case:  # for ncu: two launches of the timed shape
        for _ in range(2):
            plan.product_sum(a, bhat, out)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "product_sum 1024 groups x 8 terms, N=2048, x2"}))
        return
    ms, clocks = timed(torch, lambda: plan.product_sum(a, bhat, out), args.steps, args.warmup, local, world)
    per = ms * 1e-3 / args.steps
    n = N // 2
    ops = groups * (T * (fp64_ops_per_transform(n, 1024, 2) + 4 * n + 4 * n + 2 * n) - 2 * n
                    + fp64_ops_per_transform(n, 1024, 2) + 4 * n)
    peak = fp64_peak(cf)
    peaks, peak_kind = measured_peaks()
    alg_bytes = groups * T * N * 8 + groups * T * n * 16 + groups * N * 8  # A and Bhat read, sums written
    if rank != 0:
        return
    print(json.dumps({
        "metric": "N=2048 products/s summed in the Fourier domain (8 per output)",
        "value": world * groups * T / per, "unit": "products/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded numpy PCG64)",
        "config": {"workload": "1024 groups x 8 products, one inverse per group"},
        "roofline": {"bound": "hbm", "achieved": alg_bytes / per / 1e9, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": alg_bytes / per / 1e9 / peaks["hbm_gbs"], "peak_kind": peak_kind,
                     "traffic": (profiled_traffic("u64_product_sum_n2048") or {}).get("dram_bytes_per_launch"),
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "fp64": {"achieved_ops_per_s": ops / per, "peak_ops_per_s": peak, "frac": ops / per / peak}},
        "clocks": clocks, "gpu_launches": args.steps,
    }))


def run_serving(args):
    """The Poisson request loop with the full set of variants and the capacity sweep."""
    torch, cf, rank, world, local = gpu_setup()
    if args.profile_case:  # for ncu: a short batched run only
        eng = cf.serving.ProductEngine(SERVE_SIZES)
        srv = cf.serving.Server(eng, SERVE_SIZES, operand_bytes=args.operand_gb << 30, seed=5 + rank)
        srv.run(srv.config(rate=args.rate, duration_s=0.05))
        st = srv.run(srv.config(rate=args.rate, duration_s=0.1))
        print(json.dumps({"profile_case": "serving 0.1 s", "launches": st.get("launches")}))
        return
    entry = measure_serving(torch, cf, local, world, rate=args.rate, seconds=args.serve_seconds,
                            operand_gb=args.operand_gb, full=True, cpu=not args.no_cpu_baseline and rank == 0,
                            cpu_seconds=args.cpu_seconds, seed=5 + rank)
    if rank == 0:
        print_line(entry, world, data="synthetic (seeded Poisson stream, resident operands %d GiB)" % args.operand_gb)


def measure_latency(torch, cf, local, world, cpu=True, cpu_seconds=0.5, profile_case=False):
    """One call at a time on device-resident data, device time per call (20 calls in a CUDA
    graph): u64 products of N = 2048 to 65536 (Method::Measure plans) on the automatic path
    (a cluster over the base's residue classes for a few products), on one CTA and as five
    launches; u128 products of N = 1024 and 8192; fft128 and unordered transforms.  Beside them the
    restated reference pipeline on one host core."""
    import numpy as np
    po = _oracle() if cpu and world == 1 else None
    rng = np.random.default_rng(21)
    if profile_case:
        # ncu case: 20 lone products of N = 2048 (Dif4, base 1024) and 20 fft128 forwards of 512,
        # then 20 fft128 forwards of 16384
        plan = cf.product.U64ProductPlan(2048, cf.FftAlgo.Dif4, 1024)
        a = torch.from_numpy(rng.integers(0, 2 ** 64, (1, 2048), dtype=np.uint64).view(np.int64)).cuda()
        bh = torch.empty((1, 1024), dtype=torch.complex128, device="cuda")
        plan.prepare_operand(torch.from_numpy(rng.integers(-128, 128, (1, 2048))).cuda(), bh)
        out = torch.empty_like(a)
        fp = cf.fft128.Plan(512)
        arrs = [torch.rand((1, 512), dtype=torch.float64, device="cuda") for _ in range(4)]
        for _ in range(20):
            plan.product(a, bh, out)
            fp.fwd(*arrs)
        # then 20 fft128 forwards of 16384 points, batch 1 (half-butterfly stages and blocks)
        fb = cf.fft128.Plan(16384)
        big = [torch.rand((1, 16384), dtype=torch.float64, device="cuda") for _ in range(4)]
        for _ in range(20):
            fb.fwd(*big)
        torch.cuda.synchronize()
        return {"profile_case": "20 lone u64 products N=2048 (Dif4/1024) and 20 fft128 forwards n=512, "
                                "then 20 fft128 forwards n=16384"}
    rows = {}
    with ClockSampler(local) as clk:
        t0 = time.time()
        for N in (2048, 4096, 8192, 16384, 32768, 65536):
            plan = cf.product.U64ProductPlan(N, measure_seconds=0.002)
            algo, base = plan.algo()
            a_np = rng.integers(0, 2 ** 64, (1, N), dtype=np.uint64)
            b_np = rng.integers(-128, 128, (1, N))
            a = torch.from_numpy(a_np.view(np.int64)).cuda()
            bh = torch.empty((1, N // 2), dtype=torch.complex128, device="cuda")
            plan.prepare_operand(torch.from_numpy(b_np).cuda(), bh)
            out = torch.empty_like(a)
            z = torch.empty((1, N // 2), dtype=torch.complex128, device="cuda")
            row = {"plan": "%s/%d" % (ALGO_NAMES[int(algo)], base),
                   "auto_us": graph_device_us(torch, lambda: plan.product(a, bh, out))}
            ok = out.clone()
            plan.set_cluster_size(1)
            row["one_cta_us"] = graph_device_us(torch, lambda: plan.product(a, bh, out))
            plan.set_cluster_size(0)
            row["five_launches_us"] = graph_device_us(torch, lambda: plan.product_unfused(a, bh, out, z))
            if N >= 16384:  # the kernel with level-0 slices only, on 8 CTAs
                plan.set_cluster_size(8)
                row["level_slices_8_ctas_us"] = graph_device_us(torch, lambda: plan.product(a, bh, out))
                plan.set_cluster_size(0)
            row["paths_agree"] = bool(torch.equal(out, ok))
            if po is not None and N <= 16384:  # per product, over calls of 32 (the plan's set-up spread)
                ca = rng.integers(0, 2 ** 64, (32, N), dtype=np.uint64)
                wb = po.u64_prepare(N, int(algo), base, rng.integers(-128, 128, (32, N)))
                reps, el = cpu_loop(lambda: po.u64_product(N, int(algo), base, ca, wb, nthreads=1), cpu_seconds)
                row["cpu_one_core_us"] = el / (32 * reps) * 1e6
            rows["u64_product_N%d" % N] = {k: (round(v, 2) if isinstance(v, float) else v) for k, v in row.items()}
        # one external product of a blind-rotation step: 2 outputs, each the Fourier-domain
        # sum of 4 products (k + 1 = 2, l = 2), N = 2048 and 4096
        for N in (2048, 4096):
            plan = cf.product.U64ProductPlan(N, measure_seconds=0.002)
            algo, base = plan.algo()
            a_np = rng.integers(0, 2 ** 64, (2, 4, N), dtype=np.uint64)
            b_np = rng.integers(-128, 128, (8, N))
            a = torch.from_numpy(a_np.view(np.int64)).cuda()
            bh = torch.empty((2, 4, N // 2), dtype=torch.complex128, device="cuda")
            plan.prepare_operand(torch.from_numpy(b_np).cuda(), bh)
            out = torch.empty((2, N), dtype=torch.int64, device="cuda")
            row = {"plan": "%s/%d" % (ALGO_NAMES[int(algo)], base),
                   "auto_us": graph_device_us(torch, lambda: plan.product_sum(a, bh, out))}
            ok = out.clone()
            plan.set_cluster_size(1)
            row["one_cta_per_output_us"] = graph_device_us(torch, lambda: plan.product_sum(a, bh, out))
            plan.set_cluster_size(0)
            row["paths_agree"] = bool(torch.equal(out, ok))
            if po is not None:  # per external product, over calls of 16 (32 outputs of 4 terms)
                ca = rng.integers(0, 2 ** 64, (32, 4, N), dtype=np.uint64)
                wb = po.u64_prepare(N, int(algo), base, rng.integers(-128, 128, (128, N))).reshape(32, 4, N // 2)
                reps, el = cpu_loop(lambda: po.u64_product_sum(N, int(algo), base, ca, wb, nthreads=1), cpu_seconds)
                row["cpu_one_core_us"] = el / (16 * reps) * 1e6
            rows["external_product_N%d_2x4" % N] = {k: (round(v, 2) if isinstance(v, float) else v)
                                                    for k, v in row.items()}
        # u128 products N = 1024 and 8192
        for N in (1024, 8192):
            p128 = cf.product.U128ProductPlan(N)
            a_np = rng.integers(0, 2 ** 64, (1, N, 2), dtype=np.uint64)
            b_np = rng.integers(-2 ** 15, 2 ** 15, (1, N))
            a = torch.from_numpy(a_np.view(np.int64)).cuda()
            bh = torch.empty((1, 4, N // 2), dtype=torch.float64, device="cuda")
            p128.prepare_operand(torch.from_numpy(b_np).cuda(), bh)
            out = torch.empty_like(a)
            row = {"auto_us": round(graph_device_us(torch, lambda: p128.product(a, bh, out)), 2)}
            if po is not None:
                ca = rng.integers(0, 2 ** 64, (8, N, 2), dtype=np.uint64)
                wb = po.u128_prepare(N, rng.integers(-2 ** 15, 2 ** 15, (8, N)))
                reps, el = cpu_loop(lambda: po.u128_product(N, ca, wb, nthreads=1), cpu_seconds)
                row["cpu_one_core_us"] = round(el / (8 * reps) * 1e6, 2)
            rows["u128_product_N%d" % N] = row
        clk.mark(t0, time.time())
    return {"rows": rows, "clocks": clk.summary(),
            "gpu": "device time per call: 20 calls captured in a CUDA graph, replayed 10 times, CUDA events",
            "cpu": "the restated reference pipeline on one host core with the plan's algorithm, per product over "
                   "calls of 32 products (8 for u128), so that the plan's set-up is spread as for a prepared plan"}


def run_latency(args):
    torch, cf, rank, world, local = gpu_setup()
    res = measure_latency(torch, cf, local, world, cpu=not args.no_cpu_baseline, profile_case=args.profile_case)
    if rank == 0:
        print(json.dumps({"workload": "one call at a time (latency)", "results": res}))


def run_u64_large(args):
    """Fused u64 products from N = 8192 (one product per thread-block cluster) against the
    plain five-launch path on the same products: N = 8192 (also against one CTA per
    product), 16384, 32768, 65536."""
    import numpy as np
    torch, cf, rank, world, local = gpu_setup()
    peak = fp64_peak(cf)
    rows = {}
    clocks = None
    for N in ((16384,) if args.profile_case else (8192, 16384, 32768, 65536)):
        count = 8192 * 2048 // N
        plan = cf.product.U64ProductPlan(N, cf.FftAlgo.Dif4, 1024)
        rng = np.random.default_rng(N)
        a = torch.from_numpy(rng.integers(0, 2 ** 64, (count, N), dtype=np.uint64).view(np.int64)).cuda()
        b = torch.from_numpy(rng.integers(-2 ** 7, 2 ** 7, (count, N))).cuda()
        bhat = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
        plan.prepare_operand(b, bhat)
        out = torch.empty_like(a)
        ms, clocks = timed(torch, lambda: plan.product(a, bhat, out), args.steps, args.warmup, local, world)
        plan.set_cluster_size(8)  # one cluster per product, whatever the batch
        out3 = torch.empty_like(a)
        ms_c, _ = timed(torch, lambda: plan.product(a, bhat, out3), args.steps, args.warmup, local, world)
        ms_1 = None
        if N <= 8192:  # one CTA per product (4096 points: one CTA per SM)
            plan.set_cluster_size(1)
            out4 = torch.empty_like(a)
            ms_1, _ = timed(torch, lambda: plan.product(a, bhat, out4), args.steps, args.warmup, local, world)
            assert torch.equal(out4, out)
        plan.set_cluster_size(0)
        z = torch.empty((count, N // 2), dtype=torch.complex128, device="cuda")
        out2 = torch.empty_like(a)
        ms_u, _ = timed(torch, lambda: plan.product_unfused(a, bhat, out2, z), max(3, args.steps // 4), 2, local,
                        world)
        per = ms * 1e-3 / args.steps
        ops = fp64_ops_per_product(N, 1024, int(cf.FftAlgo.Dif4)) * count
        rows[N] = {"products_per_s": world * count / per, "fp64_frac": ops / per / peak,
                   "cluster_products_per_s": world * count * args.steps / (ms_c * 1e-3),
                   "unfused_products_per_s": world * count * max(3, args.steps // 4) / (ms_u * 1e-3),
                   "matches_unfused": bool(torch.equal(out, out2) and torch.equal(out3, out2)), "count": count}
        if ms_1 is not None:
            rows[N]["one_cta_products_per_s"] = world * count * args.steps / (ms_1 * 1e-3)
    if rank != 0:
        return
    print(json.dumps({
        "metric": "u64 products/s at N=16384 (automatic path: clusters up to N = 16384, five launches from 32768)",
        "value": rows[16384]["products_per_s"], "unit": "products/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded numpy PCG64)",
        "config": {"workload": "u64 products N=8192/16384/32768/65536, Dif4 base 1024, 16 MiB of A per launch",
                   "by_N": rows},
        "clocks": clocks, "gpu_launches": 3 * args.steps,
    }))


def run_serde(args):
    """Permuted <-> standard order conversion (serialize/deserialize_fourier_buffer's element
    order) of 65536 unordered transforms of n = 1024 (base 32): 1 GiB in, 1 GiB out per call.
    HBM-bound: 32 bytes moved per point."""
    torch, cf, rank, world, local = gpu_setup()
    n, base = 1024, 32
    batch = args.count or 65536
    plan = cf.unordered.Plan(n, cf.unordered.Method.UserProvided(2, base))
    src = torch.randn(batch, n, dtype=torch.complex128, device="cuda")
    dst = torch.empty_like(src)
    if args.profile_case:  # for ncu: two to_standard calls of the batch
        for _ in range(2):
            plan.to_standard(src, dst)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "to_standard %d x 1024 points, base 32, x2" % batch}))
        return
    ms_to, clocks = timed(torch, lambda: plan.to_standard(src, dst), args.steps, args.warmup, local, world)
    ms_from, _ = timed(torch, lambda: plan.from_standard(dst, src), args.steps, args.warmup, local, world)
    nbytes = 2 * batch * n * 16
    gbs_to = nbytes * args.steps / (ms_to * 1e-3) / 1e9
    gbs_from = nbytes * args.steps / (ms_from * 1e-3) / 1e9
    # the wire format across the host link: page-locked standard-order host data straight into
    # the device's permuted order and back, the permutation kernel reading (writing) host memory
    wire = torch.empty((batch, n), dtype=torch.complex128).pin_memory()
    ms_h2d, _ = timed(torch, lambda: plan.from_standard(wire, src), max(3, args.steps // 4), 2, local, world)
    ms_d2h, _ = timed(torch, lambda: plan.to_standard(src, wire), max(3, args.steps // 4), 2, local, world)
    link_bytes = batch * n * 16  # each direction crosses the link once per call
    gbs_h2d = link_bytes * max(3, args.steps // 4) / (ms_h2d * 1e-3) / 1e9
    gbs_d2h = link_bytes * max(3, args.steps // 4) / (ms_d2h * 1e-3) / 1e9
    del wire
    peaks, peak_kind = measured_peaks()
    prof = profiled_traffic("permute_tile_n1024")
    traffic = prof["dram_bytes_per_point"] * batch * n if prof else None
    if rank != 0:
        return
    print(json.dumps({
        "metric": "unordered permuted->standard order conversion, n=1024 (GB/s moved)", "value": world * gbs_to,
        "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_to / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 copy", "data": "synthetic (torch.randn)",
        "config": {"workload": "to_standard / from_standard, %d x 1024 points, base 32, %.2f GiB per call"
                               % (batch, nbytes / 2 ** 30),
                   "from_standard_gbs": world * gbs_from, "l2": "inputs larger than L2",
                   "from_standard_h2d_gbs": world * gbs_h2d, "to_standard_d2h_gbs": world * gbs_d2h,
                   "host_side": "page-locked, read or written by the permutation kernel across the link"},
        "e2e": {"value": world * gbs_d2h, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": link_bytes,
                "note": "device permuted order -> serialized standard order in host memory (to_standard_d2h)"},
        "roofline": {"bound": "hbm", "achieved": gbs_to, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": gbs_to / peaks["hbm_gbs"], "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": nbytes,
                     "from_standard_frac": gbs_from / peaks["hbm_gbs"]},
        "clocks": clocks, "gpu_launches": 2 * args.steps,
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--cpu-seconds", type=float, default=5.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--count", type=int, default=None,
                    help="products per launch (u64_product, default %d) or transforms per call (serde, default 65536)" % COUNT)
    ap.add_argument("--base-algo", default=None, help="fix the base algorithm (e.g. Dif4) instead of measuring")
    ap.add_argument("--base-n", type=int, default=1024)
    ap.add_argument("--int-adds", type=int, default=None,
                    help="eighths of butterfly additions on the integer pipe (default: the plan's tuned value)")
    ap.add_argument("--profile-case", action="store_true",
                    help="small fixed case for ncu: 1 warm-up + 1 launch, no timing")
    ap.add_argument("--rate", type=float, default=20000.0)
    ap.add_argument("--serve-seconds", type=float, default=1.0)
    ap.add_argument("--operand-gb", type=int, default=8)
    ap.add_argument("--workload", choices=["u64_product", "mixed", "ordered", "u128_product", "serving", "product_sum", "serde",
                             "u64_large", "reference_cases", "latency"],
                    default="u64_product",
                    help="u64_product (default headline) or one of the other benchmark configurations")
    ap.add_argument("--mixed-items", type=int, default=100000)
    ap.add_argument("--no-configs", action="store_true",
                    help="headline only: skip the other benchmark configurations in the default line")
    ap.add_argument("--cluster-size", type=int, default=None, help="--profile-case of the ordered workload: CTAs per transform")
    ap.add_argument("--tune-seconds", type=float, default=0.0005)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "mixed":
        run_mixed(args)
    elif args.workload == "ordered":
        run_ordered(args)
    elif args.workload == "u128_product":
        run_u128(args)
    elif args.workload == "serde":
        run_serde(args)
    elif args.workload == "u64_large":
        run_u64_large(args)
    elif args.workload == "serving":
        run_serving(args)
    elif args.workload == "product_sum":
        run_product_sum(args)
    elif args.workload == "latency":
        run_latency(args)
    elif args.workload == "reference_cases":
        torch, cf, rank, world, local = gpu_setup()
        res = measure_reference_cases(torch, cf, local, world, cpu=not args.no_cpu_baseline)
        if rank == 0:
            print(json.dumps({"workload": "reference bench cases (benches/fft.rs)", "results": res}))
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()

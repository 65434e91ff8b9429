"""Benchmark: converged POIs/s of the 2D subset-DIC hot path on one GB300 (per rank).

Workload: a 2048 x 2048 uint8 synthetic speckle pair (24000 blobs,
u = 0.5 sin(2 pi x / 256), v = 0.3 cos(2 pi y / 192), noise 1), first-order ZNSSD ICGN, bicubic
B-spline, subset radius 15, POI step 5 (410 x 410 grid, 163,216 interior POIs), threshold 1e-3,
20 iterations, seed from the reference initializer.

One step = the hot path over one image pair with the inputs resident in HBM: the pair set-up
(K1, one launch: float32 copies of both images and the B-spline prefilter), then the
propagation over every grid POI (K3, dataflow order by default), with device outputs.  ``value`` = converged POIs (valid, strictly converged, accepted) / step time.
``e2e`` = the same through the public API ``subset.compute`` with pinned host images: upload,
seed selection, prefilter, propagation and the device->host result dict, every step.
L2 (129 MB) is flushed with a 256 MB write between timed steps.

``cpu_baseline`` is the FP64 C++ port of the reference path (oracle/) on every host thread over
the whole workload (dataflow order, each diagonal's solves spread over the threads);
``cpu_baseline_serial`` is the same port on one thread in the reference's heap order, on a prefix.

``prefilter`` times the pair set-up launch alone (L2 flushed before each) on the benchmark pair
and on a 5120 x 5120 uint16 pair, against the measured HBM bandwidth.

The default run also carries the uneven 48-pair batch in one graph-replayed launch
(``batched_uneven``) and the served Poisson request stream with its p50 / p99 latency
(``served``); ``--no-batch`` / ``--no-serve`` skip them.

``--impl reference`` times the reference algorithm's CPU implementation (the FP64 C++ port in
oracle/, the reference itself does not build without Eigen) on the same workload and
configuration: each step propagates the whole grid in the dataflow order on every host thread.
It imports neither this build's package nor its CUDA library (the seeded input generator is
loaded from its file on its own).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "converged POIs/s, 2048^2 r=15 (FP32 vs FP64, <=1e-3 px)"
UNIT = "POI/s"
WORKLOAD = {
    "workload": "synthetic speckle 2048x2048 uint8, sinusoidal u/v, radius 15, POI step 5",
    "image": [2048, 2048], "dtype_in": "uint8", "subset_radius": 15, "poi_step": 5, "grid": [410, 410],
    "bspline_degree": 3, "threshold": 1e-3, "max_iterations": 20, "shape_function": "first_order",
    "optimizer": "icgn", "l2": "flushed (256 MB write) between timed steps",
}


PROPAGATE_DRAM_BYTES = 37_934_080 + 6_583_552  # ncu, propagate_kernel, 2048^2 r=15, one launch


def workload_desc(side: int) -> dict:
    """WORKLOAD for a side x side case of the same generator (2048 = the benchmark itself)."""
    if side == 2048:
        return dict(WORKLOAD)
    g = (side + 4) // 5
    return dict(WORKLOAD, workload=f"synthetic speckle {side}x{side} uint8 (profiling case), sinusoidal u/v, "
                                   f"radius 15, POI step 5", image=[side, side], grid=[g, g])


def run_config(side: int, mode: str) -> dict:
    """The ``config`` object of both arms' lines: the workload and the propagation order (the
    arithmetic and the hardware of an arm are top-level keys, so the two arms' configs compare
    equal when they run the same work)."""
    return dict(workload_desc(side), propagation=mode)


CONFIG = {
    "subset": {"radius": 15},
    "optimization": {"max_iterations": 20, "convergence_threshold": 1e-3},
    "interpolation": {"degree": 3},
    "initialization": {"method": "integer_search",
                       "integer_search": {"subset_radius": 10, "search_radius": 20, "sift_enabled": False,
                                          "pyramid_enabled": True},
                       "subpixel_refinement": {"enabled": True, "subset_radius": 15, "max_iterations": 20,
                                               "convergence_threshold": 1e-3}},
    "seed_selection": {"seed_count": 64, "max_znssd": 0.3, "min_texture_std": 0.02},
    "reliability_propagation": {"spacing": 4, "max_znssd": 0.5},
}


def prefilter_bytes(side: int, in_bytes: int, coef_bytes: int, border: int = 3) -> int:
    """Algorithmic bytes of one pair set-up launch on a side x side pair: both raw images read,
    both float32 images and the (side + 2 border)^2 coefficients written."""
    c = side + 2 * border
    return 2 * side * side * in_bytes + 2 * side * side * 4 + c * c * coef_bytes


def run_prefilter(ctx, stream, flush, pair, ref_d, def_d, hbm_gbs) -> dict:
    """The pair set-up launch (prefilter_fused_kernel) alone, CUDA events on its stream, L2
    flushed before each launch: the benchmark pair and a 5120^2 uint16 pair (seeded uniform
    pixels; the kernel's work does not depend on the pixel values)."""
    import torch
    from traditional_dic_gb300 import subset as S

    def timed(p, r, d, reps=20):
        for _ in range(3):
            p.update(r, d, stream=stream)
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            with torch.cuda.stream(stream):
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                p.update(r, d, stream=stream)
                b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b) * 1e-3)
        return statistics.median(ts)

    out = []
    side = int(ref_d.shape[0])
    t = timed(pair, ref_d, def_d)
    nb = prefilter_bytes(side, ref_d.element_size(), 4)
    out.append({"image": f"{side}x{side} uint8", "coefficients": "float32", "us": 1e6 * t, "algorithmic_bytes": nb,
                "achieved_gbs": nb / t / 1e9, "frac": nb / t / 1e9 / hbm_gbs})
    rng = np.random.default_rng(5120)
    big = [torch.from_numpy(rng.integers(0, 65536, (5120, 5120), dtype=np.uint16)).to(ref_d.device) for _ in range(2)]
    p5 = S.Pair(ctx, big[0], big[1], degree=3, stream=stream)
    t = timed(p5, big[0], big[1])
    p5.close()
    nb = prefilter_bytes(5120, 2, 4)
    out.append({"image": "5120x5120 uint16", "coefficients": "float32", "us": 1e6 * t, "algorithmic_bytes": nb,
                "achieved_gbs": nb / t / 1e9, "frac": nb / t / 1e9 / hbm_gbs})
    del big
    return {"kernel": "prefilter_fused_kernel<In, float, 3> (pair set-up: both images to float32 + "
                      "B-spline coefficients)", "bound": "hbm", "peak_gbs": hbm_gbs,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth, of measured)", "workloads": out}


def icgn_flops(iterations: np.ndarray, n_samples: int) -> float:
    """Algorithmic FP32 flops of the ICGN solves (FMA = 2): per POI 52 N setup + per iteration
    (94 N + 150)."""
    it = iterations.astype(np.float64)
    solved = it > 0
    return float(np.sum(solved * 52.0 * n_samples + it * (94.0 * n_samples + 150.0)))


def n_samples(r: int) -> int:
    return sum(1 for dy in range(-r, r + 1) for dx in range(-r, r + 1) if dx * dx + dy * dy <= r * r)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="tdic_clocks_", suffix=".csv")
        os.close(fd)

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self, device: int = 0) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        lines = open(self.path).read().splitlines()
        os.unlink(self.path)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9 or parts[0] != str(device):
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def fp32_peak_tflops(torch) -> float:
    """Measured FP32 CUDA-core throughput: cuBLAS SGEMM 8192^3 with TF32 disabled, best of 5."""
    torch.backends.cuda.matmul.allow_tf32 = False
    a = torch.randn(8192, 8192, device="cuda", dtype=torch.float32)
    b = torch.randn(8192, 8192, device="cuda", dtype=torch.float32)
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        a @ b
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    del a, b
    return 2.0 * 8192 ** 3 / best / 1e12


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v: float) -> float:
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, v: float) -> float:
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------------------------------
def standalone_synthetic():
    """The seeded workload generator (numpy only), loaded from its file as a module of its own:
    the reference arm imports neither this build's package nor its CUDA library."""
    import importlib.util
    path = os.path.join(ROOT, "traditional-dic_gb300", "synthetic.py")
    spec = importlib.util.spec_from_file_location("tdic_workload_generator", path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod
    spec.loader.exec_module(mod)
    return mod


def oracle_config(O, d: dict, mode: int):
    """The oracle's configuration for a config dict of this benchmark (the keys CONFIG uses),
    over the oracle's own defaults (the reference's C++ defaults)."""
    cfg = O.default_config()
    cfg.subset_radius = d["subset"]["radius"]
    cfg.max_iterations = d["optimization"]["max_iterations"]
    cfg.convergence_threshold = d["optimization"]["convergence_threshold"]
    cfg.degree = d["interpolation"]["degree"]
    ini = d["initialization"]
    cfg.is_subset_radius = ini["integer_search"]["subset_radius"]
    cfg.is_search_radius = ini["integer_search"]["search_radius"]
    cfg.sift_enabled = int(ini["integer_search"]["sift_enabled"])
    cfg.pyramid_enabled = int(ini["integer_search"]["pyramid_enabled"])
    sp = ini["subpixel_refinement"]
    cfg.sp_enabled = int(sp["enabled"])
    cfg.sp_subset_radius = sp["subset_radius"]
    cfg.sp_max_iterations = sp["max_iterations"]
    cfg.sp_convergence_threshold = sp["convergence_threshold"]
    ss = d["seed_selection"]
    cfg.seed_count = ss["seed_count"]
    cfg.seed_max_znssd = ss["max_znssd"]
    cfg.min_texture_std = ss["min_texture_std"]
    cfg.propagation_spacing = d["reliability_propagation"]["spacing"]
    cfg.propagation_max_znssd = d["reliability_propagation"]["max_znssd"]
    cfg.propagation_mode = mode
    return cfg


def run_reference(args, world, rank, pg):
    """Reference arm: the FP64 C++ port of the reference path (oracle/; the reference itself
    does not build without Eigen) on the host cores of rank 0, on the GPU arm's workload and
    configuration.  A step propagates the whole 2048^2 grid from the seed, the solves of each
    dataflow diagonal spread over every host thread (the same visit order, work and results as
    one thread; the GPU arm's default order).  The reference's own serial heap order is timed
    once on one thread over a prefix and reported beside it."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    synthetic = standalone_synthetic()
    pair = synthetic.workload(1)
    threads = host_threads()
    cfg = oracle_config(O, CONFIG, 2)
    t0 = time.perf_counter()
    seed, _ = O.select_seed(pair.reference, pair.deformed, cfg)
    t_seed = time.perf_counter() - t0
    assert seed.found, "no seed found"
    t0 = time.perf_counter()
    coef = O.prefilter(pair.deformed, 3, 3, True)
    grads = O.reference_gradient(pair.reference)
    t_pre = time.perf_counter() - t0
    for _ in range(args.warmup):  # warm-up steps: a bounded prefix each
        O.propagate(pair.reference, coef, cfg, seed, gradients=grads, max_solves=2000, threads=threads)
    conv_total, t_total = 0, 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r = O.propagate(pair.reference, coef, cfg, seed, gradients=grads, threads=threads)
        t_total += time.perf_counter() - t0
        conv_total += int(np.sum(r["valid"] & r["converged"]))
    value = conv_total / t_total
    heap = oracle_config(O, CONFIG, 1)
    t0 = time.perf_counter()
    rh = O.propagate(pair.reference, coef, heap, seed, gradients=grads, max_solves=args.ref_solves)
    t_heap = time.perf_counter() - t0
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": run_config(2048, "dataflow"),
        "precision": "fp64", "parallelism": f"{threads} host threads",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"the whole 2048x2048 workload per step: {r['solves']} solves, dataflow order, "
                                   f"{threads} threads (FP64 C++ port of the reference path; seed selection "
                                   f"{t_seed:.2f} s and prefilter + gradients {t_pre:.2f} s once, untimed)"},
        "heap_order_serial": {"value": int(np.sum(rh["valid"] & rh["converged"])) / t_heap, "unit": UNIT, "cores": 1,
                              "sample": f"first {rh['solves']} solves in the reference's heap order, one thread"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def cpu_baselines(reference, deformed, cfg, seed, ref_solves: int, threads: int | None = None):
    """The FP64 C++ port of the reference path (oracle/) on the host cores, from the same seed:
    (1) every host thread on the whole workload in dataflow order, the solves of each diagonal
    spread over the threads (the visit order and results of one thread); (2) one thread in the
    reference's own heap order on its first ``ref_solves`` solves.  Returns (parallel, serial)
    ``cpu_baseline`` objects; a leg that fails reports its error instead of a value."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    threads = threads or host_threads()
    coef = O.prefilter(deformed, 3, 3, True)
    grads = O.reference_gradient(reference)
    oseed = O.make_seed(seed.x, seed.y, list(seed.p), seed.correlation)
    legs = []
    # a full 2048^2 propagation is about 50 s of one core: below 4 threads, time a prefix
    budget = -1 if threads >= 4 else ref_solves * threads
    for mode, n_threads, max_solves in ((2, threads, budget), (1, 1, ref_solves)):
        ocfg = O.as_config(cfg)
        ocfg.propagation_mode = mode
        try:
            t0 = time.perf_counter()
            rr = O.propagate(reference, coef, ocfg, oseed, gradients=grads, max_solves=max_solves, threads=n_threads)
            dt = time.perf_counter() - t0
        except Exception as e:  # the GPU figures above stand without the baseline
            legs.append({"value": None, "unit": UNIT, "cores": n_threads, "kind": "port", "error": repr(e)})
            continue
        conv = int(np.sum(rr["valid"] & rr["converged"]))
        size = "x".join(str(n) for n in reversed(np.shape(reference)))
        what = (f"the whole {size} workload, dataflow order" if max_solves < 0 and mode == 2 else
                f"first {rr['solves']} {'heap-order' if mode == 1 else 'dataflow-order'} solves of the same "
                f"{size} workload")
        legs.append({"value": conv / dt, "unit": UNIT, "cores": n_threads, "kind": "port",
                     "sample": f"{what}: {rr['solves']} solves, {conv} converged in {dt:.1f} s "
                               f"(FP64 C++ port of the reference path, {n_threads} thread"
                               f"{'s' if n_threads > 1 else ''})"})
    return legs[0], legs[1]


def run_ours(args, world, rank, local, pg):
    import torch
    from traditional_dic_gb300 import subset as S, synthetic, _lib as L
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = S.Context(local)
    pair_np = synthetic.workload(1, side=args.side)
    h, w = pair_np.reference.shape
    cfg = S.config_from_dict(CONFIG)
    cfg.precision = L.FP64 if args.precision == "fp64" else L.FP32_MIXED
    cfg.propagation_mode = S.PROPAGATION_MODES[args.mode]
    r = cfg.subset_radius
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    ref_d = torch.from_numpy(pair_np.reference).to(dev)
    def_d = torch.from_numpy(pair_np.deformed).to(dev)
    gw, gh = L.grid_dims(w, h, cfg.propagation_spacing)
    n = gw * gh
    outs = {k: torch.empty(n, dtype=torch.float64, device=dev) for k in
            ("x", "y", "u", "v", "du_dx", "du_dy", "dv_dx", "dv_dy", "correlation", "zncc")}
    outs["valid"] = torch.empty(n, dtype=torch.uint8, device=dev)
    outs["status"] = torch.empty(n, dtype=torch.int8, device=dev)
    outs["iterations"] = torch.empty(n, dtype=torch.int32, device=dev)
    outs["converged"] = torch.empty(n, dtype=torch.uint8, device=dev)
    grid = L.GridOut(**{k: outs[k].data_ptr() for k in L.GRID_FIELDS})
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # Seed from the reference initializer (tdic_select_seed), once, untimed: it is an input of
    # the hot path.  The e2e leg below re-runs it every step.
    gpu_cfg = {"precision": args.precision, "propagation": args.mode}
    _, seed = S.compute(pair_np.reference, pair_np.deformed, dict(CONFIG, gpu=gpu_cfg),
                        context=ctx, return_seed=True)
    assert seed.found, "no seed found"
    pair = S.Pair(ctx, ref_d, def_d, degree=3, precision=cfg.precision, stream=stream)
    pc = C.c_int32()

    def step():
        pair.update(ref_d, def_d, stream=stream)
        ctx.check(ctx.lib.tdic_propagate(ctx.handle, pair.handle, C.byref(cfg),
                                         C.byref(seed), None, C.byref(grid),
                                         L.DEVICE, C.byref(pc), sptr))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks()
    barrier(pg)
    torch.cuda.synchronize()
    clocks.start()
    times, prop_times = [], []
    conv_counts = []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            pair.update(ref_d, def_d, stream=stream)
            e1.record(stream)
            ctx.check(ctx.lib.tdic_propagate(ctx.handle, pair.handle, C.byref(cfg),
                                             C.byref(seed), None, C.byref(grid),
                                             L.DEVICE, C.byref(pc), sptr))
            e2.record(stream)
        e2.synchronize()
        times.append(e0.elapsed_time(e2) / 1e3)
        prop_times.append(e1.elapsed_time(e2) / 1e3)
        conv_counts.append(int(((outs["valid"] != 0) & (outs["converged"] != 0)).sum().item()))
    torch.cuda.synchronize()
    barrier(pg)
    clk = clocks.stop(local)
    t_step = max_over_ranks(pg, sum(times) / len(times))
    conv = conv_counts[-1]
    total_conv = sum_over_ranks(pg, float(conv))
    value = total_conv / t_step

    iters = outs["iterations"].cpu().numpy()
    flops = icgn_flops(iters, n_samples(r))
    t_prop = statistics.median(prop_times)
    peaks = measured_peaks()
    fp32_peak = fp32_peak_tflops(torch)
    roofline = {"kernel": "propagate_kernel (ICGN, FP32 mixed)", "bound": "fp32",
                "achieved": flops / t_prop / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": flops / t_prop / 1e12 / fp32_peak,
                "peak_source": "measured in this run: cuBLAS SGEMM 8192^3, TF32 off (MEASURED_PEAKS.json holds "
                               "HBM and bf16 only)",
                "algorithmic_flops_per_launch": flops,
                # DRAM bytes (read + write) of one launch on this workload, from one ncu capture
                # (dram__bytes_read.sum + dram__bytes_write.sum after the L2 flush); recorded for
                # the benchmark workload only
                "traffic": PROPAGATE_DRAM_BYTES if args.side == 2048 else None,
                "hbm_peak_gbs": peaks.get("hbm_gbs")}

    pre = run_prefilter(ctx, stream, flush, pair, ref_d, def_d, peaks.get("hbm_gbs") or 6795.8)

    # FP64 GPU path on the same configuration, for the precision comparison.
    res32 = {k: outs[k].cpu().numpy().copy() for k in ("u", "v", "valid", "converged", "zncc")}
    fp64 = None
    if args.precision == "fp32" and not args.skip_fp64:
        cfg64 = S.config_from_dict(dict(CONFIG, gpu={"precision": "fp64", "propagation": args.mode}))
        pair64 = S.Pair(ctx, ref_d, def_d, degree=3, precision=L.FP64, stream=stream)
        t64 = []
        for i in range(2):
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            pair64.update(ref_d, def_d, stream=stream)
            ctx.check(ctx.lib.tdic_propagate(ctx.handle, pair64.handle, C.byref(cfg64),
                                             C.byref(seed), None, C.byref(grid),
                                             L.DEVICE, C.byref(pc), sptr))
            b.record(stream)
            b.synchronize()
            if i:
                t64.append(a.elapsed_time(b) / 1e3)
        v64 = outs["valid"].cpu().numpy() != 0
        c64 = outs["converged"].cpu().numpy() != 0
        res64 = {k: outs[k].cpu().numpy().copy() for k in ("u", "v", "valid", "converged", "zncc")}
        both = v64 & (res32["valid"] != 0)
        du = np.abs(outs["u"].cpu().numpy()[both] - res32["u"][both])
        dv = np.abs(outs["v"].cpu().numpy()[both] - res32["v"][both])
        dz = np.abs(outs["zncc"].cpu().numpy()[both] - res32["zncc"][both])
        fp64 = {"value": float(np.sum(v64 & c64)) / t64[0], "ms_per_step": 1e3 * t64[0],
                "speedup_fp32_over_fp64": value / (float(np.sum(v64 & c64)) / t64[0]),
                "fp32_vs_fp64": {"max_abs_u_px": float(du.max()), "max_abs_v_px": float(dv.max()),
                                 "p99_abs_u_px": float(np.quantile(du, 0.99)), "max_abs_zncc": float(dz.max()),
                                 "flag_agreement": float(np.mean(v64 == (res32["valid"] != 0))),
                                 "within_1e-3_px": float(np.mean((du <= 1e-3) & (dv <= 1e-3)))}}
        pair64.close()

    # The reference's own visit order on the device (propagation_mode 1: heap simulation on the
    # host, device rounds), FP32-mixed and FP64, against the dataflow order of the same build.
    heap = None
    if not args.skip_heap:
        heap = {}
        res_flow = {args.precision: res32}   # the main timed run's results
        if fp64 is not None:
            res_flow["fp64"] = res64
        for prec in res_flow:
            hcfg = S.config_from_dict(dict(CONFIG, gpu={"precision": prec, "propagation": "heap"}))
            hpair = pair if prec == args.precision else S.Pair(ctx, ref_d, def_d, degree=3, precision=hcfg.precision,
                                                               stream=stream)
            th = []
            for i in range(3):
                torch.cuda.synchronize()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                ctx.check(ctx.lib.tdic_propagate(ctx.handle, hpair.handle, C.byref(hcfg), C.byref(seed), None,
                                                 C.byref(grid), L.DEVICE, C.byref(pc), sptr))
                b.record(stream)
                b.synchronize()
                if i:
                    th.append(a.elapsed_time(b) / 1e3)
            if hpair is not pair:
                hpair.close()
            hv = outs["valid"].cpu().numpy() != 0
            hc = outs["converged"].cpu().numpy() != 0
            f = res_flow[prec]
            both = hv & (f["valid"] != 0)
            d = np.maximum(np.abs(outs["u"].cpu().numpy()[both] - f["u"][both]),
                           np.abs(outs["v"].cpu().numpy()[both] - f["v"][both]))
            t_h = statistics.median(th)
            rounds, solves, sim_ms = ctx.heap_stats()
            heap[prec] = {"ms": 1e3 * t_h, "value": float(np.sum(hv & hc)) / t_h, "unit": UNIT,
                          "device_rounds": rounds, "round_solves": solves, "host_simulation_ms": sim_ms,
                          "dataflow_vs_heap": {"flag_agreement": float(np.mean(hv == (f["valid"] != 0))),
                                               "within_1e-3_px": float(np.mean(d <= 1e-3)),
                                               "max_abs_px": float(d.max()), "p99_abs_px": float(np.quantile(d, 0.99))}}

    # e2e through the public API with pinned host images.
    ref_pin = torch.from_numpy(pair_np.reference).pin_memory()
    def_pin = torch.from_numpy(pair_np.deformed).pin_memory()
    ref_h, def_h = ref_pin.numpy(), def_pin.numpy()
    e2e_cfg = dict(CONFIG, gpu=gpu_cfg)
    S.compute(ref_h, def_h, e2e_cfg, context=ctx)
    barrier(pg)
    t0 = time.perf_counter()
    e2e_conv = 0
    for _ in range(args.steps):
        res = S.compute(ref_h, def_h, e2e_cfg, context=ctx)
        e2e_conv = int(np.sum(res["valid"] & res["converged"]))
    t_e2e = max_over_ranks(pg, (time.perf_counter() - t0) / args.steps)
    e2e_value = sum_over_ranks(pg, float(e2e_conv)) / t_e2e
    d2h = n * (10 * 8 + 1 + 1 + 4 + 1)

    cpu = cpu_serial = None
    if rank == 0 and not args.skip_cpu:
        cpu, cpu_serial = cpu_baselines(pair_np.reference, pair_np.deformed, cfg, seed, args.ref_solves)

    routes = run_routes(args, ctx, stream) if (args.routes and rank == 0) else None
    batched = run_batch(args, ctx, stream) if (not args.no_batch and rank == 0) else None
    served = run_serve(args, ctx) if (not args.no_serve and rank == 0) else None

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64 (mixed)" if args.precision == "fp32" else "f64",
            "data": "synthetic", "config": run_config(args.side, args.mode),
            "precision": args.precision, "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
            "converged_pois_per_step": conv,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "cpu_baseline_serial": cpu_serial,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(2 * h * w),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": 1e3 * t_e2e,
                    "includes": "H2D of both images (pinned), seed selection, prefilter, propagation, D2H of the "
                                "result dict"},
            "fp64_path": fp64,
            "heap_order": heap,
            # per step: prefilter_fused_kernel (pair set-up), init_grid_kernel, propagate_kernel
            "gpu_launches": 3 * args.steps,
            "clocks": clk,
            "stages_ms": {"pair_setup": 1e3 * (statistics.median(times) - t_prop),
                          "propagate": 1e3 * t_prop},
            "prefilter": pre,
        }
        if routes is not None:
            line["routes"] = routes
        if batched is not None:
            line["batched_uneven"] = batched
        if served is not None:
            line["served"] = served
        print(json.dumps(line), flush=True)
    pair.close()
    ctx.close()


ROUTES = [("icgn", "first_order", "znssd"), ("icgn", "first_order", "ssd"), ("icgn", "second_order", "znssd"),
          ("icgn", "second_order", "ssd"), ("fgn", "first_order", "znssd"), ("fgn", "first_order", "ssd"),
          ("fgn", "second_order", "znssd"), ("fgn", "second_order", "ssd")]


def compare_builds(a, b) -> dict:
    """FP32-mixed against FP64 results of one propagation, each (valid, u, v, strictly converged):
    flag agreement, and the share of points within 1e-3 px in u and v over the jointly valid points
    and over the points that converged strictly in both builds (the metric's converged POIs; the
    others report the last of max_iterations iterates, which rounding moves in any precision)."""
    v32, u32, w32, s32 = a
    v64, u64, w64, s64 = b
    both, strict = v32 & v64, s32 & s64
    du, dv = np.abs(u32 - u64), np.abs(w32 - w64)
    close = (du <= 1e-3) & (dv <= 1e-3)
    return {"flag_agreement": float(np.mean(v32 == v64)),
            "within_1e-3_px": float(np.mean(close[both])) if both.any() else None,
            "within_1e-3_px_converged": float(np.mean(close[strict])) if strict.any() else None,
            "p99_abs_u_px": float(np.quantile(du[both], 0.99)) if both.any() else None}


def run_routes(args, ctx, stream) -> list:
    """Every solver route (optimizer x shape function x criterion) on the same 2048^2 pair, scaled
    to [0, 1] float32 (the range the reference's Python facade documents, so SSD values meet the
    acceptance threshold): propagation time of one pair with device outputs, FP32-mixed and FP64,
    the seed of each route from its own seed selection (untimed)."""
    import torch
    from traditional_dic_gb300 import subset as S, synthetic, _lib as L
    pair_np = synthetic.workload(1, side=args.side)
    ref = (pair_np.reference.astype(np.float32) / 255.0)
    de = (pair_np.deformed.astype(np.float32) / 255.0)
    h, w = ref.shape
    dev = torch.device("cuda", torch.cuda.current_device())
    ref_d, def_d = torch.from_numpy(ref).to(dev), torch.from_numpy(de).to(dev)
    sptr = stream.cuda_stream
    out = []
    for opt, order, crit in ROUTES:
        conf = dict(CONFIG, optimization=dict(CONFIG["optimization"], method=opt), correlation={"criterion": crit},
                    shape_function={"order": order})
        t_route = time.perf_counter()
        _, seed = S.compute(ref, de, conf, context=ctx, return_seed=True)
        print(f"[routes] {opt} {order} {crit}: seed {time.perf_counter() - t_route:.2f} s", file=sys.stderr, flush=True)
        entry = {"optimizer": opt, "shape_function": order, "criterion": crit}
        res = {}
        for prec in ("fp32", "fp64"):
            cfg = S.config_from_dict(dict(conf, gpu={"precision": prec, "propagation": args.mode}))
            gw, gh = L.grid_dims(w, h, cfg.propagation_spacing)
            n = gw * gh
            outs = {k: torch.empty(n, dtype=torch.float64, device=dev) for k in ("x", "y", "u", "v", "du_dx", "du_dy",
                                                                                 "dv_dx", "dv_dy", "correlation", "zncc")}
            outs["valid"] = torch.empty(n, dtype=torch.uint8, device=dev)
            outs["status"] = torch.empty(n, dtype=torch.int8, device=dev)
            outs["iterations"] = torch.empty(n, dtype=torch.int32, device=dev)
            outs["converged"] = torch.empty(n, dtype=torch.uint8, device=dev)
            grid = L.GridOut(**{k: outs[k].data_ptr() for k in L.GRID_FIELDS})
            pair = S.Pair(ctx, ref_d, def_d, degree=3, precision=cfg.precision, stream=stream)
            pc = C.c_int32()
            ts = []
            for i in range(3):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                ctx.check(ctx.lib.tdic_propagate(ctx.handle, pair.handle, C.byref(cfg), C.byref(seed), None,
                                                 C.byref(grid), L.DEVICE, C.byref(pc), sptr))
                b.record(stream)
                b.synchronize()
                if i:
                    ts.append(a.elapsed_time(b) / 1e3)
            pair.close()
            t = statistics.median(ts)
            print(f"[routes] {opt} {order} {crit} {prec}: {1e3 * t:.1f} ms per propagation", file=sys.stderr, flush=True)
            valid = outs["valid"].cpu().numpy() != 0
            strict = valid & (outs["converged"].cpu().numpy() != 0)
            conv = int(np.sum(strict))
            res[prec] = (t, conv, valid, outs["u"].cpu().numpy(), outs["v"].cpu().numpy(), strict)
            entry[prec] = {"ms": 1e3 * t, "converged": conv, "value": conv / t}
        entry["fp32_vs_fp64"] = compare_builds(res["fp32"][2:], res["fp64"][2:])
        entry["speedup_fp32_over_fp64"] = entry["fp64"]["ms"] / entry["fp32"]["ms"]
        out.append(entry)
    return out


def run_batch(args, ctx, stream) -> dict:
    """The uneven batch (48 pairs, sides log-uniform in [512, 4096], half uint8 / half uint16,
    radius in {7, 11, 15, 21, 25}, step in {3, 5, 8}, affine fields): one graph-captured,
    autotuned persistent launch over every pair against one plain launch per pair.  Inputs are
    resident (1.5 GB of images, larger than L2); seeds come from the seed selection, untimed."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    import torch
    import __graft_entry__
    from traditional_dic_gb300 import subset as S, synthetic, _lib as L
    t0 = time.perf_counter()
    with ProcessPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1)), mp_context=mp.get_context("spawn"),
                             initializer=__graft_entry__.load_package) as ex:
        pairs_np = synthetic.batch_workload(args.batch_pairs, pool=ex)
    t_gen = time.perf_counter() - t0
    pairs, cfgs, seeds = [], [], []
    for p in pairs_np:
        d = dict(CONFIG, subset={"radius": p.meta["radius"]},
                 reliability_propagation={"spacing": p.meta["step"] - 1, "max_znssd": 0.5},
                 gpu={"precision": "fp32", "propagation": "dataflow"})
        cfg = S.config_from_dict(d)
        lazy = S.Pair(ctx, p.reference, p.deformed, degree=3, exact=False)
        seed = S.select_seed(ctx, lazy, p.reference.astype(np.float32), cfg)
        lazy.close()
        pairs.append(S.Pair(ctx, p.reference, p.deformed, degree=3))
        cfgs.append(cfg)
        seeds.append(seed)
    batch = S.Batch(ctx, pairs, cfgs, seeds)
    g, k, staging = batch.tune()
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        batch.launch(stream=torch.cuda.current_stream())
    for _ in range(args.warmup):
        graph.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        graph.replay()
    e1.record()
    e1.synchronize()
    t_batch = e0.elapsed_time(e1) / 1e3 / args.steps
    batch.finish()
    conv, points = 0, 0
    for j in range(len(pairs)):
        o = batch.outputs(j)
        conv += int(np.sum(o["valid"] & o["converged"]))
        points += o["valid"].size
    # one plain launch per pair, device outputs, same seeds and configurations
    pc = C.c_int32()
    t_pairs = 0.0
    for rep in range(2):
        t_rep = 0.0
        for j in range(len(pairs)):
            grid = batch.device_outputs(j)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.check(ctx.lib.tdic_propagate(ctx.handle, pairs[j].handle, C.byref(cfgs[j]), C.byref(seeds[j]), None,
                                             C.byref(grid), L.DEVICE, C.byref(pc), stream.cuda_stream))
            b.record(stream)
            b.synchronize()
            t_rep += a.elapsed_time(b) / 1e3
        t_pairs = t_rep  # the second repetition (warm)
    del graph
    batch.close()
    for p in pairs:
        p.close()
    return {"pairs": len(pairs), "grid_points": points, "converged_per_launch": conv,
            "value": conv / t_batch, "unit": UNIT, "ms_per_launch": 1e3 * t_batch,
            "per_pair_launches": {"value": conv / t_pairs, "ms_total": 1e3 * t_pairs},
            "speedup_over_per_pair": t_pairs / t_batch,
            "launch_config": {"warps_per_poi": g, "groups_per_block": k, "staging": staging, "tuned": True,
                              "cuda_graph": True},
            "generation_s": t_gen}


def _request_config(p, precision: str) -> dict:
    return dict(CONFIG, subset={"radius": p.meta["radius"]},
                reliability_propagation={"spacing": p.meta["step"] - 1, "max_znssd": 0.5},
                gpu={"precision": precision, "propagation": "dataflow"})


def _latency_stats(lat_s, conv, span_s) -> dict:
    lat = np.asarray(lat_s) * 1e3
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "value": conv / span_s, "unit": UNIT, "span_s": span_s}


def run_serve(args, ctx) -> dict:
    """The served request stream (Poisson arrivals at 40/s; sides 1024-4096; uint8/uint16; bump
    or affine; radius and step as the uneven batch): the continuous-batching server against the
    same stream solved one request at a time (FP64 and FP32 plain compute calls)."""
    import multiprocessing as mp
    import threading
    from concurrent.futures import ProcessPoolExecutor
    import __graft_entry__
    from traditional_dic_gb300 import subset as S, synthetic, serve
    with ProcessPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1)), mp_context=mp.get_context("spawn"),
                             initializer=__graft_entry__.load_package) as ex:
        stream = synthetic.serve_workload(args.serve_requests, pool=ex)

    def served_run(server):
        reqs = [None] * len(stream)

        def feed():
            t0 = time.perf_counter()
            for i, (arrival, p) in enumerate(stream):
                delay = t0 + arrival - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                reqs[i] = server.submit(p.reference, p.deformed, _request_config(p, "fp32"))
        th = threading.Thread(target=feed)
        th.start()
        th.join()
        res = [r.wait(600) for r in reqs]
        conv = sum(int(np.sum(r["valid"] & r["converged"])) for r in res)
        span = max(r.finished for r in reqs) - min(r.arrival for r in reqs)
        return [r.latency for r in reqs], conv, span

    with serve.Server(ctx, reserve_sms=args.serve_reserve_sms) as server:
        served_run(server)                    # warm: the device pool holds buffers for every shape
        nb = len(server.batches)
        marks = {k: len(v) for k, v in server.stats.items()}
        lat, conv, span = served_run(server)
        sizes = server.batches[nb:]
        stage = {k: 1e3 * float(np.mean(v[marks[k]:])) for k, v in server.stats.items() if len(v) > marks[k]}
    out = _latency_stats(lat, conv, span)
    out.update(requests=len(stream), rate_per_s=40.0, batches=len(sizes), propagation_sms=server._sms,
               mean_batch=float(np.mean(sizes)) if sizes else 0.0,
               mean_ms={"prepare_per_request": stage.get("prepare"), "propagate_per_batch": stage.get("propagate"),
                        "collect_per_batch": stage.get("collect")})

    def plain(precision):
        for arrival, p in stream[:2]:         # warm
            S.compute(p.reference, p.deformed, _request_config(p, precision), context=ctx)
        t0 = time.perf_counter()
        free, lat, conv = t0, [], 0
        for arrival, p in stream:
            start = max(free, t0 + arrival)
            while time.perf_counter() < start:
                time.sleep(0.0002)
            r = S.compute(p.reference, p.deformed, _request_config(p, precision), context=ctx)
            free = time.perf_counter()
            lat.append(free - (t0 + arrival))
            conv += int(np.sum(r["valid"] & r["converged"]))
        return _latency_stats(lat, conv, free - t0 - stream[0][0])

    out["per_request_fp64"] = plain("fp64")
    out["per_request_fp32"] = plain("fp32")
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--mode", default="dataflow", choices=["dataflow", "waves"])
    ap.add_argument("--ref-solves", type=int, default=20000)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-heap", action="store_true",
                    help="skip the reference's heap order on the device (FP32 and FP64, against dataflow)")
    ap.add_argument("--routes", action="store_true",
                    help="also time every solver route (ICGN/FGN x first/second order x ZNSSD/SSD), FP32 and FP64")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the uneven 48-pair batch (one launch, against per-pair launches)")
    ap.add_argument("--batch-pairs", type=int, default=48)
    ap.add_argument("--no-serve", action="store_true",
                    help="skip the served Poisson request stream (continuous batching, against per-request solves)")
    ap.add_argument("--serve-requests", type=int, default=40)
    ap.add_argument("--serve-reserve-sms", type=int, default=None,
                    help="SMs the served propagation leaves to request preparation (default: a tenth)")
    ap.add_argument("--side", type=int, default=2048,
                    help="image side; 2048 is the benchmark workload, smaller sides are profiling cases")
    args = ap.parse_args()
    world, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank, pg)
    else:
        import __graft_entry__
        __graft_entry__.build()
        run_ours(args, world, rank, local, pg)


if __name__ == "__main__":
    main()

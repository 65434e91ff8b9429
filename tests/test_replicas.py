"""The multi-GPU mode of bench.py runs independent replicas (the propagation does not shard:
each image pair's grid depends on its own seed chain).  Its host-side harness - process group,
barrier, max / sum over ranks - is checked here with two gloo ranks on the CPU, each solving
its own small job with the oracle.  The CPU-baseline legs that bench.py adds to its line run here
too, on the small workload."""
import os
import socket
import sys

import numpy as np
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import bench
    import oracle as O
    w, r, local, pg = bench.dist_setup(None)
    assert (w, r, local) == (world, rank, rank) and pg is not None
    # a rank-local job: one translated image pair, solved by the oracle
    rng = np.random.default_rng(100 + rank)
    img = rng.uniform(0, 255, (48, 48))
    from scipy.ndimage import gaussian_filter, shift
    ref = gaussian_filter(img, 1.5).astype(np.float32)
    de = shift(ref.astype(np.float64), (0.0, 0.3 + 0.1 * rank), order=3, mode="nearest").astype(np.float32)
    cfg = O.default_config()
    cfg.subset_radius, cfg.degree = 8, 3
    coef = O.prefilter(de, 3, 3, True)
    res = O.solve_pois(ref, coef, cfg, [[24.0, 24.0]], [[0.0] * 6], gradients=O.reference_gradient(ref))
    bench.barrier(pg)
    u_max = bench.max_over_ranks(pg, float(res["p"][0, 0]))
    n_sum = bench.sum_over_ranks(pg, float(res["converged"].sum()))
    out[rank] = (float(res["p"][0, 0]), u_max, n_sum)
    pg.destroy_process_group()


def test_two_replicas_on_gloo(oracle):
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    u = [out[r][0] for r in range(world)]
    assert abs(u[0] - 0.3) < 0.02 and abs(u[1] - 0.4) < 0.02       # each rank solved its own job
    assert all(out[r][1] == max(u) for r in range(world))           # max over ranks
    assert all(out[r][2] == 2.0 for r in range(world))              # sum over ranks


def test_cpu_baseline_legs(oracle, workload0):
    """bench.py's CPU baselines on the small workload: the threaded dataflow leg over the whole
    grid and the one-thread heap-order leg on a prefix, each a complete cpu_baseline object."""
    import __graft_entry__ as G
    import bench
    from traditional_dic_gb300 import subset as S
    cfg = S.config_from_dict(G.WORKLOAD0_CONFIG)
    seed, _ = oracle.select_seed(workload0.reference, workload0.deformed, oracle.as_config(cfg))
    par, ser = bench.cpu_baselines(workload0.reference, workload0.deformed, cfg, seed, 100, threads=4)
    for leg, cores in ((par, 4), (ser, 1)):
        assert "error" not in leg, leg
        assert leg["value"] > 0 and leg["unit"] == bench.UNIT and leg["cores"] == cores and leg["kind"] == "port"
        assert leg["sample"]
    assert "whole 256x256 workload" in par["sample"] and "576 solves" in par["sample"]
    assert "first 100 heap-order solves of the same 256x256 workload" in ser["sample"]


def test_route_comparison_counts_converged_points_apart():
    """bench.py --routes compares the FP32-mixed and FP64 builds over the jointly valid points
    and, separately, over the points both converged on strictly."""
    import bench
    valid = np.array([1, 1, 1, 1, 0], bool)
    strict = np.array([1, 1, 0, 0, 0], bool)
    u64 = np.zeros(5)
    u32 = np.array([1e-4, -2e-4, 0.05, 0.0, 9.0])
    got = bench.compare_builds((valid, u32, np.zeros(5), strict), (valid, u64, np.zeros(5), strict))
    assert got["flag_agreement"] == 1.0
    assert got["within_1e-3_px"] == 0.75 and got["within_1e-3_px_converged"] == 1.0
    none = bench.compare_builds((valid & False, u32, u64, strict), (valid, u64, u64, strict & False))
    assert none["within_1e-3_px"] is None and none["within_1e-3_px_converged"] is None

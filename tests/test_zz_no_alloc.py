"""tdic_propagate_noalloc: propagation with its scratch in a static device array instead of the
context's pool, for callers that cannot allocate device memory while they propagate.  Called
through the C ABI; its grid must equal tdic_propagate's bit for bit (the same kernel in the same
deterministic visit order) on two calls in a row (the second call finds the first call's scratch
contents), and neither the context's pool nor the device's free memory may change while it runs;
with masked subsets too (the pixel ROI in its own region of the array)."""
import ctypes as C

import numpy as np
import pytest

DOUBLE_FIELDS = ("x", "y", "u", "v", "du_dx", "du_dy", "dv_dx", "dv_dy", "correlation", "zncc")


def _device_grid(torch, n):
    t = {k: torch.full((n,), float("nan"), dtype=torch.float64, device="cuda") for k in DOUBLE_FIELDS}
    t["valid"] = torch.full((n,), 7, dtype=torch.uint8, device="cuda")
    t["status"] = torch.full((n,), 9, dtype=torch.int8, device="cuda")
    t["iterations"] = torch.full((n,), -5, dtype=torch.int32, device="cuda")
    t["converged"] = torch.full((n,), 7, dtype=torch.uint8, device="cuda")
    return t


def _grid_struct(L, t):
    return L.GridOut(**{k: t[k].data_ptr() for k in L.GRID_FIELDS})


def _roi(shape, sx, sy):
    """A rectangular hole in the quadrant diagonally opposite the seed, for the propagation
    to go around."""
    roi = np.ones(shape, np.uint8)
    h, w = shape
    y0 = h // 8 if sy >= h // 2 else h // 2 + h // 8
    x0 = w // 8 if sx >= w // 2 else w // 2 + w // 8
    roi[y0: y0 + h // 5, x0: x0 + w // 4] = 0
    return roi


@pytest.mark.gpu
@pytest.mark.parametrize("mode,masked", [(2, 0), (0, 0), (2, 1)])
def test_noalloc_matches_propagate_on_two_calls(oracle, workload0, mode, masked):
    import torch
    import __graft_entry__ as G
    from traditional_dic_gb300 import subset as S, _lib as L
    p = workload0
    cfg = S.config_from_dict(G.WORKLOAD0_CONFIG)
    cfg.propagation_spacing = 2                        # 86 x 86 grid points: two 4 KiB upload chunks
    cfg.propagation_mode = mode
    cfg.truncate_roi_subsets = masked                 # masked subsets read the pixel ROI
    seed_o, _ = oracle.select_seed(p.reference, p.deformed, oracle.as_config(cfg))
    assert seed_o.found
    seed = S.make_seed(seed_o.x, seed_o.y, list(seed_o.p), seed_o.correlation)
    roi = np.ascontiguousarray(_roi(p.reference.shape, seed_o.x, seed_o.y))

    ctx = S.Context(0)
    pair = S.Pair(ctx, p.reference, p.deformed, degree=3)
    gw, gh = L.grid_dims(pair.width, pair.height, cfg.propagation_spacing)
    n = gw * gh
    want = S.propagate(ctx, pair, cfg, seed, roi=roi)   # the allocating entry point (loads the kernels)
    grids = [_device_grid(torch, n) for _ in range(3)]   # outputs made before the calls
    torch.cuda.synchronize()
    held = ctx.device_bytes

    def call(t):
        g = _grid_struct(L, t)
        pc = C.c_int32(-1)
        ctx.check(ctx.lib.tdic_propagate_noalloc(ctx.handle, pair.handle, C.byref(cfg), C.byref(seed),
                                                 roi.ctypes.data, C.byref(g), C.byref(pc), None))
        return pc.value

    # the first call on the device is the set-up: looking up the static array makes the driver
    # load it (its ~16 MiB appear in the device's used memory then, once)
    got = [call(grids[0])]
    free_before = torch.cuda.mem_get_info()[0]
    got += [call(t) for t in grids[1:]]                 # two calls in a row
    free_after = torch.cuda.mem_get_info()[0]
    assert ctx.device_bytes == held                    # nothing taken from the context's pool
    assert free_after == free_before                   # nor from the device
    for t, pc in zip(grids, got):
        out = {k: v.cpu().numpy() for k, v in t.items()}
        assert pc == want["points_computed"] and pc > 1
        assert out["valid"].astype(bool).sum() > 0.5 * n
        # every field of every grid point, bit for bit (the device arrays started as NaN and
        # out-of-range codes, so a point left unwritten shows)
        for k in DOUBLE_FIELDS:
            assert np.array_equal(out[k], want[k], equal_nan=True), k
        for k in ("valid", "converged"):
            assert np.array_equal(out[k].astype(bool), want[k]), k
        assert np.array_equal(out["status"], want["status"])
        assert np.array_equal(out["iterations"], want["iterations"])
    pair.close()
    ctx.close()


@pytest.mark.gpu
def test_noalloc_rejects_grids_beyond_its_scratch():
    import torch
    from traditional_dic_gb300 import subset as S, _lib as L
    rng = np.random.default_rng(3)
    img = rng.integers(0, 255, (400, 400), dtype=np.uint8)
    ctx = S.Context(0)
    pair = S.Pair(ctx, img, img, degree=3)
    cfg = L.default_config()
    cfg.propagation_spacing = 0                       # 400 x 400 = 160000 grid points
    cfg.propagation_mode = 2
    seed = S.make_seed(200.0, 200.0, [0.0] * 6, 0.0)
    t = _device_grid(torch, 400 * 400)
    g = _grid_struct(L, t)
    pc = C.c_int32(-1)
    st = ctx.lib.tdic_propagate_noalloc(ctx.handle, pair.handle, C.byref(cfg), C.byref(seed), None, C.byref(g),
                                        C.byref(pc), None)
    assert st == L.TDIC_INVALID_ARG
    assert b"static scratch" in ctx.lib.tdic_last_error(ctx.handle)
    pair.close()
    ctx.close()

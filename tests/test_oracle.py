"""CPU tests that pin the FP64 oracle to the reference's algorithm.

The reference cannot be built here (Eigen is absent), so the oracle is pinned by numpy
transcriptions of the reference's own arithmetic -- the FFT deconvolution of
src/interpolation/bspline.cpp:177-244 and the local polynomial block evaluation of
bspline.cpp:96-175 / 320-367 -- and by analytic known-answer tests.
"""
import numpy as np
import pytest
from math import comb, factorial


# ---------------------------------------------------------------------------------------
# numpy transcriptions of the reference (bspline.cpp)
# ---------------------------------------------------------------------------------------
def ref_basis(x, r, d):  # bspline.cpp:342-367
    if r < 0 or r > d:
        return 0.0
    dfac = factorial(d) // factorial(d - r)
    s = 0.0
    for k in range(d + 2):
        sign = 1.0 if k % 2 == 0 else -1.0
        shift = (d + 1) / 2.0 - k
        xx = x + shift
        s += sign * comb(d + 1, k) * dfac * (xx ** (d - r) if xx > 0 else 0.0)
    return s / factorial(d)


def ref_qk(d):  # bspline.cpp:320-340
    n, off = d + 1, d // 2
    q = np.zeros((n, n))
    for r in range(n):
        for c in range(n):
            q[r, c] = (1.0 if r % 2 == 0 else -1.0) * ref_basis(float(-off + c), r, d) / factorial(r)
    return q


def ref_symmetric_index(v, size):  # bspline.cpp:78-89
    period = 2 * size
    w = v % period
    return w if w < size else period - 1 - w


def ref_form_coefficients(img, d, border):  # bspline.cpp:369-392 with the FFT path of :177-244
    h, w = img.shape
    border = max(3, border)
    ch, cw = h + 2 * border, w + 2 * border
    c = np.empty((ch, cw))
    for y in range(ch):
        sy = ref_symmetric_index(y - border, h)
        for x in range(cw):
            c[y, x] = float(img[sy, ref_symmetric_index(x - border, w)])

    def kernel(length):
        k = np.zeros(length)
        k[0] = ref_basis(0.0, 0, d)
        for o in range(1, d // 2 + 1):
            k[o] = ref_basis(float(o), 0, d)
            k[length - o] = ref_basis(float(o), 0, d)
        return k

    kr = np.fft.fft(kernel(cw))
    assert np.all(np.abs(kr) ** 2 > 1e-14)
    c = np.real(np.fft.ifft(np.fft.fft(c, axis=1) / kr[None, :], axis=1))
    kc = np.fft.fft(kernel(ch))
    c = np.real(np.fft.ifft(np.fft.fft(c, axis=0) / kc[:, None], axis=0))
    return c


def ref_value(coef, w, h, d, border, x, y, q):  # bspline.cpp:458-474 via the polynomial block
    n, off = d + 1, d // 2
    ix = min(max(int(np.floor(x)), 0), w - 1)
    iy = min(max(int(np.floor(y)), 0), h - 1)
    dx, dy = x - ix, y - iy
    top, left = iy + border - off, ix + border - off
    cb = coef[top:top + n, left:left + n]
    P = q @ cb @ q.T
    return sum(P[r, c] * dy ** r * dx ** c for r in range(n) for c in range(n))


def ref_gradient(coef, w, h, d, border, x, y, q):  # bspline.cpp:476-500
    n, off = d + 1, d // 2
    ix = min(max(int(np.floor(x)), 0), w - 1)
    iy = min(max(int(np.floor(y)), 0), h - 1)
    dx, dy = x - ix, y - iy
    top, left = iy + border - off, ix + border - off
    P = q @ coef[top:top + n, left:left + n] @ q.T
    gx = sum(c * P[r, c] * dy ** r * dx ** (c - 1) for r in range(n) for c in range(1, n))
    gy = sum(r * P[r, c] * dy ** (r - 1) * dx ** c for r in range(1, n) for c in range(n))
    return gx, gy


def rng_image(h, w, seed=0, dtype=np.uint8):
    return np.random.default_rng(seed).integers(0, 255, (h, w)).astype(dtype)


# ---------------------------------------------------------------------------------------
@pytest.mark.parametrize("d", [1, 3, 5])
def test_basis_and_qk_match_transcription(oracle, d):
    for x in np.linspace(-3.5, 3.5, 29):
        for r in range(d + 1):
            assert oracle.basis(x, r, d) == pytest.approx(ref_basis(x, r, d), abs=1e-14)
    assert np.allclose(oracle.qk(d), ref_qk(d), atol=1e-15)


@pytest.mark.parametrize("d", [1, 3, 5])
def test_basis_partition_of_unity(oracle, d):
    for x in np.linspace(0.0, 0.999, 17):
        s = sum(oracle.basis(x - k, 0, d) for k in range(-4, 5))
        assert s == pytest.approx(1.0, abs=1e-12)  # truncated-power form cancels at ~1e-13
        g = sum(oracle.basis(x - k, 1, d) for k in range(-4, 5)) if d > 1 else 0.0
        assert abs(g) < 1e-11


@pytest.mark.parametrize("d", [1, 3, 5])
@pytest.mark.parametrize("shape,border", [((1, 1), 3), ((2, 3), 3), ((5, 7), 4), ((23, 17), 3), ((40, 33), 6)])
def test_prefilter_equals_fft_deconvolution(oracle, d, shape, border):
    img = rng_image(*shape, seed=sum(shape) + d)
    got = oracle.prefilter(img, d, border, True)
    want = ref_form_coefficients(img, d, border)
    assert got.shape == want.shape
    assert np.max(np.abs(got - want)) < 1e-10 * max(1.0, np.abs(want).max())


def test_lazy_prefilter_is_clamp_padding(oracle):
    img = rng_image(9, 11, seed=3)
    got = oracle.prefilter(img, 5, 3, False)
    ys = np.clip(np.arange(-3, 12) , 0, 8)
    xs = np.clip(np.arange(-3, 14), 0, 10)
    assert np.array_equal(got, img[np.ix_(ys, xs)].astype(np.float64))


@pytest.mark.parametrize("d", [1, 3, 5])
def test_interpolation_equals_polynomial_block(oracle, d):
    img = rng_image(30, 26, seed=11)
    coef = oracle.prefilter(img, d, 3, True)
    q = ref_qk(d)
    rs = np.random.default_rng(5)
    for _ in range(40):
        x, y = rs.uniform(0, 25), rs.uniform(0, 29)
        assert oracle.interp_value(coef, 26, 30, d, 3, x, y) == pytest.approx(ref_value(coef, 26, 30, d, 3, x, y, q),
                                                                               abs=1e-10)
        gx, gy = oracle.interp_gradient(coef, 26, 30, d, 3, x, y)
        rx, ry = ref_gradient(coef, 26, 30, d, 3, x, y, q)
        assert gx == pytest.approx(rx, abs=1e-9) and gy == pytest.approx(ry, abs=1e-9)


@pytest.mark.parametrize("d", [1, 3, 5])
def test_interpolating_at_pixels(oracle, d):
    """The exact prefilter makes the spline interpolate the image at integer positions."""
    img = rng_image(21, 19, seed=2)
    coef = oracle.prefilter(img, d, 3, True)
    for y in range(0, 21, 4):
        for x in range(0, 19, 3):
            assert oracle.interp_value(coef, 19, 21, d, 3, x, y) == pytest.approx(float(img[y, x]), abs=1e-9)


def test_reference_gradient_formula(oracle):
    img = rng_image(6, 5, seed=9).astype(np.float32)
    gx, gy = oracle.reference_gradient(img)
    f = img.astype(np.float64)
    ex = np.empty_like(f)
    ex[:, 1:-1] = (f[:, 2:] - f[:, :-2]) / 2
    ex[:, 0] = f[:, 1] - f[:, 0]
    ex[:, -1] = f[:, -1] - f[:, -2]
    ey = np.empty_like(f)
    ey[1:-1] = (f[2:] - f[:-2]) / 2
    ey[0] = f[1] - f[0]
    ey[-1] = f[-1] - f[-2]
    assert np.array_equal(gx, ex) and np.array_equal(gy, ey)


def smooth_image(h, w, shift=(0.0, 0.0)):
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    X, Y = x - shift[0], y - shift[1]
    return (120 + 40 * np.sin(2 * np.pi * X / 23.0) * np.cos(2 * np.pi * Y / 17.0)
            + 30 * np.sin(2 * np.pi * (X + 2 * Y) / 31.0)).astype(np.float32)


@pytest.mark.parametrize("optimizer", [0, 1])
@pytest.mark.parametrize("d", [3, 5])
def test_translation_known_answer(oracle, optimizer, d):
    ref = smooth_image(80, 80)
    de = smooth_image(80, 80, shift=(0.3, -0.7))
    coef = oracle.prefilter(de, d, 3, True)
    cfg = oracle.default_config(subset_radius=12, max_iterations=50, convergence_threshold=1e-8, degree=d,
                                optimizer=optimizer)
    xy = np.array([[40.0, 40.0], [30.0, 45.0], [50.0, 33.0]])
    res = oracle.solve_pois(ref, coef, cfg, xy, np.zeros((3, 6)))
    assert np.all(res["status"] == 0) and np.all(res["converged"])
    assert np.allclose(res["p"][:, 0], 0.3, atol=2e-3) and np.allclose(res["p"][:, 1], -0.7, atol=2e-3)
    assert np.all(np.abs(res["p"][:, 2:]) < 2e-3)


def test_zero_hessian_is_positive_semidefinite(oracle):
    """A period-2 pattern has zero central differences: the Hessian is zero, Eigen's LDLT
    reports ZeroSign (isPositive() true), the solve returns dp = 0 and ICGN converges at the
    first iteration (icgn.cpp:538-542, 594-615)."""
    y, x = np.mgrid[0:40, 0:40]
    ref = (100 + 50 * ((x + y) % 2)).astype(np.float32)
    coef = oracle.prefilter(ref, 3, 3, True)
    cfg = oracle.default_config(subset_radius=5, max_iterations=10, degree=3)
    res = oracle.solve_pois(ref, coef, cfg, np.array([[20.0, 20.0]]), np.zeros((1, 6)))
    assert res["status"][0] == 0 and res["iterations"][0] == 1 and res["converged"][0]
    assert np.all(res["p"] == 0.0)


def test_solver_edge_statuses(oracle):
    ref = rng_image(40, 40, seed=4).astype(np.float32)
    ref[:12, :12] = 50
    coef = oracle.prefilter(ref, 3, 3, True)
    cfg = oracle.default_config(subset_radius=5, max_iterations=10, degree=3)
    xy = np.array([[2.0, 20.0], [20.0, 20.0], [6.0, 6.0]])
    p0 = np.zeros((3, 6))
    p0[1, 0] = 30.0
    res = oracle.solve_pois(ref, coef, cfg, xy, p0, confidence0=np.array([0.1, 0.2, 0.3]))
    assert list(res["status"]) == [2, 2, 3]
    assert list(res["correlation"]) == [0.1, 0.2, 0.3]       # initial.confidence on early exits
    assert res["p"][1, 0] == 30.0 and np.all(res["p"][:, 2:] == 0)
    cfg0 = oracle.default_config(subset_radius=5, max_iterations=0, degree=3)
    r0 = oracle.solve_pois(ref, coef, cfg0, xy[1:2], np.zeros((1, 6)))
    assert r0["status"][0] == 1 and not r0["valid"][0]          # inf correlation -> NotConverged


def test_integer_search_known_shift(oracle):
    ref = rng_image(90, 90, seed=21).astype(np.float32)
    de = np.roll(np.roll(ref, 3, axis=1), -2, axis=0)
    cfg = oracle.default_config(is_subset_radius=8, is_search_radius=6)
    u, v, z = oracle.integer_search(ref, de, cfg, 45, 45)
    assert (u, v) == (3.0, -2.0) and z == pytest.approx(1.0, abs=1e-12)


def test_grid_dims(oracle):
    assert oracle.grid_dims(2048, 2048, 4) == (410, 410)
    assert oracle.grid_dims(256, 256, 9) == (26, 26)
    assert oracle.grid_dims(5120, 5120, 2) == (1707, 1707)


def test_heap_and_frontier_orders(oracle, workload0):
    """The two visit orders accept the same points; converged values differ only at the
    convergence-threshold level (the reference's own output is that far from the exact
    minimiser)."""
    import __graft_entry__ as G
    from traditional_dic_gb300 import subset as S
    cfg = oracle.as_config(S.config_from_dict(G.WORKLOAD0_CONFIG))
    seed, _ = oracle.select_seed(workload0.reference, workload0.deformed, cfg)
    coef = oracle.prefilter(workload0.deformed, 3, 3, True)
    cfg.propagation_mode = 1
    heap = oracle.propagate(workload0.reference, coef, cfg, seed)
    cfg.propagation_mode = 0
    front = oracle.propagate(workload0.reference, coef, cfg, seed)
    assert heap["points_computed"] == front["points_computed"] > 500
    assert np.array_equal(heap["valid"], front["valid"])
    both = heap["valid"]
    d = np.hypot(heap["u"][both] - front["u"][both], heap["v"][both] - front["v"][both])
    assert np.median(d) < 1e-4 and d.max() < 1e-2


@pytest.mark.parametrize("mode", [0, 2])
@pytest.mark.parametrize("max_solves", [-1, 150])
def test_threaded_propagation_is_the_serial_one(oracle, workload0, mode, max_solves):
    """The threaded CPU baseline solves each frontier wave (mode 0) or dataflow diagonal (mode 2)
    on several host threads: every output array, the solve count and the point count are those
    of one thread, with and without a solve budget."""
    import __graft_entry__ as G
    from traditional_dic_gb300 import subset as S
    cfg = oracle.as_config(S.config_from_dict(G.WORKLOAD0_CONFIG))
    cfg.propagation_mode = mode
    seed, _ = oracle.select_seed(workload0.reference, workload0.deformed, cfg)
    coef = oracle.prefilter(workload0.deformed, 3, 3, True)
    grads = oracle.reference_gradient(workload0.reference)
    one = oracle.propagate(workload0.reference, coef, cfg, seed, gradients=grads, max_solves=max_solves)
    many = oracle.propagate(workload0.reference, coef, cfg, seed, gradients=grads, max_solves=max_solves, threads=5)
    assert one["solves"] == many["solves"] and one["points_computed"] == many["points_computed"] > 100
    for k, a in one.items():
        if isinstance(a, np.ndarray):
            assert np.array_equal(a, many[k], equal_nan=a.dtype.kind == "f"), k

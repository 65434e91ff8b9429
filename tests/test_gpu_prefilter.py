"""The pair set-up launch (prefilter_fused_kernel) against the oracle's prefilter on shapes that
cut the 224/192/144-column and 32/16-row output tiles at every kind of edge (images smaller than
one tile, one pixel, thin strips, several tiles with ragged last tiles), for every input dtype,
both coefficient precisions, cubic and quintic splines and several border widths; and the
float32 images the same launch leaves in the pair equal the input as dic::Image holds it.
Widths of 701 and more put integer-pixel tiles on the staged path (rows copied to shared memory
by 16-byte asynchronous copies), with row starts at every alignment (odd widths)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1), (5, 300), (300, 7), (70, 90), (33, 250), (97, 701), (250, 33)]
DTYPES = [np.uint8, np.uint16, np.float32, np.float64]


def _image(shape, dtype, seed):
    rng = np.random.default_rng(seed)
    if dtype == np.uint8:
        return rng.integers(0, 256, shape).astype(np.uint8)
    if dtype == np.uint16:
        return rng.integers(0, 65536, shape).astype(np.uint16)
    return (rng.random(shape) * 255.0).astype(dtype)


def _check(oracle, pair, ref, de, degree, border, precision):
    got = pair.coefficients().astype(np.float64)
    want = oracle.prefilter(de.astype(np.float32), degree, border, True)
    assert got.shape == want.shape
    tol = 1e-11 if precision == 1 else 2e-5
    assert np.max(np.abs(got - want)) <= tol * max(1.0, np.abs(want).max())
    r, d = pair.images()
    assert np.array_equal(r, ref.astype(np.float32)) and np.array_equal(d, de.astype(np.float32))


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("degree", [3, 5])
@pytest.mark.parametrize("precision", [0, 1])
def test_pair_setup_shapes(oracle, gpu_ctx, shape, degree, precision):
    from traditional_dic_gb300 import subset as S
    ref, de = _image(shape, np.uint8, 1), _image(shape, np.uint8, 2)
    pair = S.Pair(gpu_ctx, ref, de, degree=degree, border=3, precision=precision)
    _check(oracle, pair, ref, de, degree, 3, precision)
    pair.close()


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("border", [3, 6])
def test_pair_setup_dtypes_and_borders(oracle, gpu_ctx, dtype, border):
    from traditional_dic_gb300 import subset as S
    ref, de = _image((61, 729), dtype, 3), _image((61, 729), dtype, 4)
    for precision in (0, 1):
        pair = S.Pair(gpu_ctx, ref, de, degree=3, border=border, precision=precision)
        _check(oracle, pair, ref, de, 3, border, precision)
        pair.close()


def test_pair_setup_device_input_and_update(oracle, gpu_ctx):
    """Device images are read in place; an update from host images replaces all three outputs."""
    import torch
    from traditional_dic_gb300 import subset as S
    ref, de = _image((130, 470), np.uint8, 5), _image((130, 470), np.uint8, 6)
    ref2, de2 = _image((130, 470), np.uint8, 7), _image((130, 470), np.uint8, 8)
    pair = S.Pair(gpu_ctx, torch.from_numpy(ref).cuda(), torch.from_numpy(de).cuda(), degree=5, precision=0)
    _check(oracle, pair, ref, de, 5, 3, 0)
    pair.update(ref2, de2)
    _check(oracle, pair, ref2, de2, 5, 3, 0)
    pair.update(torch.from_numpy(ref).cuda(), torch.from_numpy(de).cuda())
    _check(oracle, pair, ref, de, 5, 3, 0)
    pair.close()


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
def test_pair_setup_unaligned_device_rows(oracle, gpu_ctx, dtype):
    """Device images whose first pixel is one element past a 16-byte boundary, with a row pitch
    that is a multiple of 16 bytes (one alignment shift for every staged row) and without one."""
    import torch
    from traditional_dic_gb300 import subset as S
    for shape in ((200, 1024), (120, 1001)):
        ref, de = _image(shape, dtype, 11), _image(shape, dtype, 12)
        tdt = torch.uint8 if dtype == np.uint8 else torch.uint16
        imgs = []
        for a in (ref, de):
            flat = torch.empty(a.size + 1, dtype=tdt, device="cuda")
            flat[1:] = torch.from_numpy(a.ravel()).to("cuda")
            imgs.append(flat[1:].view(shape))
        assert imgs[0].data_ptr() % 16 != 0 and imgs[0].is_contiguous()
        pair = S.Pair(gpu_ctx, imgs[0], imgs[1], degree=3, precision=0)
        _check(oracle, pair, ref, de, 3, 3, 0)
        pair.close()


def test_pair_setup_large(oracle, gpu_ctx):
    """A 2048 x 1536 uint8 pair (whole tiles plus ragged edges in both directions)."""
    from traditional_dic_gb300 import subset as S
    ref, de = _image((1536, 2048), np.uint8, 9), _image((1536, 2048), np.uint8, 10)
    pair = S.Pair(gpu_ctx, ref, de, degree=3, precision=0)
    _check(oracle, pair, ref, de, 3, 3, 0)
    pair.close()

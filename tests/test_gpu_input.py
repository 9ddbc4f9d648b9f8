"""Input preparation kernels (gray, thumbnail resize, FP16 pyramid) against
the oracle's restatements: bit-exact."""
import numpy as np
import pytest

from oracle import oracle as O
from patchmatch_gb300 import native

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    return torch


@pytest.mark.parametrize("ch,order", [(3, native.ORDER_BGR), (3, native.ORDER_RGB), (4, native.ORDER_BGR), (1, 0)])
def test_gray_bit_exact(ctx, torch_cuda, ch, order):
    rng = np.random.default_rng(ch + 10 * order)
    img = rng.integers(0, 256, (97, 131, ch) if ch > 1 else (97, 131), dtype=np.uint8)
    g = ctx.to_gray(torch_cuda.from_numpy(img).cuda(), order).cpu().numpy()
    assert np.array_equal(g, O.to_gray(img[..., :3] if ch == 4 else img, rgb=order == native.ORDER_RGB))


@pytest.mark.parametrize("src,dst,ch", [((3840, 1920), (1920, 960), 1), ((1920, 960), (1280, 640), 3),
                                        ((640, 320), (1000, 500), 1), ((257, 129), (100, 50), 3)])
def test_resize_bit_exact(ctx, torch_cuda, src, dst, ch):
    rng = np.random.default_rng(src[0])
    shape = (src[1], src[0], ch) if ch > 1 else (src[1], src[0])
    img = rng.integers(0, 256, shape, dtype=np.uint8)
    g = ctx.resize(torch_cuda.from_numpy(img).cuda(), *dst).cpu().numpy()
    o = O.resize_linear(img, *dst)
    assert g.shape == o.shape and np.array_equal(g, o)
    if src == (3840, 1920):  # exact 2x: the mean of each 2x2 block, rounded half up
        blk = img.reshape(960, 2, 1920, 2).astype(np.int64).sum(axis=(1, 3))
        assert np.array_equal(g, ((blk * 1024 * 1024 + (1 << 21)) >> 22).astype(np.uint8))


def test_pyramid_bit_exact(ctx, torch_cuda):
    rng = np.random.default_rng(3)
    img = rng.integers(0, 256, (961, 1923), dtype=np.uint8)
    g = [t.cpu().numpy() for t in ctx.pyramid_f16(torch_cuda.from_numpy(img).cuda(), 3)]
    o = O.pyramid_f16(img, 3)
    assert [x.shape for x in g] == [(961, 1923), (481, 962), (241, 481)]
    for a, b in zip(g, o):
        assert np.array_equal(a.view(np.uint16), b.view(np.uint16))

"""Lookahead analysis on the GPU: the lowres_filter drop-in and the
picture-level low-resolution picture + block MAD maps against the oracle
(lowres_filter pinned to the reference's mc.c, MAD to pixel.c)."""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def test_lowres_dropin(gpu, olib):
    import xavs2_gb300 as xg
    rng = np.random.default_rng(98)
    for w, h in ((32, 18), (7, 5), (64, 64), (1, 1), (100, 3)):
        src = rng.integers(0, 256, (2 * h + 3, 2 * w + 5), dtype=np.uint8)
        a = np.full((h, w + 3), 7, np.uint8)
        b = a.copy()
        xg.fn("xavs2gpu_lowres_filter")(xg.ptr(src), src.shape[1], xg.ptr(a), w + 3, w, h)
        olib.xo_lowres_filter(oracle.ptr(src), src.shape[1], oracle.ptr(b), w + 3, w, h)
        assert np.array_equal(a, b), (w, h)


@pytest.mark.parametrize("w,h", [(128, 64), (200, 136), (72, 40), (1920, 1080), (3840, 2160), (66, 34)])
def test_lookahead_picture(gpu, olib, w, h):
    import torch
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(w + h)
    img = synth.base_picture(rng, w, h)
    img[: h // 3, : w // 4] = rng.integers(0, 256, (h // 3, w // 4))
    stride = w + 12
    src = np.zeros((h, stride), np.uint8)
    src[:, :w] = img
    ls = w // 2 + 4
    n = [((w + s - 1) // s) * ((h + s - 1) // s) for s in (16, 32, 64)]
    el = np.zeros((h // 2, ls), np.uint8)
    em = [np.zeros(k, np.int32) for k in n]
    olib.xo_lookahead_picture(oracle.ptr(src), stride, w, h, oracle.ptr(el), ls, *[oracle.ptr(m) for m in em])
    d_src = torch.from_numpy(src).cuda()
    d_l = torch.zeros((h // 2, ls), dtype=torch.uint8, device="cuda")
    d_m = [torch.full((k,), 12345, dtype=torch.int32, device="cuda") for k in n]
    rc = gpu.xavs2gpu_lookahead_picture(ctypes.c_void_p(d_src.data_ptr()), stride, w, h,
                                        ctypes.c_void_p(d_l.data_ptr()), ls,
                                        *[ctypes.c_void_p(m.data_ptr()) for m in d_m], None)
    assert rc == 0
    torch.cuda.synchronize()
    assert np.array_equal(d_l.cpu().numpy()[:, : w // 2], el[:, : w // 2])
    for k in range(3):
        assert np.array_equal(d_m[k].cpu().numpy(), em[k]), k
    d_l2 = torch.zeros((h // 2, ls), dtype=torch.uint8, device="cuda")
    assert gpu.xavs2gpu_lowres_picture(ctypes.c_void_p(d_src.data_ptr()), stride, ctypes.c_void_p(d_l2.data_ptr()),
                                       ls, w // 2, h // 2, None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(d_l2.cpu().numpy()[:, : w // 2], el[:, : w // 2])


@pytest.mark.parametrize("w,h,pad,lpad,content", [(128, 64, 0, 0, "max"), (128, 64, 16, 4, "checker"),
                                                  (200, 136, 8, 0, "random"), (1920, 1080, 0, 0, "checker"),
                                                  (3840, 2160, 0, 4, "random"), (200, 136, 8, 4, "zero")])
def test_lookahead_aligned_rows(gpu, olib, w, h, pad, lpad, content):
    """The 16-byte row path (source and stride 16-byte aligned; partial
    strips at the right edge when the width is not a multiple of 16), the
    8-byte and the bytewise half-resolution stores (row alignment of the
    low-resolution plane), and sums at their extremes (all 255, 0/255
    checkerboards: the largest MADs)."""
    import torch
    rng = np.random.default_rng(w * 3 + h + pad)
    stride = w + pad
    assert stride % 16 == 0
    if content == "max":
        img = np.full((h, w), 255, np.uint8)
    elif content == "zero":
        img = np.zeros((h, w), np.uint8)
    elif content == "checker":
        img = (((np.arange(h)[:, None] + np.arange(w)[None, :]) & 1) * 255).astype(np.uint8)
    else:
        img = rng.integers(0, 256, (h, w), dtype=np.uint8)
    src = np.zeros((h, stride), np.uint8)
    src[:, :w] = img
    ls = w // 2 + lpad
    n = [((w + s - 1) // s) * ((h + s - 1) // s) for s in (16, 32, 64)]
    el = np.zeros((h // 2, ls), np.uint8)
    em = [np.zeros(k, np.int32) for k in n]
    olib.xo_lookahead_picture(oracle.ptr(src), stride, w, h, oracle.ptr(el), ls, *[oracle.ptr(m) for m in em])
    d_src = torch.from_numpy(src).cuda()
    d_l = torch.zeros((h // 2, ls), dtype=torch.uint8, device="cuda")
    d_m = [torch.full((k,), 12345, dtype=torch.int32, device="cuda") for k in n]
    rc = gpu.xavs2gpu_lookahead_picture(ctypes.c_void_p(d_src.data_ptr()), stride, w, h,
                                        ctypes.c_void_p(d_l.data_ptr()), ls,
                                        *[ctypes.c_void_p(m.data_ptr()) for m in d_m], None)
    assert rc == 0
    torch.cuda.synchronize()
    assert np.array_equal(d_l.cpu().numpy()[:, : w // 2], el[:, : w // 2])
    for k in range(3):
        assert np.array_equal(d_m[k].cpu().numpy(), em[k]), k
    if content == "checker":
        # a 0/255 checkerboard: block average 128, MAD 128 * 127 + 128 * 128 per 16x16
        assert em[0][0] == 128 * 127 + 128 * 128

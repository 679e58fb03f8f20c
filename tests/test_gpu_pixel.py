"""GPU drop-ins of pixel_funcs_t against the oracle (bit-exact)."""
import ctypes

import numpy as np
import pytest

import oracle
from oracle import PU_W, PU_H

pytestmark = pytest.mark.gpu


def _pairs(rng):
    out = []
    for mode in range(4):
        a = rng.integers(0, 256, (64, 72), dtype=np.uint8)
        b = rng.integers(0, 256, (64, 80), dtype=np.uint8)
        if mode == 1:
            a[:] = 255; b[:] = 0
        elif mode == 2:
            sgn = rng.integers(0, 2, (64, 80))
            a[:] = np.where(sgn[:, :72] == 1, 255, 0); b[:] = np.where(sgn == 1, 0, 255)
        elif mode == 3:
            a[:] = np.where(np.indices(a.shape).sum(0) % 2 == 0, 255, 0)
        out.append((a, b))
    return out


@pytest.fixture(params=[1, 0], ids=["in_place", "staged"])
def percall_mode(request, gpu):
    """Per-call block costs read in place (where the device reads pageable
    host memory) and through the staged copies."""
    gpu.xavs2gpu_set_percall_mode(request.param)
    yield request.param
    gpu.xavs2gpu_set_percall_mode(1)


@pytest.mark.parametrize("kind", ["sad", "satd", "sa8d", "ssd"])
def test_costs(gpu, olib, kind, percall_mode):
    import xavs2_gb300 as xg
    rng = np.random.default_rng(3)
    ofn = getattr(olib, "xo_" + kind)
    for a, b in _pairs(rng):
        for part in range(25):
            got = xg.pixel_fn(kind, part)(xg.ptr(a, 3), 72, xg.ptr(b, 5), 80)
            exp = ofn(part, oracle.ptr(a, 3), 72, oracle.ptr(b, 5), 80)
            assert got == exp, (kind, part, got, exp)


def test_sad_x3_x4(gpu, olib, percall_mode):
    import xavs2_gb300 as xg
    rng = np.random.default_rng(4)
    fenc = rng.integers(0, 256, (64, 64), dtype=np.uint8)
    ref = rng.integers(0, 256, (80, 100), dtype=np.uint8)
    for part in range(25):
        offs = [0, 3, 105, 1001]
        g3 = (ctypes.c_int * 3)(); o3 = (ctypes.c_int32 * 3)()
        xg.pixel_fn("sad_x3", part)(xg.ptr(fenc), *[xg.ptr(ref, o) for o in offs[:3]], 100, g3)
        olib.xo_sad_x3(part, oracle.ptr(fenc), *[oracle.ptr(ref, o) for o in offs[:3]], 100, o3)
        assert list(g3) == list(o3)
        g4 = (ctypes.c_int * 4)(); o4 = (ctypes.c_int32 * 4)()
        xg.pixel_fn("sad_x4", part)(xg.ptr(fenc), *[xg.ptr(ref, o) for o in offs], 100, g4)
        olib.xo_sad_x4(part, oracle.ptr(fenc), *[oracle.ptr(ref, o) for o in offs], 100, o4)
        assert list(g4) == list(o4)


def test_block_ops(gpu, olib):
    import xavs2_gb300 as xg
    rng = np.random.default_rng(5)
    for part in range(25):
        a = rng.integers(0, 256, (64, 70), dtype=np.uint8)
        b = rng.integers(0, 256, (64, 66), dtype=np.uint8)
        s = rng.integers(-600, 600, (64, 72), dtype=np.int16)
        d1 = np.zeros((64, 68), np.uint8); d2 = d1.copy()
        xg.pixel_fn("avg", part)(xg.ptr(d1), 68, xg.ptr(a), 70, xg.ptr(b), 66, 32)
        olib.xo_avg(part, oracle.ptr(d2), 68, oracle.ptr(a), 70, oracle.ptr(b), 66)
        assert np.array_equal(d1, d2)
        e1 = np.zeros((64, 64), np.int16); e2 = e1.copy()
        xg.pixel_fn("sub_ps", part)(xg.ptr(e1), 64, xg.ptr(a), xg.ptr(b), 70, 66)
        olib.xo_sub_ps(part, oracle.ptr(e2), 64, oracle.ptr(a), oracle.ptr(b), 70, 66)
        assert np.array_equal(e1, e2)
        d1[:] = 7; d2[:] = 7
        xg.pixel_fn("add_ps", part)(xg.ptr(d1), 68, xg.ptr(a), xg.ptr(s), 70, 72)
        olib.xo_add_ps(part, oracle.ptr(d2), 68, oracle.ptr(a), oracle.ptr(s), 70, 72)
        assert np.array_equal(d1, d2)
        for kind, src, dt in (("copy_pp", a, np.uint8), ("copy_ps", a, np.int16),
                              ("copy_sp", (np.abs(s) % 256).astype(np.int16), np.uint8), ("copy_ss", s, np.int16)):
            x1 = np.zeros((64, 80), dt); x2 = x1.copy()
            xg.pixel_fn(kind, part)(xg.ptr(x1), 80, xg.ptr(src), src.shape[1])
            getattr(olib, "xo_" + kind)(part, oracle.ptr(x2), 80, oracle.ptr(src), src.shape[1])
            assert np.array_equal(x1, x2), kind
    for (w, h) in ((13, 7), (64, 64), (100, 3)):
        a = rng.integers(0, 256, (h, 128), dtype=np.uint8)
        b = rng.integers(0, 256, (h, 128), dtype=np.uint8)
        assert xg.fn("xavs2gpu_get_block_ssd")(xg.ptr(a), 128, xg.ptr(b), 128, w, h) == \
            olib.xo_ssd_block(oracle.ptr(a), 128, oracle.ptr(b), 128, w, h)
        d1 = np.zeros((h, 128), np.uint8); d2 = d1.copy()
        xg.fn("xavs2gpu_pixel_average")(xg.ptr(d1), 128, xg.ptr(a), 128, xg.ptr(b), 128, w, h)
        olib.xo_average(oracle.ptr(d2), 128, oracle.ptr(a), 128, oracle.ptr(b), 128, w, h)
        assert np.array_equal(d1, d2)
    for size in (16, 32, 64):
        a = rng.integers(0, 256, (64, 90), dtype=np.uint8)
        assert xg.fn("xavs2gpu_mad_NxN")(xg.ptr(a), 90, size) == olib.xo_mad(oracle.ptr(a), 90, size)


def test_pixel_table_install(gpu, olib):
    """xavs2gpu_pixel_init fills a pixel_funcs_t-shaped table; call through it."""
    import xavs2_gb300 as xg
    fptr = ctypes.CFUNCTYPE(ctypes.c_int32, ctypes.c_void_p, ctypes.c_ssize_t, ctypes.c_void_p, ctypes.c_ssize_t)
    nptr = 13 * 25 + 2 + 4 + 2
    table = (ctypes.c_void_p * nptr)()
    xg.fn("xavs2gpu_pixel_init")(0, ctypes.byref(table))
    rng = np.random.default_rng(6)
    a = rng.integers(0, 256, (64, 64), dtype=np.uint8)
    b = rng.integers(0, 256, (64, 64), dtype=np.uint8)
    for row, kind in ((0, "xo_sad"), (1, "xo_satd"), (2, "xo_sa8d"), (3, "xo_ssd")):
        for part in range(25):
            f = fptr(table[row * 25 + part])
            assert f(xg.ptr(a), 64, xg.ptr(b), 64) == getattr(olib, kind)(part, oracle.ptr(a), 64, oracle.ptr(b), 64)


def test_cost_batch(gpu, olib):
    import torch
    import xavs2_gb300 as xg
    rng = np.random.default_rng(7)
    base1 = rng.integers(0, 256, 1 << 16, dtype=np.uint8)
    base2 = rng.integers(0, 256, 1 << 16, dtype=np.uint8)
    n = 300
    jobs = np.zeros(n, xg.COST_JOB_DTYPE)
    jobs["part"] = rng.integers(0, 25, n)
    jobs["s1"] = 128
    jobs["s2"] = 160
    jobs["off1"] = rng.integers(0, (1 << 16) - 64 * 128 - 64, n)
    jobs["off2"] = rng.integers(0, (1 << 16) - 64 * 160 - 64, n)
    d1 = torch.from_numpy(base1).cuda(); d2 = torch.from_numpy(base2).cuda()
    dj = torch.from_numpy(jobs.view(np.uint8).copy()).cuda()
    for kind, name in enumerate(["xo_sad", "xo_satd", "xo_sa8d", "xo_ssd"]):
        out = torch.zeros(n, dtype=torch.int32, device="cuda")
        rc = xg.fn("xavs2gpu_cost_batch")(kind, dj.data_ptr(), n, d1.data_ptr(), d2.data_ptr(), out.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        exp = [getattr(olib, name)(int(j["part"]), oracle.ptr(base1, int(j["off1"])), 128,
                                   oracle.ptr(base2, int(j["off2"])), 160) for j in jobs]
        assert np.array_equal(got, exp), name

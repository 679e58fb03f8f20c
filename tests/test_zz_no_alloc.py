"""The allocation-free motion search (xavs2gpu_me_search_noalloc), for callers
that cannot allocate device memory while they run, against the session
entry point (xavs2gpu_me_run): identical results on two calls in a row
through the C ABI.  Collected last on purpose."""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _noalloc(lib):
    f = lib.xavs2gpu_me_search_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                  ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f


def test_noalloc_matches_session_entry(gpu):
    import torch
    import xavs2_gb300 as xg
    lib = xg.load()
    rng = np.random.default_rng(2024)
    w, h = 192, 128
    cur = rng.integers(0, 256, (h, w), dtype=np.uint8)
    refs = [np.clip(np.roll(cur, s, axis=(0, 1)).astype(np.int16) + rng.integers(-4, 5, (h, w)), 0, 255)
            .astype(np.uint8) for s in ((1, -2), (-3, 2))]
    layout = xg.frame_pus(w, h, 2)[::3]
    n = 200
    extra = np.zeros(n, xg.PU_DTYPE)
    extra["part"] = rng.integers(0, 25, n)
    pw, ph = np.array(xg.PU_W)[extra["part"]], np.array(xg.PU_H)[extra["part"]]
    extra["x"] = (rng.random(n) * (w - pw + 1)).astype(int)
    extra["y"] = (rng.random(n) * (h - ph + 1)).astype(int)
    extra["ref"] = rng.integers(0, 2, n)
    extra["mvp_x"] = rng.integers(-30, 31, n)
    extra["mvp_y"] = rng.integers(-30, 31, n)
    pus = np.concatenate([layout, xg.set_limits(extra, w, h)])
    prm = xg.MeParams(12, oracle.lambda_factor(32), 1, 2, 0, 0)

    sess = xg.MeSession(w, h, 2, len(pus))
    sess.set_picture(-1, cur)
    for i, r in enumerate(refs):
        sess.set_picture(i, r)
    sess.set_pus(pus)
    sess.run(prm)
    expected = sess.results()

    planes = (ctypes.c_void_p * 32)(*[sess.plane_ptr(r, k) for r in range(2) for k in range(16)])
    d_pus = torch.from_numpy(pus.view(np.uint8).copy()).cuda()
    f = _noalloc(lib)
    for call in range(2):
        d_out = torch.full((len(pus) * xg.RESULT_DTYPE.itemsize,), 0xAB, dtype=torch.uint8, device="cuda")
        rc = f(sess.plane_ptr(-1, 0), sess.plane_stride(), w, h, planes, 2, d_pus.data_ptr(), len(pus),
               ctypes.byref(prm), d_out.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        got = d_out.cpu().numpy().view(xg.RESULT_DTYPE)
        assert got.tobytes() == expected.tobytes(), "call %d differs from xavs2gpu_me_run" % call
    sess.close()


def test_noalloc_rejects_oversized_requests(gpu):
    import xavs2_gb300 as xg
    lib = xg.load()
    f = _noalloc(lib)
    prm = xg.MeParams(8, oracle.lambda_factor(32), 1, 2, 0, 0)
    planes = (ctypes.c_void_p * 16)(*([1] * 16))
    lib.xavs2gpu_set_abort_on_error(0)
    try:
        rc = f(ctypes.c_void_p(1), 400, 128, 64, planes, 1, ctypes.c_void_p(1), 65537, ctypes.byref(prm),
               ctypes.c_void_p(1), None)
        assert rc == 5   # XAVS2GPU_ERR_CAPACITY, nothing launched
        assert b"65536" in lib.xavs2gpu_get_error()
    finally:
        lib.xavs2gpu_clear_error()
        lib.xavs2gpu_set_abort_on_error(1)


def test_noalloc_invalid_pus_report_no_candidate(gpu):
    """PUs the entry cannot search (outside the picture, shape or reference
    index out of range, limits beyond the plane margin) come back with
    bcost = 1 << 30 and leave the valid PUs' results unchanged."""
    import torch
    import xavs2_gb300 as xg
    lib = xg.load()
    rng = np.random.default_rng(77)
    w, h = 128, 96
    cur = rng.integers(0, 256, (h, w), dtype=np.uint8)
    ref = np.clip(np.roll(cur, (2, -1), axis=(0, 1)).astype(np.int16) + rng.integers(-3, 4, (h, w)), 0, 255) \
        .astype(np.uint8)
    valid = xg.set_limits(xg.frame_pus(w, h, 1)[::5].copy(), w, h)
    prm = xg.MeParams(8, oracle.lambda_factor(32), 1, 2, 0, 0)
    sess = xg.MeSession(w, h, 1, len(valid))
    sess.set_picture(-1, cur)
    sess.set_picture(0, ref)
    sess.set_pus(valid)
    sess.run(prm)
    expected = sess.results()

    bad = np.repeat(valid[:1], 5)
    bad[0]["x"] = w - 4            # x + w beyond the picture (part 0 is 4x4: use a 16x16)
    bad[0]["part"] = 2
    bad[1]["ref"] = 1              # reference index >= num_refs
    bad[2]["part"] = 25            # no such shape
    bad[3]["max_x"] = w + 80       # limit reaching beyond the 80-pixel margin
    bad[4]["min_y"] = -200
    pus = np.concatenate([valid[:7], bad, valid[7:]])
    bad_idx = np.arange(7, 12)
    ok_idx = np.setdiff1d(np.arange(len(pus)), bad_idx)

    planes = (ctypes.c_void_p * 16)(*[sess.plane_ptr(0, k) for k in range(16)])
    d_pus = torch.from_numpy(pus.view(np.uint8).copy()).cuda()
    f = _noalloc(lib)
    for call in range(2):
        d_out = torch.full((len(pus) * xg.RESULT_DTYPE.itemsize,), 0x5A, dtype=torch.uint8, device="cuda")
        rc = f(sess.plane_ptr(-1, 0), sess.plane_stride(), w, h, planes, 1, d_pus.data_ptr(), len(pus),
               ctypes.byref(prm), d_out.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        got = d_out.cpu().numpy().view(xg.RESULT_DTYPE)
        assert (got["bcost"][bad_idx] == 1 << 30).all(), "call %d: %s" % (call, got["bcost"][bad_idx])
        assert got[ok_idx].tobytes() == expected.tobytes(), "call %d: valid PUs differ" % call
    sess.close()

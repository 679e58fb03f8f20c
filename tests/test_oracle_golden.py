"""The oracle against the golden fixtures recorded from the reference's own C
primitives (tests/golden/make_golden.py).  Runs on CPU everywhere, including
machines without the reference tree."""
import ctypes
import hashlib
import os

import numpy as np
import pytest

import oracle
from oracle import PU_W, PU_H, TU_PARTS, ptr

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz")


@pytest.fixture(scope="module")
def g():
    return dict(np.load(GOLDEN))


def test_costs(olib, g):
    a, b = g["cost_a"], g["cost_b"]
    fns = [olib.xo_sad, olib.xo_satd, olib.xo_sa8d, olib.xo_ssd]
    for i in range(4):
        for kind in range(4):
            got = [fns[kind](p, ptr(a[i]), 72, ptr(b[i]), 80) for p in range(25)]
            assert got == list(g["costs"][i, kind]), (i, kind)
    for part in range(25):
        res = (ctypes.c_int32 * 4)()
        olib.xo_sad_x4(part, ptr(a[0]), ptr(b[0], 0), ptr(b[0], 1), ptr(b[0], 81), ptr(b[0], 163), 80, res)
        assert list(res) == list(g["sad_x4"][part])


def test_block_ops(olib, g):
    a, b, s = g["cost_a"][0], g["cost_b"][0], g["ops_s"]
    for part in range(25):
        avg = np.zeros((64, 64), np.uint8); sub = np.zeros((64, 64), np.int16); add = avg.copy()
        olib.xo_avg(part, ptr(avg), 64, ptr(a), 72, ptr(b), 80)
        olib.xo_sub_ps(part, ptr(sub), 64, ptr(a), ptr(b), 72, 80)
        olib.xo_add_ps(part, ptr(add), 64, ptr(a), ptr(s), 72, 64)
        assert np.array_equal(avg, g["avg"][part])
        assert np.array_equal(sub, g["sub_ps"][part])
        assert np.array_equal(add, g["add_ps"][part])


def test_interpolation(olib, g):
    planes = oracle.interpolate_frame(olib, g["intp_img"], mode=2, ref=False)
    for k in range(1, 16):
        assert hashlib.sha256(planes[k].tobytes()).hexdigest() == str(g["intp_sha"][k]), k
    assert np.array_equal(planes[:, 80:152, 80:216], g["intp_center"])


def test_transforms(olib, g):
    for part in TU_PARTS:
        w, h = PU_W[part], PU_H[part]
        wav = w == 64 or h == 64
        n = (w // 2) * (h // 2) if wav else w * h
        res = np.ascontiguousarray(g["dct_in_%d" % part])
        out = np.zeros(64 * 64, np.int16)
        olib.xo_dct(part, ptr(res), ptr(out), w)
        assert np.array_equal(out[:n], g["dct_out_%d" % part]), part
        cbuf = np.zeros(64 * 64, np.int16); cbuf[:n] = g["idct_in_%d" % part]
        rec = np.zeros(64 * 64, np.int16)
        olib.xo_idct(part, ptr(cbuf), ptr(rec), w)
        assert np.array_equal(rec[:w * h], g["idct_out_%d" % part]), part
    t = g["sec_in"].copy(); olib.xo_transform_4x4_2nd(ptr(t), 4)
    assert np.array_equal(t, g["sec_fwd"])
    t = g["sec_in"].copy(); olib.xo_inv_transform_4x4_2nd(ptr(t), 4)
    assert np.array_equal(t, g["sec_inv"])


def test_quant(olib, g):
    for i, qp in enumerate(g["q_qps"]):
        c = g["q_in"][i].copy()
        shift = 17
        nz = olib.xo_quant(ptr(c), 1024, olib.xo_q_scale(int(qp)), shift, olib.xo_quant_fwd_add(shift, 0))
        assert nz == g["q_nz"][i] and np.array_equal(c, g["q_out"][i])
        olib.xo_dequant(ptr(c), 1024, olib.xo_iq_scale(int(qp)), olib.xo_iq_shift(int(qp)) + 9 + 5 - 16)
        assert np.array_equal(c, g["dq_out"][i])


def test_motion_search(olib, g):
    cur, refimg = g["me_cur"], g["me_ref"]
    h, w = cur.shape
    planes = oracle.interpolate_frame(olib, refimg, mode=2, ref=False)
    flat = np.ascontiguousarray(planes.reshape(16, -1))
    stride = w + 160
    off = 80 * stride + 80
    frefs = (ctypes.c_void_p * 16)(*[ptr(flat[k], off).value for k in range(16)])
    prm = oracle.MeParams(*[int(v) for v in g["me_params"]])
    pus = np.ascontiguousarray(g["me_pus"])
    out = np.zeros(len(pus), oracle.RESULT_DTYPE)
    olib.xo_me_search_list(ctypes.byref(prm), ptr(pus), len(pus), ptr(cur), w, frefs, stride, ptr(out), 1)
    assert np.array_equal(out, g["me_out"])


def _intra_golden():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_intra_prediction(olib, g):
    """Every intra mode on every block shape, three edge sets, DC with all
    four availabilities, destination pre-filled (the reference's mode 31 on
    16x64 leaves columns 4..15 alone)."""
    mg = _intra_golden()
    for e, edge in enumerate(g["intra_edges"]):
        edge = np.ascontiguousarray(edge)
        for s, (bw, bh) in enumerate(mg.INTRA_SHAPES):
            for m in range(36):
                mode, avail = (0, mg.INTRA_DC_AVAIL[m - 33]) if m >= 33 else (m, mg.INTRA_DC_AVAIL[3])
                dst = mg.intra_prefill(bw, bh)
                olib.xo_intra_pred(mode, ptr(edge, 256), ptr(dst), bw + 8, avail, bw, bh)
                assert hashlib.sha256(dst.tobytes()).hexdigest() == g["intra_sha"][e, s, m], (e, bw, bh, m)


def test_deblock_lcu_order_equals_two_passes(olib):
    """The picture deblocked in the reference's LCU order equals all vertical
    edges then all horizontal edges (edges 8 samples apart, each reading 3
    and writing at most 3 samples on either side), for LCU sizes 16..64."""
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(93)
    for (w, h, lcu) in ((128, 96, 6), (136, 72, 5), (64, 48, 4), (200, 120, 6), (64, 48, 6), (56, 40, 6),
                        (32, 64, 5)):
        y, u, v, scus = synth.deblock_picture(rng, w, h)
        outs = []
        for lcu_order in (1, 0):
            yy, uu, vv = y.copy(), u.copy(), v.copy()
            olib.xo_deblock_picture(ptr(yy), w, ptr(uu), ptr(vv), w // 2, w, h, ptr(scus), lcu, lcu_order)
            outs.append((yy, uu, vv))
        for a, b in zip(*outs):
            assert np.array_equal(a, b), (w, h, lcu)
        assert not np.array_equal(outs[0][0], y)      # something was filtered


def test_intra_fill_edges(olib, g):
    """Edge filling of a block inside a picture, every availability mask,
    against digests of the reference's fill_reference_samples; the batch
    entry writes the same samples and repeats each run's last one out to
    the RMD window."""
    import xavs2_gb300 as xg
    mg = _intra_golden()
    pic = mg.intra_fill_picture()
    for s, (bw, bh) in enumerate(mg.INTRA_SHAPES):
        def fill(p, buf, avail):
            olib.xo_intra_fill_edge(ptr(p), 272, 72, 72, bw, bh, avail, ptr(buf, 512))
        win = mg.intra_fill_windows(fill, bw, bh)
        assert hashlib.sha256(win.tobytes()).hexdigest() == g["intra_fill_sha"][s], (bw, bh)
        lo, hi = bh + (11 * bw) // 4 + 6, bw + (11 * bh) // 4 + 6
        jobs = np.zeros(32, xg.INTRA_EDGE_JOB_DTYPE)
        jobs["edge_offset"] = 512 + 1024 * np.arange(32)
        jobs["x"], jobs["y"], jobs["width"], jobs["height"], jobs["avail"] = 72, 72, bw, bh, np.arange(32)
        edges = np.zeros(32 * 1024, np.uint8)
        olib.xo_intra_fill_edges(ptr(jobs), 32, ptr(pic), 272, 272, 272, ptr(edges), len(edges))
        rlo, rhi = lo - 2, hi - 2
        ref = win.reshape(32, rlo + rhi + 1)
        for a in range(32):
            ep = 512 + 1024 * a
            got = edges[ep - lo:ep + hi + 1]
            assert np.array_equal(got[2:-2], ref[a]), (bw, bh, a)
            hi_ref = 2 * bw + max(bh * 11 // 4 - bw + 4, 0)
            lo_ref = 2 * bh + max(bw * 11 // 4 - bh + 4, 0)
            if hi > hi_ref:
                assert (edges[ep + hi_ref:ep + hi + 1] == edges[ep + hi_ref]).all()
            if lo > lo_ref:
                assert (edges[ep - lo:ep - lo_ref + 1] == edges[ep - lo_ref]).all()

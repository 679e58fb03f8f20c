"""Pins the oracle restatement against the reference's own C primitives
(oracle/_ref, compiled from the xavs2 sources).  Runs on CPU; skipped where
the reference tree is absent."""
import ctypes

import numpy as np
import pytest

import oracle
from oracle import PU_W, PU_H, TU_PARTS, ptr

pytestmark = pytest.mark.filterwarnings("ignore")


def _blocks(rng, n, stride_extra=(0, 7, 33)):
    """Seeded pixel pairs plus adversarial patterns (flat 0/255, checkerboard,
    random +-255 signs) that push the Hadamard sums to their extremes."""
    out = []
    for i in range(n):
        s1 = 64 + stride_extra[i % len(stride_extra)]
        s2 = 64 + stride_extra[(i + 1) % len(stride_extra)]
        a = rng.integers(0, 256, (64, s1), dtype=np.uint8)
        b = rng.integers(0, 256, (64, s2), dtype=np.uint8)
        mode = i % 5
        if mode == 1:
            a[:] = 255
            b[:] = 0
        elif mode == 2:
            a[:] = np.where((np.indices(a.shape).sum(0) % 2) == 0, 255, 0)
            b[:] = 255 - a[:, :s2] if s2 <= s1 else 0
        elif mode == 3:
            sgn = rng.integers(0, 2, (64, max(s1, s2)))
            a[:] = np.where(sgn[:, :s1] == 1, 255, 0)
            b[:] = np.where(sgn[:, :s2] == 1, 0, 255)
        out.append((np.ascontiguousarray(a), s1, np.ascontiguousarray(b), s2))
    return out


@pytest.mark.parametrize("kind,name", [(0, "xo_sad"), (1, "xo_satd"), (2, "xo_sa8d"), (3, "xo_ssd")])
def test_block_costs(olib, rlib, kind, name):
    rng = np.random.default_rng(100 + kind)
    fn = getattr(olib, name)
    for a, s1, b, s2 in _blocks(rng, 12):
        for part in range(25):
            r = rlib.xr_cmp(kind, part, ptr(a), s1, ptr(b), s2)
            o = fn(part, ptr(a), s1, ptr(b), s2)
            assert r == o, (name, part, r, o)


def test_sad_x3_x4(olib, rlib):
    rng = np.random.default_rng(7)
    fenc = rng.integers(0, 256, (64, 64), dtype=np.uint8)
    ref = rng.integers(0, 256, (80, 100), dtype=np.uint8)
    for part in range(25):
        ptrs = [ptr(ref, o) for o in (0, 3, 105, 1001)]
        r3 = (ctypes.c_int * 3)(); o3 = (ctypes.c_int32 * 3)()
        rlib.xr_sad_x3(part, ptr(fenc), *ptrs[:3], 100, r3)
        olib.xo_sad_x3(part, ptr(fenc), *ptrs[:3], ctypes.c_ssize_t(100), o3)
        assert list(r3) == list(o3)
        r4 = (ctypes.c_int * 4)(); o4 = (ctypes.c_int32 * 4)()
        rlib.xr_sad_x4(part, ptr(fenc), *ptrs, 100, r4)
        olib.xo_sad_x4(part, ptr(fenc), *ptrs, ctypes.c_ssize_t(100), o4)
        assert list(r4) == list(o4)


def test_block_ops(olib, rlib):
    rng = np.random.default_rng(11)
    for part in range(25):
        w, h = PU_W[part], PU_H[part]
        a = rng.integers(0, 256, (64, 70), dtype=np.uint8)
        b = rng.integers(0, 256, (64, 66), dtype=np.uint8)
        s = rng.integers(-600, 600, (64, 72), dtype=np.int16)
        # avg
        d1 = np.zeros((64, 68), np.uint8); d2 = d1.copy()
        rlib.xr_avg(part, ptr(d1), 68, ptr(a), 70, ptr(b), 66)
        olib.xo_avg(part, ptr(d2), 68, ptr(a), 70, ptr(b), 66)
        assert np.array_equal(d1, d2)
        # sub_ps
        e1 = np.zeros((64, 64), np.int16); e2 = e1.copy()
        rlib.xr_sub_ps(part, ptr(e1), 64, ptr(a), ptr(b), 70, 66)
        olib.xo_sub_ps(part, ptr(e2), 64, ptr(a), ptr(b), 70, 66)
        assert np.array_equal(e1, e2)
        # add_ps
        d1[:] = 0; d2[:] = 0
        rlib.xr_add_ps(part, ptr(d1), 68, ptr(a), ptr(s), 70, 72)
        olib.xo_add_ps(part, ptr(d2), 68, ptr(a), ptr(s), 70, 72)
        assert np.array_equal(d1, d2)
        # copies
        for kind, (dt_d, src) in enumerate([(np.uint8, a), (np.int16, a), (np.uint8, np.abs(s) % 256), (np.int16, s)]):
            src = np.ascontiguousarray(src.astype(np.int16) if kind >= 2 else src)
            x1 = np.zeros((64, 80), dt_d); x2 = x1.copy()
            ss = src.shape[1]
            rlib.xr_copy(kind, part, ptr(x1), 80, ptr(src), ss)
            fn = [olib.xo_copy_pp, olib.xo_copy_ps, olib.xo_copy_sp, olib.xo_copy_ss][kind]
            fn(part, ptr(x2), 80, ptr(src), ss)
            assert np.array_equal(x1, x2), kind
        # ssd_block / average on the PU size
        assert rlib.xr_ssd_block(ptr(a), 70, ptr(b), 66, w, h) == olib.xo_ssd_block(ptr(a), 70, ptr(b), 66, w, h)
        d1[:] = 0; d2[:] = 0
        rlib.xr_average(ptr(d1), 68, ptr(a), 70, ptr(b), 66, w, h)
        olib.xo_average(ptr(d2), 68, ptr(a), 70, ptr(b), 66, w, h)
        assert np.array_equal(d1, d2)
    for size in (16, 32, 64):
        a = rng.integers(0, 256, (64, 90), dtype=np.uint8)
        assert rlib.xr_mad(ptr(a), 90, size) == olib.xo_mad(ptr(a), 90, size)


def test_interp_primitives(olib, rlib):
    rng = np.random.default_rng(21)
    src = rng.integers(0, 256, (96, 120), dtype=np.uint8)
    src[10:20] = 255
    src[30:40, :] = 0
    o = 8 * 120 + 8          # room for the taps
    w, h = 64, 48
    for frac in range(1, 4):
        c = olib.xo_luma_filter(frac)
        d1 = np.zeros((h, 100), np.uint8); d2 = d1.copy()
        t1 = np.zeros((h, 100), np.int16); t2 = t1.copy()
        rlib.xr_intpl_luma_hor(ptr(d1), 100, ptr(t1), 100, ptr(src, o), 120, w, h, c)
        olib.xo_intpl_luma_hor(ptr(d2), 100, ptr(t2), 100, ptr(src, o), 120, w, h, c)
        assert np.array_equal(d1, d2) and np.array_equal(t1, t2)
        d1[:] = 0; d2[:] = 0
        rlib.xr_intpl_luma_ver(ptr(d1), 100, ptr(src, o), 120, w, h, c)
        olib.xo_intpl_luma_ver(ptr(d2), 100, ptr(src, o), 120, w, h, c)
        assert np.array_equal(d1, d2)
        tmp = rng.integers(-6000, 22000, (64, 100), dtype=np.int16)
        d1[:] = 0; d2[:] = 0
        rlib.xr_intpl_luma_ext(ptr(d1), 100, ptr(tmp, 4 * 100), 100, w, h - 8, c)
        olib.xo_intpl_luma_ext(ptr(d2), 100, ptr(tmp, 4 * 100), 100, w, h - 8, c)
        assert np.array_equal(d1, d2)
    for fx in range(4):
        for fy in range(4):
            cx, cy = olib.xo_luma_filter(fx), olib.xo_luma_filter(fy)
            for kind, fn in ((0, olib.xo_intpl_luma_block_hor), (1, olib.xo_intpl_luma_block_ver),
                             (2, olib.xo_intpl_luma_block_ext)):
                for (bw, bh) in ((64, 64), (16, 12), (8, 4)):
                    d1 = np.zeros((64, 64), np.uint8); d2 = d1.copy()
                    rlib.xr_intpl_block(kind, ptr(d1), 64, ptr(src, o), 120, bw, bh, cx, cy)
                    if kind == 2:
                        fn(ptr(d2), 64, ptr(src, o), 120, bw, bh, cx, cy)
                    else:
                        fn(ptr(d2), 64, ptr(src, o), 120, bw, bh, cx if kind == 0 else cy)
                    assert np.array_equal(d1, d2), (kind, fx, fy, bw, bh)
    for fx in range(8):
        for fy in range(8):
            cx, cy = olib.xo_chroma_filter(fx), olib.xo_chroma_filter(fy)
            for kind, fn in ((3, olib.xo_intpl_chroma_block_hor), (4, olib.xo_intpl_chroma_block_ver),
                             (5, olib.xo_intpl_chroma_block_ext)):
                for (bw, bh) in ((32, 32), (8, 6), (2, 8)):
                    d1 = np.zeros((32, 32), np.uint8); d2 = d1.copy()
                    rlib.xr_intpl_block(kind, ptr(d1), 32, ptr(src, o), 120, bw, bh, cx, cy)
                    if kind == 5:
                        fn(ptr(d2), 32, ptr(src, o), 120, bw, bh, cx, cy)
                    else:
                        fn(ptr(d2), 32, ptr(src, o), 120, bw, bh, cx if kind == 3 else cy)
                    assert np.array_equal(d1, d2), (kind, fx, fy, bw, bh)


@pytest.mark.parametrize("w,h,lcu,mode", [(128, 72, 6, 2), (96, 64, 5, 2), (72, 40, 6, 1), (200, 136, 6, 2)])
def test_frame_interpolation(olib, rlib, w, h, lcu, mode):
    rng = np.random.default_rng(w * h)
    img = rng.integers(0, 256, (h, w), dtype=np.uint8)
    img[: h // 3, : w // 4] = 255
    a = oracle.interpolate_frame(rlib, img, mode=mode, ref=True, lcu_level=lcu)
    b = oracle.interpolate_frame(olib, img, mode=mode, ref=False)
    planes = range(1, 16) if mode == 2 else (2, 8, 10)
    for k in planes:
        assert np.array_equal(a[k], b[k]), k


def _residual(rng, w, h, kind):
    if kind == 0:
        return np.clip(np.round(rng.laplace(0, 12, (h, w))), -255, 255).astype(np.int16)
    if kind == 1:
        return rng.integers(-255, 256, (h, w)).astype(np.int16)
    if kind == 2:
        return np.where(rng.integers(0, 2, (h, w)) == 1, 255, -255).astype(np.int16)
    return rng.integers(-32768, 32768, (h, w)).astype(np.int16)   # far outside the residual range


@pytest.mark.parametrize("part", TU_PARTS)
def test_dct_idct(olib, rlib, part):
    w, h = PU_W[part], PU_H[part]
    rng = np.random.default_rng(part)
    wavelet = w == 64 or h == 64
    for kind in range(4):
        for flag in ((0, 1) if part in (3, 19, 20) else (0,)):
            res = _residual(rng, w, h, kind)
            stride = w if wavelet else w
            src = np.zeros((h, stride + 8), np.int16)
            src[:, :w] = res
            src_c = np.ascontiguousarray(src) if not wavelet else np.ascontiguousarray(res)
            ss = (stride + 8 if not wavelet else w) | flag
            d1 = np.zeros(64 * 64, np.int16); d2 = d1.copy()
            rlib.xr_dct(0, part, ptr(src_c), ptr(d1), ss)
            olib.xo_dct(part, ptr(src_c), ptr(d2), ss)
            # the 64-point transforms output (w/2)x(h/2) coefficients; the
            # reference leaves wavelet scratch in the rest of its buffer
            ncoef = (w // 2) * (h // 2) if wavelet else w * h
            assert np.array_equal(d1[:ncoef], d2[:ncoef]), ("dct", part, kind, flag)
            if part in (3, 4):
                d1[:] = 0; d2[:] = 0
                rlib.xr_dct(2, part, ptr(src_c), ptr(d1), ss)
                olib.xo_dct_half(part, ptr(src_c), ptr(d2), ss)
                assert np.array_equal(d1[:1024], d2[:1024]), ("dct_half", part, kind)
            # inverse on random coefficients
            n = (w // 2) * (h // 2) if wavelet else w * h
            coef = np.zeros(64 * 64, np.int16)
            coef[:n] = _residual(rng, n, 1, kind).reshape(-1) * (4 if kind < 2 else 1)
            o1 = np.zeros(64 * 72, np.int16); o2 = o1.copy()
            ds = (w + 8 if not wavelet else w) | flag
            rlib.xr_dct(1, part, ptr(coef), ptr(o1), ds)
            olib.xo_idct(part, ptr(coef), ptr(o2), ds)
            assert np.array_equal(o1, o2), ("idct", part, kind, flag)


def test_secondary_transforms(olib, rlib):
    rng = np.random.default_rng(5)
    for trial in range(60):
        blk = rng.integers(-2000, 2000, (8, 12)).astype(np.int16)
        if trial % 4 == 3:
            blk = rng.integers(-32768, 32768, (8, 12)).astype(np.int16)
        mode, top, left = int(rng.integers(0, 33)), int(rng.integers(0, 2)), int(rng.integers(0, 2))
        for kind, fn in enumerate([olib.xo_transform_4x4_2nd, olib.xo_inv_transform_4x4_2nd,
                                   olib.xo_transform_2nd, olib.xo_inv_transform_2nd]):
            a = blk.copy(); b = blk.copy()
            rlib.xr_2nd(kind, ptr(a), 12, mode, top, left)
            if kind < 2:
                fn(ptr(b), 12)
            else:
                fn(ptr(b), 12, mode, top, left)
            assert np.array_equal(a, b), (kind, mode, top, left)


def test_quant_family(olib, rlib):
    rng = np.random.default_rng(9)
    for qp in range(0, 80, 3):
        assert rlib.xr_q_scale(qp) == olib.xo_q_scale(qp)
        assert rlib.xr_iq_scale(qp) == olib.xo_iq_scale(qp)
        assert rlib.xr_iq_shift(qp) == olib.xo_iq_shift(qp)
    for qp in range(0, 64):
        assert rlib.xr_iq_shift(qp) == olib.xo_iq_shift(qp)
        for level in range(2, 7):
            for intra in (0, 1):
                n = 1 << (2 * level) if level < 6 else 1024
                c = rng.integers(-32768, 32768, n).astype(np.int16)
                c[rng.random(n) < 0.3] = 0
                shift = 22 - level
                add = olib.xo_quant_fwd_add(shift, intra)
                a = c.copy(); b = c.copy()
                assert rlib.xr_quant(ptr(a), n, rlib.xr_q_scale(qp), shift, add) == \
                    olib.xo_quant(ptr(b), n, olib.xo_q_scale(qp), shift, add)
                assert np.array_equal(a, b)
                dshift = olib.xo_iq_shift(qp) + 9 + level - 16
                a2 = a.copy(); b2 = a.copy()
                rlib.xr_dequant(ptr(a2), n, rlib.xr_iq_scale(qp), dshift)
                olib.xo_dequant(ptr(b2), n, olib.xo_iq_scale(qp), dshift)
                assert np.array_equal(a2, b2)
    for n in (16, 64, 1024):
        c = rng.integers(-32768, 32768, n).astype(np.int16)
        a = np.zeros(n, np.int16); b = a.copy()
        rlib.xr_abs_coeff(ptr(a), ptr(c), n)
        olib.xo_abs_coeff(ptr(b), ptr(c), n)
        assert np.array_equal(a, b)
        d = rng.integers(-5, 5, n).astype(np.int16)
        a = d.copy(); b = d.copy()
        assert rlib.xr_add_sign(ptr(a), ptr(np.abs(c).astype(np.int16)), n) == \
            olib.xo_add_sign(ptr(b), ptr(np.abs(c).astype(np.int16)), n)
        assert np.array_equal(a, b)
        ls = rng.integers(1, 4096, n).astype(np.int32)
        a = c.copy(); b = c.copy()
        assert rlib.xr_wquant(ptr(a), n, 5000, 18, 1000, ptr(ls)) == \
            olib.xo_wquant(ptr(b), n, 5000, 18, 1000, ptr(ls))
        assert np.array_equal(a, b)


def test_mvbits(olib, rlib):
    for d in list(range(-300, 301)) + [1023, -1024, 4095, 16383, -16383]:
        assert rlib.xr_mvbits(d) == olib.xo_mvbits(d)


def _me_setup(seed, w=96, h=64, pad=80):
    rng = np.random.default_rng(seed)
    cur = rng.integers(0, 256, (h, w), dtype=np.uint8)
    # reference: the current picture moved by a few pixels plus noise
    refimg = np.roll(cur, (3, -5), axis=(0, 1)).astype(np.int16) + rng.integers(-6, 7, (h, w))
    refimg = np.clip(refimg, 0, 255).astype(np.uint8)
    return rng, cur, refimg


@pytest.mark.parametrize("hadamard,frac,fast,pmvr", [(1, 2, 0, 0), (0, 1, 0, 0), (1, 2, 1, 0), (1, 2, 0, 1), (0, 0, 0, 0), (0, 2, 0, 0)])
def test_me_search(olib, rlib, hadamard, frac, fast, pmvr):
    rng, cur, refimg = _me_setup(31 + 7 * frac + hadamard)
    h, w = cur.shape
    planes_r = oracle.interpolate_frame(rlib, refimg, mode=2, ref=True)
    pad = 80
    stride = w + 2 * pad
    flat = np.ascontiguousarray(planes_r.reshape(16, -1))
    off = pad * stride + pad
    frefs = (ctypes.c_void_p * 16)(*[ptr(flat[k], off).value for k in range(16)])
    prm = oracle.MeParams(12, oracle.lambda_factor(32), hadamard, frac, fast, pmvr)
    n = 0
    for part in range(25):
        pw, ph = PU_W[part], PU_H[part]
        for t in range(3):
            x = int(rng.integers(0, w - pw + 1)) // 4 * 4
            y = int(rng.integers(0, h - ph + 1)) // 4 * 4
            pu = oracle.Pu(x, y, part, 0, int(rng.integers(-40, 41)), int(rng.integers(-40, 41)))
            olib.xo_pu_set_limits(ctypes.byref(pu), w, h, -2048, 2047)
            r1 = oracle.MeResult(); r2 = oracle.MeResult()
            cr = rlib.xr_me_search(ctypes.byref(prm), ctypes.byref(pu), ptr(cur, y * w + x), w, frefs, stride, ctypes.byref(r1))
            co = olib.xo_me_search(ctypes.byref(prm), ctypes.byref(pu), ptr(cur, y * w + x), ctypes.c_ssize_t(w), frefs, ctypes.c_ssize_t(stride), ctypes.byref(r2))
            got = [getattr(r2, f) for f, _ in oracle.MeResult._fields_]
            exp = [getattr(r1, f) for f, _ in oracle.MeResult._fields_]
            assert cr == co and got == exp, (part, x, y, exp, got)
            n += 1
    assert n == 75


INTRA_SHAPES = [(4, 4), (8, 8), (16, 16), (32, 32), (64, 64), (4, 16), (16, 4), (8, 32), (32, 8), (16, 64), (64, 16)]


def test_intra_prediction(olib, rlib):
    """xo_intra_pred against the reference's intraf[] table on seeded edges,
    with edge buffers built by the reference's own fill_edge_f for random
    neighbour availabilities as well as plain random edges."""
    rng = np.random.default_rng(77)
    edges = []
    for i in range(6):
        edges.append(rng.integers(0, 256, 512).astype(np.uint8))
    for i in range(6):
        t = np.arange(512)
        edges.append(np.clip(120 + 90 * np.sin(t / (5.0 + 7 * i)) + rng.integers(-9, 10, 512), 0, 255).astype(np.uint8))
    for edge in edges:
        for bw, bh in INTRA_SHAPES:
            for mode in range(33):
                for avail in ((0x000, 0x001, 0x100, 0x101) if mode == 0 else (mode,)):
                    fill = rng.integers(0, 256, (bh, bw + 5), dtype=np.uint8)
                    a, b = fill.copy(), fill.copy()
                    olib.xo_intra_pred(mode, ptr(edge, 256), ptr(a), bw + 5, avail, bw, bh)
                    rlib.xr_intra_pred(mode, ptr(edge, 256), ptr(b), bw + 5, avail, bw, bh)
                    assert np.array_equal(a, b), (bw, bh, mode, avail)


def test_intra_fill_edge_prediction(olib, rlib):
    """Edges as the encoder builds them (fill_edge_f, every availability
    combination of left / top / top-right / left-down / top-left), then
    every mode through both."""
    rng = np.random.default_rng(78)
    pic = rng.integers(0, 256, (320, 320), dtype=np.uint8)
    pic = np.ascontiguousarray((pic.astype(np.int32) + np.roll(pic, 1, 0) + np.roll(pic, 1, 1)) // 3).astype(np.uint8)
    lcu_ep = rng.integers(0, 256, 512).astype(np.uint8)
    for bw, bh in [(8, 8), (16, 16), (32, 8), (4, 16), (64, 64)]:
        for avail in range(32):
            for xy in range(4):
                ebuf = np.zeros(1024, np.uint8)
                rlib.xr_intra_fill_edge(xy, ptr(pic, 40 * 320 + 40), 320, ptr(lcu_ep, 200), ptr(ebuf, 512),
                                        avail, bw, bh)
                for mode in range(33):
                    a = np.zeros((bh, bw), np.uint8)
                    b = np.zeros((bh, bw), np.uint8)
                    olib.xo_intra_pred(mode, ptr(ebuf, 512), ptr(a), bw, 0x101, bw, bh)
                    rlib.xr_intra_pred(mode, ptr(ebuf, 512), ptr(b), bw, 0x101 if mode == 0 else mode, bw, bh)
                    assert np.array_equal(a, b), (bw, bh, avail, xy, mode)


ALPHA_TAB_SAMPLES = [(2, 1), (6, 2), (13, 3), (24, 5), (36, 8), (50, 15), (64, 27), (0, 0), (255, 255)]


def _deblock_area(rng, n):
    """n 16x16 areas (a vertical and a horizontal edge through the centre)
    with flat or ramped sides, a step of random size and small noise, so that
    every filter strength occurs."""
    out = []
    for i in range(n):
        base = int(rng.integers(20, 230))
        a = np.full((16, 16), base, np.int32)
        kind = i % 4
        if kind == 1:
            a += np.arange(16)[None, :] * int(rng.integers(-3, 4))
        elif kind == 2:
            a += rng.integers(-2, 3, (16, 16))
        elif kind == 3:
            a += rng.integers(-12, 13, (16, 16))
        step = int(rng.integers(-30, 31))
        a[:, 8:] += step
        a[8:, :] += int(rng.integers(-30, 31))
        if i % 7 == 0:
            a[:, 7] = a[:, 6]          # L0 == L1 / R0 == R1 patterns
            a[:, 8] = a[:, 9]
        out.append(np.clip(a, 0, 255).astype(np.uint8))
    return out


def test_deblock_edges(olib, rlib):
    rng = np.random.default_rng(91)
    for area in _deblock_area(rng, 160):
        for alpha, beta in ALPHA_TAB_SAMPLES:
            for flags in ((1, 1), (1, 0), (0, 1)):
                fl = np.array(flags, np.uint8)
                for d in (0, 1):
                    a, b = area.copy(), area.copy()
                    olib.xo_deblock_luma(d, ptr(a, 4 * 16 + 8 if d == 0 else 8 * 16 + 4), 16, alpha, beta, ptr(fl))
                    rlib.xr_deblock_luma(d, ptr(b, 4 * 16 + 8 if d == 0 else 8 * 16 + 4), 16, alpha, beta, ptr(fl))
                    assert np.array_equal(a, b), (d, alpha, beta, flags)
                    u1, v1 = area.copy(), area[::-1].copy()
                    u2, v2 = u1.copy(), v1.copy()
                    o = 4 * 16 + 8 if d == 0 else 8 * 16 + 4
                    olib.xo_deblock_chroma(d, ptr(u1, o), ptr(v1, o), 16, alpha, beta, ptr(fl))
                    rlib.xr_deblock_chroma(d, ptr(u2, o), ptr(v2, o), 16, alpha, beta, ptr(fl))
                    assert np.array_equal(u1, u2) and np.array_equal(v1, v2), (d, alpha, beta, flags)


def test_sao_block(olib, rlib):
    """Every SAO type over every combination of the four side
    availabilities (diagonals are the conjunctions, as the encoder derives
    them), several block sizes, random offsets."""
    rng = np.random.default_rng(92)
    for trial in range(6):
        img = rng.integers(0, 256, (80, 96), dtype=np.uint8)
        if trial % 2:
            img = np.clip(128 + np.cumsum(rng.integers(-3, 4, (80, 96)), 1), 0, 255).astype(np.uint8)
        for w, h in ((64, 64), (68, 60), (60, 68), (8, 8), (36, 4), (4, 36)):
            for sides in range(16):
                T, D, L, R = sides & 1, (sides >> 1) & 1, (sides >> 2) & 1, (sides >> 3) & 1
                avail = np.array([T, D, L, R, T & L, T & R, D & L, D & R], np.int32)
                for typ in range(5):
                    prm = np.zeros(36, np.int32)
                    prm[1] = typ
                    prm[4:] = rng.integers(-7, 8, 32)
                    dst1 = rng.integers(0, 256, (80, 96), dtype=np.uint8)
                    dst2 = dst1.copy()
                    o = 6 * 96 + 8
                    olib.xo_sao_block(ptr(dst1, o), 96, ptr(img, o), 96, w, h, ptr(avail), ptr(prm))
                    rlib.xr_sao_block(ptr(dst2, o), 96, ptr(img, o), 96, w, h, ptr(avail), ptr(prm))
                    assert np.array_equal(dst1, dst2), (trial, w, h, sides, typ)


def test_lowres_filter(olib, rlib):
    rng = np.random.default_rng(94)
    for w, h in ((32, 18), (7, 5), (64, 64), (1, 1)):
        src = rng.integers(0, 256, (2 * h + 3, 2 * w + 5), dtype=np.uint8)
        a = np.zeros((h, w + 3), np.uint8)
        b = a.copy()
        olib.xo_lowres_filter(ptr(src), src.shape[1], ptr(a), w + 3, w, h)
        rlib.xr_lowres_filter(ptr(src), src.shape[1], ptr(b), w + 3, w, h)
        assert np.array_equal(a, b), (w, h)


def test_intra_fill_edge_restated(olib, rlib):
    """xo_intra_fill_edge against the reference's fill_edge_f: variant xy
    (block inside its CTU: neighbours from the reconstruction) and variant 0
    (block at the CTU's corner: neighbours from the border buffer, here
    built from the same picture), every availability mask, several shapes."""
    rng = np.random.default_rng(79)
    pic = rng.integers(0, 256, (320, 320), dtype=np.uint8)
    x0, y0 = 120, 96
    for bw, bh in INTRA_SHAPES:
        # border buffer of variant 0: [k] = top row (k >= 0, k = 0 the corner), [-j] = left column
        buf = np.zeros(1024, np.uint8)
        for k in range(0, 2 * bw + 1):
            buf[512 + k] = pic[y0 - 1, x0 - 1 + k]
        for j in range(1, 2 * bh + 1):
            buf[512 - j] = pic[y0 + j - 1, x0 - 1]
        for avail in range(32):
            want = np.zeros(1024, np.uint8)
            olib.xo_intra_fill_edge(ptr(pic), 320, x0, y0, bw, bh, avail, ptr(want, 512))
            lo, hi = 512 - (bh + (11 * bw) // 4 + 4), 512 + bw + (11 * bh) // 4 + 4
            for xy, ptl, lcu in ((3, ptr(pic, (y0 - 1) * 320 + x0 - 1), ptr(buf, 512)),
                                 (0, ptr(pic, (y0 - 1) * 320 + x0 - 1), ptr(buf, 512))):
                got = np.zeros(1024, np.uint8)
                rlib.xr_intra_fill_edge(xy, ptl, 320, lcu, ptr(got, 512), avail, bw, bh)
                assert np.array_equal(got[lo:hi + 1], want[lo:hi + 1]), (bw, bh, avail, xy)


def test_intra_neighbor_rule(rlib):
    """The synthetic availability (xavs2_gb300.synth.intra_neighbors: picture
    bounds plus the z-scan of 4x4 units) equals get_intra_neighbors' lookup
    in the reference's tab_TR_Avail / tab_DL_Avail tables (block_info.c),
    read from its source, for every block of every shape of a 256x192
    picture and every LCU size."""
    import os
    import re
    import xavs2_gb300.synth as synth
    path = os.path.join(oracle.REF_SRC, "common", "block_info.c")
    src = open(path, encoding="latin-1").read()

    def table(name, n):
        body = re.search(r"%s\[[^\]]*\] = \{(.*?)\};" % name, src, re.S).group(1)
        return np.array([int(v) for v in re.findall(r"\b[01]\b", re.sub(r"//.*", "", body))]).reshape(n, n)

    W, H = 256, 192
    for lcu in (16, 32, 64):
        n = lcu // 4
        tr, dl = table("tab_TR_Avail%d" % lcu, n), table("tab_DL_Avail%d" % lcu, n)
        rects = [(x, y, bw, bh) for bw, bh in synth.INTRA_ALL_SHAPES if bw <= lcu and bh <= lcu
                 for y in range(0, H - bh + 1, bh) for x in range(0, W - bw + 1, bw)]
        got = synth.intra_neighbors(rects, W, H, lcu)
        for (x, y, bw, bh), a in zip(rects, got):
            x4, y4 = x // 4, y // 4

            def inside(dx, dy):
                return 0 <= x4 + dx < W // 4 and 0 <= y4 + dy < H // 4
            ld = inside(-1, bh // 2 - 1) and dl[(y4 % n) + bh // 4 - 1][x4 % n]
            trr = inside(bw // 2 - 1, -1) and tr[y4 % n][(x4 % n) + bw // 4 - 1]
            want = int(inside(-1, 0)) | int(inside(0, -1)) << 1 | int(bool(ld)) << 2 | int(bool(trr)) << 3 \
                | int(inside(-1, -1)) << 4
            assert want == int(a), (lcu, x, y, bw, bh)

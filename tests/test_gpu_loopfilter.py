"""In-loop filters on the GPU: the deblocking and SAO drop-ins against the
oracle (which is pinned to the reference's filter_deblock.c / filter_sao.c),
and the picture-level forms against the oracle's picture functions (the
deblocking one in the reference's LCU order)."""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def test_deblock_table_init(gpu):
    table = (ctypes.c_void_p * 4)()
    gpu.xavs2gpu_deblock_init(0, table)
    addr = lambda name: ctypes.cast(getattr(gpu, name), ctypes.c_void_p).value
    assert list(table) == [addr("xavs2gpu_deblock_luma_ver"), addr("xavs2gpu_deblock_luma_hor"),
                           addr("xavs2gpu_deblock_chroma_ver"), addr("xavs2gpu_deblock_chroma_hor")]
    sao = (ctypes.c_void_p * 1)()
    gpu.xavs2gpu_sao_init(0, sao)
    assert sao[0] == addr("xavs2gpu_sao_block")


def test_deblock_dropins(gpu, olib):
    import xavs2_gb300 as xg
    rng = np.random.default_rng(95)
    import xavs2_gb300.synth as synth
    for trial in range(40):
        area = synth._blocky(rng, 16, 16, 12 + trial % 20)
        if trial % 5 == 0:
            area[:, 7] = area[:, 6]
            area[:, 8] = area[:, 9]
        alpha, beta = int(rng.integers(0, 70)), int(rng.integers(0, 30))
        fl = np.array(rng.integers(0, 2, 2), np.uint8)
        for d in (0, 1):
            o = 4 * 16 + 8 if d == 0 else 8 * 16 + 4
            a, b = area.copy(), area.copy()
            xg.fn("xavs2gpu_deblock_luma_" + ("ver" if d == 0 else "hor"))(xg.ptr(a, o), 16, alpha, beta, xg.ptr(fl))
            olib.xo_deblock_luma(d, oracle.ptr(b, o), 16, alpha, beta, oracle.ptr(fl))
            assert np.array_equal(a, b), (trial, d)
            u1, v1 = area.copy(), area[::-1].copy()
            u2, v2 = u1.copy(), v1.copy()
            xg.fn("xavs2gpu_deblock_chroma_" + ("ver" if d == 0 else "hor"))(xg.ptr(u1, o), xg.ptr(v1, o), 16,
                                                                           alpha, beta, xg.ptr(fl))
            olib.xo_deblock_chroma(d, oracle.ptr(u2, o), oracle.ptr(v2, o), 16, alpha, beta, oracle.ptr(fl))
            assert np.array_equal(u1, u2) and np.array_equal(v1, v2), (trial, d)


def test_sao_block_dropin(gpu, olib):
    import xavs2_gb300 as xg
    rng = np.random.default_rng(96)
    img = rng.integers(0, 256, (80, 96), dtype=np.uint8)
    img[40:] = np.clip(128 + np.cumsum(rng.integers(-3, 4, (40, 96)), 1), 0, 255)
    for w, h in ((64, 64), (68, 60), (8, 8), (36, 4)):
        for sides in (0, 5, 10, 15, 3, 12):
            T, D, L, R = sides & 1, (sides >> 1) & 1, (sides >> 2) & 1, (sides >> 3) & 1
            avail = np.array([T, D, L, R, T & L, T & R, D & L, D & R], np.int32)
            for typ in range(5):
                prm = np.zeros(36, np.int32)
                prm[1] = typ
                prm[4:] = rng.integers(-7, 8, 32)
                d1 = rng.integers(0, 256, (80, 96), dtype=np.uint8)
                d2 = d1.copy()
                o = 6 * 96 + 8
                xg.fn("xavs2gpu_sao_block")(xg.ptr(d1, o), 96, xg.ptr(img, o), 96, w, h, xg.ptr(avail), xg.ptr(prm))
                olib.xo_sao_block(oracle.ptr(d2, o), 96, oracle.ptr(img, o), 96, w, h, oracle.ptr(avail),
                                  oracle.ptr(prm))
                assert np.array_equal(d1, d2), (w, h, sides, typ)


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("w,h,lcu", [(128, 96, 6), (136, 72, 5), (200, 120, 6), (64, 48, 6), (56, 40, 6),
                                     (64, 48, 4), (1920, 1080, 6)])
def test_deblock_picture(gpu, olib, w, h, lcu):
    import torch
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(w * 7 + h)
    y, u, v, scus = synth.deblock_picture(rng, w, h)
    ey, eu, ev = y.copy(), u.copy(), v.copy()
    olib.xo_deblock_picture(oracle.ptr(ey), w, oracle.ptr(eu), oracle.ptr(ev), w // 2, w, h, oracle.ptr(scus), lcu,
                            1)
    dy, du, dv, ds = _dev(y), _dev(u), _dev(v), _dev(scus.view(np.uint8))
    rc = gpu.xavs2gpu_deblock_picture(ctypes.c_void_p(dy.data_ptr()), w, ctypes.c_void_p(du.data_ptr()),
                                      ctypes.c_void_p(dv.data_ptr()), w // 2, w, h, lcu,
                                      ctypes.c_void_p(ds.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    assert np.array_equal(dy.cpu().numpy(), ey)
    assert np.array_equal(du.cpu().numpy(), eu) and np.array_equal(dv.cpu().numpy(), ev)
    assert not np.array_equal(ey, y)


@pytest.mark.parametrize("w,h,lcu", [(128, 96, 6), (136, 72, 5), (200, 120, 6), (64, 48, 4), (1920, 1080, 6)])
def test_sao_picture(gpu, olib, w, h, lcu):
    import torch
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(w * 5 + h + lcu)
    y, u, v, _ = synth.deblock_picture(rng, w, h)
    lcus = synth.sao_params(rng, w, h, lcu)
    for fill in ("same", "random", "copy_rest"):
        if fill == "same":
            dst = [y.copy(), u.copy(), v.copy()]
        else:
            dst = [rng.integers(0, 256, p.shape, dtype=np.uint8) for p in (y, u, v)]
        # copy_rest: the expected picture is the reference's, whose dst held
        # the source before filtering
        exp = [p.copy() for p in ((y, u, v) if fill == "copy_rest" else dst)]
        src = [y, u, v]
        dptr = (ctypes.c_void_p * 3)(*[oracle.ptr(p).value for p in exp])
        sptr = (ctypes.c_void_p * 3)(*[oracle.ptr(p).value for p in src])
        olib.xo_sao_picture(dptr, sptr, w, w // 2, w, h, lcu, oracle.ptr(lcus))
        dd = [_dev(p) for p in dst]
        ds = [_dev(p) for p in src]
        dl = _dev(lcus.view(np.uint8))
        rc = gpu.xavs2gpu_sao_picture(*[ctypes.c_void_p(t.data_ptr()) for t in dd + ds], w, w // 2, w, h, lcu,
                                      ctypes.c_void_p(dl.data_ptr()), 1 if fill == "copy_rest" else 0, None)
        assert rc == 0
        torch.cuda.synchronize()
        for k in range(3):
            assert np.array_equal(dd[k].cpu().numpy(), exp[k]), (fill, k)


def test_loopfilter_bad_args(gpu):
    import xavs2_gb300 as xg
    lib = xg.load()
    lib.xavs2gpu_set_abort_on_error(0)
    try:
        assert lib.xavs2gpu_deblock_picture(None, 64, None, None, 32, 60, 48, 6, None, None) != 0
        assert lib.xavs2gpu_sao_picture(None, None, None, None, None, None, 64, 32, 64, 48, 7, None, 0, None) != 0
    finally:
        lib.xavs2gpu_clear_error()
        lib.xavs2gpu_set_abort_on_error(1)


def test_sao_picture_inconsistent_avail(gpu, olib):
    """Interior availability bits drawn at random (neighbouring LCUs
    disagree, so regions overlap or leave gaps): the later LCU in raster
    order wins where regions overlap, gaps keep dst, as in the reference's
    LCU loop.  Picture-border bits stay off, so no filtered sample has a
    neighbour outside the picture."""
    import torch
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(97)
    w, h, lcu = 256, 192, 5
    y, u, v, _ = synth.deblock_picture(rng, w, h)
    lcus = synth.sao_params(rng, w, h, lcu, p_off=0.0)
    wl, hl = w >> lcu, h >> lcu
    lx, ly = np.arange(wl * hl) % wl, np.arange(wl * hl) // wl
    bits = rng.integers(0, 16, wl * hl)
    border = (ly > 0) | ((ly < hl - 1) << 1) | ((lx > 0) << 2) | ((lx < wl - 1) << 3)
    lcus["avail"] = bits & border
    dst = [rng.integers(0, 256, p.shape, dtype=np.uint8) for p in (y, u, v)]
    exp = [p.copy() for p in dst]
    dptr = (ctypes.c_void_p * 3)(*[oracle.ptr(p).value for p in exp])
    sptr = (ctypes.c_void_p * 3)(*[oracle.ptr(p).value for p in (y, u, v)])
    olib.xo_sao_picture(dptr, sptr, w, w // 2, w, h, lcu, oracle.ptr(lcus))
    dd = [_dev(p) for p in dst]
    ds = [_dev(p) for p in (y, u, v)]
    dl = _dev(lcus.view(np.uint8))
    rc = gpu.xavs2gpu_sao_picture(*[ctypes.c_void_p(t.data_ptr()) for t in dd + ds], w, w // 2, w, h, lcu,
                                  ctypes.c_void_p(dl.data_ptr()), 0, None)
    assert rc == 0
    torch.cuda.synchronize()
    for k in range(3):
        assert np.array_equal(dd[k].cpu().numpy(), exp[k]), k


@pytest.mark.parametrize("w,h,lcu", [(128, 96, 6), (136, 72, 5), (200, 120, 6), (64, 48, 6), (56, 40, 6),
                                     (64, 48, 4), (1920, 1080, 6)])
def test_loopfilter_fused(gpu, olib, w, h, lcu):
    """Deblocking + SAO in one pass equals the reference's two loops: the
    picture deblocked in LCU order, then SAO over every LCU region with the
    deblocked picture as both source and starting destination."""
    import torch
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(w * 3 + h + lcu)
    y, u, v, scus = synth.deblock_picture(rng, w, h)
    lcus = synth.sao_params(rng, w, h, lcu)
    dy, du, dv = y.copy(), u.copy(), v.copy()
    olib.xo_deblock_picture(oracle.ptr(dy), w, oracle.ptr(du), oracle.ptr(dv), w // 2, w, h, oracle.ptr(scus), lcu, 1)
    exp = [dy.copy(), du.copy(), dv.copy()]
    dptr = (ctypes.c_void_p * 3)(*[oracle.ptr(p).value for p in exp])
    sptr = (ctypes.c_void_p * 3)(*[oracle.ptr(p).value for p in (dy, du, dv)])
    olib.xo_sao_picture(dptr, sptr, w, w // 2, w, h, lcu, oracle.ptr(lcus))
    src = [_dev(p) for p in (y, u, v)]
    out = [torch.full(p.shape, 7, dtype=torch.uint8, device="cuda") for p in (y, u, v)]
    ds, dl = _dev(scus.view(np.uint8)), _dev(lcus.view(np.uint8))
    rc = gpu.xavs2gpu_loopfilter_picture(*[ctypes.c_void_p(t.data_ptr()) for t in src + out], w, w // 2, w, h, lcu,
                                         ctypes.c_void_p(ds.data_ptr()), ctypes.c_void_p(dl.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    for k in range(3):
        assert np.array_equal(out[k].cpu().numpy(), exp[k]), k
        assert np.array_equal(src[k].cpu().numpy(), (y, u, v)[k])   # source untouched


@pytest.mark.parametrize("w,h,lcu", [(200, 120, 6), (136, 72, 5), (64, 48, 4)])
def test_loopfilter_extreme_params(gpu, olib, w, h, lcu):
    """The word-wise filters at the edges of their value ranges: alpha and
    beta over the whole byte range (0, 1, 2 and 255 included), pictures of
    flat 8x8 blocks with small steps between them (so every filter strength,
    including the one that needs L1 == L0 and R1 == R0, occurs), and SAO
    offsets over the whole int8 range (the saturating byte arithmetic).
    Both the fused pass and the two picture passes against the oracle."""
    import torch
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(w * 11 + h + lcu)
    y, u, v, scus = synth.deblock_picture(rng, w, h, p_edge=0.95)
    for p, bs in ((y, 8), (u, 4), (v, 4)):
        # about half the blocks flat: their value plus a step of -3..3
        for by in range(0, p.shape[0], bs):
            for bx in range(0, p.shape[1], bs):
                if rng.random() < 0.5:
                    blk = p[by:by + bs, bx:bx + bs]
                    blk[:] = np.clip(int(blk.mean()) + int(rng.integers(-3, 4)), 0, 255)
    for f in ("alpha", "beta", "alpha_c", "beta_c"):
        scus[f] = rng.integers(0, 256, scus[f].shape)
        k = rng.integers(0, len(scus), 8)
        scus[f][k[:2]] = 0
        scus[f][k[2:4]] = 1
        scus[f][k[4:6]] = 2
        scus[f][k[6:]] = 255
    lcus = synth.sao_params(rng, w, h, lcu, p_off=0.05)
    lcus["offset"] = rng.integers(-128, 128, lcus["offset"].shape)
    lcus["offset"][0::3] = 127
    lcus["offset"][1::5] = -128
    dy, du, dv = y.copy(), u.copy(), v.copy()
    olib.xo_deblock_picture(oracle.ptr(dy), w, oracle.ptr(du), oracle.ptr(dv), w // 2, w, h, oracle.ptr(scus), lcu, 1)
    assert not np.array_equal(dy, y)
    exp = [dy.copy(), du.copy(), dv.copy()]
    dptr = (ctypes.c_void_p * 3)(*[oracle.ptr(p).value for p in exp])
    sptr = (ctypes.c_void_p * 3)(*[oracle.ptr(p).value for p in (dy, du, dv)])
    olib.xo_sao_picture(dptr, sptr, w, w // 2, w, h, lcu, oracle.ptr(lcus))
    ds, dl = _dev(scus.view(np.uint8)), _dev(lcus.view(np.uint8))
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    # fused
    src = [_dev(p) for p in (y, u, v)]
    out = [torch.full(p.shape, 7, dtype=torch.uint8, device="cuda") for p in (y, u, v)]
    rc = gpu.xavs2gpu_loopfilter_picture(*[P(t) for t in src + out], w, w // 2, w, h, lcu, P(ds), P(dl), None)
    assert rc == 0
    torch.cuda.synchronize()
    for k in range(3):
        assert np.array_equal(out[k].cpu().numpy(), exp[k]), ("fused", k)
    # two passes: deblocking in place, then SAO writing the picture whole
    work = [_dev(p) for p in (y, u, v)]
    rc = gpu.xavs2gpu_deblock_picture(P(work[0]), w, P(work[1]), P(work[2]), w // 2, w, h, lcu, P(ds), None)
    assert rc == 0
    out2 = [torch.full(p.shape, 7, dtype=torch.uint8, device="cuda") for p in (y, u, v)]
    rc = gpu.xavs2gpu_sao_picture(*[P(t) for t in out2 + work], w, w // 2, w, h, lcu, P(dl), 1, None)
    assert rc == 0
    torch.cuda.synchronize()
    for k in range(3):
        assert np.array_equal(work[k].cpu().numpy(), (dy, du, dv)[k]), ("deblock", k)
        assert np.array_equal(out2[k].cpu().numpy(), exp[k]), ("two-pass", k)

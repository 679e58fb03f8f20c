"""GPU interpolation and transform/quant drop-ins and batched forms against
the oracle (bit-exact)."""
import ctypes

import numpy as np
import pytest

import oracle
from oracle import PU_W, PU_H, TU_PARTS

pytestmark = pytest.mark.gpu


def test_intpl_dropins(gpu, olib):
    import xavs2_gb300 as xg
    rng = np.random.default_rng(21)
    src = rng.integers(0, 256, (96, 120), dtype=np.uint8)
    src[10:20] = 255
    o = 8 * 120 + 8
    w, h = 40, 24
    for frac in range(1, 4):
        c = olib.xo_luma_filter(frac)
        d1 = np.zeros((h, 100), np.uint8); d2 = d1.copy()
        t1 = np.zeros((h, 100), np.int16); t2 = t1.copy()
        xg.fn("xavs2gpu_intpl_luma_hor")(xg.ptr(d1), 100, xg.ptr(t1), 100, xg.ptr(src, o), 120, w, h, c)
        olib.xo_intpl_luma_hor(oracle.ptr(d2), 100, oracle.ptr(t2), 100, oracle.ptr(src, o), 120, w, h, c)
        assert np.array_equal(d1, d2) and np.array_equal(t1, t2)
        d1[:] = 0; d2[:] = 0
        xg.fn("xavs2gpu_intpl_luma_ver")(xg.ptr(d1), 100, xg.ptr(src, o), 120, w, h, c)
        olib.xo_intpl_luma_ver(oracle.ptr(d2), 100, oracle.ptr(src, o), 120, w, h, c)
        assert np.array_equal(d1, d2)
        tmp = rng.integers(-6000, 22000, (64, 100), dtype=np.int16)
        d1[:] = 0; d2[:] = 0
        xg.fn("xavs2gpu_intpl_luma_ext")(xg.ptr(d1), 100, xg.ptr(tmp, 400), 100, w, h - 8, c)
        olib.xo_intpl_luma_ext(oracle.ptr(d2), 100, oracle.ptr(tmp, 400), 100, w, h - 8, c)
        assert np.array_equal(d1, d2)
    for fx in range(4):
        for fy in range(4):
            cx, cy = olib.xo_luma_filter(fx), olib.xo_luma_filter(fy)
            for (bw, bh) in ((64, 64), (16, 12), (8, 4)):
                d1 = np.zeros((64, 64), np.uint8); d2 = d1.copy()
                xg.fn("xavs2gpu_intpl_luma_block_ext")(xg.ptr(d1), 64, xg.ptr(src, o), 120, bw, bh, cx, cy)
                olib.xo_intpl_luma_block_ext(oracle.ptr(d2), 64, oracle.ptr(src, o), 120, bw, bh, cx, cy)
                assert np.array_equal(d1, d2)
                d1[:] = 0; d2[:] = 0
                xg.fn("xavs2gpu_intpl_luma_block_hor")(xg.ptr(d1), 64, xg.ptr(src, o), 120, bw, bh, cx)
                olib.xo_intpl_luma_block_hor(oracle.ptr(d2), 64, oracle.ptr(src, o), 120, bw, bh, cx)
                assert np.array_equal(d1, d2)
    for fx in range(8):
        for fy in range(8):
            cx, cy = olib.xo_chroma_filter(fx), olib.xo_chroma_filter(fy)
            for kind in ("hor", "ver", "ext"):
                d1 = np.zeros((32, 32), np.uint8); d2 = d1.copy()
                g = xg.fn("xavs2gpu_intpl_chroma_block_" + kind)
                e = getattr(olib, "xo_intpl_chroma_block_" + kind)
                if kind == "ext":
                    g(xg.ptr(d1), 32, xg.ptr(src, o), 120, 8, 6, cx, cy)
                    e(oracle.ptr(d2), 32, oracle.ptr(src, o), 120, 8, 6, cx, cy)
                else:
                    cc = cx if kind == "hor" else cy
                    g(xg.ptr(d1), 32, xg.ptr(src, o), 120, 32, 32, cc)
                    e(oracle.ptr(d2), 32, oracle.ptr(src, o), 120, 32, 32, cc)
                assert np.array_equal(d1, d2), (kind, fx, fy)


@pytest.mark.parametrize("w,h", [(136, 72), (64, 8), (200, 120), (416, 240), (330, 190), (1920, 1080)])
def test_frame_planes(gpu, olib, w, h):
    """The 15 sub-pel planes (with their 80-pixel replicated margin) computed
    on the device when a reference picture is loaded."""
    import xavs2_gb300 as xg
    rng = np.random.default_rng(w + h)
    img = rng.integers(0, 256, (h, w), dtype=np.uint8)
    img[: h // 3, : w // 4] = 255
    s = xg.MeSession(w, h, 1, 16)
    s.set_picture(0, img)
    exp = oracle.interpolate_frame(olib, img, mode=2)
    for k in range(16):
        assert np.array_equal(s.get_plane(0, k), exp[k]), k
    s.close()


@pytest.mark.parametrize("w,h,pad,extra,mode", [(300, 170, 9, 3, 2), (256, 128, 12, 0, 1), (97, 61, 8, 1, 2)])
def test_interpolate_frame_api(gpu, olib, w, h, pad, extra, mode):
    """xavs2gpu_interpolate_frame on device buffers with other margins,
    strides that are not multiples of 4 (byte stores, byte source loads)
    and the half-pel-only mode: every requested plane equals the oracle's
    over the whole padded area; planes not requested stay untouched."""
    import ctypes
    import torch
    import xavs2_gb300 as xg
    lib = xg.load()
    rng = np.random.default_rng(w * h + pad)
    img = rng.integers(0, 256, (h, w), dtype=np.uint8)
    exp = oracle.interpolate_frame(olib, img, mode=2)      # 80-pixel margins
    stride = w + 2 * pad + extra
    rows = h + 2 * pad
    src = np.zeros((rows, stride), np.uint8)
    src[:, :w + 2 * pad] = exp[0][80 - pad:80 + h + pad, 80 - pad:80 + w + pad]
    d_src = torch.from_numpy(src.reshape(-1).copy()).cuda()
    d_planes = torch.full((16, rows * stride + 16), 0x5A, dtype=torch.uint8, device="cuda")
    org = pad * stride + pad
    off = 1 if extra else 0          # misaligned planes where the stride is odd anyway
    ptrs = (ctypes.c_void_p * 16)(*[d_planes[k].data_ptr() + off + org for k in range(16)])
    rc = lib.xavs2gpu_interpolate_frame(ctypes.c_void_p(d_src.data_ptr() + org), stride, w, h, pad, ptrs, mode, None)
    assert rc == 0
    torch.cuda.synchronize()
    got = d_planes.cpu().numpy()
    for k in range(1, 16):
        plane = got[k][off:off + rows * stride].reshape(rows, stride)[:, :w + 2 * pad]
        if mode == 2 or k in (2, 8, 10):
            assert np.array_equal(plane, exp[k][80 - pad:80 + h + pad, 80 - pad:80 + w + pad]), k
        else:
            assert (plane == 0x5A).all(), k


@pytest.mark.parametrize("part", TU_PARTS)
def test_dct_dropins(gpu, olib, part):
    import xavs2_gb300 as xg
    w, h = PU_W[part], PU_H[part]
    wav = w == 64 or h == 64
    rng = np.random.default_rng(part)
    n = (w // 2) * (h // 2) if wav else w * h
    for kind in range(3):
        for flag in ((0, 1) if part in (3, 19, 20) else (0,)):
            if kind == 0:
                res = np.clip(np.round(rng.laplace(0, 12, (h, w + 8))), -255, 255).astype(np.int16)
            elif kind == 1:
                res = rng.integers(-255, 256, (h, w + 8)).astype(np.int16)
            else:
                res = rng.integers(-32768, 32768, (h, w + 8)).astype(np.int16)
            if wav:
                res = np.ascontiguousarray(res[:, :w])
            stride = (w if wav else w + 8) | flag
            g = np.zeros(64 * 64, np.int16); e = g.copy()
            xg.dct_fn("dct", part)(xg.ptr(res), xg.ptr(g), stride)
            olib.xo_dct(part, oracle.ptr(res), oracle.ptr(e), stride)
            assert np.array_equal(g[:n], e[:n]), ("dct", kind, flag)
            coef = np.zeros(64 * 64, np.int16)
            coef[:n] = (rng.integers(-600, 600, n) if kind < 2 else rng.integers(-32768, 32768, n))
            g = np.zeros(64 * 72, np.int16); e = g.copy()
            ds = (w if wav else w + 8) | flag
            xg.dct_fn("idct", part)(xg.ptr(coef), xg.ptr(g), ds)
            olib.xo_idct(part, oracle.ptr(coef), oracle.ptr(e), ds)
            assert np.array_equal(g, e), ("idct", kind, flag)
    if part in (3, 4):
        res = rng.integers(-255, 256, (w, w)).astype(np.int16)
        g = np.zeros(64 * 64, np.int16); e = g.copy()
        name = "xavs2gpu_dct_32x32_half" if part == 3 else "xavs2gpu_dct_64x64_half"
        xg.fn(name)(xg.ptr(res), xg.ptr(g), w)
        olib.xo_dct_half(part, oracle.ptr(res), oracle.ptr(e), w)
        assert np.array_equal(g[:1024], e[:1024])


def test_secondary_and_quant(gpu, olib):
    import xavs2_gb300 as xg
    rng = np.random.default_rng(8)
    for t in range(40):
        blk = rng.integers(-3000, 3000, (8, 12)).astype(np.int16)
        mode, top, left = int(rng.integers(0, 33)), int(rng.integers(0, 2)), int(rng.integers(0, 2))
        for gname, oname, extra in (("xavs2gpu_transform_4x4_2nd", "xo_transform_4x4_2nd", ()),
                                    ("xavs2gpu_inv_transform_4x4_2nd", "xo_inv_transform_4x4_2nd", ()),
                                    ("xavs2gpu_transform_2nd", "xo_transform_2nd", (mode, top, left)),
                                    ("xavs2gpu_inv_transform_2nd", "xo_inv_transform_2nd", (mode, top, left))):
            a = blk.copy(); b = blk.copy()
            xg.fn(gname)(xg.ptr(a), 12, *extra)
            getattr(olib, oname)(oracle.ptr(b), 12, *extra)
            assert np.array_equal(a, b), gname
    for qp in (0, 13, 22, 32, 40, 51, 63, 79):
        for n in (16, 64, 256, 1024):
            c = rng.integers(-32768, 32768, n).astype(np.int16)
            c[rng.random(n) < 0.3] = 0
            shift = 22 - 4
            add = olib.xo_quant_fwd_add(shift, qp & 1)
            a = c.copy(); b = c.copy()
            assert xg.fn("xavs2gpu_quant")(xg.ptr(a), n, olib.xo_q_scale(qp), shift, add) == \
                olib.xo_quant(oracle.ptr(b), n, olib.xo_q_scale(qp), shift, add)
            assert np.array_equal(a, b)
            ds = olib.xo_iq_shift(qp) + 9 + 4 - 16
            xg.fn("xavs2gpu_dequant")(xg.ptr(a), n, olib.xo_iq_scale(qp), ds)
            olib.xo_dequant(oracle.ptr(b), n, olib.xo_iq_scale(qp), ds)
            assert np.array_equal(a, b)
    n = 512
    c = rng.integers(-32768, 32768, n).astype(np.int16)
    a = np.zeros(n, np.int16); b = a.copy()
    xg.fn("xavs2gpu_abs_coeff")(xg.ptr(a), xg.ptr(c), n)
    olib.xo_abs_coeff(oracle.ptr(b), oracle.ptr(c), n)
    assert np.array_equal(a, b)
    d = rng.integers(-3, 3, n).astype(np.int16)
    av = np.abs(c).astype(np.int16)
    a = d.copy(); b = d.copy()
    assert xg.fn("xavs2gpu_add_sign")(xg.ptr(a), xg.ptr(av), n) == olib.xo_add_sign(oracle.ptr(b), oracle.ptr(av), n)
    assert np.array_equal(a, b)
    ls = rng.integers(1, 4096, n).astype(np.int32)
    a = c.copy(); b = c.copy()
    assert xg.fn("xavs2gpu_quant_weighted")(xg.ptr(a), n, 5000, 18, 1000, xg.ptr(ls)) == \
        olib.xo_wquant(oracle.ptr(b), n, 5000, 18, 1000, oracle.ptr(ls))
    assert np.array_equal(a, b)


def _tq_blocks(rng, n, parts=(0, 1, 2, 3, 4)):
    sizes = {p: PU_W[p] * PU_H[p] for p in TU_PARTS}
    ncoef = {p: (sizes[p] // 4 if (PU_W[p] == 64 or PU_H[p] == 64) else sizes[p]) for p in TU_PARTS}
    blocks = np.zeros(n, np.dtype([("offset", "<i8"), ("coef_offset", "<i8"), ("part", "<i4"), ("qp", "<i4"),
                                   ("flags", "<i4"), ("pad_", "<i4")]))
    blocks["part"] = rng.choice(parts, n)
    blocks["qp"] = rng.integers(22, 52, n)
    sec = (blocks["part"] == 0) & (rng.random(n) < 0.5)
    blocks["flags"] = np.where(sec, 3, 0)
    off = coff = 0
    for i in range(n):
        blocks["offset"][i] = off
        blocks["coef_offset"][i] = coff
        off += sizes[int(blocks["part"][i])]
        coff += ncoef[int(blocks["part"][i])]
    res = np.clip(np.round(rng.laplace(0, 12, off)), -255, 255).astype(np.int16)
    zero = rng.random(n) < 0.1
    for i in np.nonzero(zero)[0]:
        o = int(blocks["offset"][i])
        res[o:o + sizes[int(blocks["part"][i])]] = 0
    return blocks, res, off, coff


def test_tq_batch(gpu, olib):
    import torch
    import xavs2_gb300 as xg
    rng = np.random.default_rng(12)
    blocks, res, nres, ncoef = _tq_blocks(rng, 400, parts=TU_PARTS)
    d_blocks = torch.from_numpy(blocks.view(np.uint8).copy()).cuda()
    d_res = torch.from_numpy(res).cuda()
    d_coef = torch.zeros(ncoef, dtype=torch.int16, device="cuda")
    d_rec = torch.zeros(nres, dtype=torch.int16, device="cuda")
    d_nnz = torch.zeros(len(blocks), dtype=torch.int32, device="cuda")
    rc = xg.fn("xavs2gpu_tq_batch")(d_blocks.data_ptr(), len(blocks), d_res.data_ptr(), d_coef.data_ptr(),
                                     d_rec.data_ptr(), d_nnz.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    coef, rec, nnz = d_coef.cpu().numpy(), d_rec.cpu().numpy(), d_nnz.cpu().numpy()
    for i, b in enumerate(blocks):
        p = int(b["part"])
        w, h = PU_W[p], PU_H[p]
        o, co = int(b["offset"]), int(b["coef_offset"])
        blk = res[o:o + w * h].copy()
        cf = np.zeros(w * h, np.int16)
        nz = olib.xo_tq_chain(p, oracle.ptr(blk), oracle.ptr(cf), int(b["qp"]), int(b["flags"]) & 1,
                              (int(b["flags"]) >> 1) & 1)
        n = (w // 2) * (h // 2) if (w == 64 or h == 64) else w * h
        assert nnz[i] == nz, i
        assert np.array_equal(coef[co:co + n], cf[:n]), i
        assert np.array_equal(rec[o:o + w * h], blk), i


def _run_tq_batch(blocks, res, nres, ncoef):
    import torch
    import xavs2_gb300 as xg
    d_blocks = torch.from_numpy(blocks.view(np.uint8).copy()).cuda()
    d_res = torch.from_numpy(res).cuda()
    d_coef = torch.full((ncoef,), 0x5A5A, dtype=torch.int16, device="cuda")
    d_rec = torch.full((nres,), 0x5A5A, dtype=torch.int16, device="cuda")
    d_nnz = torch.zeros(len(blocks), dtype=torch.int32, device="cuda")
    rc = xg.fn("xavs2gpu_tq_batch")(d_blocks.data_ptr(), len(blocks), d_res.data_ptr(), d_coef.data_ptr(),
                                     d_rec.data_ptr(), d_nnz.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    return d_coef.cpu().numpy(), d_rec.cpu().numpy(), d_nnz.cpu().numpy()


def test_tq_batch_edges(gpu, olib):
    """Extreme residuals (the int16 wrap of the forward passes and the 16-bit
    clips), blocks at unaligned offsets (element-granular packing), invalid
    descriptors (a non-TU shape, QP out of range): levels, recon and nnz
    equal the oracle's chain; invalid blocks report nnz = -1."""
    rng = np.random.default_rng(77)
    parts = list(TU_PARTS) * 6
    n = len(parts) + 2
    blocks = np.zeros(n, np.dtype([("offset", "<i8"), ("coef_offset", "<i8"), ("part", "<i4"), ("qp", "<i4"),
                                   ("flags", "<i4"), ("pad_", "<i4")]))
    off = coff = 0
    chunks = []
    for i in range(n):
        p = parts[i] if i < len(parts) else 0
        w, h = PU_W[p], PU_H[p]
        gap = int(rng.integers(0, 3))          # 0..2 elements: breaks 16-byte alignment
        off += gap
        chunks.append(np.zeros(gap, np.int16))
        kind = i % 4
        if kind == 0:
            blk = rng.integers(-32768, 32768, w * h)
        elif kind == 1:
            blk = np.where(rng.random(w * h) < 0.5, -32768, 32767)
        elif kind == 2:
            blk = rng.integers(-2048, 2048, w * h)
        else:
            blk = np.clip(np.round(rng.laplace(0, 40, w * h)), -255, 255)
        chunks.append(blk.astype(np.int16))
        blocks[i] = (off, coff, p, int(rng.integers(0, 80)), int(rng.integers(0, 4)) if p == 0 else int(rng.integers(0, 2)), 0)
        off += w * h
        coff += (w // 2) * (h // 2) if (w == 64 or h == 64) else w * h
    blocks["part"][-2] = 5            # 8x4 is not a TU shape
    blocks["qp"][-1] = 80             # out of range
    res = np.concatenate(chunks)
    coef, rec, nnz = _run_tq_batch(blocks, res, off, coff)
    for i, b in enumerate(blocks[:-2]):
        p = int(b["part"])
        w, h = PU_W[p], PU_H[p]
        o, co = int(b["offset"]), int(b["coef_offset"])
        blk = res[o:o + w * h].copy()
        cf = np.zeros(w * h, np.int16)
        nz = olib.xo_tq_chain(p, oracle.ptr(blk), oracle.ptr(cf), int(b["qp"]), int(b["flags"]) & 1,
                              (int(b["flags"]) >> 1) & 1)
        nc = (w // 2) * (h // 2) if (w == 64 or h == 64) else w * h
        assert nnz[i] == nz, (i, p)
        assert np.array_equal(coef[co:co + nc], cf[:nc]), (i, p)
        assert np.array_equal(rec[o:o + w * h], blk), (i, p)
    assert nnz[-2] == -1 and nnz[-1] == -1


@pytest.mark.parametrize("pinned,chunks", [(True, 7), (False, 4), (True, 1), (True, 0)])
def test_tq_batch_host(gpu, pinned, chunks):
    """The host-buffer TU chain (chunked copies overlapped with the chain)
    gives exactly the device entry's outputs, for page-locked and pageable
    host buffers, with descriptors out of offset order and invalid ones."""
    import torch
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth
    n = 5000
    blocks, nres, ncoef, zero = synth.tq_blocks(n, seed=12)
    res = synth.tq_residual(blocks, zero, nres, seed=13).numpy()
    rng = np.random.default_rng(14)
    perm = rng.permutation(n)
    blocks = np.ascontiguousarray(blocks[perm])      # offsets no longer monotone
    blocks["part"][::97] = 30                          # invalid descriptors: nnz = -1, nothing written
    d = {k: torch.from_numpy(v).cuda() for k, v in (("b", blocks.view(np.uint8).copy()), ("r", res))}
    d_coef = torch.zeros(ncoef, dtype=torch.int16, device="cuda")
    d_rec = torch.zeros(nres, dtype=torch.int16, device="cuda")
    d_nnz = torch.zeros(n, dtype=torch.int32, device="cuda")
    assert xg.fn("xavs2gpu_tq_batch")(d["b"].data_ptr(), n, d["r"].data_ptr(), d_coef.data_ptr(), d_rec.data_ptr(),
                                      d_nnz.data_ptr(), None) == 0
    torch.cuda.synchronize()

    def host(a):
        t = torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy())
        return t.pin_memory() if pinned else t
    hb, hr = host(blocks), host(res)
    hc, hrec, hn = host(np.zeros(ncoef, np.int16)), host(np.zeros(nres, np.int16)), host(np.zeros(n, np.int32))
    # regions owned by valid descriptors (others are unspecified after the host call)
    valid = blocks["part"] < 25
    w, h = np.asarray(xg.PU_W)[blocks["part"][valid]], np.asarray(xg.PU_H)[blocks["part"][valid]]
    sz = (w * h).astype(np.int64)
    nc = np.where((w == 64) | (h == 64), sz // 4, sz)
    own_r = np.concatenate([np.arange(o, o + k) for o, k in zip(blocks["offset"][valid], sz)])
    own_c = np.concatenate([np.arange(o, o + k) for o, k in zip(blocks["coef_offset"][valid], nc)])
    want_c, want_r = d_coef.cpu().numpy()[own_c], d_rec.cpu().numpy()[own_r]
    for _ in range(2):
        assert xg.fn("xavs2gpu_tq_batch_host")(hb.data_ptr(), n, hr.data_ptr(), hc.data_ptr(), hrec.data_ptr(),
                                               hn.data_ptr(), chunks) == 0
        assert np.array_equal(hn.numpy().view(np.int32), d_nnz.cpu().numpy())
        assert np.array_equal(hc.numpy().view(np.int16)[own_c], want_c)
        assert np.array_equal(hrec.numpy().view(np.int16)[own_r], want_r)
    assert (hn.numpy().view(np.int32)[::97] == -1).all()

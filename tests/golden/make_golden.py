"""Generates tests/golden/golden.npz from the reference's own C primitives.

Run where the xavs2 sources are present (it builds oracle/_ref from them):

    python tests/golden/make_golden.py

Every input is seeded; every output comes from the reference build
(oracle/_ref/libxavs2ref.so, pure-C primitive table), never from this
project's code.  Large outputs (sub-pel planes) are stored as SHA-256 digests.
"""
import ctypes
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402
from oracle import PU_W, PU_H, TU_PARTS, ptr  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")


# intra block shapes (square CUs, SDIP / NSQT partitions) and the DC
# availability words (top << 8 | left); entries 33..35 of a digest row are DC
# with the first three availabilities, entry 0 with both neighbours
INTRA_SHAPES = [(4, 4), (8, 8), (16, 16), (32, 32), (64, 64), (4, 16), (16, 4), (8, 32), (32, 8), (16, 64), (64, 16)]
INTRA_DC_AVAIL = [0x000, 0x001, 0x100, 0x101]


def intra_edges(rng):
    """512-sample edge arrays (top-left sample at 256): random, a smooth ramp
    with noise, and alternating 0 / 255 runs."""
    a = rng.integers(0, 256, 512).astype(np.uint8)
    t = np.arange(512)
    b = np.clip(128 + 100 * np.sin(t / 37.0) + rng.integers(-6, 7, 512), 0, 255).astype(np.uint8)
    c = np.where((t // 3) % 2 == 0, 255, 0).astype(np.uint8)
    return [a, b, c]


def intra_fill_picture():
    """272x272 picture for the edge-fill digests (a closed formula, so the
    fixture stores only digests)."""
    y, x = np.mgrid[0:272, 0:272]
    return ((x * 37 + y * 101 + (x * y) // 3) % 251).astype(np.uint8)


def intra_fill_windows(fill, bw, bh):
    """The edges of a bw x bh block at (72, 72) of intra_fill_picture for
    availability masks 0..31, the window the reference writes
    (-(bh + 11*bw/4 + 4) .. bw + 11*bh/4 + 4), concatenated; fill(pic, ep,
    avail) writes one edge around ep (an index into a 1024-sample array)."""
    pic = intra_fill_picture()
    lo, hi = bh + (11 * bw) // 4 + 4, bw + (11 * bh) // 4 + 4
    out = []
    for avail in range(32):
        buf = np.zeros(1024, np.uint8)
        fill(pic, buf, avail)
        out.append(buf[512 - lo:512 + hi + 1])
    return np.concatenate(out)


def intra_prefill(bw, bh):
    """Destination with stride bw + 8, pre-filled so that samples a mode
    leaves alone are visible."""
    return ((np.arange(bh * (bw + 8)) * 7 + 3) % 251).astype(np.uint8).reshape(bh, bw + 8)


def main():
    r = oracle.ref_lib()
    if r is None:
        raise SystemExit("reference sources not found; set XAVS2_REF_SRC")
    rng = np.random.default_rng(20240601)
    g = {}

    # --- block costs: 4 pixel pairs, every shape, sad/satd/sa8d/ssd --------
    a = rng.integers(0, 256, (4, 64, 72), dtype=np.uint8)
    b = rng.integers(0, 256, (4, 64, 80), dtype=np.uint8)
    a[1] = 255; b[1] = 0
    a[2] = np.where(rng.integers(0, 2, (64, 72)) == 1, 255, 0)
    b[2] = np.where(rng.integers(0, 2, (64, 80)) == 1, 255, 0)
    costs = np.zeros((4, 4, 25), np.int32)
    for i in range(4):
        for kind in range(4):
            for part in range(25):
                costs[i, kind, part] = r.xr_cmp(kind, part, ptr(a[i]), 72, ptr(b[i]), 80)
    g["cost_a"], g["cost_b"], g["costs"] = a, b, costs
    x3 = np.zeros((25, 4), np.int32)
    for part in range(25):
        res = (ctypes.c_int * 4)()
        r.xr_sad_x4(part, ptr(a[0]), ptr(b[0], 0), ptr(b[0], 1), ptr(b[0], 81), ptr(b[0], 163), 80, res)
        x3[part] = list(res)
    g["sad_x4"] = x3

    # --- block ops on one input set ---------------------------------------
    s = rng.integers(-300, 300, (64, 64), dtype=np.int16)
    g["ops_s"] = s
    avg = np.zeros((25, 64, 64), np.uint8)
    sub = np.zeros((25, 64, 64), np.int16)
    add = np.zeros((25, 64, 64), np.uint8)
    for part in range(25):
        r.xr_avg(part, ptr(avg[part]), 64, ptr(a[0]), 72, ptr(b[0]), 80)
        r.xr_sub_ps(part, ptr(sub[part]), 64, ptr(a[0]), ptr(b[0]), 72, 80)
        r.xr_add_ps(part, ptr(add[part]), 64, ptr(a[0]), ptr(s), 72, 64)
    g["avg"], g["sub_ps"], g["add_ps"] = avg, sub, add

    # --- frame sub-pel planes (digests) -------------------------------------
    img = rng.integers(0, 256, (72, 136), dtype=np.uint8)
    img[:20, :40] = 255
    planes = oracle.interpolate_frame(r, img, mode=2, ref=True, lcu_level=6)
    g["intp_img"] = img
    g["intp_sha"] = np.array([hashlib.sha256(planes[k].tobytes()).hexdigest() for k in range(16)])
    g["intp_center"] = planes[:, 80:80 + 72, 80:80 + 136].copy()

    # --- transforms -----------------------------------------------------------
    for part in TU_PARTS:
        w, h = PU_W[part], PU_H[part]
        wav = w == 64 or h == 64
        n = (w // 2) * (h // 2) if wav else w * h
        res = np.clip(np.round(rng.laplace(0, 12, (h, w))), -255, 255).astype(np.int16)
        dct = np.zeros(64 * 64, np.int16)
        r.xr_dct(0, part, ptr(res), ptr(dct), w)
        coef = (rng.integers(-400, 400, n)).astype(np.int16)
        cbuf = np.zeros(64 * 64, np.int16); cbuf[:n] = coef
        rec = np.zeros(64 * 64, np.int16)
        r.xr_dct(1, part, ptr(cbuf), ptr(rec), w)
        g["dct_in_%d" % part] = res
        g["dct_out_%d" % part] = dct[:n].copy()
        g["idct_in_%d" % part] = coef
        g["idct_out_%d" % part] = rec[:w * h].copy()
    blk = rng.integers(-1500, 1500, (4, 4)).astype(np.int16)
    t = blk.copy(); r.xr_2nd(0, ptr(t), 4, 0, 0, 0)
    it = blk.copy(); r.xr_2nd(1, ptr(it), 4, 0, 0, 0)
    g["sec_in"], g["sec_fwd"], g["sec_inv"] = blk, t, it

    # --- quant/dequant chain on a few QPs -----------------------------------
    qps = np.array([22, 27, 32, 37, 42, 51], np.int32)
    qin = rng.integers(-4000, 4000, (len(qps), 1024)).astype(np.int16)
    qout = qin.copy(); dqout = qin.copy(); nz = np.zeros(len(qps), np.int32)
    for i, qp in enumerate(qps):
        shift = 22 - 5
        nz[i] = r.xr_quant(ptr(qout[i]), 1024, r.xr_q_scale(int(qp)), shift, (1 << shift) * 5 // 31)
        dqout[i] = qout[i]
        r.xr_dequant(ptr(dqout[i]), 1024, r.xr_iq_scale(int(qp)), r.xr_iq_shift(int(qp)) + 9 + 5 - 16)
    g["q_qps"], g["q_in"], g["q_out"], g["q_nz"], g["dq_out"] = qps, qin, qout, nz, dqout

    # --- motion search: small frame, FS +-16, quarter-pel SATD --------------
    h, w = 72, 96
    cur = rng.integers(0, 256, (h, w), dtype=np.uint8)
    refimg = np.clip(np.roll(cur, (2, -3), axis=(0, 1)).astype(np.int16) + rng.integers(-5, 6, (h, w)), 0, 255).astype(np.uint8)
    planes = oracle.interpolate_frame(r, refimg, mode=2, ref=True)
    flat = np.ascontiguousarray(planes.reshape(16, -1))
    stride = w + 160
    off = 80 * stride + 80
    frefs = (ctypes.c_void_p * 16)(*[ptr(flat[k], off).value for k in range(16)])
    prm = oracle.MeParams(16, oracle.lambda_factor(32), 1, 2, 0, 0)
    pus, outs = [], []
    olib = oracle.lib()
    for part in range(25):
        for t in range(2):
            pw, ph = PU_W[part], PU_H[part]
            x = int(rng.integers(0, w - pw + 1)) // 4 * 4
            y = int(rng.integers(0, h - ph + 1)) // 4 * 4
            pu = oracle.Pu(x, y, part, 0, int(rng.integers(-20, 21)), int(rng.integers(-20, 21)))
            olib.xo_pu_set_limits(ctypes.byref(pu), w, h, -2048, 2047)
            res = oracle.MeResult()
            r.xr_me_search(ctypes.byref(prm), ctypes.byref(pu), ptr(cur, y * w + x), w, frefs, stride, ctypes.byref(res))
            pus.append(bytes(pu))
            outs.append(bytes(res))
    g["me_cur"], g["me_ref"] = cur, refimg
    g["me_params"] = np.array([16, oracle.lambda_factor(32), 1, 2, 0, 0], np.int32)
    g["me_pus"] = np.frombuffer(b"".join(pus), oracle.PU_DTYPE)
    g["me_out"] = np.frombuffer(b"".join(outs), oracle.RESULT_DTYPE)

    # --- intra prediction: every mode and shape on three edge sets (digests)
    edges = intra_edges(rng)
    dig = np.zeros((len(edges), len(INTRA_SHAPES), 33 + 3), "<U64")
    for e, edge in enumerate(edges):
        for s_, (bw, bh) in enumerate(INTRA_SHAPES):
            for m in range(36):
                mode, dir_mode = (0, INTRA_DC_AVAIL[m - 33]) if m >= 33 else (m, INTRA_DC_AVAIL[3] if m == 0 else m)
                dst = intra_prefill(bw, bh)
                r.xr_intra_pred(mode, ptr(edge, 256), ptr(dst), bw + 8, dir_mode, bw, bh)
                dig[e, s_, m] = hashlib.sha256(dst.tobytes()).hexdigest()
    g["intra_edges"], g["intra_sha"] = np.stack(edges), dig

    # --- intra edge filling: a block inside a picture, every availability
    fill_dig = []
    for bw, bh in INTRA_SHAPES:
        def fill(pic, buf, avail, bw=bw, bh=bh):
            ptl = ptr(pic, 71 * 272 + 71)
            r.xr_intra_fill_edge(3, ptl, 272, ptr(buf, 512), ptr(buf, 512), avail, bw, bh)
        fill_dig.append(hashlib.sha256(intra_fill_windows(fill, bw, bh).tobytes()).hexdigest())
    g["intra_fill_sha"] = np.array(fill_dig)

    np.savez_compressed(OUT, **g)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()

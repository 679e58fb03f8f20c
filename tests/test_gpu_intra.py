"""Intra prediction on the GPU: the intraf[] drop-ins (one block per call,
host buffers) against the oracle and the golden digests recorded from the
reference, and the batched rough mode decision (every mode's cost and the
candidate list) against the oracle's restatement of the encoder's search."""
import ctypes
import hashlib
import importlib.util
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden_mod():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_intra_table_init(gpu):
    import xavs2_gb300 as xg
    table = (ctypes.c_void_p * 33)()
    gpu.xavs2gpu_intra_pred_init(0, table)
    addr = lambda name: ctypes.cast(getattr(gpu, name), ctypes.c_void_p).value
    want = [addr("xavs2gpu_intra_pred_ang")] * 33
    want[0], want[1], want[2] = addr("xavs2gpu_intra_pred_dc"), addr("xavs2gpu_intra_pred_plane"), \
        addr("xavs2gpu_intra_pred_bilinear")
    want[12], want[24] = addr("xavs2gpu_intra_pred_ver"), addr("xavs2gpu_intra_pred_hor")
    assert list(table) == want


def test_intra_dropins_golden(gpu, olib):
    """Every mode and shape through the table, destination pre-filled with a
    stride wider than the block: the digests equal the reference's."""
    import xavs2_gb300 as xg
    g = dict(np.load(os.path.join(HERE, "golden", "golden.npz")))
    mg = _golden_mod()
    table = (ctypes.c_void_p * 33)()
    gpu.xavs2gpu_intra_pred_init(0, table)
    proto = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                             ctypes.c_int)
    fns = [proto(a) for a in table]
    for e, edge in enumerate(g["intra_edges"]):
        edge = np.ascontiguousarray(edge)
        for s, (bw, bh) in enumerate(mg.INTRA_SHAPES):
            for m in range(36):
                mode, avail = (0, mg.INTRA_DC_AVAIL[m - 33]) if m >= 33 else (m, mg.INTRA_DC_AVAIL[3])
                dst = mg.intra_prefill(bw, bh)
                fns[mode](xg.ptr(edge, 256).value, xg.ptr(dst).value, bw + 8, avail if mode == 0 else mode, bw, bh)
                assert hashlib.sha256(dst.tobytes()).hexdigest() == g["intra_sha"][e, s, m], (e, bw, bh, m)


def test_intra_dropins_random(gpu, olib):
    import xavs2_gb300 as xg
    rng = np.random.default_rng(5)
    for trial in range(3):
        edge = rng.integers(0, 256, 512).astype(np.uint8)
        for bw, bh in _golden_mod().INTRA_SHAPES:
            for mode in range(33):
                fill = rng.integers(0, 256, (bh, bw + 3), dtype=np.uint8)
                a, b = fill.copy(), fill.copy()
                avail = int(rng.integers(0, 2)) << 8 | int(rng.integers(0, 2))
                name = {0: "dc", 1: "plane", 2: "bilinear", 12: "ver", 24: "hor"}.get(mode, "ang")
                xg.fn("xavs2gpu_intra_pred_" + name)(xg.ptr(edge, 256), xg.ptr(a), bw + 3,
                                                     avail if mode == 0 else mode, bw, bh)
                olib.xo_intra_pred(mode, oracle.ptr(edge, 256), oracle.ptr(b), bw + 3, avail, bw, bh)
                assert np.array_equal(a, b), (bw, bh, mode)


def _rmd_expected(olib, blocks, edges, src, prm):
    width = src.shape[1]
    flat = np.ascontiguousarray(src).reshape(-1)
    cost = np.zeros((len(blocks), 33))
    modes = np.zeros((len(blocks), 9), np.int32)
    ccost = np.zeros((len(blocks), 9))
    nrdo = np.zeros(len(blocks), np.int32)
    for i, b in enumerate(blocks):
        mpm = np.array(b["mpm"], np.int32)
        c = np.zeros(33)
        olib.xo_intra_mode_costs(oracle.ptr(edges, int(b["edge_offset"])), oracle.ptr(flat, int(b["fenc_offset"])),
                                 width, int(b["width"]), int(b["height"]), int(b["dc_avail"]), oracle.ptr(mpm),
                                 prm.lambda_, prm.use_hadamard, oracle.ptr(c))
        cost[i] = c
        nrdo[i] = olib.xo_intra_candidates(oracle.ptr(c), prm.rough, prm.dist2, prm.dist1, int(b["num_for_rdo"]),
                                           oracle.ptr(mpm), oracle.ptr(modes[i]), oracle.ptr(ccost[i]))
    return cost, modes, ccost, nrdo


def _rmd_gpu(gpu, blocks, edges, src, prm):
    import torch
    import xavs2_gb300 as xg
    dev = torch.device("cuda:0")
    d_blocks = torch.from_numpy(blocks.view(np.uint8).copy()).to(dev)
    d_edges = torch.from_numpy(edges).to(dev)
    d_src = torch.from_numpy(np.ascontiguousarray(src)).to(dev)
    d_out = torch.zeros(len(blocks) * xg.INTRA_RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    rc = gpu.xavs2gpu_intra_rmd_batch(ctypes.c_void_p(d_blocks.data_ptr()), len(blocks),
                                      ctypes.c_void_p(d_edges.data_ptr()), ctypes.c_void_p(d_src.data_ptr()),
                                      src.shape[1], ctypes.byref(prm), ctypes.c_void_p(d_out.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(xg.INTRA_RESULT_DTYPE)


@pytest.mark.parametrize("hadamard,rough", [(1, 0), (1, 1), (0, 1)])
def test_intra_rmd_batch(gpu, olib, hadamard, rough):
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(40 + 2 * hadamard + rough)
    src = synth.base_picture(rng, 256, 192)
    src[64:128, 128:192] = rng.integers(0, 256, (64, 64))          # a noisy CTU
    recon = np.clip(src.astype(np.int32) + rng.integers(-4, 5, src.shape), 0, 255).astype(np.uint8)
    blocks, edges = synth.intra_blocks(rng, src, recon, all_shapes=True, block_dtype=xg.INTRA_BLOCK_DTYPE)
    prm = xg.IntraParams(oracle.lambda_factor(32) / 65536.0 * 1.7, hadamard, rough, synth.INTRA_DIST2,
                         synth.INTRA_DIST1)
    got = _rmd_gpu(gpu, blocks, edges, src, prm)
    cost, modes, ccost, nrdo = _rmd_expected(olib, blocks, edges, src, prm)
    assert np.array_equal(got["cost"], cost)
    assert np.array_equal(got["cand_mode"], modes)
    assert np.array_equal(got["cand_cost"], ccost)
    assert np.array_equal(got["num_for_rdo"], nrdo)


def test_intra_rmd_edges(gpu, olib):
    """Empty batch, flat content (ties between modes resolved in mode
    order), MPMs equal to the best modes, and blocks that are not intra
    shapes (reported with num_for_rdo = -1)."""
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth
    prm = xg.IntraParams(12.5, 1, 1, 4, 2)
    assert gpu.xavs2gpu_intra_rmd_batch(None, 0, None, None, 64, ctypes.byref(prm), None, None) == 0
    rng = np.random.default_rng(9)
    src = np.full((128, 128), 77, np.uint8)
    blocks, edges = synth.intra_blocks(rng, src, src.copy(), all_shapes=True, block_dtype=xg.INTRA_BLOCK_DTYPE)
    blocks["mpm"][::3] = (0, 1)
    got = _rmd_gpu(gpu, blocks, edges, src, prm)
    cost, modes, ccost, nrdo = _rmd_expected(olib, blocks, edges, src, prm)
    assert np.array_equal(got["cost"], cost) and np.array_equal(got["cand_mode"], modes)
    assert np.array_equal(got["num_for_rdo"], nrdo)
    bad = blocks[:5].copy()
    bad["width"] = (12, 4, 128, 8, 4)
    bad["height"] = (4, 0, 64, 8, 32)
    bad["mpm"][3] = (40, 2)
    got = _rmd_gpu(gpu, bad, edges, src, prm)
    assert list(got["num_for_rdo"]) == [-1] * 5


def test_intra_rmd_every_shape(gpu, olib):
    """All 19 shapes with power-of-two sides and aspect ratio <= 4 in one
    shuffled batch (classes of 1 .. 40 blocks, partial tiles)."""
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(12)
    src = synth.base_picture(rng, 256, 256)
    recon = np.clip(src.astype(np.int32) + rng.integers(-6, 7, src.shape), 0, 255).astype(np.uint8)
    rects = []
    for a in range(5):
        for b in range(5):
            if abs(a - b) > 2:
                continue
            w, h = 4 << a, 4 << b
            for _ in range(int(rng.integers(1, 41))):
                rects.append((int(rng.integers(0, (256 - w) // 4 + 1)) * 4, int(rng.integers(0, 256 - h + 1)), w, h))
    rects = [rects[i] for i in rng.permutation(len(rects))]
    blocks, edges = synth.intra_pack(rects, recon, rng, xg.INTRA_BLOCK_DTYPE)
    for hadamard in (1, 0):
        prm = xg.IntraParams(7.25, hadamard, 1, 4, 2)
        got = _rmd_gpu(gpu, blocks, edges, src, prm)
        cost, modes, ccost, nrdo = _rmd_expected(olib, blocks, edges, src, prm)
        assert np.array_equal(got["cost"], cost), hadamard
        assert np.array_equal(got["cand_mode"], modes) and np.array_equal(got["num_for_rdo"], nrdo)


def _fill_gpu(gpu, jobs, pic, size, width=None, height=None, prefill=0):
    import torch
    dev = torch.device("cuda:0")
    d_jobs = torch.from_numpy(jobs.view(np.uint8).copy()).to(dev)
    d_pic = torch.from_numpy(np.ascontiguousarray(pic)).to(dev)
    d_edges = torch.full((size,), prefill, dtype=torch.uint8, device=dev)
    h, w = pic.shape
    rc = gpu.xavs2gpu_intra_fill_edges(ctypes.c_void_p(d_jobs.data_ptr()), len(jobs), ctypes.c_void_p(d_pic.data_ptr()),
                                       w, width or w, height or h, ctypes.c_void_p(d_edges.data_ptr()), size, None)
    assert rc == 0
    torch.cuda.synchronize()
    return d_edges.cpu().numpy()


def _fill_oracle(olib, jobs, pic, size, width=None, height=None, prefill=0):
    edges = np.full(size, prefill, np.uint8)
    h, w = pic.shape
    olib.xo_intra_fill_edges(oracle.ptr(jobs), len(jobs), oracle.ptr(pic), w, width or w, height or h,
                             oracle.ptr(edges), size)
    return edges


def test_intra_fill_edges(gpu, olib):
    """Edges of every block of every shape of a 320x256 picture, with the
    encoder's availability, built on the device from the reconstruction:
    equal to the oracle's fill_reference_samples; then the rough mode
    decision on those edges equals the oracle's on the oracle's edges."""
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(31)
    W, H = 320, 256
    src = synth.base_picture(rng, W, H)
    recon = np.clip(src.astype(np.int32) + rng.integers(-5, 6, src.shape), 0, 255).astype(np.uint8)
    rects = synth.intra_level_blocks(W, H, synth.INTRA_ALL_SHAPES)
    blocks, jobs, size = synth.intra_fill_jobs(rects, W, H, rng, xg.INTRA_BLOCK_DTYPE, xg.INTRA_EDGE_JOB_DTYPE)
    assert len(np.unique(jobs["avail"])) > 8
    got = _fill_gpu(gpu, jobs, recon, size, prefill=0xA5)
    want = _fill_oracle(olib, jobs, recon, size, prefill=0xA5)
    assert np.array_equal(got, want)
    sel = rng.choice(len(blocks), 600, replace=False)
    prm = xg.IntraParams(9.5, 1, 1, synth.INTRA_DIST2, synth.INTRA_DIST1)
    res = _rmd_gpu(gpu, blocks[sel], got, src, prm)
    cost, modes, ccost, nrdo = _rmd_expected(olib, blocks[sel], want, src, prm)
    assert np.array_equal(res["cost"], cost) and np.array_equal(res["cand_mode"], modes)
    assert np.array_equal(res["num_for_rdo"], nrdo)


def test_intra_fill_edges_edge_cases(gpu, olib):
    """Empty batch; availability claimed outside the picture (treated as
    missing), every mask at the picture's corners, a picture smaller than
    its stride; jobs with a bad shape or a window outside the buffer are
    skipped (their samples keep the buffer's value)."""
    import xavs2_gb300 as xg
    assert gpu.xavs2gpu_intra_fill_edges(None, 0, None, 64, 64, 64, None, 0, None) == 0
    rng = np.random.default_rng(8)
    pic = rng.integers(0, 256, (136, 200), dtype=np.uint8)
    W, H = 184, 128                    # inside a 200-stride, 136-row allocation
    shapes = [(4, 4), (8, 8), (64, 64), (16, 64), (64, 16), (4, 16), (32, 8)]
    pos = [(0, 0), (W - 64, 0), (0, H - 64), (W - 64, H - 64), (8, 8), (W - 4, H - 4), (60, 36)]
    jobs = []
    off = 256
    for bw, bh in shapes:
        for x, y in pos:
            if x + bw > W or y + bh > H:
                x, y = min(x, W - bw), min(y, H - bh)
            for avail in range(32):
                jobs.append((off, x, y, bw, bh, avail))
                off += 512
    bad = [(off, 8, 8, 12, 4, 31), (off + 512, 8, 8, 4, 32, 31), (3, 8, 8, 8, 8, 31),
           (off + 1024 + 400, 8, 8, 64, 64, 31)]
    size = off + 1024 + 500
    arr = np.array(jobs + bad, dtype=[("edge_offset", "<i8"), ("x", "<i4"), ("y", "<i4"), ("width", "<i2"),
                                      ("height", "<i2"), ("avail", "<i4")]).astype(xg.INTRA_EDGE_JOB_DTYPE)
    got = _fill_gpu(gpu, arr, pic, size, W, H, prefill=0x3C)
    want = _fill_oracle(olib, arr, pic, size, W, H, prefill=0x3C)
    assert np.array_equal(got, want)
    assert (got[off:] == 0x3C).all() and (got[:100] == 0x3C).all()

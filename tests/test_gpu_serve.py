"""The serving form (xavs2gpu_server_*): pictures of several streams of
different sizes, batched as they arrive, give per-picture outputs that do
not depend on the batch they shared -- the same checksum when every picture
runs alone (max_batch_frames = 1) and in the mix -- and equal to the
full-picture chain on the same pictures (the chain is pinned against the
oracle in test_gpu_chain.py)."""
import ctypes
import time

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

SIZES = [(192, 136), (128, 64), (256, 200)]
QP, R, NFRAMES = 32, 12, 5


def _streams(xg):
    import xavs2_gb300.synth as synth
    out = []
    for i, (w, h) in enumerate(SIZES):
        rng = np.random.default_rng(100 + i)
        frames = [synth.base_picture(rng, w, h)]
        for _ in range(NFRAMES - 1):
            frames.append(synth.next_picture(rng, frames[-1], 4, 5))
        pus, cus = xg.cu_pus(xg.split_map_cus(w, h, 7 + i), w, h, 2)
        out.append((w, h, frames, pus, cus))
    return out


def _serve(xg, streams, max_frames, target=0):
    prm = xg.MeParams(R, oracle.lambda_factor(QP), 1, 2, 0, 0)
    cfg = xg.ServerConfig(0, 1 << 20, max_frames, QP, prm, hbm_reserve_bytes=0, batch_pixels_target=target)
    srv = xg.Server(cfg)
    ids = [srv.open_stream(w, h, pus, cus, ring=NFRAMES) for (w, h, _, pus, cus) in streams]
    assert all(i >= 0 for i in ids)
    for f in range(NFRAMES):                      # interleaved arrivals
        for sid, (_, _, frames, _, _) in zip(ids, streams):
            assert srv.submit(sid, frames[f], tag=1000 * sid + f) == 0
    got = []
    t0 = time.time()
    while len(got) < NFRAMES * len(streams) and time.time() - t0 < 60:
        got.extend(srv.poll(256, 200).tolist())
    srv.close()
    res = np.array(got, dtype=xg.SERVER_RESULT_DTYPE)
    assert len(res) == NFRAMES * len(streams)
    return {(int(r["stream"]), int(r["frame"])): r for r in res}


def test_server_alone_equals_mixed_and_chain(gpu):
    import xavs2_gb300 as xg
    streams = _streams(xg)
    alone = _serve(xg, streams, 1)
    mixed = _serve(xg, streams, 8)
    assert max(int(r["batch_frames"]) for r in mixed.values()) > 1
    for key, a in alone.items():
        m = mixed[key]
        assert int(a["ref_only"]) == int(m["ref_only"]) == (1 if key[1] < 2 else 0)
        assert int(a["hash"]) == int(m["hash"]), key
        assert m["t_done_ns"] >= m["t_submit_ns"]
    # picture 2 of every stream through the chain (refs = pictures 1, 0)
    lib = xg.load()
    for sid, (w, h, frames, pus, cus) in enumerate(streams):
        sess = xg.MeSession(w, h, 2, len(pus))
        sess.set_pus(pus)
        chain = xg.Chain(sess, cus, QP)
        for idx, img in enumerate([frames[2], frames[1], frames[0]]):
            assert lib.xavs2gpu_copy_h2d(ctypes.c_void_p(chain.source(idx)), oracle.ptr(img), img.nbytes) == 0
        chain.run(xg.MeParams(R, oracle.lambda_factor(QP), 1, 2, 0, 0))
        o = chain.outputs()
        sess.sync()
        recon = np.zeros(w * h, np.uint8)
        coef = np.zeros(o.n_coef, np.int16)
        assert lib.xavs2gpu_copy_d2h(oracle.ptr(recon), ctypes.c_void_p(o.recon), recon.nbytes) == 0
        assert lib.xavs2gpu_copy_d2h(oracle.ptr(coef), ctypes.c_void_p(o.coef), coef.nbytes) == 0
        want = xg.output_hash(recon, coef, sess.results())
        assert int(mixed[(sid, 2)]["hash"]) == want, sid
        chain.close()
        sess.close()


def test_server_batch_target(gpu):
    """A batch target below every picture but the smallest: batches grow to
    the full size only while the backlog exceeds twice the target, a batch's
    first picture always fits, every picture is served, and the outputs equal
    the pictures run alone."""
    import xavs2_gb300 as xg
    streams = _streams(xg)
    alone = _serve(xg, streams, 1)
    small = _serve(xg, streams, 8, target=128 * 64)
    assert set(small) == set(alone)
    for key, a in alone.items():
        assert int(a["hash"]) == int(small[key]["hash"]), key


def test_server_admission_budget(gpu):
    """A stream that does not fit the device-memory budget is refused."""
    import xavs2_gb300 as xg
    w, h, frames, pus, cus = _streams(xg)[1]
    prm = xg.MeParams(R, oracle.lambda_factor(QP), 1, 2, 0, 0)
    srv = xg.Server(xg.ServerConfig(0, 1 << 18, 4, QP, prm))
    used = srv.stats()["hbm_used"]
    srv.close()
    srv = xg.Server(xg.ServerConfig(used + 1, 1 << 18, 4, QP, prm))
    lib = xg.load()
    lib.xavs2gpu_set_abort_on_error(0)
    try:
        assert srv.open_stream(w, h, pus, cus) == -5      # -XAVS2GPU_ERR_CAPACITY
    finally:
        lib.xavs2gpu_clear_error()
        lib.xavs2gpu_set_abort_on_error(1)
    srv.close()


def test_server_admission_free_memory(gpu):
    """Streams are admitted against the device's free memory: with a
    reserve that leaves less free memory than one stream needs, opening it
    is refused; with the default reserve it is admitted, and a stream
    refused earlier does not count against later ones."""
    import torch
    import xavs2_gb300 as xg
    w, h, frames, pus, cus = _streams(xg)[1]
    prm = xg.MeParams(R, oracle.lambda_factor(QP), 1, 2, 0, 0)
    free_b, _ = torch.cuda.mem_get_info()
    lib = xg.load()
    srv = xg.Server(xg.ServerConfig(0, 1 << 18, 4, QP, prm, max(free_b - (1 << 20), 1)))
    lib.xavs2gpu_set_abort_on_error(0)
    try:
        assert srv.open_stream(w, h, pus, cus) == -5      # -XAVS2GPU_ERR_CAPACITY: 1 MiB is not enough
        assert b"free device memory" in lib.xavs2gpu_get_error()
    finally:
        lib.xavs2gpu_clear_error()
        lib.xavs2gpu_set_abort_on_error(1)
    srv.close()
    srv = xg.Server(xg.ServerConfig(0, 1 << 18, 4, QP, prm))
    assert srv.open_stream(w, h, pus, cus) >= 0
    srv.close()

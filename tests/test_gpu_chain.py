"""The full-picture chain (xavs2gpu_chain_*) against the oracle: the motion
search of every leaf-CU PU, each CU's best reference and prediction, the
residual through dct -> quant -> dequant -> idct, and the reconstructed
picture; the captured CUDA graph gives the same outputs as the eager run,
the autotuner's launch shapes change no output, and the feedback loop makes
the reconstruction the next reference."""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

W, H, NREFS, QP = 192, 136, 2, 32


def _pictures(seed=11):
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(seed)
    f0 = synth.base_picture(rng, W, H)
    f1 = synth.next_picture(rng, f0, 4, 6)
    f2 = synth.next_picture(rng, f1, 4, 6)
    return f2, [f1, f0]


def _oracle_chain(cur, refs, pus, cus, prm_tuple, qp):
    olib = oracle.lib()
    stride = W + 160
    flats = [np.ascontiguousarray(oracle.interpolate_frame(olib, r, mode=2).reshape(16, -1)) for r in refs]
    frefs = (ctypes.c_void_p * (16 * len(refs)))(*[oracle.ptr(f[k], 80 * stride + 80).value
                                                   for f in flats for k in range(16)])
    res = np.zeros(len(pus), oracle.RESULT_DTYPE)
    prm = oracle.MeParams(*prm_tuple)
    olib.xo_me_search_list(ctypes.byref(prm), oracle.ptr(pus), len(pus), oracle.ptr(cur), W, frefs, stride,
                           oracle.ptr(res), 1)
    planes = [f.reshape(16, H + 160, W + 160) for f in flats]
    n_res = int((cus["size"].astype(np.int64) ** 2).sum())
    n_coef = int(cus["coef_offset"][-1]) + (1024 if cus["size"][-1] == 64 else int(cus["size"][-1]) ** 2)
    coef = np.zeros(n_coef, np.int16)
    rres = np.zeros(n_res, np.int16)
    nnz = np.zeros(len(cus), np.int32)
    recon = np.zeros((H, W), np.uint8)
    choice = np.zeros(len(cus), [("ref", "<i4"), ("mv_x", "<i2"), ("mv_y", "<i2")])
    part_of = {8: 1, 16: 2, 32: 3, 64: 4}
    for i, c in enumerate(cus):
        x, y, s = int(c["x"]), int(c["y"]), int(c["size"])
        best = 0
        for r in range(NREFS):
            if r == 0 or res["bcost"][c["pu"][r]] < res["bcost"][c["pu"][best]]:
                best = r
        q = res[c["pu"][best]]
        mvx, mvy = int(q["bmv_x"]), int(q["bmv_y"])
        pl = planes[best][((mvy & 3) << 2) + (mvx & 3)]
        pred = pl[80 + y + (mvy >> 2):80 + y + (mvy >> 2) + s, 80 + x + (mvx >> 2):80 + x + (mvx >> 2) + s].astype(np.int32)
        blk = (cur[y:y + s, x:x + s].astype(np.int32) - pred).astype(np.int16).reshape(-1).copy()
        cf = np.zeros(s * s, np.int16)
        nnz[i] = olib.xo_tq_chain(part_of[s], oracle.ptr(blk), oracle.ptr(cf), qp, 0, 0)
        nc = 1024 if s == 64 else s * s
        coef[int(c["coef_offset"]):int(c["coef_offset"]) + nc] = cf[:nc]
        rres[int(c["offset"]):int(c["offset"]) + s * s] = blk
        recon[y:y + s, x:x + s] = np.clip(pred + blk.reshape(s, s), 0, 255)
        choice[i] = (best, mvx, mvy)
    return res, coef, rres, nnz, recon, choice


def _d2h(lib, dev_ptr, n, dtype):
    out = np.zeros(n, dtype)
    assert lib.xavs2gpu_copy_d2h(oracle.ptr(out), ctypes.c_void_p(dev_ptr), out.nbytes) == 0
    return out


def _outputs(lib, chain, n_cus):
    import xavs2_gb300 as xg
    o = chain.outputs()
    lib.xavs2gpu_me_sync(chain.sess.h)
    return (_d2h(lib, o.coef, o.n_coef, np.int16), _d2h(lib, o.recon_residual, o.n_residual, np.int16),
            _d2h(lib, o.nnz, n_cus, np.int32), _d2h(lib, o.recon, W * H, np.uint8).reshape(H, W),
            _d2h(lib, o.choice, n_cus, xg.CHOICE_DTYPE))


def _setup(feedback=False, seed=11):
    import xavs2_gb300 as xg
    cur, refs = _pictures(seed)
    cus_list = xg.split_map_cus(W, H, seed=3, p_split=(0.6, 0.5, 0.5))
    pus, cus = xg.cu_pus(cus_list, W, H, NREFS)
    sess = xg.MeSession(W, H, NREFS, len(pus))
    sess.set_pus(pus)
    chain = xg.Chain(sess, cus, QP, feedback=feedback)
    lib = xg.load()
    for idx, img in enumerate([cur] + refs):
        assert lib.xavs2gpu_copy_h2d(ctypes.c_void_p(chain.source(idx)), oracle.ptr(img), img.nbytes) == 0
    return xg, lib, sess, chain, cur, refs, pus, cus


def test_chain_matches_oracle_and_graph(gpu):
    xg, lib, sess, chain, cur, refs, pus, cus = _setup()
    prm_t = (16, oracle.lambda_factor(QP), 1, 2, 0, 0)
    prm = xg.MeParams(*prm_t)
    chain.run(prm)
    eager = _outputs(lib, chain, len(cus))
    me = sess.results()
    o_me, o_coef, o_rres, o_nnz, o_recon, o_choice = _oracle_chain(cur, refs, pus, cus, prm_t, QP)
    assert me.tobytes() == o_me.tobytes()
    coef, rres, nnz, recon, choice = eager
    assert np.array_equal(choice, o_choice)
    assert np.array_equal(nnz, o_nnz)
    assert np.array_equal(coef, o_coef)
    assert np.array_equal(rres, o_rres)
    assert np.array_equal(recon, o_recon)
    # the captured graph: same outputs, and it holds the chain's kernels
    chain.capture(prm)
    assert chain.graph_kernels() >= 8
    chain.launch()
    graph = _outputs(lib, chain, len(cus))
    for a, b in zip(eager, graph):
        assert np.array_equal(a, b)
    # autotuned launch shapes change nothing
    chain.autotune(prm, reps=1)
    t = chain.tuning()
    assert t.tq_warps in (4, 8) and t.me.refine_block in (64, 128)
    chain.run(prm)
    tuned = _outputs(lib, chain, len(cus))
    for a, b in zip(eager, tuned):
        assert np.array_equal(a, b)
    chain.close()
    sess.close()


def test_chain_feedback_loop(gpu):
    """With feedback the reconstruction becomes reference 0 and reference 0
    moves to slot 1 after each picture."""
    xg, lib, sess, chain, cur, refs, pus, cus = _setup(feedback=True, seed=5)
    prm = xg.MeParams(8, oracle.lambda_factor(QP), 1, 2, 0, 0)
    chain.run(prm)
    _, _, _, recon, _ = _outputs(lib, chain, len(cus))
    src1 = _d2h(lib, chain.source(1), W * H, np.uint8).reshape(H, W)
    src2 = _d2h(lib, chain.source(2), W * H, np.uint8).reshape(H, W)
    assert np.array_equal(src1, recon)
    assert np.array_equal(src2, refs[0])
    chain.close()
    sess.close()

"""The full-picture chain (xavs2gpu_chain_*) against the oracle: the motion
search of every leaf-CU PU; for every inter candidate (each partition mode
of each CU) the prediction from each PU's best reference, the residual
through dct -> quant -> dequant -> idct as one TU and as the mode's four
split TUs (levels, nnz, reconstructed residual, SSD); each CU's choice and
the reconstructed picture; the captured CUDA graph gives the same outputs
as the eager run, the autotuner's launch shapes change no output, and the
feedback loop makes the reconstruction the next reference."""
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


def _oracle_me(cur, refs, pus, prm_tuple):
    olib = oracle.lib()
    h, w = cur.shape
    stride = w + 160
    flats = [np.ascontiguousarray(oracle.interpolate_frame(olib, r, mode=2).reshape(16, -1)) for r in refs]
    frefs = (ctypes.c_void_p * (16 * len(refs)))(*[oracle.ptr(f[k], 80 * stride + 80).value
                                                   for f in flats for k in range(16)])
    res = np.zeros(len(pus), oracle.RESULT_DTYPE)
    prm = oracle.MeParams(*prm_tuple)
    olib.xo_me_search_list(ctypes.byref(prm), oracle.ptr(pus), len(pus), oracle.ptr(cur), w, frefs, stride,
                           oracle.ptr(res), 8)
    return res, [f.reshape(16, h + 160, w + 160) for f in flats]


def check_candidates(out, cur, planes, res, cus, qp, cand_idx):
    """The GPU outputs of the candidates cand_idx against the oracle's
    chain_candidate; returns the oracle's per-candidate results."""
    olib = oracle.lib()
    exp = {}
    for i in cand_idx:
        cd = out["cands"][i]
        e = oracle.chain_candidate(olib, cur, planes, res, cus[int(cd["cu"])], int(cd["mode"]),
                                   int(cd["split_type"]), qp)
        S = int(cus[int(cd["cu"])]["size"])
        assert out["cost"][i] == e["cost"], i
        assert list(out["dist"][i]) == e["dist"], (i, out["dist"][i], e["dist"])
        assert list(out["nnz"][5 * i:5 * i + 5]) == [e["nnz"][0][0]] + e["nnz"][1], i
        ro, co = int(cd["res_offset"]), int(cd["coef_offset"])
        assert np.array_equal(out["rres"][ro:ro + S * S].reshape(S, S), e["rres"][0]), i
        n0 = len(e["levels"][0])
        assert np.array_equal(out["coef"][co:co + n0], e["levels"][0]), i
        n1 = len(e["levels"][1])
        assert np.array_equal(out["coef"][co + n0:co + n0 + n1], e["levels"][1]), i
        # the split TUs' reconstructed residual, TU by TU
        split = out["rres"][ro + S * S:ro + 2 * S * S]
        off = 0
        for (tx, ty, tw, th) in oracle._split_tus(S, int(cd["split_type"])):
            assert np.array_equal(split[off:off + tw * th].reshape(th, tw), e["rres"][1][ty:ty + th, tx:tx + tw]), i
            off += tw * th
        exp[i] = e
    return exp


def check_choices(out, cur, planes, res, cus, qp):
    """Every candidate and every CU's choice and reconstruction."""
    exp = check_candidates(out, cur, planes, res, cus, qp, range(len(out["cands"])))
    first = np.searchsorted(out["cands"]["cu"], np.arange(len(cus)))
    last = np.searchsorted(out["cands"]["cu"], np.arange(len(cus)), side="right")
    recon = np.zeros_like(cur)
    for c in range(len(cus)):
        ks = list(range(first[c], last[c]))
        best = min(ks, key=lambda k: (exp[k]["cost"], k))
        split = int(exp[best]["dist"][1] < exp[best]["dist"][0])
        ch = out["choice"][c]
        assert (int(ch["cand"]), int(ch["mode"]), int(ch["split"])) == (best, int(out["cands"][best]["mode"]), split), c
        x, y, S = int(cus[c]["x"]), int(cus[c]["y"]), int(cus[c]["size"])
        recon[y:y + S, x:x + S] = np.clip(exp[best]["pred"] + exp[best]["rres"][split], 0, 255)
    assert np.array_equal(out["recon"], recon)


def _d2h(lib, dev_ptr, n, dtype):
    out = np.zeros(n, dtype)
    assert lib.xavs2gpu_copy_d2h(oracle.ptr(out), ctypes.c_void_p(dev_ptr), out.nbytes) == 0
    return out


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
    eager = chain.download()
    me = sess.results()
    o_me, planes = _oracle_me(cur, refs, pus, prm_t)
    assert me.tobytes() == o_me.tobytes()
    # every CU has all of its partition modes (8x8: three)
    modes = np.bincount(eager["cands"]["cu"], minlength=len(cus))
    assert (modes == np.where(cus["size"] == 8, 3, 7)).all()
    assert set(np.unique(eager["cands"]["split_type"])) == {1, 2, 3}
    check_choices(eager, cur, planes, o_me, cus, QP)
    # the captured graph: same outputs, and it holds the chain's kernels
    chain.capture(prm)
    assert chain.graph_kernels() >= 8
    chain.launch()
    graph = chain.download()
    for k in eager:
        assert np.array_equal(eager[k], graph[k]), k
    # autotuned launch shapes change nothing
    chain.autotune(prm, reps=1)
    t = chain.tuning()
    assert t.tq_warps in (4, 8) and t.me.refine_block in (64, 128)
    chain.run(prm)
    tuned = chain.download()
    for k in eager:
        assert np.array_equal(eager[k], tuned[k]), k
    chain.close()
    sess.close()


def test_chain_2nx2n_only_cus(gpu):
    """CUs whose partition PUs are not in the PU list have the 2Nx2N
    candidate alone; it is chosen and reconstructed like the others."""
    import xavs2_gb300 as xg
    cur, refs = _pictures(seed=4)
    cus_list = xg.split_map_cus(W, H, seed=9)
    pus, cus = xg.cu_pus(cus_list, W, H, NREFS)
    # keep only the 2Nx2N PUs: re-index the CU records
    keep = np.unique(cus["pu"][:, :NREFS].reshape(-1))
    remap = -np.ones(len(pus), np.int64)
    remap[keep] = np.arange(len(keep))
    pus2 = np.ascontiguousarray(pus[keep])
    cus2 = cus.copy()
    cus2["pu"][:, :NREFS] = remap[cus["pu"][:, :NREFS]]
    sess = xg.MeSession(W, H, NREFS, len(pus2))
    sess.set_pus(pus2)
    chain = xg.Chain(sess, cus2, QP)
    lib = xg.load()
    for idx, img in enumerate([cur] + refs):
        assert lib.xavs2gpu_copy_h2d(ctypes.c_void_p(chain.source(idx)), oracle.ptr(img), img.nbytes) == 0
    prm_t = (8, oracle.lambda_factor(QP), 1, 2, 0, 0)
    chain.run(xg.MeParams(*prm_t))
    out = chain.download()
    assert len(out["cands"]) == len(cus2) and (out["cands"]["mode"] == 0).all()
    o_me, planes = _oracle_me(cur, refs, pus2, prm_t)
    check_choices(out, cur, planes, o_me, cus2, QP)
    chain.close()
    sess.close()


def test_chain_feedback_loop(gpu):
    """With feedback the reconstruction becomes reference 0 and reference 0
    moves to slot 1 after each picture."""
    xg, lib, sess, chain, cur, refs, pus, cus = _setup(feedback=True, seed=5)
    prm = xg.MeParams(8, oracle.lambda_factor(QP), 1, 2, 0, 0)
    chain.run(prm)
    recon = chain.download()["recon"]
    src1 = _d2h(lib, chain.source(1), W * H, np.uint8).reshape(H, W)
    src2 = _d2h(lib, chain.source(2), W * H, np.uint8).reshape(H, W)
    assert np.array_equal(src1, recon)
    assert np.array_equal(src2, refs[0])
    chain.close()
    sess.close()


def test_chain_rejects_bad_cus(gpu):
    """CU lists the chain cannot serve fail at creation with an error: a CU
    off the 8x8 grid, a size other than 8..64, a CU past the picture, a
    2Nx2N PU index of another position."""
    import xavs2_gb300 as xg
    cus_list = xg.split_map_cus(W, H, seed=9)
    pus, cus = xg.cu_pus(cus_list, W, H, NREFS)
    sess = xg.MeSession(W, H, NREFS, len(pus))
    sess.set_pus(pus)
    lib = xg.load()
    lib.xavs2gpu_set_abort_on_error(0)      # report failures instead of aborting
    try:
        for field, value in (("x", 4), ("size", 12), ("y", H)):
            bad = cus.copy()
            bad[field][3] = value
            with pytest.raises(RuntimeError):
                xg.Chain(sess, bad, QP)
        bad = cus.copy()
        bad["pu"][3, 0] = bad["pu"][4, 0]
        with pytest.raises(RuntimeError):
            xg.Chain(sess, bad, QP)
    finally:
        lib.xavs2gpu_clear_error()
        lib.xavs2gpu_set_abort_on_error(1)
    xg.Chain(sess, cus, QP).close()     # the valid list still builds
    sess.close()

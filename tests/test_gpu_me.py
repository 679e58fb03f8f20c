"""Batched motion search on the GPU against the oracle's restatement of
xavs2_me_search (full search + sub-pel refinement), bit-exact."""
import ctypes
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _frames(rng, w, h, shift=(2, -3), noise=5):
    cur = rng.integers(0, 256, (h, w), dtype=np.uint8)
    # smooth it a little so that the search has real minima
    cur = ((cur.astype(np.int32) + np.roll(cur, 1, 0) + np.roll(cur, 1, 1) + np.roll(cur, (1, 1), (0, 1))) // 4).astype(np.uint8)
    ref = np.clip(np.roll(cur, shift, axis=(0, 1)).astype(np.int16) + rng.integers(-noise, noise + 1, (h, w)),
                  0, 255).astype(np.uint8)
    return cur, ref


def _oracle(olib, cur, refs, pus, prm, threads=8):
    h, w = cur.shape
    stride = w + 160
    flats = [np.ascontiguousarray(oracle.interpolate_frame(olib, r, mode=2).reshape(16, -1)) for r in refs]
    frefs = (ctypes.c_void_p * (16 * len(refs)))(
        *[oracle.ptr(f[k], 80 * stride + 80).value for f in flats for k in range(16)])
    out = np.zeros(len(pus), oracle.RESULT_DTYPE)
    oprm = oracle.MeParams(prm.search_range, prm.lambda_factor, prm.use_hadamard, prm.fractional_me,
                           prm.fast_sub_me, prm.enable_pmvr)
    olib.xo_me_search_list(ctypes.byref(oprm), oracle.ptr(pus), len(pus), oracle.ptr(cur), w, frefs, stride,
                           oracle.ptr(out), threads)
    return out


def _run(cur, refs, pus, prm):
    import xavs2_gb300 as xg
    h, w = cur.shape
    s = xg.MeSession(w, h, len(refs), len(pus))
    s.set_picture(-1, cur)
    for i, r in enumerate(refs):
        s.set_picture(i, r)
    s.set_pus(pus)
    assert s.window_tma(), "no tensor map for the window copies"
    s.run(prm)
    out = s.results()
    stats = s.plan_stats()
    s.close()
    return out, stats


def _assert_same(got, exp, pus):
    bad = np.nonzero(got.view(np.uint8).reshape(len(got), -1).any(axis=1) != exp.view(np.uint8).reshape(len(exp), -1).any(axis=1))
    diff = [i for i in range(len(got)) if got[i].tobytes() != exp[i].tobytes()]
    assert not diff, "first mismatches: %s" % [(int(pus[i]["x"]), int(pus[i]["y"]), int(pus[i]["part"]),
                                                 int(pus[i]["ref"]), got[i], exp[i]) for i in diff[:5]]


@pytest.mark.parametrize("R,w,h", [(16, 256, 192), (8, 136, 72), (64, 320, 256), (96, 256, 192)])
def test_ctu_layout_all_pus(gpu, olib, R, w, h):
    """Every PU of the CTU quadtree layout (all 25 shapes), two references,
    MVP (0,0): the shared-window CTU kernel, edge CTUs included.  R = 96 is a
    range where the launch leaves out the TMA staging area (it would cost a
    CTA per SM) and the windows are filled with 16-byte loads."""
    import xavs2_gb300 as xg
    rng = np.random.default_rng(R + w)
    cur, ref0 = _frames(rng, w, h)
    _, ref1 = _frames(rng, w, h, shift=(-3, 4))
    pus = xg.frame_pus(w, h, 2)
    if R >= 64:
        pus = pus[rng.random(len(pus)) < (0.25 if R == 64 else 0.15)]     # keep the CPU oracle quick
    prm = xg.MeParams(R, oracle.lambda_factor(32), 1, 2, 0, 0)
    got, stats = _run(cur, [ref0, ref1], pus, prm)
    assert stats[0] == len(pus) and stats[1] == 0, stats
    exp = _oracle(olib, cur, [ref0, ref1], pus, prm)
    _assert_same(got, exp, pus)


@pytest.mark.parametrize("lam,on_ctu", [(1 << 25, True), (1 << 27, False)])
def test_large_lambda(gpu, olib, lam, on_ctu):
    """Large MV costs: lambda 2^25 keeps the CTU search (its 32-bit keys hold
    costs with MV costs up to 2^14), lambda 2^27 plans every PU for the
    per-PU search; both equal the oracle."""
    import xavs2_gb300 as xg
    rng = np.random.default_rng(lam & 0xffff)
    cur, ref0 = _frames(rng, 136, 72)
    pus = xg.frame_pus(136, 72, 1)
    prm = xg.MeParams(8, lam, 1, 2, 0, 0)
    got, stats = _run(cur, [ref0], pus, prm)
    assert (stats[0] == len(pus)) if on_ctu else (stats[0] == 0), stats
    _assert_same(got, _oracle(olib, cur, [ref0], pus, prm), pus)


def test_generic_pus(gpu, olib):
    """PUs at arbitrary positions with arbitrary predictors take the per-PU
    kernel; both paths in one run."""
    import xavs2_gb300 as xg
    rng = np.random.default_rng(77)
    w, h = 160, 96
    cur, ref0 = _frames(rng, w, h)
    n = 300
    pus = np.zeros(n, xg.PU_DTYPE)
    pus["part"] = rng.integers(0, 25, n)
    pw = np.array(xg.PU_W)[pus["part"]]
    ph = np.array(xg.PU_H)[pus["part"]]
    pus["x"] = (rng.random(n) * (w - pw + 1)).astype(int) // 2 * 2
    pus["y"] = (rng.random(n) * (h - ph + 1)).astype(int)
    pus["mvp_x"] = rng.integers(-40, 41, n)
    pus["mvp_y"] = rng.integers(-40, 41, n)
    pus = xg.set_limits(pus, w, h)
    layout = xg.frame_pus(w, h, 1)[::3]
    allp = np.concatenate([pus, layout])
    for prm in (xg.MeParams(12, oracle.lambda_factor(32), 1, 2, 0, 0),
                xg.MeParams(6, oracle.lambda_factor(40), 0, 1, 0, 0),
                xg.MeParams(10, oracle.lambda_factor(27), 1, 2, 1, 1),
                xg.MeParams(7, oracle.lambda_factor(32), 1, 2, 0, 0),
                xg.MeParams(13, oracle.lambda_factor(35), 0, 2, 0, 0)):
        got, stats = _run(cur, [ref0], allp, prm)
        assert stats[1] >= n
        exp = _oracle(olib, cur, [ref0], allp, prm)
        _assert_same(got, exp, allp)


def test_golden_me(gpu):
    """The GPU reproduces the reference's own xavs2_me_search results stored
    in the golden fixtures."""
    import os
    import xavs2_gb300 as xg
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz"))
    p = [int(v) for v in g["me_params"]]
    prm = xg.MeParams(*p)
    pus = np.ascontiguousarray(g["me_pus"]).view(xg.PU_DTYPE)
    got, _ = _run(g["me_cur"], [g["me_ref"]], pus, prm)
    assert got.tobytes() == g["me_out"].tobytes()


def test_pinned_host_pictures_and_results(gpu):
    """Page-locked host pictures take the asynchronous upload path and a
    page-locked result array the direct download; results equal the
    pageable path's."""
    import torch
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(91)
    w, h = 160, 96
    f0 = synth.base_picture(rng, w, h)
    f1 = synth.next_picture(rng, f0, 4, 5)
    pus = xg.frame_pus(w, h, 1)
    prm = xg.MeParams(8, oracle.lambda_factor(32), 1, 2, 0, 0)
    s = xg.MeSession(w, h, 1, len(pus))
    s.set_pus(pus)
    s.set_picture(-1, f1)
    s.set_picture(0, f0)
    s.run(prm)
    want = s.results()

    def pinned(a):
        t = torch.empty(a.nbytes, dtype=torch.uint8).pin_memory()
        v = t.numpy().view(a.dtype).reshape(a.shape)
        v[...] = a
        return t, v

    keep = [pinned(f1), pinned(f0), pinned(np.zeros(len(pus), xg.RESULT_DTYPE))]
    s2 = xg.MeSession(w, h, 1, len(pus))
    s2.set_pus(pus)
    s2.set_picture(-1, keep[0][1])
    s2.set_picture(0, keep[1][1])
    s2.run(prm)
    got = s2.results(keep[2][1])
    assert got.tobytes() == want.tobytes()
    s.close()
    s2.close()


@pytest.mark.parametrize("had,frac,fast,pmvr", [(1, 2, 0, 0), (0, 2, 0, 0), (1, 1, 0, 0), (1, 2, 1, 0), (0, 0, 0, 0),
                                                (1, 2, 0, 1)])
def test_cu_partition_refinement(gpu, olib, had, frac, fast, pmvr):
    """The partitions of leaf CUs (every mode of 16..64 CUs, 8x8 CUs),
    searched and refined together per CU (CU-grouped refinement; per-PU
    kernels with PMVR), predictors varying between the partitions of a CU,
    content with several motions (partitions that disagree on the centre),
    duplicated searches (groups split at 32 members): equal to the oracle."""
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(300 + 8 * had + 4 * frac + 2 * fast + pmvr)
    w, h = 256, 192
    f0 = synth.base_picture(rng, w, h)
    f1 = synth.next_picture(rng, f0, 6, 6)
    f2 = synth.next_picture(rng, f1, 6, 6)
    pus, _ = xg.cu_pus(xg.split_map_cus(w, h, 17), w, h, 2)
    pus["mvp_x"] = rng.integers(-12, 13, len(pus))
    pus["mvp_y"] = rng.integers(-12, 13, len(pus))
    pus = xg.set_limits(pus, w, h)
    big = np.nonzero(np.array(xg.PU_W)[pus["part"]] == 64)[0][:1]
    dup = np.repeat(pus[big], 40) if len(big) else pus[:0]
    allp = np.concatenate([pus, pus[:200], dup])
    prm = xg.MeParams(10, oracle.lambda_factor(30), had, frac, fast, pmvr)
    got, _ = _run(f2, [f1, f0], allp, prm)
    exp = _oracle(olib, f2, [f1, f0], allp, prm)
    _assert_same(got, exp, allp)


def test_tuning_cu_groups(gpu, olib):
    """The CU-grouped refinement on and off (xavs2gpu_me_set_tuning) give the
    same results; bad tuning values are refused."""
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(5150)
    w, h = 192, 128
    f0 = synth.base_picture(rng, w, h)
    f1 = synth.next_picture(rng, f0, 3, 5)
    pus, _ = xg.cu_pus(xg.split_map_cus(w, h, 23), w, h, 1)
    prm = xg.MeParams(12, oracle.lambda_factor(32), 1, 2, 0, 0)
    s = xg.MeSession(w, h, 1, len(pus))
    s.set_pus(pus)
    s.set_picture(-1, f1)
    s.set_picture(0, f0)
    outs = []
    for groups in (1, 0, 1):
        assert s.lib.xavs2gpu_me_set_tuning(s.h, ctypes.byref(xg.MeTuning(256, 128, groups))) == 0
        t = xg.MeTuning()
        s.lib.xavs2gpu_me_get_tuning(s.h, ctypes.byref(t))
        assert (t.refine_split_px, t.refine_block, t.cu_groups) == (256, 128, groups)
        s.run(prm)
        outs.append(s.results().tobytes())
    assert outs[0] == outs[1] == outs[2]
    s.lib.xavs2gpu_set_abort_on_error(0)
    try:
        assert s.lib.xavs2gpu_me_set_tuning(s.h, ctypes.byref(xg.MeTuning(256, 128, 2))) != 0
    finally:
        s.lib.xavs2gpu_clear_error()
        s.lib.xavs2gpu_set_abort_on_error(1)
    s.close()
    exp = _oracle(olib, f1, [f0], pus, prm)
    assert outs[0] == exp.tobytes()


def test_headline_1080p_sample(gpu, olib):
    """The benchmark's own workload at its own size: 1920x1080, 2 references,
    FS +-64, quarter-pel SATD at QP 32, every PU of the CTU layout searched
    on the GPU; checked against the oracle on a seeded sample of about 3,000
    PU searches made of every PU of six CTUs at the picture's corners and
    bottom edge (the partial 56-row CTU row) plus a random draw over the
    rest."""
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth
    W, H, R = 1920, 1080, 64
    cur, refs = synth.me_workload(seed=1, width=W, height=H)
    pus = xg.frame_pus(W, H, 2)
    prm = xg.MeParams(R, oracle.lambda_factor(32), 1, 2, 0, 0)
    got, stats = _run(cur, refs, pus, prm)
    assert stats[0] == len(pus) and stats[1] == 0, stats
    ctu = (pus["x"] // 64).astype(int) * 1000 + (pus["y"] // 64).astype(int)
    corners = [(0, 0), (29, 0), (0, 16), (29, 16), (14, 16), (15, 8)]
    edge = np.isin(ctu, [cx * 1000 + cy for cx, cy in corners])
    rng = np.random.default_rng(1080)
    rest = np.flatnonzero(~edge)
    idx = np.sort(np.concatenate([np.flatnonzero(edge), rng.choice(rest, 1500, replace=False)]))
    assert (pus["y"][idx] >= 1024).any() and (pus["x"][idx] >= 1856).any()
    sel = np.ascontiguousarray(pus[idx])
    exp = _oracle(olib, cur, refs, sel, prm, threads=os.cpu_count() or 1)
    _assert_same(np.ascontiguousarray(got[idx]), exp, sel)


def test_generic_pus_large_range(gpu, olib):
    """The per-PU search at R = 64 (and the maximum R = 128 on a few PUs):
    every shape with predictors far from (0,0), PUs at the picture corners
    whose windows leave the padded plane, both references."""
    import xavs2_gb300 as xg
    rng = np.random.default_rng(640)
    w, h = 256, 192
    cur, ref0 = _frames(rng, w, h, shift=(5, -7))
    _, ref1 = _frames(rng, w, h, shift=(-9, 3))
    n = 60
    pus = np.zeros(n, xg.PU_DTYPE)
    pus["part"] = np.arange(n) % 25
    pw = np.array(xg.PU_W)[pus["part"]]
    ph = np.array(xg.PU_H)[pus["part"]]
    corner = np.arange(n) % 3
    pus["x"] = np.where(corner == 0, 0, np.where(corner == 1, w - pw, (rng.random(n) * (w - pw + 1)).astype(int)))
    pus["y"] = np.where(corner == 0, h - ph, np.where(corner == 1, 0, (rng.random(n) * (h - ph + 1)).astype(int)))
    pus["ref"] = np.arange(n) % 2
    mvx = rng.integers(-120, 121, n)
    pus["mvp_x"] = np.where(np.abs(mvx) < 3, 9, mvx)     # never rounds to (0, 0): the per-PU path
    pus["mvp_y"] = rng.integers(-120, 121, n)
    pus = xg.set_limits(pus, w, h)
    for prm in (xg.MeParams(64, oracle.lambda_factor(32), 1, 2, 0, 0),
                xg.MeParams(128, oracle.lambda_factor(30), 0, 2, 0, 0)):
        sel = pus if prm.search_range == 64 else pus[::6].copy()
        got, stats = _run(cur, [ref0, ref1], sel, prm)
        assert stats[1] == len(sel)
        exp = _oracle(olib, cur, [ref0, ref1], sel, prm, threads=os.cpu_count() or 1)
        _assert_same(got, exp, sel)

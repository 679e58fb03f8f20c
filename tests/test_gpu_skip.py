"""Skip / direct rough cost on the GPU (xavs2gpu_skip_costs) against the
oracle: SA8D of single- and bi-predicted candidates with one or four PUs
from the session's sub-pel planes, rdcost with the reference's rounding,
repeated motion left unevaluated, the first strictly smallest per CU."""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _planes(olib, refs):
    h, w = refs[0].shape
    stride = w + 160
    flats = [np.ascontiguousarray(oracle.interpolate_frame(olib, r, mode=2).reshape(16, -1)) for r in refs]
    tab = (ctypes.c_void_p * (16 * len(refs)))(*[oracle.ptr(f[k], 80 * stride + 80).value for f in flats
                                                 for k in range(16)])
    return flats, tab, stride


@pytest.mark.parametrize("w,h,nrefs", [(256, 192, 2), (136, 72, 1), (320, 128, 3), (416, 240, 2)])
def test_skip_costs(gpu, olib, w, h, nrefs):
    import torch
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(w + h + nrefs)
    frames = [synth.base_picture(rng, w, h)]
    for _ in range(nrefs):
        frames.append(synth.next_picture(rng, frames[-1], 2, 4))
    cur, refs = frames[-1], frames[-2::-1][:nrefs]
    cands, n_cu = synth.skip_candidates(rng, w, h, nrefs, motion=(-4, 6), cand_dtype=xg.SKIP_CAND_DTYPE)
    # malformed candidates: outside the picture, no list, a reference beyond the session
    cands[7]["x"] = w - 4
    cands[11]["ref"][0] = (-1, -1)
    cands[13]["ref"][0, 0] = nrefs
    # the last candidate predicts from the last reference at quarter-pel (3, 3)
    # with its block ending exactly at the bottom-right plane margin (the
    # word-wise plane readers then touch the end of the planes' allocation;
    # at 416x240 a plane's bytes are a multiple of 256)
    last = cands[-1]
    S = 1 << int(last["size_log2"])
    last["n_pu"] = 1
    last["ref"][:] = -1
    last["ref"][0, 0] = nrefs - 1
    last["mv"][0, 0] = (4 * (w + 80 - S - int(last["x"])) + 3, 4 * (h + 80 - S - int(last["y"])) + 3)
    cands[-1] = last
    lam = 17.375
    flats, tab, stride = _planes(olib, refs)
    e_dist = np.zeros(len(cands), np.int32)
    e_cost = np.zeros(len(cands))
    e_best = np.zeros(n_cu, np.int32)
    olib.xo_skip_costs(oracle.ptr(cur), w, tab, stride, w, h, nrefs, oracle.ptr(cands), len(cands), lam, n_cu,
                       oracle.ptr(e_dist), oracle.ptr(e_cost), oracle.ptr(e_best))
    assert (e_dist == -1).sum() > 3 and (e_dist > 0).sum() > len(cands) // 2
    assert e_dist[-1] > 0
    sess = xg.MeSession(w, h, nrefs, 1)
    sess.set_picture(-1, cur)
    for i, r in enumerate(refs):
        sess.set_picture(i, r)
    sess.sync()
    d_c = torch.from_numpy(cands.view(np.uint8).copy()).cuda()
    d_dist = torch.zeros(len(cands), dtype=torch.int32, device="cuda")
    d_cost = torch.zeros(len(cands), dtype=torch.float64, device="cuda")
    d_best = torch.zeros(n_cu, dtype=torch.int32, device="cuda")
    rc = gpu.xavs2gpu_skip_costs(ctypes.c_void_p(sess.h), ctypes.c_void_p(d_c.data_ptr()), len(cands), lam,
                                 n_cu, ctypes.c_void_p(d_dist.data_ptr()), ctypes.c_void_p(d_cost.data_ptr()),
                                 ctypes.c_void_p(d_best.data_ptr()), None)
    assert rc == 0
    sess.sync()
    assert np.array_equal(d_dist.cpu().numpy(), e_dist)
    assert np.array_equal(d_cost.cpu().numpy(), e_cost)
    assert np.array_equal(d_best.cpu().numpy(), e_best)
    sess.close()

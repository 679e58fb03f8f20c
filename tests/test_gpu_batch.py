"""Several motion-search sessions -- pictures of different sizes, each with
its own references and PU list -- searched by one launch of each kernel
(xavs2gpu_me_batch_run): every session's results equal its own
xavs2gpu_me_run; reference rotation keeps the search equal to a session
loaded in the rotated order."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _session(xg, w, h, seed, leaf=True):
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(seed)
    f0 = synth.base_picture(rng, w, h)
    f1 = synth.next_picture(rng, f0, 4, 5)
    f2 = synth.next_picture(rng, f1, 4, 5)
    if leaf:
        pus, _ = xg.cu_pus(xg.split_map_cus(w, h, seed), w, h, 2)
    else:
        pus = xg.frame_pus(w, h, 2)
    s = xg.MeSession(w, h, 2, len(pus))
    s.set_pus(pus)
    s.set_picture(-1, f2)
    s.set_picture(0, f1)
    s.set_picture(1, f0)
    return s, (f2, f1, f0)


@pytest.mark.parametrize("R", [8, 16])
def test_batch_equals_single_sessions(gpu, R):
    import xavs2_gb300 as xg
    sizes = [(192, 136, True), (128, 64, False), (256, 200, True)]
    sess = [_session(xg, w, h, 40 + i, leaf)[0] for i, (w, h, leaf) in enumerate(sizes)]
    prm = xg.MeParams(R, oracle.lambda_factor(32), 1, 2, 0, 0)
    alone = []
    for s in sess:
        s.run(prm)
        alone.append(s.results())
    for s in sess:   # clobber: the batch must recompute everything
        s.run(xg.MeParams(R, oracle.lambda_factor(40), 0, 1, 0, 0))
        s.sync()
    batch = xg.MeBatch()
    for s in sess:
        s.set_stream(sess[0].stream())
    batch.run(sess, prm, sess[0].stream())
    for s, a in zip(sess, alone):
        assert s.results().tobytes() == a.tobytes()
    for s in sess:
        s.set_stream(None)
    batch.close()
    for s in sess:
        s.close()


def test_rotate_refs(gpu):
    import xavs2_gb300 as xg
    s, (f2, f1, f0) = _session(xg, 160, 96, 7)
    prm = xg.MeParams(8, oracle.lambda_factor(32), 1, 2, 0, 0)
    # after a rotation, slot 1 holds what slot 0 held; load f0 into slot 0
    s.rotate_refs()
    s.set_picture(0, f0)
    s.run(prm)
    got = s.results()
    t = xg.MeSession(160, 96, 2, s.n)
    t.set_pus(s._pus)
    t.set_picture(-1, f2)
    t.set_picture(0, f0)
    t.set_picture(1, f1)
    t.run(prm)
    assert got.tobytes() == t.results().tobytes()
    s.close()
    t.close()

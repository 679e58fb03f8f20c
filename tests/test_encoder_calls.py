"""The config-0 oracle on the CPU: primitive calls recorded from a real xavs2
encode (tests/golden/encoder_calls.npz) replay bit-exactly through the
oracle's restatements, and -- where the reference sources are present -- the
fixture equals a fresh recording and the reference encoder's bitstream is
unchanged when the oracle's functions replace its primitive table."""
import hashlib
import os
import sys

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import encoder_calls as ec            # noqa: E402
import make_encoder_calls as mk       # noqa: E402

need_ref = pytest.mark.skipif(not mk.reference_available(), reason="reference sources not present")


@pytest.fixture(scope="module")
def fixture():
    return np.load(mk.FIXTURE)


@pytest.mark.parametrize("preset", sorted(mk.PRESETS))
def test_recorded_calls_replay_through_oracle(fixture, preset):
    records, counts = ec.parse(fixture["records_p%d" % preset].tobytes())
    assert len(records) > 1000
    entry = ec.oracle_entry(oracle.lib())
    for fill in (0, 0xA5):    # bytes outside the recorded regions must not matter
        done, skipped, bad = ec.replay(records, entry, fill)
        assert not skipped, skipped
        assert not bad, bad[:10]
    assert sum(done.values()) == len(records)
    # every recorded entry was called by the encoder, and the sample holds
    # at least one call of every entry it called
    called = {(ec.KINDS[k], s) for k, s in zip(*np.nonzero(counts))}
    sampled = {(r[0], r[1]) for r in records}
    assert sampled == called


def test_recorded_calls_cover_the_table(fixture):
    """Between them the two presets exercise the hot-path entries the
    library replaces: every SAD / SATD shape, the DCTs of every TU shape,
    all 33 intra modes, quant/dequant, the interpolation planes and blocks,
    deblocking and SAO."""
    kinds = set()
    per_kind = {}
    for preset in mk.PRESETS:
        records, _ = ec.parse(fixture["records_p%d" % preset].tobytes())
        for r in records:
            kinds.add(r[0])
            per_kind.setdefault(r[0], set()).add(r[1])
    for k in ("sad", "satd", "ssd", "sad_x3", "sad_x4", "sub_ps", "add_ps", "avg", "copy_pp", "dct", "idct",
              "quant", "dequant", "intra", "luma_hor_x3", "luma_block_ext", "chroma_block_ext", "deblock_luma",
              "deblock_chroma", "sao", "t4_2nd", "t_2nd"):
        assert k in kinds, k
    assert len(per_kind["sad"]) == 25 and len(per_kind["satd"]) == 25
    assert len(per_kind["intra"]) == 33
    assert len(per_kind["dct"]) == 11 and len(per_kind["idct"]) == 11


@need_ref
def test_fixture_equals_fresh_recording(fixture, tmp_path):
    runs = mk.record_all(str(tmp_path))
    for preset, (blob, bs) in runs.items():
        assert blob == fixture["records_p%d" % preset].tobytes(), "preset %d" % preset
        assert hashlib.sha256(bs).digest() == fixture["bitstream_sha256_p%d" % preset].tobytes()


@need_ref
@pytest.mark.parametrize("preset", sorted(mk.PRESETS))
def test_oracle_table_keeps_the_bitstream(tmp_path, preset):
    """The oracle's functions installed in the reference encoder's table the
    way the GPU drop-ins are installed (after xavs2_init_all_primitives)
    leave every byte of the bitstream unchanged."""
    mk.build_recorder()
    yuv = str(tmp_path / "config0.yuv")
    mk.write_sequence(yuv)
    plain, _ = mk.run_encoder("plain", preset, str(tmp_path), yuv)
    replaced, side = mk.run_encoder("oracle", preset, str(tmp_path), yuv)
    assert len(side.splitlines()) > 300        # entries replaced by the oracle
    assert replaced == plain

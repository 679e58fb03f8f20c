"""The config-0 oracle on the GPU: every primitive call recorded from a real
xavs2 encode (tests/golden/encoder_calls.npz: the reference encoder at
presets 0 and 9 on the seeded 416x240 sequence) replayed through the GPU
library's drop-in tables -- filled by its table initialisers, as an encoder
installs them -- with the encoder's own strides, aliasing (in-place
transforms) and wavelet flag bits; every written region and return value
must equal the reference's."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import encoder_calls as ec            # noqa: E402

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(HERE, "golden", "encoder_calls.npz")


@pytest.mark.parametrize("preset", [0, 9])
def test_recorded_encoder_calls_replay_on_gpu(gpu, preset):
    records, _ = ec.parse(np.load(FIXTURE)["records_p%d" % preset].tobytes())
    entry = ec.gpu_entry(gpu)
    for fill in (0, 0xA5):
        done, skipped, bad = ec.replay(records, entry, fill)
        assert not skipped, skipped
        assert not bad, bad[:10]
        assert sum(done.values()) == len(records)
    assert gpu.xavs2gpu_get_status() == 0

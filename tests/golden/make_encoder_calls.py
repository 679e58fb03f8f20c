"""Records the config-0 oracle: the primitive-table calls of a real xavs2
encode, written to tests/golden/encoder_calls.npz.  TEST INFRASTRUCTURE ONLY.

The reference encoder is built from its own source files by oracle/Makefile
(target _ref/xavs2_record, with oracle/enc_record.c as its driver) and run
on the seeded config-0 sequence (8 pictures of 416x240, 4:2:0,
xavs2_gb300.synth.config0_sequence) with the reference's random-access
configuration (config/encoder_ra.cfg), QP 32, one frame thread and one row
thread, at two presets:

* preset 0 -- the configuration the workload names; every sampled call is
  kept;
* preset 9 -- the slowest preset, which reaches entries preset 0 never calls
  (SATD, every PU shape, the non-square TUs, SAO, the plane-level x3
  interpolation); six records per entry are kept.

The fixture also keeps each run's bitstream digest and per-entry call
counts.  Run: python tests/golden/make_encoder_calls.py (needs the
reference sources; XAVS2_REF_SRC overrides the recipe's location).
"""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import oracle                       # noqa: E402
import encoder_calls as ec          # noqa: E402

FIXTURE = os.path.join(HERE, "encoder_calls.npz")
RECORDER = os.path.join(ROOT, "oracle", "_ref", "xavs2_record")
PRESETS = {0: None, 9: 6}           # preset -> records kept per entry (None: all)
WIDTH, HEIGHT, FRAMES, QP, SEED = 416, 240, 8, 32, 0


def reference_available():
    return os.path.isdir(oracle.REF_SRC)


def build_recorder():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "REF_SRC=" + oracle.REF_SRC,
                    "_ref/xavs2_record", "liboracle.so"], check=True)
    return RECORDER


def write_sequence(path):
    import xavs2_gb300.synth as synth
    with open(path, "wb") as f:
        for planes in synth.config0_sequence(FRAMES, WIDTH, HEIGHT, seed=SEED):
            for p in planes:
                f.write(np.ascontiguousarray(p).tobytes())


def run_encoder(mode, preset, workdir, yuv):
    """Runs the reference encoder in `mode` (plain, record, oracle); returns
    (bitstream bytes, side-file bytes)."""
    cfg = os.path.join(os.path.dirname(oracle.REF_SRC), "config", "encoder_ra.cfg")
    bs = os.path.join(workdir, "%s_%d.avs" % (mode, preset))
    side = os.path.join(workdir, "%s_%d.side" % (mode, preset))
    args = [RECORDER, mode, side, "--", "-f", cfg, "-p", "preset=%d" % preset, "-p", "initial_qp=%d" % QP,
            "-p", "input=" + yuv, "-p", "output=" + bs, "-p", "frames=%d" % FRAMES, "-p", "ThreadFrames=1",
            "-p", "ThreadRows=1", "-p", "LogLevel=0", "-p", "ReconFile=" + os.devnull,
            "-p", "SourceWidth=%d" % WIDTH, "-p", "SourceHeight=%d" % HEIGHT]
    subprocess.run(args, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    with open(bs, "rb") as f, open(side, "rb") as g:
        return f.read(), g.read()


def record_all(workdir):
    """{preset: (selected records blob, plain bitstream)} from fresh runs."""
    build_recorder()
    yuv = os.path.join(workdir, "config0.yuv")
    write_sequence(yuv)
    out = {}
    for preset, keep in PRESETS.items():
        plain, _ = run_encoder("plain", preset, workdir, yuv)
        recorded_bs, raw = run_encoder("record", preset, workdir, yuv)
        if recorded_bs != plain:
            raise RuntimeError("the recorder changed the bitstream at preset %d" % preset)
        out[preset] = (ec.select(raw, keep), plain)
    return out


def main():
    if not reference_available():
        raise SystemExit("reference sources not found; set XAVS2_REF_SRC")
    with tempfile.TemporaryDirectory() as d:
        runs = record_all(d)
    arrays = {}
    for preset, (blob, bs) in runs.items():
        arrays["records_p%d" % preset] = np.frombuffer(blob, np.uint8)
        arrays["bitstream_sha256_p%d" % preset] = np.frombuffer(hashlib.sha256(bs).digest(), np.uint8)
        arrays["bitstream_bytes_p%d" % preset] = np.array(len(bs), np.int64)
    np.savez_compressed(FIXTURE, **arrays)
    for preset, (blob, bs) in runs.items():
        recs, counts = ec.parse(blob)
        print("preset %d: %d records, %d table entries called, %d calls, bitstream %d bytes"
              % (preset, len(recs), int((counts > 0).sum()), int(counts.sum()), len(bs)))
    print("wrote", FIXTURE, os.path.getsize(FIXTURE), "bytes")


if __name__ == "__main__":
    main()

"""Times the reference's own motion search (xavs2_me_search, full-search mode,
through oracle/_ref's xr_me_search_list) beside the oracle's C port
(xo_me_search_list) on the same sample of the 1080p batched-search workload
(2 references, FS +-64, quarter-pel SATD at QP 32), with the same thread
count, and checks that both return identical results.  TEST INFRASTRUCTURE:
it needs the reference sources (the reference build), so it runs where they
are; the port is what the GPU host times as its CPU baseline.

Run: python oracle/time_me_search.py [--fraction 0.005] [--threads N]
"""
import argparse
import ctypes
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle                      # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--fraction", type=float, default=0.005)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--seed", type=int, default=7)
    args = ap.parse_args()
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth
    oracle.build(with_ref=True)
    olib, rlib = oracle.lib(), oracle.ref_lib()
    W, H, R = 1920, 1080, 64
    cur, refs = synth.me_workload(seed=1, width=W, height=H)
    pus = xg.frame_pus(W, H, 2)
    rng = np.random.default_rng(args.seed)
    sel = np.ascontiguousarray(pus[rng.random(len(pus)) < args.fraction])
    stride = W + 160
    flats = [np.ascontiguousarray(oracle.interpolate_frame(olib, r, mode=2).reshape(16, -1)) for r in refs]
    frefs = (ctypes.c_void_p * 32)(*[oracle.ptr(f[k], 80 * stride + 80).value for f in flats for k in range(16)])
    prm = oracle.MeParams(R, oracle.lambda_factor(32), 1, 2, 0, 0)
    out = {}
    for name, fn in (("port", olib.xo_me_search_list), ("reference", rlib.xr_me_search_list)):
        res = np.zeros(len(sel), oracle.RESULT_DTYPE)
        t0 = time.perf_counter()
        fn(ctypes.byref(prm), oracle.ptr(sel), len(sel), oracle.ptr(cur), W, frefs, stride, oracle.ptr(res),
           args.threads)
        out[name] = (time.perf_counter() - t0, res)
    same = out["port"][1].tobytes() == out["reference"][1].tobytes()
    evals = int(((2 * R) ** 2 + 18) * len(sel))
    line = {"sample_pu_searches": int(len(sel)), "threads": args.threads,
            "port_s": out["port"][0], "reference_s": out["reference"][0],
            "port_evals_per_s": evals / out["port"][0], "reference_evals_per_s": evals / out["reference"][0],
            "reference_over_port_time": out["reference"][0] / out["port"][0], "results_identical": same}
    print(json.dumps(line))
    if not same:
        sys.exit("results differ")


if __name__ == "__main__":
    main()

#!/usr/bin/env python
"""Benchmark: bit-exact batched motion-search block-cost evaluation.

Workload (one step = one picture): 1920x1080 8-bit luma, two reference
pictures (k-1, k-2), synthetic content with 16 block-local motions
U[-32, 32] px in quarter-pel steps.  Every PU of the CU-quadtree layout of
every CTU (all 25 AVS2 PU shapes, 849 per CTU, those fully inside the
picture) is searched against both references: integer full search over
[-64, 64)^2 around the best of {MVP, (0,0)} with SAD + lambda*MV bits, then
half- and quarter-pel refinement with SATD + lambda*MV bits at QP 32 (P
picture lambda), exactly as xavs2_me_search + me_subpel_refine.  A step also
loads the three pictures and computes the 15 sub-pel planes of both
references.

Metric: block-cost evaluations per second (one evaluation = one (PU,
reference, candidate) cost: MVP/zero candidates, every full-search position
inside the PU's search limits, and the 17 sub-pel costs).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NREFS, RANGE, QP = 2, 64, 32
METRIC = "bit-exact block-cost evals/s (1080p batched ME, 2 refs, FS +-64 + quarter-pel SATD)"
UNIT = "evals/s"


def lambda_factor(qp, factor=0.68):
    lam = 2.0 ** ((qp - 11) / 4.0) * factor
    return int(65536.0 * np.sqrt(lam) + 0.5)


def count_evals(pus, R, frac=2, hadamard=1):
    """Evaluations per search: 1 candidate (MVP rounds to (0,0)), every
    full-search position inside the limits, 1 + 8 + 8 sub-pel costs."""
    nx = np.minimum(pus["max_x"].astype(np.int64), R - 1) - np.maximum(pus["min_x"].astype(np.int64), -R) + 1
    ny = np.minimum(pus["max_y"].astype(np.int64), R - 1) - np.maximum(pus["min_y"].astype(np.int64), -R) + 1
    sub = (1 if hadamard else 0) + 8 + (8 if frac > 1 else 0)
    return int((1 + np.clip(nx, 0, None) * np.clip(ny, 0, None) + sub).sum())


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region.  start()
    returns once the first sample has arrived, so that a timed region
    shorter than the sampling interval still has the sample that opens it."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line)

    def start(self):
        import threading
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.reader = threading.Thread(target=self._read, daemon=True)
        self.reader.start()
        t0 = time.time()
        while not self.lines and self.proc.poll() is None and time.time() - t0 < 10:
            time.sleep(0.01)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            self.proc.wait()
        self.reader.join(timeout=5)
        text = "".join(self.lines)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in text.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch / step
# of the dominant kernels at the default configurations, from one ncu capture
# of each workload; None for other configurations
MEASURED_TRAFFIC = {
    "me": 15083008 + 5165824,          # fs_ctu_kernel<0> + <1>, one picture
    "tq": 5013000000,                  # tq_chain_kernel, 10^6 blocks (scaled from 10^5)
    "intra": 39612928 + 31689984,      # rmd_tile_kernel
    "lookahead": 8311040,              # lookahead_kernel (16x4 strips)
    "skip": 106347008 + 5720832,       # skip_cost_kernel
    "loopfilter": 14746368,            # loopfilter_lcu_kernel (deblocking + SAO in one pass)
}


def measured_traffic(name, default_config):
    return MEASURED_TRAFFIC.get(name) if default_config else None


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0}, "fallback"


def cpu_sample_search(pus, cur, refs, prm_tuple, fraction, seed, threads, want_results=False):
    """The oracle's restatement of xavs2_me_search over a random sample of
    the PU list, on `threads` host threads; returns (evals, seconds, sample
    size) and, with want_results, the sampled indices and their results."""
    import oracle
    olib = oracle.lib()
    rng = np.random.default_rng(seed)
    idx = np.flatnonzero(rng.random(len(pus)) < fraction)
    sel = np.ascontiguousarray(pus[idx])
    h, w = cur.shape
    stride = w + 160
    flats = [np.ascontiguousarray(oracle.interpolate_frame(olib, r, mode=2).reshape(16, -1)) for r in refs]
    frefs = (ctypes.c_void_p * (16 * len(refs)))(*[oracle.ptr(f[k], 80 * stride + 80).value
                                                   for f in flats for k in range(16)])
    out = np.zeros(len(sel), oracle.RESULT_DTYPE)
    prm = oracle.MeParams(*prm_tuple)
    t0 = time.perf_counter()
    olib.xo_me_search_list(ctypes.byref(prm), oracle.ptr(sel), len(sel), oracle.ptr(cur), w, frefs, stride,
                           oracle.ptr(out), threads)
    dt = time.perf_counter() - t0
    if want_results:
        return count_evals(sel, prm_tuple[0]), dt, len(sel), idx, out
    return count_evals(sel, prm_tuple[0]), dt, len(sel)


def parity_check(gpu_results, idx, oracle_results, what):
    """Compares the GPU's results at the sampled indices with the oracle's
    (byte for byte: every field of every result); returns the bench line's
    parity object."""
    got = np.ascontiguousarray(gpu_results[idx]).view(np.uint8).reshape(len(idx), -1)
    exp = np.ascontiguousarray(oracle_results).view(np.uint8).reshape(len(idx), -1)
    bad = np.flatnonzero((got != exp).any(axis=1))
    return {"checked": int(len(idx)), "mismatches": int(len(bad)), "against": "oracle", "sample": what,
            "first_mismatch": int(idx[bad[0]]) if len(bad) else None}


def sm_count():
    """SM count of the current CUDA device (the integer roofs scale with it)."""
    import torch
    return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count


def reduce_max(value, device):
    """Max of a per-rank scalar over all ranks (replicas: the slowest rank
    sets the job's time); the value itself without a process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank, seconds_per_rank, device):
    """Whole-job throughput of independent replicas: all ranks' units over
    the slowest rank's time."""
    import torch.distributed as dist
    world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    return units_per_rank * world / reduce_max(seconds_per_rank, device)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def run_reference(args):
    WIDTH, HEIGHT = args.width, args.height
    """CPU arm: the oracle port of the reference's search (the reference tree
    itself is not on this machine), all host threads, a bounded random sample
    of the picture's PU searches per step."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import xavs2_gb300.synth as synth
    import xavs2_gb300 as xg
    cur, refs = synth.me_workload(seed=1, width=WIDTH, height=HEIGHT)
    pus = xg.frame_pus(WIDTH, HEIGHT, NREFS)
    prm = (RANGE, lambda_factor(QP), 1, 2, 0, 0)
    threads = os.cpu_count() or 1
    frac = args.cpu_fraction
    for i in range(args.warmup):
        cpu_sample_search(pus, cur, refs, prm, frac / 4, 100 + i, threads)
    ev = 0
    tt = 0.0
    n = 0
    for i in range(args.steps):
        e, dt, k = cpu_sample_search(pus, cur, refs, prm, frac, 200 + i, threads)
        ev += e
        tt += dt
        n += k
    value = ev / tt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic", "config": {"workload": "me_1080p_2ref_fs64_qpel_satd", "width": WIDTH,
                                            "height": HEIGHT, "refs": NREFS, "search_range": RANGE, "qp": QP},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "per step a random %.2f%% of the picture's %d PU searches" % (100 * frac, len(pus))},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def per_pu_line(pus, phases, n_gen, peaks, peak_src):
    """The per-PU search's share and rate: PU-area absolute differences
    (w*h per displacement, (2R)^2 displacements) of the PUs whose predictor
    does not round to (0,0) -- the PUs outside the CTU plan -- per second of
    the per-PU kernel, against the same integer roof as the CTU search."""
    import xavs2_gb300 as xg
    off = ((pus["mvp_x"].astype(np.int64) + 2) >> 2 != 0) | ((pus["mvp_y"].astype(np.int64) + 2) >> 2 != 0)
    area = (np.asarray(xg.PU_W)[pus["part"][off]] * np.asarray(xg.PU_H)[pus["part"][off]]).astype(np.int64).sum()
    ms = float(phases[2])
    px = float(area) * (2 * RANGE) ** 2
    peak = sm_count() * 64 * 4 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
    ach = px / (ms / 1e3) / 1e12 if ms > 0 and n_gen else 0.0
    return {"pus": int(n_gen), "kernel_ms": ms, "share_of_step": ms / float(sum(phases)) if sum(phases) else 0.0,
            "achieved": ach, "peak": peak, "unit": "Tpx-absdiff/s (PU area)", "frac": ach / peak,
            "peak_source": peak_src}


def temporal_mvps(xg, pus, refs, W, H, prm):
    """Predictors from the previous picture's motion, the way an encoder's
    temporal candidate supplies one: the previous picture (refs[0]) is
    searched against the one before it (refs[1]) with zero predictors, and
    every PU of the current picture takes the vector its co-located PU
    found there, scaled by the temporal distance of its reference (x1 for
    reference 0, x2 for reference 1) and kept inside its search limits."""
    per_ref = len(pus) // NREFS
    prev = xg.MeSession(W, H, NREFS, len(pus))
    prev.set_picture(-1, refs[0])
    for r in range(NREFS):
        prev.set_picture(r, refs[1])
    prev.set_pus(pus)
    prev.run(prm)
    res = prev.results()[:per_ref]
    prev.close()
    out = pus.copy()
    for r in range(NREFS):
        sl = slice(r * per_ref, (r + 1) * per_ref)
        mx = res["bmv_x"].astype(np.int64) * (r + 1)
        my = res["bmv_y"].astype(np.int64) * (r + 1)
        out["mvp_x"][sl] = np.clip(mx, 4 * out["min_x"][sl], 4 * out["max_x"][sl])
        out["mvp_y"][sl] = np.clip(my, 4 * out["min_y"][sl], 4 * out["max_y"][sl])
    return out


# The other measured configurations, run once each in a child process after
# the config-1 measurement of a default single-GPU run, so that one default
# run also carries configs 2-4: the batched TU chain, the 4K full-picture
# chain, and the 64-stream server with the configuration's FS +-64 job and
# with the serving-size FS +-16 search (4 s of arrivals each).  A child that
# fails or runs past its limit is recorded as such; the config-1 line stands.
OTHER_CONFIGS = {
    "config2_tq": ["--workload", "tq", "--steps", "5", "--warmup", "3"],
    "config3_chain": ["--workload", "chain", "--steps", "5", "--warmup", "3"],
    "config4_serve_fs64": ["--workload", "serve", "--serve-seconds", "4", "--serve-warm", "1"],
    "config4_serve_fs16": ["--workload", "serve", "--serve-range", "16", "--serve-seconds", "4", "--serve-warm", "1"],
}


def condense(d):
    keep = {k: d[k] for k in ("metric", "value", "unit", "ms_per_step", "higher_is_better", "parity",
                              "sample_bit_exact", "offered_pictures", "submit_failures") if k in d}
    if isinstance(d.get("e2e"), dict):
        keep["e2e"] = {k: d["e2e"][k] for k in ("value", "unit") if k in d["e2e"]}
    if isinstance(d.get("roofline"), dict):
        keep["roofline"] = {k: d["roofline"][k] for k in ("bound", "kernel", "achieved", "peak", "unit", "frac")
                            if k in d["roofline"]}
    if isinstance(d.get("batched"), dict):
        keep["served"] = {k: d["batched"][k] for k in ("p50_ms", "p99_ms", "frames_per_s", "mean_batch_frames")
                          if k in d["batched"]}
    if isinstance(d.get("cpu_baseline"), dict):
        keep["cpu_baseline"] = {k: d["cpu_baseline"][k] for k in ("value", "unit", "cores", "kind")
                                if k in d["cpu_baseline"]}
    if isinstance(d.get("clocks"), dict):
        keep["clocks"] = {k: d["clocks"][k] for k in ("sm_mhz", "reasons") if k in d["clocks"]}
    return keep


def other_configs(limit_s=300):
    out = {}
    for name, extra in OTHER_CONFIGS.items():
        t0 = time.time()
        try:
            r = subprocess.run([sys.executable, os.path.abspath(__file__)] + extra, capture_output=True, text=True,
                               timeout=limit_s)
            lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
            if r.returncode != 0 or not lines:
                out[name] = {"error": "exit status %d" % r.returncode, "tail": (r.stderr or r.stdout)[-400:]}
            else:
                out[name] = condense(json.loads(lines[-1]))
        except subprocess.TimeoutExpired:
            out[name] = {"error": "no line within %d s" % limit_s}
        out[name]["wall_s"] = round(time.time() - t0, 1)
        out[name]["command"] = "python bench.py " + " ".join(extra)
    return out


def run_ours(args):
    import torch
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth

    WIDTH, HEIGHT = args.width, args.height
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = xg.load()
    lib.xavs2gpu_init(local)

    cur, refs = synth.me_workload(seed=1 + rank, width=WIDTH, height=HEIGHT)
    if args.me_leaf:
        # the serving-shaped search (device timing only): every partition of
        # the leaf CUs of a seeded split map, FS +-16, content panned by a
        # global quarter-pel motion
        if not args.quick:
            raise SystemExit("--me-leaf is a --quick (device timing) workload")
        frames = serve_content(WIDTH, HEIGHT, 3, 52)
        cur, refs = frames[2], [frames[1], frames[0]]
        pus, _ = xg.cu_pus(xg.split_map_cus(WIDTH, HEIGHT, 1002), WIDTH, HEIGHT, NREFS)
        prm = xg.MeParams(16, lambda_factor(QP), 1, 2, 0, 0)
        evals = count_evals(pus, 16)
    else:
        pus = xg.frame_pus(WIDTH, HEIGHT, NREFS)
        prm = xg.MeParams(RANGE, lambda_factor(QP), 1, 2, 0, 0)
        if args.mvp == "temporal":
            pus = temporal_mvps(xg, pus, refs, WIDTH, HEIGHT, prm)
        evals = count_evals(pus, RANGE)
    sess = xg.MeSession(WIDTH, HEIGHT, NREFS, len(pus))
    sess.set_pus(pus)
    stream = torch.cuda.ExternalStream(sess.stream())
    d_cur = torch.from_numpy(cur).cuda()
    d_refs = [torch.from_numpy(r).cuda() for r in refs]
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")   # > L2 (129 MB)
    torch.cuda.synchronize()

    def step_device():
        sess.set_picture_device(-1, d_cur.data_ptr(), WIDTH)
        for i, r in enumerate(d_refs):
            sess.set_picture_device(i, r.data_ptr(), WIDTH)
        sess.run(prm)

    # the library's autotuner picks the refinement launch shapes (results do
    # not depend on them) before the warm-up
    step_device()
    tune_ms, tuning = sess.autotune(prm, reps=2)
    for _ in range(args.warmup):
        step_device()
    sess.sync()
    # correctness spot check against the last warm-up (cheap: a few PUs)
    res = sess.results()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- device-resident timing: per-step events, L2 flushed between steps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clk = ClockSampler(local)
    launches0 = lib.xavs2gpu_kernel_launches()
    barrier()
    clk.start()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            step_device()
            ends[i].record(stream)
    sess.sync()
    barrier()
    clocks = clk.stop()
    launches = lib.xavs2gpu_kernel_launches() - launches0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = float(sum(step_ms))
    total_ms = reduce_max(total_ms, "cuda")
    value = evals * world * args.steps / (total_ms / 1e3)

    # ---- per-kernel timing on the session stream (separate pass)
    sess.set_profiling(True)
    phases = np.zeros(4)
    interp_ms = 0.0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.zero_()
            ev0.record(stream)
            for j, r in enumerate(d_refs):
                sess.set_picture_device(j, r.data_ptr(), WIDTH)
            ev1.record(stream)
            sess.set_picture_device(-1, d_cur.data_ptr(), WIDTH)
            sess.run(prm)
            phases += np.array(sess.phase_ms())
            interp_ms += ev0.elapsed_time(ev1)
    sess.set_profiling(False)
    phases /= args.steps
    interp_ms /= args.steps
    n_ctu, n_gen, n_jobs = sess.plan_stats()

    peaks, peak_src = measured_peaks()
    n_pos = (2 * RANGE) ** 2
    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": total_ms / args.steps,
                              "kernels_ms": list(phases), "interp_ms": interp_ms,
                              "config": {"width": WIDTH, "height": HEIGHT, "leaf_partitions": bool(args.me_leaf),
                                         "search_range": prm.search_range, "pus": int(len(pus))},
                              "autotuned": list(tuning), "plan": [n_ctu, n_gen, n_jobs]}))
        sess.close()
        return
    # ---- end to end through the C ABI with host buffers: the pictures and
    # the result array live in page-locked host memory
    h2d = WIDTH * HEIGHT * (1 + NREFS)
    d2h = len(pus) * xg.RESULT_DTYPE.itemsize

    def pinned(a):
        t = torch.empty(a.nbytes, dtype=torch.uint8).pin_memory()
        v = t.numpy().view(a.dtype).reshape(a.shape)
        v[...] = a
        return t, v

    keep = [pinned(cur)] + [pinned(r) for r in refs] + [pinned(np.zeros(len(pus), xg.RESULT_DTYPE))]
    h_cur, h_refs, out = keep[0][1], [k[1] for k in keep[1:1 + NREFS]], keep[-1][1]
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        sess.set_picture(-1, h_cur)
        for j, r in enumerate(h_refs):
            sess.set_picture(j, r)
        sess.run(prm)
        sess.results(out)
    barrier()
    e2e_s = time.perf_counter() - t0
    e2e_s = reduce_max(e2e_s, "cuda")
    e2e = evals * world * args.steps / e2e_s
    same = bool(np.array_equal(out, res))

    # ---- per-call drop-in (one SAD per call, host buffers)
    rng = np.random.default_rng(5)
    a = rng.integers(0, 256, (64, 64), dtype=np.uint8)
    b = rng.integers(0, 256, (64, 64), dtype=np.uint8)
    f = xg.pixel_fn("sad", 2)
    expect_sad = int(np.abs(a[:16, :16].astype(np.int32) - b[:16, :16].astype(np.int32)).sum())
    per_call_modes = {}
    for mode in (0, 1):            # staged copies; blocks read in place where the device allows it
        lib.xavs2gpu_set_percall_mode(mode)
        for _ in range(50):
            f(xg.ptr(a), 64, xg.ptr(b), 64)
        if f(xg.ptr(a), 64, xg.ptr(b), 64) != expect_sad:
            sys.exit("bench: per-call SAD differs from the host sum (mode %d)" % mode)
        n_calls = 2000
        t0 = time.perf_counter()
        for _ in range(n_calls):
            f(xg.ptr(a), 64, xg.ptr(b), 64)
        per_call_modes[mode] = n_calls / (time.perf_counter() - t0)
    per_call_in_place = lib.xavs2gpu_percall_in_place()
    per_call = per_call_modes[1]

    if rank != 0:
        return
    # roofline of the dominant kernel (shared-window CTU search): the
    # algorithmic work is 4096 absolute differences (one 64x64 CTU) per
    # (CTU, reference, displacement); the SM peak is the device's SMs x 64
    # lanes/clk of VABSDIFF4 (4 pixels each, half the INT32 issue rate) x max
    # SM clock.
    ctu_px = n_jobs * n_pos * 4096
    ctu_ms = phases[1]
    achieved = ctu_px / (ctu_ms / 1e3) / 1e12
    peak = sm_count() * 64 * 4 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
    # interpolation (HBM-bound): 15 planes written with their margin + the source read, per reference
    plane_bytes = (WIDTH + 160) * (HEIGHT + 160)
    interp_bytes = NREFS * (15 * plane_bytes + WIDTH * HEIGHT)
    interp_gbs = interp_bytes / (interp_ms / 1e3) / 1e9

    cpu_e, cpu_s, cpu_n, cpu_idx, cpu_res = cpu_sample_search(pus, cur, refs, (RANGE, prm.lambda_factor, 1, 2, 0, 0),
                                                              args.cpu_fraction, 7, os.cpu_count() or 1,
                                                              want_results=True)
    # the timed run's results (last warm-up; the e2e run's download equals
    # it) against the oracle on the CPU sample: every field of every sampled
    # PU search, border CTUs and the partial bottom CTU row included
    parity = parity_check(res, cpu_idx, cpu_res, "the CPU baseline's random %.2f%% of the picture's PU searches"
                          % (100 * args.cpu_fraction))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": "me_1080p_2ref_fs64_qpel_satd" + ("_temporal_mvp" if args.mvp == "temporal" else ""),
                   "mvp": "zero" if args.mvp == "zero" else "previous picture's co-located vectors, distance-scaled",
                   "width": WIDTH, "height": HEIGHT, "refs": NREFS,
                   "search_range": RANGE, "qp": QP, "pus_per_picture": int(len(pus)),
                   "evals_per_step": evals, "l2": "flushed between steps (512 MiB write)",
                   "autotuned": {"refine_split_px": tuning[0], "refine_block": tuning[1], "cu_groups": tuning[2],
                                 "search_ms": tune_ms},
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "results_equal_device_run": same},
        "gpu_launches": int(launches),
        "roofline": {"bound": "int", "kernel": "fs_ctu_kernel", "achieved": achieved, "peak": peak,
                     "unit": "Tpx-absdiff/s", "frac": achieved / peak,
                     "traffic": measured_traffic("me", (WIDTH, HEIGHT, RANGE) == (1920, 1080, 64)),
                     "peak_source": "%d SMs x 64 VABSDIFF4 lanes/clk x 4 px x sm_max_mhz (%s)" % (sm_count(), peak_src),
                     "work_per_launch": "%d CTU-ref jobs x %d displacements x 4096 px" % (n_jobs, n_pos),
                     "kernel_ms": ctu_ms},
        "kernels_ms": {"candidates": phases[0], "ctu_search": phases[1], "per_pu_search": phases[2],
                       "subpel_refine": phases[3], "interpolation_2refs": interp_ms},
        "interpolation_roofline": {"bound": "hbm", "achieved": interp_gbs, "peak": peaks.get("hbm_gbs"),
                                   "unit": "GB/s", "frac": interp_gbs / peaks.get("hbm_gbs", 6800.0)},
        "plan": {"ctu_pus": n_ctu, "per_pu_pus": n_gen, "ctu_jobs": n_jobs},
        "per_pu_search": per_pu_line(pus, phases, n_gen, peaks, peak_src),
        "per_call": {"value": per_call, "unit": UNIT, "what": "xavs2gpu_pixel_sad_16x16 with host buffers",
                     "staged_value": per_call_modes[0],
                     "in_place": bool(per_call_in_place)},
        "cpu_baseline": {"value": cpu_e / cpu_s, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                         "sample": "random %.2f%% (%d) of the picture's PU searches, oracle C port, OpenMP"
                                   % (100 * args.cpu_fraction, cpu_n)},
        "parity": parity,
        "clocks": clocks,
    }
    sess.close()
    if (args.configs and world == 1 and not args.quick and args.mvp == "zero"
            and (WIDTH, HEIGHT) == (1920, 1080)):
        torch.cuda.empty_cache()
        line["other_configs"] = other_configs()
    print(json.dumps(line))
    if parity["mismatches"] or not same:
        sys.exit("bench: motion-search results differ from the oracle on %d of %d sampled PU searches"
                 " (e2e equal to device run: %s)" % (parity["mismatches"], parity["checked"], same))


# ---- batched transform + quant ---------------------------------------------
TQ_METRIC = "bit-exact TU blocks/s (batched dct->quant->dequant->idct, 10^6 blocks, TU 4..64)"


def tq_bytes(blocks):
    """Algorithmic bytes of a batch: residual in, levels out, recon out
    (int16 each), the 32-byte descriptor and the 4-byte nnz per block."""
    import xavs2_gb300 as xg
    w = np.asarray(xg.PU_W)[blocks["part"]].astype(np.int64)
    h = np.asarray(xg.PU_H)[blocks["part"]].astype(np.int64)
    size = w * h
    ncoef = np.where((w == 64) | (h == 64), size // 4, size)
    return int((2 * size + 2 * ncoef + 2 * size).sum() + 36 * len(blocks))


def cpu_sample_tq(blocks, residual, fraction, seed, threads):
    """The oracle's chain over a random sample of the blocks; returns
    (blocks done, seconds, sample descriptors, levels, recon, nnz)."""
    import oracle
    import xavs2_gb300 as xg
    olib = oracle.lib()
    rng = np.random.default_rng(seed)
    sel = np.ascontiguousarray(blocks[rng.random(len(blocks)) < fraction])
    # repack the sample so its buffers are small
    w = np.asarray(xg.PU_W)[sel["part"]].astype(np.int64)
    h = np.asarray(xg.PU_H)[sel["part"]].astype(np.int64)
    size = w * h
    ncoef = np.where((w == 64) | (h == 64), size // 4, size)
    src_off = sel["offset"].copy()
    sel["offset"] = np.cumsum(size) - size
    sel["coef_offset"] = np.cumsum(ncoef) - ncoef
    idx = np.concatenate([np.arange(o, o + n) for o, n in zip(src_off, size)]) if len(sel) else np.zeros(0, np.int64)
    res = np.ascontiguousarray(residual[idx])
    coef = np.zeros(int(ncoef.sum()), np.int16)
    rec = np.zeros(int(size.sum()), np.int16)
    nnz = np.zeros(len(sel), np.int32)
    t0 = time.perf_counter()
    olib.xo_tq_batch(oracle.ptr(sel), len(sel), oracle.ptr(res), oracle.ptr(coef), oracle.ptr(rec),
                     oracle.ptr(nnz), threads)
    dt = time.perf_counter() - t0
    return len(sel), dt, sel, src_off, coef, rec, nnz


def run_tq(args):
    import torch
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth

    rank, world, local = dist_env()
    n = args.tq_blocks
    parts = tuple(int(x) for x in args.tq_parts.split(","))
    blocks, nres, ncoef, zero = synth.tq_blocks(n, seed=3 + rank, parts=parts)
    algo_bytes = tq_bytes(blocks)
    cfg = {"workload": "tq_batch_1e6_tu4to64", "blocks": n, "tu_sizes": "4,8,16,32,64 uniform",
           "qp": "uniform 22..51", "secondary_4x4": "50% of 4x4 blocks", "zero_blocks": "10%",
           "l2": "inputs larger than L2 (%.1f GB per step)" % (algo_bytes / 1e9)}
    if args.impl == "reference":
        if rank != 0:
            return
        res = synth.tq_residual(blocks, zero, nres, seed=4 + rank).numpy()
        threads = os.cpu_count() or 1
        for i in range(args.warmup):
            cpu_sample_tq(blocks, res, args.cpu_fraction / 4, 100 + i, threads)
        done = 0
        tt = 0.0
        for i in range(args.steps):
            k, dt, *_ = cpu_sample_tq(blocks, res, args.cpu_fraction, 200 + i, threads)
            done += k
            tt += dt
        value = done / tt
        print(json.dumps({"impl": "reference", "metric": TQ_METRIC, "value": value, "unit": "blocks/s",
                          "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": 1e3 * tt / args.steps, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "int16", "data": "synthetic", "config": cfg,
                          "cpu_baseline": {"value": value, "unit": "blocks/s", "cores": threads, "kind": "port",
                                           "sample": "per step a random %.2f%% of the %d blocks" %
                                                     (100 * args.cpu_fraction, n)},
                          "e2e": {"value": value, "unit": "blocks/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}))
        return

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = xg.load()
    lib.xavs2gpu_init(local)
    dev = torch.device("cuda", local)
    d_res = synth.tq_residual(blocks, zero, nres, seed=4 + rank, device=dev)
    d_blocks = torch.from_numpy(blocks.view(np.uint8).copy()).to(dev)
    d_coef = torch.empty(ncoef, dtype=torch.int16, device=dev)
    d_rec = torch.empty(nres, dtype=torch.int16, device=dev)
    d_nnz = torch.empty(n, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(dev)
    tq = xg.fn("xavs2gpu_tq_batch")

    def step(s):
        rc = tq(d_blocks.data_ptr(), n, d_res.data_ptr(), d_coef.data_ptr(), d_rec.data_ptr(), d_nnz.data_ptr(),
                s.cuda_stream)
        assert rc == 0

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step(stream)
    barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clk = ClockSampler(local)
    launches0 = lib.xavs2gpu_kernel_launches()
    clk.start()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            starts[i].record(stream)
            step(stream)
            ends[i].record(stream)
    barrier()
    clocks = clk.stop()
    launches = lib.xavs2gpu_kernel_launches() - launches0
    step_ms = [s_.elapsed_time(e) for s_, e in zip(starts, ends)]
    total_ms = float(sum(step_ms))
    total_ms = reduce_max(total_ms, dev)
    value = n * world * args.steps / (total_ms / 1e3)
    kernel_ms = min(step_ms)
    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": TQ_METRIC, "value": value, "unit": "blocks/s", "ms_per_step": kernel_ms,
                              "GBs": algo_bytes / (kernel_ms / 1e3) / 1e9, "parts": args.tq_parts, "blocks": n}))
        return

    # end to end through the host-buffer entry (xavs2gpu_tq_batch_host):
    # page-locked descriptors and residual in, levels + recon + nnz out, the
    # copies overlapped with the chain in chunks
    h_res = d_res.cpu().pin_memory()
    h_blocks = torch.from_numpy(blocks.view(np.uint8).copy()).pin_memory()
    h_coef = torch.empty(ncoef, dtype=torch.int16).pin_memory()
    h_rec = torch.empty(nres, dtype=torch.int16).pin_memory()
    h_nnz = torch.empty(n, dtype=torch.int32).pin_memory()
    tq_host = xg.fn("xavs2gpu_tq_batch_host")

    # what the host link itself moves: one page-locked copy of the residual
    # array each way, and both directions at once on two streams (before the
    # host entry runs, which then overwrite the output arrays)
    link = {}
    tmp = torch.empty_like(d_res)
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    nbytes = d_res.numel() * 2
    for name, pairs in (("h2d", [(tmp, h_res, s_in)]), ("d2h", [(h_rec, d_res, s_out)]),
                        ("both", [(tmp, h_res, s_in), (h_rec, d_res, s_out)])):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for dst, src, st in pairs:
            with torch.cuda.stream(st):
                dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        link[name] = nbytes * len(pairs) / (time.perf_counter() - t0) / 1e9
    del tmp
    # both forms of the host entry: chunked copies, and the chain reading and
    # writing the page-locked arrays in place (chunks = 0); the faster one is
    # the e2e figure, both are reported
    host_forms = {}
    for chunks in (args.tq_chunks, 0):
        args_chunks = chunks

        def step_host_c():
            rc = tq_host(h_blocks.data_ptr(), n, h_res.data_ptr(), h_coef.data_ptr(), h_rec.data_ptr(),
                         h_nnz.data_ptr(), args_chunks)
            assert rc == 0
        step_host_c()    # device buffers of the host entry allocated outside the timed region
        barrier()
        t0 = time.perf_counter()
        for i in range(args.steps):
            step_host_c()
        barrier()
        host_forms[chunks] = reduce_max(time.perf_counter() - t0, dev)
    best_chunks = min(host_forms, key=host_forms.get)
    e2e_s = host_forms[best_chunks]
    e2e = n * world * args.steps / e2e_s
    if rank != 0:
        return
    # bit-exactness of a random sample against the oracle (the sample timed
    # as the CPU baseline)
    res_np = h_res.numpy()
    k, cpu_s, sel, src_off, coef, rec, nnz = cpu_sample_tq(blocks, res_np, args.cpu_fraction, 7,
                                                          os.cpu_count() or 1)
    g_coef, g_rec, g_nnz = h_coef.numpy(), h_rec.numpy(), h_nnz.numpy()
    idx = np.searchsorted(blocks["offset"], src_off)
    exact = bool(np.array_equal(g_nnz[idx], nnz))
    for j in range(len(sel)):
        b = blocks[idx[j]]
        o, co = int(b["offset"]), int(b["coef_offset"])
        n_in = xg.PU_W[int(b["part"])] * xg.PU_H[int(b["part"])]
        n_c = n_in // 4 if n_in == 4096 else n_in
        so, sco = int(sel["offset"][j]), int(sel["coef_offset"][j])
        if not (np.array_equal(g_rec[o:o + n_in], rec[so:so + n_in]) and
                np.array_equal(g_coef[co:co + n_c], coef[sco:sco + n_c])):
            exact = False
            break
    peaks, peak_src = measured_peaks()
    achieved = algo_bytes / (kernel_ms / 1e3) / 1e9
    line = {
        "metric": TQ_METRIC, "value": value, "unit": "blocks/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int16", "data": "synthetic", "config": cfg,
        "e2e": {"value": e2e, "unit": "blocks/s", "h2d_bytes_per_step": int(2 * nres + 32 * n),
                "d2h_bytes_per_step": int(2 * ncoef + 2 * nres + 4 * n),
                "call": "xavs2gpu_tq_batch_host, page-locked buffers, %s" %
                        ("in place over the host link (chunks = 0)" if best_chunks == 0 else "%d chunks" % best_chunks),
                "host_link_gbs": (4 * nres + 2 * ncoef + 36 * n) * args.steps / e2e_s / 1e9,
                "host_link_copy_gbs": link,
                "forms_s_per_step": {("in_place" if k == 0 else "chunks_%d" % k): v / args.steps
                                     for k, v in host_forms.items()}},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "tq_batch", "achieved": achieved,
                     "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                     "frac": achieved / peaks.get("hbm_gbs", 6800.0),
                     "traffic": measured_traffic("tq", n == 1000000 and args.tq_parts == "0,1,2,3,4"),
                     "peak_source": peak_src, "algorithmic_bytes_per_launch": algo_bytes,
                     "kernel_ms": kernel_ms},
        "sample_bit_exact": exact,
        "cpu_baseline": {"value": k / cpu_s, "unit": "blocks/s", "cores": os.cpu_count() or 1, "kind": "port",
                         "sample": "random %.2f%% (%d) of the blocks, oracle C chain, OpenMP"
                                   % (100 * args.cpu_fraction, k)},
        "clocks": clocks,
    }
    print(json.dumps(line))
    if not exact:
        sys.exit("bench: sampled outputs differ from the oracle")


# ---- intra rough mode decision over every CU level of a 1080p picture --------
INTRA_METRIC = ("bit-exact intra RMD mode-samples/s (1080p, every CU level 64..4 + SDIP strips, 33 modes, "
                "SATD + lambda*bits, rough candidate search)")
# integer-op model of one mode-sample: 4-tap filter (4 multiply-adds + round /
# shift), difference, 2-D 4-point Hadamard (4 add/sub), |x| accumulate
INTRA_OPS_PER_SAMPLE = 11


def intra_workload(rank, width, height):
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(61 + rank)
    src = synth.base_picture(rng, width, height)
    recon = np.clip(src.astype(np.int32) + rng.integers(-3, 4, src.shape), 0, 255).astype(np.uint8)
    rects = synth.intra_level_blocks(width, height)
    blocks, jobs, size = synth.intra_fill_jobs(rects, width, height, rng, xg.INTRA_BLOCK_DTYPE,
                                               xg.INTRA_EDGE_JOB_DTYPE)
    prm = xg.IntraParams(np.sqrt(2.0 ** ((QP - 11) / 4.0) * 0.68), 1, 1, synth.INTRA_DIST2, synth.INTRA_DIST1)
    return src, recon, blocks, jobs, size, prm


def cpu_sample_intra(blocks, jobs, size, recon, src, prm, fraction, seed, threads):
    """The oracle's edge filling and batched RMD over a random sample of the
    blocks; returns (mode-samples done, seconds, sample indices, results)."""
    import oracle
    import xavs2_gb300 as xg
    rng = np.random.default_rng(seed)
    idx = np.nonzero(rng.random(len(blocks)) < fraction)[0]
    sel = np.ascontiguousarray(blocks[idx])
    sjobs = np.ascontiguousarray(jobs[idx])
    edges = np.zeros(size, np.uint8)
    out = np.zeros(len(sel), xg.INTRA_RESULT_DTYPE)
    lib = oracle.lib()
    t0 = time.perf_counter()
    lib.xo_intra_fill_edges(oracle.ptr(sjobs), len(sjobs), oracle.ptr(recon), recon.shape[1], recon.shape[1],
                            recon.shape[0], oracle.ptr(edges), size)
    lib.xo_intra_rmd_batch(oracle.ptr(sel), len(sel), oracle.ptr(edges), oracle.ptr(src), src.shape[1],
                           prm.lambda_, prm.use_hadamard, prm.rough, prm.dist2, prm.dist1, oracle.ptr(out), threads)
    dt = time.perf_counter() - t0
    done = int((sel["width"].astype(np.int64) * sel["height"]).sum()) * 33
    return done, dt, idx, out


def run_intra(args):
    import torch
    import xavs2_gb300 as xg

    rank, world, local = dist_env()
    W, H = args.width, args.height
    src, recon, blocks, jobs, esize, prm = intra_workload(rank, W, H)
    n = len(blocks)
    mode_samples = int((blocks["width"].astype(np.int64) * blocks["height"]).sum()) * 33
    cfg = {"workload": "intra_rmd_1080p_all_levels", "width": W, "height": H, "blocks": n,
           "shapes": "64x64,32x32,16x16,8x8,4x4,32x8,8x32,16x4,4x16 tiling the picture", "qp": QP,
           "rough": {"dist2": prm.dist2, "dist1": prm.dist1}, "cost": "SATD",
           "content": "blurred-noise picture, edges from a +-3 noisy reconstruction",
           "edges": "built on the device from the reconstruction each step (fill_reference_samples, "
                    "encoder availability: picture bounds + z-scan within the 64x64 LCU)",
           "l2": "flushed between steps (512 MB write)"}
    if args.impl == "reference":
        if rank != 0:
            return
        threads = os.cpu_count() or 1
        frac = min(1.0, 8 * args.cpu_fraction)
        cpu_sample_intra(blocks, jobs, esize, recon, src, prm, frac / 4, 100, threads)
        done, tt = 0, 0.0
        for i in range(args.steps):
            k, dt, *_ = cpu_sample_intra(blocks, jobs, esize, recon, src, prm, frac, 200 + i, threads)
            done += k
            tt += dt
        value = done / tt
        print(json.dumps({"impl": "reference", "metric": INTRA_METRIC, "value": value, "unit": "mode-samples/s",
                          "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": 1e3 * tt / args.steps, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "u8", "data": "synthetic", "config": cfg,
                          "cpu_baseline": {"value": value, "unit": "mode-samples/s", "cores": threads,
                                           "kind": "port",
                                           "sample": "per step a random %.2f%% of the %d blocks (edge fill + RMD)"
                                                     % (100 * frac, n)},
                          "e2e": {"value": value, "unit": "mode-samples/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}))
        return

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = xg.load()
    lib.xavs2gpu_init(local)
    dev = torch.device("cuda", local)
    h_blocks = torch.from_numpy(blocks.view(np.uint8).copy()).pin_memory()
    h_jobs = torch.from_numpy(jobs.view(np.uint8).copy()).pin_memory()
    h_recon = torch.from_numpy(np.ascontiguousarray(recon).reshape(-1)).pin_memory()
    h_src = torch.from_numpy(np.ascontiguousarray(src).reshape(-1)).pin_memory()
    out_bytes = n * xg.INTRA_RESULT_DTYPE.itemsize
    h_out = torch.empty(out_bytes, dtype=torch.uint8).pin_memory()
    d_blocks, d_jobs, d_recon, d_src = h_blocks.to(dev), h_jobs.to(dev), h_recon.to(dev), h_src.to(dev)
    d_edges = torch.zeros(esize, dtype=torch.uint8, device=dev)
    d_out = torch.empty(out_bytes, dtype=torch.uint8, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(dev)
    rmd = lib.xavs2gpu_intra_rmd_batch
    fill = lib.xavs2gpu_intra_fill_edges

    def fill_step(s):
        rc = fill(ctypes.c_void_p(d_jobs.data_ptr()), n, ctypes.c_void_p(d_recon.data_ptr()), W, W, H,
                  ctypes.c_void_p(d_edges.data_ptr()), esize, ctypes.c_void_p(s.cuda_stream))
        assert rc == 0

    def step(s):
        fill_step(s)
        rc = rmd(ctypes.c_void_p(d_blocks.data_ptr()), n, ctypes.c_void_p(d_edges.data_ptr()),
                 ctypes.c_void_p(d_src.data_ptr()), W, ctypes.byref(prm), ctypes.c_void_p(d_out.data_ptr()),
                 ctypes.c_void_p(s.cuda_stream))
        assert rc == 0

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step(stream)
    barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clk = ClockSampler(local)
    launches0 = lib.xavs2gpu_kernel_launches()
    clk.start()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            step(stream)
            ends[i].record(stream)
    barrier()
    clocks = clk.stop()
    launches = lib.xavs2gpu_kernel_launches() - launches0
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_ms = reduce_max(float(sum(step_ms)), dev)
    value = mode_samples * world * args.steps / (total_ms / 1e3)
    kernel_ms = float(np.median(step_ms))
    # the edge filling alone (events around it, L2 flushed before each)
    f0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    f1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.zero_()
            f0[i].record(stream)
            fill_step(stream)
            f1[i].record(stream)
    barrier()
    fill_ms = float(np.median([x.elapsed_time(y) for x, y in zip(f0, f1)]))
    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": INTRA_METRIC, "value": value, "ms_per_step": kernel_ms, "fill_ms": fill_ms,
                              "blocks": n}))
        return

    # end to end with host buffers: descriptors, reconstruction and source in, results out
    barrier()
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            d_blocks.copy_(h_blocks, non_blocking=True)
            d_jobs.copy_(h_jobs, non_blocking=True)
            d_recon.copy_(h_recon, non_blocking=True)
            d_src.copy_(h_src, non_blocking=True)
            step(stream)
            h_out.copy_(d_out, non_blocking=True)
        stream.synchronize()
    barrier()
    e2e_s = reduce_max(time.perf_counter() - t0, dev)
    e2e = mode_samples * world * args.steps / e2e_s
    if rank != 0:
        return
    got = h_out.numpy().view(xg.INTRA_RESULT_DTYPE)
    import oracle
    want_edges = np.zeros(esize, np.uint8)
    oracle.lib().xo_intra_fill_edges(oracle.ptr(jobs), n, oracle.ptr(recon), W, W, H, oracle.ptr(want_edges), esize)
    edges_exact = bool(np.array_equal(d_edges.cpu().numpy(), want_edges))
    done, cpu_s, idx, want = cpu_sample_intra(blocks, jobs, esize, recon, src, prm, args.cpu_fraction, 7,
                                              os.cpu_count() or 1)
    exact = bool(np.array_equal(got[idx]["cost"], want["cost"]) and
                 np.array_equal(got[idx]["cand_mode"], want["cand_mode"]) and
                 np.array_equal(got[idx]["num_for_rdo"], want["num_for_rdo"]))
    peaks, peak_src = measured_peaks()
    rmd_ms = max(kernel_ms - fill_ms, 1e-6)
    achieved = mode_samples / (rmd_ms / 1e3) / 1e12
    peak = sm_count() * 128 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / INTRA_OPS_PER_SAMPLE / 1e12
    line = {
        "metric": INTRA_METRIC, "value": value, "unit": "mode-samples/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic", "config": cfg,
        "e2e": {"value": e2e, "unit": "mode-samples/s",
                "h2d_bytes_per_step": int(h_blocks.numel() + h_jobs.numel() + h_recon.numel() + h_src.numel()),
                "d2h_bytes_per_step": int(out_bytes)},
        "gpu_launches": int(launches),
        "fill_edges_ms": fill_ms, "edges_bit_exact": edges_exact,
        "roofline": {"bound": "int", "kernel": "intra_rmd_batch (sort, tiles, candidates)", "achieved": achieved, "peak": peak,
                     "unit": "T mode-samples/s", "frac": achieved / peak,
                     "traffic": measured_traffic("intra", (W, H) == (1920, 1080)),
                     "peak_source": "%d SMs x 128 INT32 lanes/clk x sm_max_mhz / %d ops per mode-sample (%s)"
                                    % (sm_count(), INTRA_OPS_PER_SAMPLE, peak_src),
                     "work_per_launch": "%d blocks, %d mode-samples" % (n, mode_samples),
                     "kernel_ms": rmd_ms},
        "sample_bit_exact": exact,
        "cpu_baseline": {"value": done / cpu_s, "unit": "mode-samples/s", "cores": os.cpu_count() or 1,
                         "kind": "port", "sample": "random %.2f%% (%d) of the blocks, oracle C edge fill + RMD, OpenMP"
                                                   % (100 * args.cpu_fraction, len(idx))},
        "clocks": clocks,
    }
    print(json.dumps(line))
    if not exact:
        sys.exit("bench: sampled outputs differ from the oracle")


# ---- in-loop filters: 4K 4:2:0 deblocking + SAO -----------------------------------
LF_METRIC = "bit-exact 3840x2160 4:2:0 pictures/s (deblocking + SAO, per-8x8 edge parameters, LCU 64)"


def lf_workload(rank, width, height):
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(71 + rank)
    y, u, v, scus = synth.deblock_picture(rng, width, height)
    lcus = synth.sao_params(rng, width, height, 6)
    return y, u, v, scus, lcus


def cpu_lf(y, u, v, scus, lcus, width, height):
    """The oracle's picture deblocking (reference LCU order), the copy and the
    SAO of one picture on one core; returns (seconds, y, u, v)."""
    import oracle
    olib = oracle.lib()
    ey, eu, ev = y.copy(), u.copy(), v.copy()
    t0 = time.perf_counter()
    olib.xo_deblock_picture(oracle.ptr(ey), width, oracle.ptr(eu), oracle.ptr(ev), width // 2, width, height,
                            oracle.ptr(scus), 6, 1)
    src = [ey.copy(), eu.copy(), ev.copy()]
    dptr = (ctypes.c_void_p * 3)(*[oracle.ptr(p).value for p in (ey, eu, ev)])
    sptr = (ctypes.c_void_p * 3)(*[oracle.ptr(p).value for p in src])
    olib.xo_sao_picture(dptr, sptr, width, width // 2, width, height, 6, oracle.ptr(lcus))
    return time.perf_counter() - t0, ey, eu, ev


def run_loopfilter(args):
    import torch
    import xavs2_gb300 as xg

    rank, world, local = dist_env()
    W, H = args.chain_width, args.chain_height
    y, u, v, scus, lcus = lf_workload(rank, W, H)
    pic_bytes = y.nbytes + u.nbytes + v.nbytes
    cfg = {"workload": "loopfilter_2160p", "width": W, "height": H, "chroma": "4:2:0", "lcu": 64,
           "edges": "per 8x8 block: type none/luma/both (0.2/0.2/0.6), half-edge flags 0.9, alpha 4..64, beta 1..27",
           "sao": "per LCU and component: off 10 %, else EO_0/EO_90/EO_135/EO_45/BO uniform",
           "content": "blurred noise plus a random offset per 8x8 block (blocking artefacts)",
           "l2": "flushed between steps (512 MB write)"}
    if args.impl == "reference":
        if rank != 0:
            return
        cpu_lf(y, u, v, scus, lcus, W, H)
        tt = 0.0
        for i in range(args.steps):
            dt, *_ = cpu_lf(y, u, v, scus, lcus, W, H)
            tt += dt
        value = args.steps / tt
        print(json.dumps({"impl": "reference", "metric": LF_METRIC, "value": value, "unit": "pictures/s",
                          "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": 1e3 * tt / args.steps, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "u8", "data": "synthetic", "config": cfg,
                          "cpu_baseline": {"value": value, "unit": "pictures/s", "cores": 1, "kind": "port",
                                           "sample": "whole pictures, oracle C (one thread)"},
                          "e2e": {"value": value, "unit": "pictures/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}))
        return

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = xg.load()
    lib.xavs2gpu_init(local)
    dev = torch.device("cuda", local)
    h_pic = [torch.from_numpy(p).pin_memory() for p in (y, u, v)]
    h_scus = torch.from_numpy(scus.view(np.uint8).copy()).pin_memory()
    h_lcus = torch.from_numpy(lcus.view(np.uint8).copy()).pin_memory()
    pristine = [t.to(dev) for t in h_pic]
    work = [t.clone() for t in pristine]
    out = [torch.empty_like(t) for t in pristine]
    d_scus, d_lcus = h_scus.to(dev), h_lcus.to(dev)
    h_out = [torch.empty_like(t).pin_memory() for t in h_pic]
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(dev)
    P = lambda t: ctypes.c_void_p(t.data_ptr())

    def step_two_pass(s):
        # deblock in place, then SAO into a second picture written whole
        # (the reference copies the deblocked picture and filters into it)
        rc = lib.xavs2gpu_deblock_picture(P(work[0]), W, P(work[1]), P(work[2]), W // 2, W, H, 6, P(d_scus),
                                          ctypes.c_void_p(s.cuda_stream))
        assert rc == 0
        rc = lib.xavs2gpu_sao_picture(P(out[0]), P(out[1]), P(out[2]), P(work[0]), P(work[1]), P(work[2]), W,
                                      W // 2, W, H, 6, P(d_lcus), 1, ctypes.c_void_p(s.cuda_stream))
        assert rc == 0

    def step(s):
        # both filters in one pass per LCU region: the reconstruction in,
        # the filtered picture out
        rc = lib.xavs2gpu_loopfilter_picture(P(work[0]), P(work[1]), P(work[2]), P(out[0]), P(out[1]), P(out[2]), W,
                                             W // 2, W, H, 6, P(d_scus), P(d_lcus), ctypes.c_void_p(s.cuda_stream))
        assert rc == 0

    def restore():
        for k in range(3):
            work[k].copy_(pristine[k], non_blocking=True)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            restore()
            step(stream)
    barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clk = ClockSampler(local)
    launches0 = lib.xavs2gpu_kernel_launches()
    clk.start()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            restore()
            flush.zero_()
            starts[i].record(stream)
            step(stream)
            ends[i].record(stream)
    barrier()
    clocks = clk.stop()
    launches = lib.xavs2gpu_kernel_launches() - launches0
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_ms = reduce_max(float(sum(step_ms)), dev)
    value = world * args.steps / (total_ms / 1e3)
    kernel_ms = float(np.median(step_ms))
    # the two-pass form (picture deblocking, then picture SAO) for comparison
    two_ms = []
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            restore()
            flush.zero_()
            starts[i].record(stream)
            step_two_pass(stream)
            ends[i].record(stream)
    barrier()
    two_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    # end to end: host picture and edge / SAO parameters in, filtered picture out
    barrier()
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            for k in range(3):
                work[k].copy_(h_pic[k], non_blocking=True)
            d_scus.copy_(h_scus, non_blocking=True)
            d_lcus.copy_(h_lcus, non_blocking=True)
            step(stream)
            for k in range(3):
                h_out[k].copy_(out[k], non_blocking=True)
        stream.synchronize()
    barrier()
    e2e_s = reduce_max(time.perf_counter() - t0, dev)
    e2e = world * args.steps / e2e_s
    if rank != 0:
        return
    cpu_s, ey, eu, ev = cpu_lf(y, u, v, scus, lcus, W, H)
    exact = all(np.array_equal(h_out[k].numpy(), e) for k, e in enumerate((ey, eu, ev)))
    peaks, peak_src = measured_peaks()
    # algorithmic bytes: the reconstruction read once and the filtered
    # picture written once, plus the per-8x8 and per-LCU parameters
    algo = 2 * pic_bytes + h_scus.numel() + h_lcus.numel()
    achieved = algo / (kernel_ms / 1e3) / 1e9
    line = {
        "metric": LF_METRIC, "value": value, "unit": "pictures/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic", "config": cfg,
        "e2e": {"value": e2e, "unit": "pictures/s",
                "h2d_bytes_per_step": int(pic_bytes + h_scus.numel() + h_lcus.numel()),
                "d2h_bytes_per_step": int(pic_bytes)},
        "gpu_launches": int(launches),
        "two_pass_ms": float(np.median(two_ms)),
        "roofline": {"bound": "hbm", "kernel": "loopfilter_lcu_kernel (deblocking + SAO in one pass)",
                     "achieved": achieved, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                     "frac": achieved / peaks.get("hbm_gbs", 6800.0),
                     "traffic": measured_traffic("loopfilter", (W, H) == (3840, 2160)), "peak_source": peak_src,
                     "algorithmic_bytes_per_step": int(algo), "kernel_ms": kernel_ms},
        "sample_bit_exact": bool(exact),
        "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "pictures/s", "cores": 1, "kind": "port",
                         "sample": "one whole picture, oracle C (reference LCU order), one thread"},
        "clocks": clocks,
    }
    print(json.dumps(line))
    if not bool(exact):
        sys.exit("bench: sampled outputs differ from the oracle")


# ---- lookahead analysis: 4K half-resolution picture + MAD maps -------------------
LA_METRIC = "bit-exact 3840x2160 pictures/s (lookahead: half-resolution picture + 16/32/64 MAD maps)"


def cpu_lookahead(img, W, H):
    import oracle
    lw = W // 2
    low = np.zeros((H // 2, lw), np.uint8)
    n = [((W + s - 1) // s) * ((H + s - 1) // s) for s in (16, 32, 64)]
    mads = [np.zeros(k, np.int32) for k in n]
    t0 = time.perf_counter()
    oracle.lib().xo_lookahead_picture(oracle.ptr(img), W, W, H, oracle.ptr(low), lw, *[oracle.ptr(m) for m in mads])
    return time.perf_counter() - t0, low, mads


def run_lookahead(args):
    import torch
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth

    rank, world, local = dist_env()
    W, H = args.chain_width, args.chain_height
    img = synth.chain_pictures(1, W, H, seed=81 + rank)[0]
    n = [((W + s - 1) // s) * ((H + s - 1) // s) for s in (16, 32, 64)]
    cfg = {"workload": "lookahead_2160p", "width": W, "height": H,
           "outputs": "width/2 x height/2 lowres picture, MAD of every aligned 16x16 / 32x32 / 64x64 block",
           "content": "blurred-noise picture", "l2": "flushed between steps (512 MB write)"}
    if args.impl == "reference":
        if rank != 0:
            return
        cpu_lookahead(img, W, H)
        tt = sum(cpu_lookahead(img, W, H)[0] for _ in range(args.steps))
        value = args.steps / tt
        print(json.dumps({"impl": "reference", "metric": LA_METRIC, "value": value, "unit": "pictures/s",
                          "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": 1e3 * tt / args.steps, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "u8", "data": "synthetic", "config": cfg,
                          "cpu_baseline": {"value": value, "unit": "pictures/s", "cores": 1, "kind": "port",
                                           "sample": "whole pictures, oracle C (one thread)"},
                          "e2e": {"value": value, "unit": "pictures/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}))
        return
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = xg.load()
    lib.xavs2gpu_init(local)
    dev = torch.device("cuda", local)
    h_img = torch.from_numpy(img).pin_memory()
    d_img = h_img.to(dev)
    d_low = torch.empty((H // 2, W // 2), dtype=torch.uint8, device=dev)
    d_mad = [torch.empty(k, dtype=torch.int32, device=dev) for k in n]
    h_low = torch.empty_like(d_low, device="cpu").pin_memory()
    h_mad = [torch.empty(k, dtype=torch.int32).pin_memory() for k in n]
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(dev)
    P = lambda t: ctypes.c_void_p(t.data_ptr())

    def step(s):
        rc = lib.xavs2gpu_lookahead_picture(P(d_img), W, W, H, P(d_low), W // 2, *[P(m) for m in d_mad],
                                            ctypes.c_void_p(s.cuda_stream))
        assert rc == 0

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step(stream)
    barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clk = ClockSampler(local)
    launches0 = lib.xavs2gpu_kernel_launches()
    clk.start()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            step(stream)
            ends[i].record(stream)
    barrier()
    clocks = clk.stop()
    launches = lib.xavs2gpu_kernel_launches() - launches0
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_ms = reduce_max(float(sum(step_ms)), dev)
    value = world * args.steps / (total_ms / 1e3)
    kernel_ms = float(np.median(step_ms))
    barrier()
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            d_img.copy_(h_img, non_blocking=True)
            step(stream)
            h_low.copy_(d_low, non_blocking=True)
            for k in range(3):
                h_mad[k].copy_(d_mad[k], non_blocking=True)
        stream.synchronize()
    barrier()
    e2e = world * args.steps / reduce_max(time.perf_counter() - t0, dev)
    if rank != 0:
        return
    cpu_s, low, mads = cpu_lookahead(img, W, H)
    exact = bool(np.array_equal(h_low.numpy(), low) and all(np.array_equal(h_mad[k].numpy(), mads[k])
                                                           for k in range(3)))
    peaks, peak_src = measured_peaks()
    out_bytes = d_low.numel() + 4 * sum(n)
    algo = img.nbytes + out_bytes
    achieved = algo / (kernel_ms / 1e3) / 1e9
    print(json.dumps({
        "metric": LA_METRIC, "value": value, "unit": "pictures/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic", "config": cfg,
        "e2e": {"value": e2e, "unit": "pictures/s", "h2d_bytes_per_step": int(img.nbytes),
                "d2h_bytes_per_step": int(out_bytes)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": "lookahead_kernel", "achieved": achieved,
                     "peak": peaks.get("hbm_gbs"), "unit": "GB/s", "frac": achieved / peaks.get("hbm_gbs", 6800.0),
                     "traffic": measured_traffic("lookahead", (W, H) == (3840, 2160)), "peak_source": peak_src,
                     "algorithmic_bytes_per_step": int(algo),
                     "kernel_ms": kernel_ms},
        "sample_bit_exact": exact,
        "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "pictures/s", "cores": 1, "kind": "port",
                         "sample": "one whole picture, oracle C, one thread"},
        "clocks": clocks,
    }))
    if not exact:
        sys.exit("bench: sampled outputs differ from the oracle")


# ---- skip / direct rough cost: every CU of a 1080p picture, 5 candidates -------
SKIP_METRIC = ("bit-exact skip/direct candidate costs/s (1080p, CUs 8..64, 5 candidates per CU incl. 4-PU and "
               "bi-predicted, SA8D + lambda*rate, best per CU)")
SKIP_OPS_PER_SAMPLE = 10   # prediction 1, difference 1, 8x8 Hadamard 6, |x| accumulate 2


def skip_workload(rank, W, H):
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(91 + rank)
    frames = synth.chain_pictures(3, W, H, seed=93 + rank, pan_px=3)
    cur, refs = frames[2], [frames[1], frames[0]]
    cands, n_cu = synth.skip_candidates(rng, W, H, 2, motion=(-12, 0), cand_dtype=xg.SKIP_CAND_DTYPE)
    return cur, refs, cands, n_cu


def cpu_skip(olib, cur, tab, stride, W, H, cands, n_cu, lam, fraction, seed):
    """The oracle over a random sample of the CUs (all their candidates);
    returns (candidates, samples evaluated, seconds, CU ids, dist, cost, best)."""
    rng = np.random.default_rng(seed)
    pick = np.nonzero(rng.random(n_cu) < fraction)[0]
    sel = np.ascontiguousarray(cands[np.isin(cands["cu"], pick)])
    remap = np.full(n_cu, -1, np.int64)
    remap[pick] = np.arange(len(pick))
    sub = sel.copy()
    sub["cu"] = remap[sel["cu"]]
    d = np.zeros(len(sub), np.int32)
    c = np.zeros(len(sub))
    b = np.zeros(len(pick), np.int32)
    t0 = time.perf_counter()
    olib.xo_skip_costs(oracle_ptr(cur), W, tab, stride, W, H, 2, oracle_ptr(sub), len(sub), lam, len(pick),
                       oracle_ptr(d), oracle_ptr(c), oracle_ptr(b))
    dt = time.perf_counter() - t0
    samples = int((1 << (2 * sub["size_log2"].astype(np.int64))).sum())
    return len(sub), samples, dt, pick, sel, d, c, b


def oracle_ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def run_skip(args):
    import torch
    import oracle
    import xavs2_gb300 as xg

    rank, world, local = dist_env()
    W, H = args.width, args.height
    cur, refs, cands, n_cu = skip_workload(rank, W, H)
    n = len(cands)
    lam = float(np.sqrt(2.0 ** ((QP - 11) / 4.0) * 0.68))
    samples = int((1 << (2 * cands["size_log2"].astype(np.int64))).sum())
    cfg = {"workload": "skip_direct_1080p", "width": W, "height": H, "refs": 2, "cus": n_cu, "candidates": n,
           "candidates_per_cu": "1 four-PU temporal-style + 4 single-PU (35 % bi-predicted, some repeated)",
           "motion": "pan 3 px/picture + local motion; candidate vectors around (-3, 0) px", "qp": QP,
           "l2": "flushed between steps (512 MB write)"}
    olib = oracle.lib()
    stride = W + 160
    flats = [np.ascontiguousarray(oracle.interpolate_frame(olib, r, mode=2).reshape(16, -1)) for r in refs]
    tab = (ctypes.c_void_p * 32)(*[oracle.ptr(f[k], 80 * stride + 80).value for f in flats for k in range(16)])
    if args.impl == "reference":
        if rank != 0:
            return
        frac = min(1.0, 8 * args.cpu_fraction)
        cpu_skip(olib, cur, tab, stride, W, H, cands, n_cu, lam, frac / 4, 100)
        done, tt = 0, 0.0
        for i in range(args.steps):
            k, _, dt, *_ = cpu_skip(olib, cur, tab, stride, W, H, cands, n_cu, lam, frac, 200 + i)
            done += k
            tt += dt
        value = done / tt
        print(json.dumps({"impl": "reference", "metric": SKIP_METRIC, "value": value, "unit": "candidates/s",
                          "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": 1e3 * tt / args.steps, "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "u8", "data": "synthetic", "config": cfg,
                          "cpu_baseline": {"value": value, "unit": "candidates/s", "cores": 1, "kind": "port",
                                           "sample": "per step the candidates of a random %.1f%% of the CUs, "
                                                     "oracle C (one thread)" % (100 * frac)},
                          "e2e": {"value": value, "unit": "candidates/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}))
        return
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = xg.load()
    lib.xavs2gpu_init(local)
    dev = torch.device("cuda", local)
    sess = xg.MeSession(W, H, 2, 1)
    sess.set_picture(-1, cur)
    for i, r in enumerate(refs):
        sess.set_picture(i, r)
    sess.sync()
    stream = torch.cuda.ExternalStream(sess.stream())
    h_c = torch.from_numpy(cands.view(np.uint8).copy()).pin_memory()
    d_c = h_c.to(dev)
    d_dist = torch.empty(n, dtype=torch.int32, device=dev)
    d_cost = torch.empty(n, dtype=torch.float64, device=dev)
    d_best = torch.empty(n_cu, dtype=torch.int32, device=dev)
    h_dist = torch.empty(n, dtype=torch.int32).pin_memory()
    h_cost = torch.empty(n, dtype=torch.float64).pin_memory()
    h_best = torch.empty(n_cu, dtype=torch.int32).pin_memory()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    P = lambda t: ctypes.c_void_p(t.data_ptr())

    def step():
        rc = lib.xavs2gpu_skip_costs(ctypes.c_void_p(sess.h), P(d_c), n, lam, n_cu, P(d_dist), P(d_cost), P(d_best),
                                     None)
        assert rc == 0

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    sess.sync()
    barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clk = ClockSampler(local)
    launches0 = lib.xavs2gpu_kernel_launches()
    clk.start()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            step()
            ends[i].record(stream)
    sess.sync()
    barrier()
    clocks = clk.stop()
    launches = lib.xavs2gpu_kernel_launches() - launches0
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_ms = reduce_max(float(sum(step_ms)), dev)
    value = n * world * args.steps / (total_ms / 1e3)
    kernel_ms = float(np.median(step_ms))
    barrier()
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            d_c.copy_(h_c, non_blocking=True)
            step()
            h_dist.copy_(d_dist, non_blocking=True)
            h_cost.copy_(d_cost, non_blocking=True)
            h_best.copy_(d_best, non_blocking=True)
    sess.sync()
    barrier()
    e2e = n * world * args.steps / reduce_max(time.perf_counter() - t0, dev)
    dist_h, cost_h, best_h = h_dist.numpy().copy(), h_cost.numpy().copy(), h_best.numpy().copy()
    # release the tensors that were used on the session's stream before the
    # session (and its stream) goes away
    del h_c, d_c, d_dist, d_cost, d_best, h_dist, h_cost, h_best, flush, stream
    torch.cuda.synchronize()
    sess.close()
    if rank != 0:
        return
    k, smp, cpu_s, pick, sel, d, c, b = cpu_skip(olib, cur, tab, stride, W, H, cands, n_cu, lam, args.cpu_fraction, 7)
    gi = np.nonzero(np.isin(cands["cu"], pick))[0]
    gb = best_h[pick]
    exact = bool(np.array_equal(dist_h[gi], d) and np.array_equal(cost_h[gi], c) and
                 np.array_equal(np.where(gb >= 0, np.searchsorted(gi, gb), -1), b))
    peaks, peak_src = measured_peaks()
    peak = sm_count() * 128 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / SKIP_OPS_PER_SAMPLE / 1e12
    achieved = samples / (kernel_ms / 1e3) / 1e12
    print(json.dumps({
        "metric": SKIP_METRIC, "value": value, "unit": "candidates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic", "config": cfg,
        "e2e": {"value": e2e, "unit": "candidates/s", "h2d_bytes_per_step": int(cands.nbytes),
                "d2h_bytes_per_step": int(12 * n + 4 * n_cu)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "int", "kernel": "skip_count + skip_scatter + skip_cost + skip_best", "achieved": achieved,
                     "peak": peak, "unit": "T candidate-samples/s", "frac": achieved / peak,
                     "traffic": measured_traffic("skip", (W, H) == (1920, 1080)),
                     "peak_source": "%d SMs x 128 INT32 lanes/clk x sm_max_mhz / %d ops per sample (%s)"
                                    % (sm_count(), SKIP_OPS_PER_SAMPLE, peak_src),
                     "work_per_launch": "%d candidates, %d predicted samples" % (n, samples), "kernel_ms": kernel_ms},
        "sample_bit_exact": exact,
        "cpu_baseline": {"value": k / cpu_s, "unit": "candidates/s", "cores": 1, "kind": "port",
                         "sample": "the candidates of a random %.2f%% (%d) of the CUs, oracle C (one thread)"
                                   % (100 * args.cpu_fraction, len(pick))},
        "clocks": clocks,
    }), flush=True)
    if not exact:
        sys.exit("bench: sampled outputs differ from the oracle")


# ---- serving: 64 concurrent streams, continuous batching --------------------
SERVE_METRIC = "served p99 frame latency (%d streams %s, 30 fps Poisson arrivals, continuous batching)"
SERVE_RES = [(640, 360), (1280, 720), (1920, 1080), (3840, 2160)]


def serve_content(width, height, n, seed):
    """Config-0 style pictures: a blurred-noise base picture, then one global
    quarter-pel translation U[-8, 8] px per picture plus noise."""
    import xavs2_gb300.synth as synth
    rng = np.random.default_rng(seed)
    frames = [synth.base_picture(rng, width, height)]
    for _ in range(n - 1):
        frames.append(synth.next_picture(rng, frames[-1], 1, 8))
    return frames


def serve_trace(xg, srv, streams, pools, duration, warm, rate, seed):
    """Submits every stream's pictures at Poisson arrival times for
    `duration` s while a collector polls; returns the results of the
    pictures submitted after `warm` s and the submission failures."""
    import threading
    rng = np.random.default_rng(seed)
    events = []
    for sid, (res, off) in enumerate(streams):
        t = rng.uniform(0, 1.0 / rate)
        k = 0
        while t < duration:
            events.append((t, sid, res, off + k))
            t += rng.exponential(1.0 / rate)
            k += 1
    events.sort()
    results = []
    done = threading.Event()

    def collect():
        while not done.is_set() or len(results) < submitted[0]:
            r = srv.poll(4096, 20)
            if len(r):
                results.extend(r.tolist())
            elif done.is_set() and time.time() > deadline[0]:
                break

    submitted = [0]
    deadline = [0.0]
    fails = 0
    accepted = {sid: [] for sid in range(len(streams))}   # pool index of each accepted picture, in order
    th = threading.Thread(target=collect)
    th.start()
    t0 = time.perf_counter()
    t0_ns = time.monotonic_ns()
    for (t, sid, res, k) in events:
        dt = t - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        pool = pools[res]
        if srv.submit(sid, pool[k % len(pool)], tag=int(t * 1e9)) == 0:
            submitted[0] += 1
            accepted[sid].append(k % len(pool))
        else:
            fails += 1
    deadline[0] = time.time() + 30.0
    done.set()
    th.join()
    arr = np.array(results, dtype=xg.SERVER_RESULT_DTYPE)
    keep = (arr["ref_only"] == 0) & (arr["tag"] >= int(warm * 1e9))
    return arr[keep], fails, len(events), accepted


def serve_summary(arr, window):
    lat = (arr["t_done_ns"] - arr["t_submit_ns"]) / 1e6
    if len(lat) == 0:
        return {"frames": 0}
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "frames": int(len(lat)), "frames_per_s": float(len(lat) / window),
            "mean_batch_frames": float(arr["batch_frames"].mean())}


def serve_parity(xg, arr, streams, layouts, res_idx, pools, accepted, prm, n_pictures=3, n_cus=12):
    """Served pictures against the full-picture chain and the oracle: for up
    to n_pictures served pictures (the largest resolutions first), the chain
    on the same current picture and references (picture k of a stream is the
    k-th picture the server accepted from it) gives the same checksum, and
    the chain's outputs match the oracle on n_cus seeded CUs."""
    import oracle
    lib = xg.load()
    cand = arr[arr["frame"] >= 2]
    order = sorted(range(len(cand)), key=lambda i: (-int(res_idx[int(cand["stream"][i])]), i))
    seen, picked = set(), []
    for i in order:
        r = int(res_idx[int(cand["stream"][i])])
        if r not in seen:
            seen.add(r)
            picked.append(cand[i])
        if len(picked) == n_pictures:
            break
    checked, mism, first, n_pu, n_cd = 0, 0, None, 0, 0
    for rec in picked:
        sid, f = int(rec["stream"]), int(rec["frame"])
        pool = pools[streams[sid][0]]
        cur, r0, r1 = (pool[accepted[sid][k]] for k in (f, f - 1, f - 2))
        h, w = cur.shape
        pus, cus = layouts[sid]
        sess = xg.MeSession(w, h, 2, len(pus))
        sess.set_pus(pus)
        chain = xg.Chain(sess, cus, QP)
        for idx, img in enumerate([cur, r0, r1]):
            assert lib.xavs2gpu_copy_h2d(ctypes.c_void_p(chain.source(idx)), xg.ptr(img), img.nbytes) == 0
        chain.run(prm)
        out = chain.download()
        want = xg.output_hash(out["recon"], out["coef"], sess.results())
        checked += 1
        if int(rec["hash"]) != want:
            mism += 1
            first = first or "hash of stream %d picture %d" % (sid, f)
        rng = np.random.default_rng(sid)
        cu_idx = np.sort(rng.choice(len(cus), min(n_cus, len(cus)), replace=False))
        a, b, bad = oracle.chain_sample_check(oracle.lib(), out, cur, [r0, r1], pus, cus, sess.results(),
                                              (prm.search_range, prm.lambda_factor, 1, 2, 0, 0), QP, cu_idx,
                                              os.cpu_count() or 1)
        n_pu += a
        n_cd += b
        if bad:
            mism += len(bad)
            first = first or bad[0]
        chain.close()
        sess.close()
    return {"pictures": checked, "checked_pu_searches": n_pu, "checked_candidates": n_cd, "mismatches": mism,
            "first": first, "against": "full-picture chain (checksum) and oracle (sampled CUs)"}


def run_serve(args):
    import torch
    import xavs2_gb300 as xg

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    lib = xg.load()
    lib.xavs2gpu_init(local)
    rng = np.random.default_rng(11 + rank)
    nstreams, rate = args.serve_streams, 30.0
    res_idx = rng.choice(4, nstreams, p=[0.3, 0.3, 0.3, 0.1])
    if args.serve_res != "mix":
        res_idx = np.full(nstreams, ["360p", "720p", "1080p", "2160p"].index(args.serve_res))
    pools = {r: serve_content(*SERVE_RES[r], args.serve_pool, 50 + r) for r in sorted(set(res_idx.tolist()))}
    prm = xg.MeParams(args.serve_range, lambda_factor(QP), 1, 2, 0, 0)
    layouts = []
    for sid in range(nstreams):
        w, h = SERVE_RES[res_idx[sid]]
        layouts.append(xg.cu_pus(xg.split_map_cus(w, h, 1000 + sid), w, h, 2))

    def make_server(max_frames):
        cfg = xg.ServerConfig(args.serve_hbm_gb << 30, args.serve_batch_mpx << 20, max_frames, QP, prm,
                              hbm_reserve_bytes=0, batch_pixels_target=args.serve_batch_target_mpx << 20)
        srv = xg.Server(cfg)
        streams = []
        for sid in range(nstreams):
            w, h = SERVE_RES[res_idx[sid]]
            pus, cus = layouts[sid]
            got = srv.open_stream(w, h, pus, cus, ring=16)
            assert got == sid, got
            streams.append((int(res_idx[sid]), int(rng.integers(0, args.serve_pool))))
        return srv, streams

    window = args.serve_seconds - args.serve_warm
    clk = ClockSampler(local)
    launches0 = lib.xavs2gpu_kernel_launches()
    srv, streams = make_server(args.serve_batch)
    clk.start()
    arr, fails, n_events, accepted = serve_trace(xg, srv, streams, pools, args.serve_seconds, args.serve_warm, rate, 5)
    clocks = clk.stop()
    stats = srv.stats()
    srv.close()
    launches = lib.xavs2gpu_kernel_launches() - launches0
    batched = serve_summary(arr, window)
    parity = serve_parity(xg, arr, streams, layouts, res_idx, pools, accepted, prm)
    # the same trace, each picture alone (one picture per batch)
    srv1, streams1 = make_server(1)
    arr1, fails1, _, _ = serve_trace(xg, srv1, streams1, pools, args.serve_seconds, args.serve_warm, rate, 5)
    srv1.close()
    alone = serve_summary(arr1, window)
    if rank != 0:
        return
    px = {r: SERVE_RES[r][0] * SERVE_RES[r][1] for r in range(4)}
    mean_px = float(np.mean([px[r] for r in res_idx]))
    line = {
        "metric": SERVE_METRIC % (nstreams, "360p..2160p" if args.serve_res == "mix" else args.serve_res),
        "value": batched.get("p99_ms"), "unit": "ms", "n_gpus": world,
        "steps": batched.get("frames"), "warmup": args.serve_warm, "ms_per_step": batched.get("mean_ms"),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": "serve_%d_streams_%s" % (nstreams, "mixed" if args.serve_res == "mix" else args.serve_res),
                   "streams": nstreams,
                   "resolutions": {"%dx%d" % SERVE_RES[r]: int((res_idx == r).sum()) for r in range(4)},
                   "arrivals": "Poisson 30 fps per stream", "seconds": args.serve_seconds, "warm_s": args.serve_warm,
                   "search_range": args.serve_range, "qp": QP, "refs": 2,
                   "batch_cap": {"pictures": args.serve_batch, "luma_mpx": args.serve_batch_mpx,
                                 "target_luma_mpx": args.serve_batch_target_mpx},
                   "picture_job": "reference update + sub-pel planes, FS +-%d + quarter-pel SATD over the leaf-CU "
                                  "PUs of a seeded split map, every inter candidate through the TU chain (one TU and "
                                  "the TU split), choice, reconstruction" % args.serve_range},
        "batched": batched, "unbatched_same_trace": alone,
        "submit_failures": {"batched": fails, "unbatched": fails1}, "offered_pictures": n_events,
        "server": stats,
        "e2e": {"value": batched.get("frames_per_s"), "unit": "pictures/s",
                "h2d_bytes_per_step": int(mean_px), "d2h_bytes_per_step": 8},
        "gpu_launches": int(launches),
        "parity": parity,
        "clocks": clocks,
    }
    print(json.dumps(line))
    if parity.get("mismatches"):
        sys.exit("bench: served pictures differ: %s" % parity["first"])


def chain_parity(xg, chain, sess, order, pus, cus, prm_tuple, n_cus, seed):
    """The last eager picture of a chain against the oracle on n_cus seeded
    CUs: the search of each of their PUs, every candidate (levels, nnz,
    reconstructed residual, SSDs, search cost), each CU's choice and block
    of the reconstruction.  Returns the bench line's parity object."""
    import oracle
    out = chain.download()
    rng = np.random.default_rng(seed)
    cu_idx = np.sort(rng.choice(len(cus), min(n_cus, len(cus)), replace=False))
    n_pu, n_cd, bad = oracle.chain_sample_check(oracle.lib(), out, order[0], order[1:], pus, cus, sess.results(),
                                                prm_tuple, QP, cu_idx, os.cpu_count() or 1)
    return {"checked_cus": int(len(cu_idx)), "checked_pu_searches": int(n_pu), "checked_candidates": int(n_cd),
            "mismatches": len(bad), "first": bad[0] if bad else None, "against": "oracle"}


# ---- full-picture chain at 4K ------------------------------------------------
CHAIN_METRIC = ("P pictures/s, 3840x2160 hot-path chain (4 refs, FS +-64 + quarter-pel SATD, every inter candidate "
                "through the TU chain incl. TU splits, recon; CUDA graph)")


def run_chain(args):
    import torch
    import xavs2_gb300 as xg
    import xavs2_gb300.synth as synth

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    lib = xg.load()
    lib.xavs2gpu_init(local)
    W, H, NR, R = args.chain_width, args.chain_height, 4, RANGE
    frames = synth.chain_pictures(NR + 2, W, H, seed=21 + rank)
    cus_list = xg.split_map_cus(W, H, 31 + rank)
    pus, cus = xg.cu_pus(cus_list, W, H, NR)
    sess = xg.MeSession(W, H, NR, len(pus))
    sess.set_pus(pus)
    chain = xg.Chain(sess, cus, QP, feedback=True)
    prm = xg.MeParams(R, lambda_factor(QP), 1, 2, 0, 0)
    order = [frames[NR]] + [frames[NR - 1 - r] for r in range(NR)]   # current, then refs k-1 .. k-4

    def upload_sources():
        for idx, img in enumerate(order):
            assert lib.xavs2gpu_copy_h2d(ctypes.c_void_p(chain.source(idx)), xg.ptr(img), img.nbytes) == 0

    # parity at the full size: one eager picture, checked against the oracle
    # on a seeded sample of CUs (their PU searches, every candidate, choice
    # and reconstructed block); the feedback then moved the sources, so they
    # are uploaded again
    upload_sources()
    chain.run(prm)
    parity = chain_parity(xg, chain, sess, order, pus, cus, (R, prm.lambda_factor, 1, 2, 0, 0), 48, 77)
    upload_sources()
    tune_ms = chain.autotune(prm, reps=1)
    tun = chain.tuning()
    chain.capture(prm)
    nk = chain.graph_kernels()
    stream = torch.cuda.ExternalStream(sess.stream())
    for _ in range(args.warmup):
        chain.launch()
    sess.sync()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    clk = ClockSampler(local)
    launches0 = lib.xavs2gpu_kernel_launches()
    clk.start()
    ev[0].record(stream)
    for _ in range(args.steps):
        chain.launch()
    ev[1].record(stream)
    sess.sync()
    clocks = clk.stop()
    launches = lib.xavs2gpu_kernel_launches() - launches0
    total_ms = ev[0].elapsed_time(ev[1])
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    total_ms = reduce_max(total_ms, "cuda")
    fps = args.steps * world / (total_ms / 1e3)
    # end to end: each picture uploaded from pinned host memory, the
    # reconstruction read back
    h_in = torch.from_numpy(frames[NR + 1]).pin_memory()
    h_out = torch.empty(W * H, dtype=torch.uint8).pin_memory()
    o = chain.outputs()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        lib.xavs2gpu_me_sync(sess.h)
        assert lib.xavs2gpu_copy_h2d(ctypes.c_void_p(chain.source(0)), ctypes.c_void_p(h_in.data_ptr()), W * H) == 0
        chain.launch()
        lib.xavs2gpu_me_sync(sess.h)
        assert lib.xavs2gpu_copy_d2h(ctypes.c_void_p(h_out.data_ptr()), ctypes.c_void_p(o.recon), W * H) == 0
    e2e_fps = args.steps / (time.perf_counter() - t0)
    # phase timing of one eager search of the picture's PUs (the graph's
    # search kernels), for the roofline of the dominant kernel
    sess.set_profiling(True)
    ph = np.zeros(4)
    for _ in range(3):
        sess.run(prm)
        sess.sync()
        ph += np.array(sess.phase_ms())
    sess.set_profiling(False)
    ph /= 3
    n_ctu_pus, n_gen, n_jobs = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    lib.xavs2gpu_me_plan_stats(ctypes.c_void_p(sess.h), ctypes.byref(n_ctu_pus), ctypes.byref(n_gen),
                               ctypes.byref(n_jobs))
    peaks, peak_src = measured_peaks()
    ctu_px = n_jobs.value * (2 * R) * (2 * R) * 4096
    ctu_ach = ctu_px / (ph[1] / 1e3) / 1e12
    ctu_peak = sm_count() * 64 * 4 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
    # CPU baseline: the oracle's search over a sample of the picture's PU
    # searches (the search is ~99 % of the chain's work), scaled to pictures
    evals = count_evals(pus, R)
    cpu_e, cpu_s, cpu_n = cpu_sample_search(pus, order[0], order[1:], (R, prm.lambda_factor, 1, 2, 0, 0),
                                            args.cpu_fraction / 8, 9, os.cpu_count() or 1)
    cpu_fps = (cpu_e / cpu_s) / evals
    if rank != 0:
        return
    line = {
        "metric": CHAIN_METRIC, "value": fps, "unit": "pictures/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": "chain_2160p_4ref", "width": W, "height": H, "refs": NR, "search_range": R, "qp": QP,
                   "leaf_cus": int(len(cus)), "pu_searches": int(len(pus)), "evals_per_picture": evals,
                   "candidates": int(chain.outputs().n_cands), "tus_per_picture": 5 * int(chain.outputs().n_cands),
                   "content": "pan 12 px/picture + 2 block-local motions, seeded split map 64..8",
                   "l2": "inputs larger than L2 (%d MB of reference planes)" % (NR * 16 * (W + 160) * (H + 160) >> 20)},
        "graph": {"kernels_per_launch": nk, "autotuned": {"refine_split_px": tun.me.refine_split_px,
                                                            "refine_block": tun.me.refine_block,
                                                            "cu_groups": tun.me.cu_groups,
                                                            "tq_warps": tun.tq_warps, "ms_per_picture": tune_ms}},
        "e2e": {"value": e2e_fps, "unit": "pictures/s", "h2d_bytes_per_step": W * H, "d2h_bytes_per_step": W * H},
        "gpu_launches": int(launches),
        "roofline": {"bound": "int", "kernel": "fs_ctu_kernel", "achieved": ctu_ach, "peak": ctu_peak,
                     "unit": "Tpx-absdiff/s", "frac": ctu_ach / ctu_peak, "traffic": None,
                     "peak_source": "%d SMs x 64 VABSDIFF4 lanes/clk x 4 px x sm_max_mhz (%s)" % (sm_count(), peak_src),
                     "work_per_launch": "%d CTU-ref jobs x %d displacements x 4096 px" % (n_jobs.value, 4 * R * R),
                     "kernel_ms": float(ph[1]), "eager_search_phases_ms": [float(v) for v in ph]},
        "cpu_baseline": {"value": cpu_fps, "unit": "pictures/s", "cores": os.cpu_count() or 1, "kind": "port",
                         "sample": "oracle search over a random %.3f%% (%d) of the picture's PU searches, scaled"
                                   % (100 * args.cpu_fraction / 8, cpu_n)},
        "parity": parity,
        "clocks": clocks,
    }
    print(json.dumps(line))
    chain.close()
    sess.close()
    if parity["mismatches"]:
        sys.exit("bench: chain outputs differ from the oracle: %s" % parity["first"])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-fraction", type=float, default=1.0 / 64)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--quick", action="store_true", help="device timing only (for profiler runs)")
    ap.add_argument("--no-configs", dest="configs", action="store_false",
                    help="default run: skip the one-off runs of configs 2-4 added to the line")
    ap.add_argument("--me-leaf", action="store_true",
                    help="with --quick: the serving-shaped search (leaf-CU partitions, FS +-16) instead of every PU")
    ap.add_argument("--workload", choices=["me", "tq", "chain", "serve", "intra", "loopfilter", "lookahead", "skip"],
                    default="me",
                    help="me: batched motion search (default); tq: batched transform+quant; chain: 4K full-picture "
                         "chain; serve: 64-stream serving; intra: rough intra mode decision; loopfilter: 4K deblocking + SAO; "
                         "lookahead: 4K half-resolution picture + MAD maps; skip: skip/direct candidate costs")
    ap.add_argument("--chain-width", type=int, default=3840)
    ap.add_argument("--chain-height", type=int, default=2160)
    ap.add_argument("--tq-blocks", type=int, default=1000000)
    ap.add_argument("--tq-parts", default="0,1,2,3,4", help="TU shapes (LumaPU indices) of the tq workload")
    ap.add_argument("--tq-chunks", type=int, default=16, help="tq e2e: chunks the host entry overlaps")
    ap.add_argument("--mvp", choices=["zero", "temporal"], default="zero",
                    help="me: zero predictors (the shared-window CTU search) or the previous picture's vectors "
                         "(each PU its own centre: the per-PU search)")
    ap.add_argument("--serve-streams", type=int, default=64)
    ap.add_argument("--serve-seconds", type=float, default=8.0)
    ap.add_argument("--serve-warm", type=float, default=2.0)
    ap.add_argument("--serve-range", type=int, default=64)
    ap.add_argument("--serve-batch", type=int, default=64)
    # luma pixels per batch (MiB): batches of 12 Mi keep a burst of arrivals
    # from forming one long batch while the backlog is short; with more than
    # two such batches waiting they grow to 24 Mi, which carries 64 streams of
    # 1080p in full (12 Mi alone: 1,860 of 1,942 pictures/s)
    ap.add_argument("--serve-batch-mpx", type=int, default=24,
                    help="luma Mi-pixels a batch may take (sizes the batch buffers)")
    ap.add_argument("--serve-batch-target-mpx", type=int, default=12,
                    help="luma Mi-pixels a batch takes while the backlog is short (0: the full size)")
    ap.add_argument("--serve-res", choices=["mix", "360p", "720p", "1080p", "2160p"], default="mix",
                    help="stream resolutions: the 360p..2160p mix, or every stream at one size")
    ap.add_argument("--serve-pool", type=int, default=4)
    ap.add_argument("--serve-hbm-gb", type=int, default=64)
    args = ap.parse_args()
    if args.workload == "tq":
        run_tq(args)
    elif args.workload == "intra":
        run_intra(args)
    elif args.workload == "loopfilter":
        run_loopfilter(args)
    elif args.workload == "lookahead":
        run_lookahead(args)
    elif args.workload == "skip":
        run_skip(args)
    elif args.workload == "chain":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "metric": CHAIN_METRIC,
                              "unavailable": "timed as the cpu_baseline of this workload's own line"}))
        else:
            run_chain(args)
    elif args.workload == "serve":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference",
                              "metric": SERVE_METRIC % (args.serve_streams, "360p..2160p" if args.serve_res == "mix"
                                                        else args.serve_res),
                              "unavailable": "the reference has no serving path; its per-picture CPU cost is the "
                                             "--workload me reference arm"}))
        else:
            run_serve(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

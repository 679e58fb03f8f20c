"""Host logic of bench.py that needs no GPU: the condensed lines of the other
configurations a default run carries, and a child run that fails being
recorded as such (the config-1 line stands)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_condense_keeps_the_reported_keys():
    import bench
    line = {"metric": "m", "value": 2.0, "unit": "u", "ms_per_step": 1.5, "higher_is_better": True,
            "parity": {"mismatches": 0}, "sample_bit_exact": True, "config": {"big": list(range(100))},
            "e2e": {"value": 1.0, "unit": "u", "h2d_bytes_per_step": 7},
            "roofline": {"bound": "hbm", "achieved": 1.0, "peak": 2.0, "unit": "GB/s", "frac": 0.5, "traffic": 9},
            "batched": {"p50_ms": 1.0, "p99_ms": 2.0, "frames_per_s": 3.0, "mean_batch_frames": 4.0, "frames": 5},
            "cpu_baseline": {"value": 1.0, "unit": "u", "cores": 16, "kind": "port", "sample": "s"},
            "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": []}}
    c = bench.condense(line)
    assert "config" not in c
    assert c["value"] == 2.0 and c["parity"] == {"mismatches": 0} and c["sample_bit_exact"] is True
    assert c["e2e"] == {"value": 1.0, "unit": "u"}
    assert c["roofline"]["frac"] == 0.5 and "traffic" not in c["roofline"]
    assert c["served"] == {"p50_ms": 1.0, "p99_ms": 2.0, "frames_per_s": 3.0, "mean_batch_frames": 4.0}
    assert c["cpu_baseline"] == {"value": 1.0, "unit": "u", "cores": 16, "kind": "port"}
    assert c["clocks"] == {"sm_mhz": 2070.0, "reasons": []}


def test_a_failing_child_is_recorded(monkeypatch):
    import bench
    monkeypatch.setattr(bench, "OTHER_CONFIGS", {"bad": ["--workload", "no-such-workload"]})
    out = bench.other_configs(limit_s=120)
    assert set(out) == {"bad"}
    assert out["bad"]["error"].startswith("exit status")
    assert out["bad"]["command"] == "python bench.py --workload no-such-workload"
    assert out["bad"]["wall_s"] >= 0

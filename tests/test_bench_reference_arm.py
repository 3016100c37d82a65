"""The reference arm of bench.py (`--impl reference`: the reference algorithm on the
host cores, no GPU) prints one JSON line with the contract's keys, and the same
config object as the GPU arm prints for the same workload."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line(oracle_lib):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "sod", "--steps", "2", "--warmup", "3"], capture_output=True, text=True, check=True,
                         cwd=ROOT, timeout=600).stdout
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "dtype", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 2
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    case, desc = bench.workload("sod")
    ours = bench.common_config(case, desc, argparse.Namespace(steps=2), 1)
    assert d["config"] == json.loads(json.dumps(ours))


def test_reference_build_against_port(oracle_lib):
    """bench.py --impl ref-vs-port times the reference's own CPU build (oracle/_ref/HyPar)
    against the oracle port on one deck; skipped where the reference was not built."""
    if not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "HyPar")):
        import pytest
        pytest.skip("oracle/_ref/HyPar is not built here")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "ref-vs-port", "--workload",
                          "vortex", "--size", "48", "--steps", "1"], capture_output=True, text=True, check=True,
                         cwd=ROOT, timeout=600).stdout
    d = json.loads([ln for ln in out.splitlines() if ln.startswith("{")][-1])
    assert d["impl"] == "ref-vs-port"
    for row in d["threads"].values():
        assert row["reference_s_per_step"] > 0 and row["port_s_per_step"] > 0

"""bench.py --impl reference (the reference algorithm on the host cores)
prints one JSON line with the contract's keys, on the same metric and
workload names as the GPU arm; it runs without a GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "multimuon-1000trk", "--events", "16", "--steps", "2",
                        "--warmup", "3"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.strip()]
    d = json.loads(lines[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["metric"] == "events/s" and d["unit"] == "events/s" and d["higher_is_better"]
    assert d["steps"] == 2 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"] == "multimuon-1000trk"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference")
    assert cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_with_two_replicas():
    """--gpus 2 without a launcher starts two ranks itself; rank 0 alone
    runs the reference arm and prints, the other exits 0 without work."""
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "single-muon-100trk", "--events", "8", "--steps", "1",
                        "--warmup", "1", "--gpus", "2"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0


def test_gpus_flag_must_match_the_launcher():
    env = dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2"], capture_output=True, text=True, timeout=120, cwd=ROOT,
                       env=env)
    assert p.returncode == 2
    assert "disagrees" in p.stderr


def test_reference_runs_in_event_groups_its_bitmap_counts_can_hold():
    """The reference sizes its pair bitmap in 32-bit bit counts, so the arm
    runs it on event groups whose n1 * n2 bits stay below 2^31; pile-up 200
    events (~84 M bits each) go in groups of at most 25, every event once and
    in order."""
    sys.path.insert(0, ROOT)
    import numpy as np
    import bench
    from trax_gb300 import gen
    w = bench.workload_at_grid(gen.WORKLOADS["pileup200"], "tuned")

    class Batch:  # layer hit counts are all the grouping reads
        n_events = 200
        layer_nhits = np.tile(np.array([[6500, 6500, 6500, 6500]], dtype=np.uint32), (200, 1))

    groups = bench.reference_groups(Batch, w)
    assert groups[0][0] == 0 and sum(c for _, c in groups) == 200
    assert all(f2 == f1 + c1 for (f1, c1), (f2, _) in zip(groups, groups[1:]))
    per_event = 2 * 6500 * 6500
    assert all(c * per_event <= bench.REF_GROUP_BITS for _, c in groups)
    assert max(c for _, c in groups) == bench.REF_GROUP_BITS // per_event

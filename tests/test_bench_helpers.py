"""bench.py's DRAM-traffic figures come from the committed ncu summaries under
profiles/: they apply only to the launch form the capture measured."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _kv(name):
    path = os.path.join(ROOT, "profiles", name)
    return dict((k.strip(), v.strip()) for k, v in (l.split(":", 1) for l in open(path)
                                                    if ":" in l and not l.startswith("#")))


def test_frame_traffic_matches_its_launch_form():
    kv = _kv("frame_traffic.txt")
    mode, minb = (int(x) for x in kv["launch"].split(","))
    tune = {"trace_mode": mode, "minb": minb}
    per_ray = float(kv["dram_bytes_per_ray"])
    assert bench.frame_traffic(kv["workload"], tune, 1000) == per_ray * 1000
    assert bench.frame_traffic(kv["workload"], {"trace_mode": 0, "minb": 4}, 1000) is None
    assert bench.frame_traffic("cornell", tune, 1000) is None


def test_traversal_traffic_matches_its_launch_form():
    kv = _kv("traversal_traffic.txt")
    per_ray = float(kv["dram_bytes_per_ray"])
    assert bench.traversal_traffic(kv["launch"], 16) == per_ray * 16
    assert bench.traversal_traffic("plain", 16) is None


def test_compact_reference_arm_runs_on_the_cpu():
    """bench.py --impl reference --workload compact times the oracle's codec
    on the host threads (no GPU) and prints the reference arm's line."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--workload",
                        "compact", "--elems", "65536", "--steps", "3", "--warmup", "3"],
                       capture_output=True, text=True, timeout=600, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "Melem/s"
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0

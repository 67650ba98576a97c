"""The bench's reference arms run on the CPU alone (the oracle port of the
reference FP64 path) and print the contract's JSON line."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run(*args):
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", *args],
                         cwd=ROOT, capture_output=True, text=True, timeout=600, check=True)
    return json.loads(out.stdout.strip().splitlines()[-1])


def test_sites_reference_arm():
    line = run("--workload", "sites", "--sites", "12", "--tree-nodes", "201")
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["unit"] == "nodes/s"
    assert line["config"]["sites"] == 12 and line["config"]["tree_nodes"] == 201
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_dense_reference_arm():
    line = run("--workload", "dense", "--states", "8", "--trees", "3", "--tree-nodes", "150")
    assert line["impl"] == "reference"
    assert line["value"] > 0
    assert line["cpu_baseline"]["cores"] >= 1

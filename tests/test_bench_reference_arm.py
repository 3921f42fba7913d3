"""The reference arm of bench.py (the CPU port of the reference loop on the host cores) prints the
JSON line the benchmark contract asks for: impl "reference", the metric and unit of the GPU arm,
an e2e block with no device copies, and a cpu_baseline describing the timed sample.  Run on the
electrode-discharge workload (64x64x256 nodes), which the port steps in about a second."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_prints_the_contract_line(port):
    # `port` builds the oracle's C restatement that the reference arm times
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "discharge", "--steps", "1", "--warmup", "3"], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "particle-steps/s" and line["unit"] == "particle-steps/s"
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] >= 3
    assert line["value"] > 0 and line["ms_per_step"] > 0
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert "Jacobi-PCG iterations" in cb["sample"]
    # the Poisson work it charges is the GPU arm's measured count for this workload
    rec = json.load(open(os.path.join(ROOT, "profiles", "loop_poisson_iterations.json")))["discharge"]
    assert line["config"]["poisson_inner_per_step"] == rec["inner_per_step"]
